// Mixed-precision eigenpairs: FP32 eigensolve followed by an Ogita-Aishima
// refinement sweep in FP64 with Rayleigh-Ritz on near-degenerate clusters.
//
// For an approximate eigenvector matrix X of the Hermitian H (Ogita & Aishima,
// "Iterative refinement for symmetric eigenvalue decomposition", 2018):
//   R = I - X^H X,  S = X^H H X,
//   lambda_i = Re S_ii / (1 - Re R_ii),
//   F_ij = (S_ij + lambda_j R_ij) / (lambda_j - lambda_i)   for separated pairs,
//   F_ij = R_ij / 2                                        inside a cluster,
//   X <- X (I + F).
// Eigenvalues closer than delta = 1e-3 max|lambda| form a cluster; its block
// is resolved by Rayleigh-Ritz: the projected matrix
//   S~ = S_c + (R_c S_c + S_c R_c) / 2
// is diagonalised (complex Jacobi, FP64) and F_c = (I + R_c/2) W - I.

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "tbgpu_internal.cuh"

namespace tbg {

int zgemm_batched(cudaStream_t st, int N, int64_t batch, bool conj_a, const zc* A, int64_t sA, const zc* B,
                  int64_t sB, zc* C, int64_t sC);
int eig_batched_f32(cudaStream_t st, int N, int64_t batch, zc* H, double* E, cc* U, void* work,
                    size_t work_bytes, int* status_d);

namespace {

constexpr int kMaxCluster = 8;

__global__ void widen_kernel(int64_t n, const cc* __restrict__ a, zc* __restrict__ b) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        b[i] = mk((double)a[i].re, (double)a[i].im);
}

__global__ void add_kernel(int64_t n, zc* __restrict__ x, const zc* __restrict__ t) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        x[i] = x[i] + t[i];
}

// Small complex Hermitian eigenproblem (c <= kMaxCluster) by cyclic Jacobi,
// single thread.  A (c x c, row-major) is destroyed; W gets the eigenvectors
// in columns, w the eigenvalues (ascending).
__device__ void jacobi_small(int c, zc* A, zc* W, double* w) {
    for (int i = 0; i < c; ++i)
        for (int j = 0; j < c; ++j) W[i * c + j] = mk(i == j ? 1.0 : 0.0, 0.0);
    for (int sweep = 0; sweep < 30; ++sweep) {
        double off = 0.0, dia = 0.0;
        for (int i = 0; i < c; ++i)
            for (int j = 0; j < c; ++j) {
                if (i != j)
                    off += abs2(A[i * c + j]);
                else
                    dia += abs2(A[i * c + j]);
            }
        if (off <= 1e-30 * (dia + 1e-300)) break;
        for (int p = 0; p < c - 1; ++p)
            for (int q = p + 1; q < c; ++q) {
                const zc apq = A[p * c + q];
                const double mag = sqrt(abs2(apq));
                if (mag == 0.0) continue;
                const double app = A[p * c + p].re, aqq = A[q * c + q].re;
                // G = diag(1, e^{-i phi}) [[c, -s], [s, c]] with e^{i phi} = apq/|apq| and
                // tan 2 theta = 2|apq| / (app - aqq) zeroes (G^H A G)_{pq}.
                const zc ph = mk(apq.re / mag, apq.im / mag);
                const zc emi = conj(ph);
                const double theta = 0.5 * atan2(2.0 * mag, app - aqq);
                const double cs = cos(theta), sn = sin(theta);
                for (int k = 0; k < c; ++k) {
                    const zc akp = A[k * c + p], akq = emi * A[k * c + q];
                    A[k * c + p] = cs * akp + sn * akq;
                    A[k * c + q] = cs * akq - sn * akp;
                }
                for (int k = 0; k < c; ++k) {
                    const zc apk = A[p * c + k], aqk = ph * A[q * c + k];
                    A[p * c + k] = cs * apk + sn * aqk;
                    A[q * c + k] = cs * aqk - sn * apk;
                }
                for (int k = 0; k < c; ++k) {
                    const zc wkp = W[k * c + p], wkq = emi * W[k * c + q];
                    W[k * c + p] = cs * wkp + sn * wkq;
                    W[k * c + q] = cs * wkq - sn * wkp;
                }
            }
    }
    for (int i = 0; i < c; ++i) w[i] = A[i * c + i].re;
    // sort ascending with vectors
    for (int i = 0; i < c; ++i) {
        int mi = i;
        for (int j = i + 1; j < c; ++j)
            if (w[j] < w[mi]) mi = j;
        if (mi != i) {
            const double t = w[i];
            w[i] = w[mi];
            w[mi] = t;
            for (int k = 0; k < c; ++k) {
                const zc a = W[k * c + i];
                W[k * c + i] = W[k * c + mi];
                W[k * c + mi] = a;
            }
        }
    }
}

// One CTA per matrix: R (in/out: becomes F), S; E out.
__global__ void __launch_bounds__(256) oa_kernel(int N, int64_t batch, zc* __restrict__ R, const zc* __restrict__ S,
                                                 double* __restrict__ E, int64_t* __restrict__ clusters) {
    extern __shared__ double smem[];
    double* lam = smem;                                  // N
    int* cstart = reinterpret_cast<int*>(lam + N);       // N
    __shared__ double red[32];
    __shared__ double s_tnorm;
    const int64_t NN = (int64_t)N * N;
    for (int64_t b = blockIdx.x; b < batch; b += gridDim.x) {
        zc* Rb = R + b * NN;
        const zc* Sb = S + b * NN;
        double mx = 0.0;
        for (int i = threadIdx.x; i < N; i += blockDim.x) {
            const double l = Sb[(int64_t)i * N + i].re / (1.0 - Rb[(int64_t)i * N + i].re);
            lam[i] = l;
            mx = fmax(mx, fabs(l));
        }
        for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
        __syncthreads();
        if (threadIdx.x == 0) {
            double t = 0.0;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t = fmax(t, red[w]);
            s_tnorm = t;
            // clusters: runs of consecutive (sorted) eigenvalues with gaps <= delta
            const double delta = 1e-3 * fmax(t, 1e-300);
            int start = 0;
            int64_t ncl = 0;
            cstart[0] = 0;
            for (int i = 1; i < N; ++i) {
                if (fabs(lam[i] - lam[i - 1]) > delta) {
                    if (i - start > 1) ++ncl;
                    start = i;
                }
                cstart[i] = start;
            }
            if (N - start > 1) ++ncl;
            if (ncl && clusters) atomicAdd(reinterpret_cast<unsigned long long*>(clusters), (unsigned long long)ncl);
        }
        __syncthreads();
        // F for separated pairs / diagonal; cluster blocks get R/2 first
        for (int64_t idx = threadIdx.x; idx < NN; idx += blockDim.x) {
            const int i = (int)(idx / N), j = (int)(idx % N);
            const zc r = Rb[idx];
            zc f;
            if (cstart[i] == cstart[j]) {
                f = mk(0.5 * r.re, 0.5 * r.im);
            } else {
                const zc s = Sb[idx];
                const double den = lam[j] - lam[i];
                f = mk((s.re + lam[j] * r.re) / den, (s.im + lam[j] * r.im) / den);
            }
            Rb[idx] = f;  // each element read then written by the same thread
        }
        __syncthreads();
        // Rayleigh-Ritz on clusters (one thread per cluster)
        for (int i = threadIdx.x; i < N; i += blockDim.x) {
            if (cstart[i] != i) continue;
            int c = 1;
            while (i + c < N && cstart[i + c] == i) ++c;
            if (c < 2 || c > kMaxCluster) continue;
            zc A[kMaxCluster * kMaxCluster], W[kMaxCluster * kMaxCluster];
            double w[kMaxCluster];
            // S~ = S_c + (R_c S_c + S_c R_c)/2, with R_c = 2 F_c (F_c holds R_c/2 now)
            for (int p = 0; p < c; ++p)
                for (int q = 0; q < c; ++q) {
                    zc acc = Sb[(int64_t)(i + p) * N + (i + q)];
                    for (int t = 0; t < c; ++t) {
                        const zc fpt = Rb[(int64_t)(i + p) * N + (i + t)];
                        const zc stq = Sb[(int64_t)(i + t) * N + (i + q)];
                        const zc spt = Sb[(int64_t)(i + p) * N + (i + t)];
                        const zc ftq = Rb[(int64_t)(i + t) * N + (i + q)];
                        acc = acc + fpt * stq + spt * ftq;
                    }
                    A[p * c + q] = acc;
                }
            for (int p = 0; p < c; ++p)  // Hermitise
                for (int q = p; q < c; ++q) {
                    const zc a = A[p * c + q], bq = A[q * c + p];
                    const zc h = mk(0.5 * (a.re + bq.re), 0.5 * (a.im - bq.im));
                    A[p * c + q] = h;
                    A[q * c + p] = conj(h);
                }
            jacobi_small(c, A, W, w);
            // F_c = (I + R_c/2) W - I
            zc Fn[kMaxCluster * kMaxCluster];
            for (int p = 0; p < c; ++p)
                for (int q = 0; q < c; ++q) {
                    zc acc = W[p * c + q];
                    for (int t = 0; t < c; ++t) acc = acc + Rb[(int64_t)(i + p) * N + (i + t)] * W[t * c + q];
                    if (p == q) acc.re -= 1.0;
                    Fn[p * c + q] = acc;
                }
            for (int p = 0; p < c; ++p) {
                for (int q = 0; q < c; ++q) Rb[(int64_t)(i + p) * N + (i + q)] = Fn[p * c + q];
                lam[i + p] = w[p];
            }
            // rows outside the cluster: F_{t,c} <- F_{t,c} W
            for (int t = 0; t < N; ++t) {
                if (t >= i && t < i + c) continue;
                zc row[kMaxCluster];
                for (int q = 0; q < c; ++q) row[q] = Rb[(int64_t)t * N + i + q];
                for (int q = 0; q < c; ++q) {
                    zc acc = mk(0.0, 0.0);
                    for (int u = 0; u < c; ++u) acc = acc + row[u] * W[u * c + q];
                    Rb[(int64_t)t * N + i + q] = acc;
                }
            }
        }
        __syncthreads();
        for (int i = threadIdx.x; i < N; i += blockDim.x) E[b * N + i] = lam[i];
        __syncthreads();
    }
}

// Restore ascending order of E (with the columns of X) after refinement.
__global__ void sort_pairs_kernel(int N, int64_t batch, double* __restrict__ E, zc* __restrict__ X,
                                  zc* __restrict__ tmp) {
    extern __shared__ double sm2[];
    double* e = sm2;
    int* perm = reinterpret_cast<int*>(e + N);
    __shared__ int s_sorted;
    const int64_t NN = (int64_t)N * N;
    for (int64_t b = blockIdx.x; b < batch; b += gridDim.x) {
        if (threadIdx.x == 0) s_sorted = 1;
        __syncthreads();
        for (int i = threadIdx.x; i < N; i += blockDim.x) {
            e[i] = E[b * N + i];
        }
        __syncthreads();
        for (int i = threadIdx.x; i < N - 1; i += blockDim.x)
            if (e[i + 1] < e[i]) s_sorted = 0;
        __syncthreads();
        if (s_sorted) continue;
        for (int i = threadIdx.x; i < N; i += blockDim.x) {
            int rank = 0;
            for (int j = 0; j < N; ++j) rank += (e[j] < e[i]) || (e[j] == e[i] && j < i);
            perm[rank] = i;
        }
        __syncthreads();
        zc* Xb = X + b * NN;
        zc* Tb = tmp + b * NN;
        for (int64_t idx = threadIdx.x; idx < NN; idx += blockDim.x) Tb[idx] = Xb[idx];
        __syncthreads();
        for (int64_t idx = threadIdx.x; idx < NN; idx += blockDim.x) {
            const int r = (int)(idx / N), c = (int)(idx % N);
            Xb[idx] = Tb[(int64_t)r * N + perm[c]];
        }
        for (int i = threadIdx.x; i < N; i += blockDim.x) E[b * N + i] = e[perm[i]];
        __syncthreads();
    }
}

__global__ void eye_minus_kernel(int N, int64_t batch, zc* __restrict__ R) {
    const int64_t NN = (int64_t)N * N;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < batch * NN;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int e = (int)(idx % NN);
        zc r = R[idx];
        r.re = -r.re;
        r.im = -r.im;
        if (e / N == e % N) r.re += 1.0;
        R[idx] = r;
    }
}

inline unsigned blocks(int64_t total) {
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>((total + 255) / 256, 152LL * 64));
}

}  // namespace

size_t mixed_workspace_bytes(int N, int64_t batch) {
    // U32 + R + S + HX (per k) + FP32 eigensolver global workspace
    const size_t NN = (size_t)N * N;
    return (size_t)batch * NN * (sizeof(cc) + 3 * sizeof(zc)) + eig_workspace_bytes(N, batch, 1) + 1024;
}

// H (FP64, preserved), E out (FP64), U out (FP64 eigenvectors in columns).
int mixed_eig_refine(cudaStream_t st, int N, int64_t batch, const zc* H, double* E, zc* U, void* work,
                     size_t work_bytes, int* status_d, int64_t* clusters_d) {
    if (batch <= 0) return TBG_OK;
    const size_t NN = (size_t)N * N;
    if (work_bytes < mixed_workspace_bytes(N, batch)) return set_error(TBG_E_OOM, "mixed workspace too small");
    unsigned char* p = static_cast<unsigned char*>(work);
    cc* U32 = reinterpret_cast<cc*>(p);
    p += batch * NN * sizeof(cc);
    zc* R = reinterpret_cast<zc*>(p);
    p += batch * NN * sizeof(zc);
    zc* S = reinterpret_cast<zc*>(p);
    p += batch * NN * sizeof(zc);
    zc* HX = reinterpret_cast<zc*>(p);
    p += batch * NN * sizeof(zc);
    void* eigw = p;
    const size_t eigw_bytes = eig_workspace_bytes(N, batch, 1);
    int rc = eig_batched_f32(st, N, batch, const_cast<zc*>(H), E, U32, eigw, eigw_bytes, status_d);
    if (rc) return rc;
    widen_kernel<<<blocks(batch * NN), 256, 0, st>>>(batch * NN, U32, U);
    TBG_LAUNCHED("widen_kernel");
    // R = I - X^H X ; S = X^H (H X)
    if ((rc = zgemm_batched(st, N, batch, true, U, NN, U, NN, R, NN))) return rc;
    eye_minus_kernel<<<blocks(batch * NN), 256, 0, st>>>(N, batch, R);
    TBG_LAUNCHED("eye_minus_kernel");
    if ((rc = zgemm_batched(st, N, batch, false, H, NN, U, NN, HX, NN))) return rc;
    if ((rc = zgemm_batched(st, N, batch, true, U, NN, HX, NN, S, NN))) return rc;
    const size_t smem = sizeof(double) * N + sizeof(int) * N;
    {
    KTimer kt(st, "oa_kernel");
    oa_kernel<<<(unsigned)std::min<int64_t>(batch, 152 * 8), 256, smem, st>>>(N, batch, R, S, E, clusters_d);
    TBG_LAUNCHED("oa_kernel");
    }
    // X <- X + X F   (HX reused as the product buffer)
    if ((rc = zgemm_batched(st, N, batch, false, U, NN, R, NN, HX, NN))) return rc;
    add_kernel<<<blocks(batch * NN), 256, 0, st>>>(batch * NN, U, HX);
    TBG_LAUNCHED("add_kernel");
    sort_pairs_kernel<<<(unsigned)std::min<int64_t>(batch, 152 * 8), 256, smem, st>>>(N, batch, E, U, S);
    TBG_LAUNCHED("sort_pairs_kernel");
    return TBG_OK;
}

}  // namespace tbg

// ===========================================================================
// Mixed path on the tensor cores: FP32 eigensolve, Ogita-Aishima refinement
// and the velocity rotation with the exact-slice BF16 GEMM.
// ===========================================================================
namespace tbg {

int ozaki_zgemm(cudaStream_t st, bool high, bool conj_a, int fmt_a, int fmt_b, int64_t batch, int M, int Nc, int K,
                const void* A, int64_t lda, int64_t sA, const void* B, int64_t ldb, int64_t sB, float4* C, int64_t ldc,
                int64_t sC, int* EA, int* EB);
int ozaki_zgemm_tc(cudaStream_t st, bool conj_a, int fmt_a, int fmt_b, int64_t batch, int M, int Nc, int K,
                   const void* A, int64_t lda, int64_t sA, const void* B, int64_t ldb, int64_t sB, float4* C,
                   int64_t ldc, int64_t sC, int* EA, int* EB, int* err);
bool ozaki_use_tc();
size_t ozaki_exp_bytes(int64_t batch, int M, int Nc);

namespace {

enum { F64 = 0, F32 = 1, PAIR = 2 };

// pair -> FP64 complex, optionally as I - X (for R = I - X^H X)
__global__ void pairs_to_z_kernel(int N, int64_t batch, const float4* __restrict__ in, zc* __restrict__ out,
                                  int eye_minus) {
    const int64_t NN = (int64_t)N * N;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < batch * NN;
         i += (int64_t)gridDim.x * blockDim.x) {
        const float4 v = in[i];
        double re = (double)v.x + (double)v.y, im = (double)v.z + (double)v.w;
        if (eye_minus) {
            const int e = (int)(i % NN);
            re = ((e / N == e % N) ? 1.0 : 0.0) - re;
            im = -im;
        }
        out[i] = mk(re, im);
    }
}

// X' = X + X F as a float pair: hi = X (exact FP32 eigenvectors), lo = X F.
__global__ void xprime_kernel(int64_t n, const cc* __restrict__ X, const float4* __restrict__ XF,
                              float4* __restrict__ Xp) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const cc x = X[i];
        const float4 f = XF[i];
        Xp[i] = make_float4(x.re, f.x + f.y, x.im, f.z + f.w);
    }
}

// Omega_n = sum_{m != n} -2 Im(Bx[n,m] By[m,n]) / ((E_n - E_m)^2 + eta^2) from
// float-pair band-basis velocities; one warp per row n.
__global__ void berry_pairs_kernel(int N, int64_t batch, const float4* __restrict__ Bx, const float4* __restrict__ By,
                                   const double* __restrict__ E, double eta2, double* __restrict__ Omega) {
    const int lane = threadIdx.x & 31;
    const int64_t NN = (int64_t)N * N;
    const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t w = gw; w < batch * N; w += nw) {
        const int64_t b = w / N;
        const int n = (int)(w % N);
        const float4* bx = Bx + b * NN + (int64_t)n * N;
        const float4* by = By + b * NN;
        const double* Eb = E + b * N;
        const double en = Eb[n];
        double s = 0.0;
        for (int m = lane; m < N; m += 32) {
            if (m == n) continue;
            const float4 x = bx[m];
            const float4 y = by[(int64_t)m * N + n];
            const double xr = (double)x.x + (double)x.y, xi = (double)x.z + (double)x.w;
            const double yr = (double)y.x + (double)y.y, yi = (double)y.z + (double)y.w;
            const double im = xr * yi + xi * yr;
            const double de = en - Eb[m];
            s += -2.0 * im / (de * de + eta2);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) Omega[b * N + n] = s;
    }
}

// Keep E ascending (with Omega) after refinement; a no-op when already sorted.
__global__ void sort_e_om_kernel(int N, int64_t batch, double* __restrict__ E, double* __restrict__ Om) {
    extern __shared__ double sm3[];
    double* e = sm3;
    double* o = sm3 + N;
    __shared__ int s_sorted;
    for (int64_t b = blockIdx.x; b < batch; b += gridDim.x) {
        if (threadIdx.x == 0) s_sorted = 1;
        __syncthreads();
        for (int i = threadIdx.x; i < N; i += blockDim.x) {
            e[i] = E[b * N + i];
            o[i] = Om[b * N + i];
        }
        __syncthreads();
        for (int i = threadIdx.x; i < N - 1; i += blockDim.x)
            if (e[i + 1] < e[i]) s_sorted = 0;
        __syncthreads();
        if (!s_sorted) {
            for (int i = threadIdx.x; i < N; i += blockDim.x) {
                int rank = 0;
                for (int j = 0; j < N; ++j) rank += (e[j] < e[i]) || (e[j] == e[i] && j < i);
                E[b * N + rank] = e[i];
                Om[b * N + rank] = o[i];
            }
        }
        __syncthreads();
    }
}

inline unsigned nblk(int64_t total) {
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>((total + 255) / 256, 152LL * 64));
}

}  // namespace

size_t mixed_berry_workspace_bytes(int N, int64_t batch) {
    const size_t NN = (size_t)N * N;
    // X (cc) + 5 pair buffers + R, S (zc) + exponents + FP32 solver workspace
    return (size_t)batch * NN * (sizeof(cc) + 5 * sizeof(float4) + 2 * sizeof(zc)) +
           ozaki_exp_bytes(batch, N, N) + eig_workspace_bytes(N, batch, 1) + 4096;
}

// H (FP64, preserved), Vx/Vy (FP64, stride ldV) -> E (refined, ascending), Omega.
int mixed_berry(cudaStream_t st, int N, int64_t batch, const zc* H, const zc* Vx, const zc* Vy, int64_t ldV,
                double eta, double* E, double* Om, void* work, size_t work_bytes, int* status_d,
                int64_t* clusters_d) {
    if (batch <= 0) return TBG_OK;
    const int64_t NN = (int64_t)N * N;
    if (work_bytes < mixed_berry_workspace_bytes(N, batch)) return set_error(TBG_E_OOM, "mixed workspace too small");
    unsigned char* p = static_cast<unsigned char*>(work);
    auto take = [&](size_t bytes) {
        void* q = p;
        p += (bytes + 255) & ~size_t(255);
        return q;
    };
    cc* X = static_cast<cc*>(take(sizeof(cc) * batch * NN));
    float4* bA = static_cast<float4*>(take(sizeof(float4) * batch * NN));
    float4* bB = static_cast<float4*>(take(sizeof(float4) * batch * NN));
    float4* bC = static_cast<float4*>(take(sizeof(float4) * batch * NN));
    float4* bD = static_cast<float4*>(take(sizeof(float4) * batch * NN));
    float4* bE = static_cast<float4*>(take(sizeof(float4) * batch * NN));
    zc* Rz = static_cast<zc*>(take(sizeof(zc) * batch * NN));
    zc* Sz = static_cast<zc*>(take(sizeof(zc) * batch * NN));
    int* EA = static_cast<int*>(take(ozaki_exp_bytes(batch, N, N)));
    int* EB = EA + batch * N;
    const size_t eigw_bytes = eig_workspace_bytes(N, batch, 1);
    void* eigw = take(eigw_bytes);
    // FP64-class products: tcgen05 form unless the mma.sync form is selected
    auto hp = [&](bool conj_a, int fa, int fb, const void* A, int64_t sA, const void* B, int64_t sB,
                  float4* C) -> int {
        if (ozaki_use_tc())
            return ozaki_zgemm_tc(st, conj_a, fa, fb, batch, N, N, N, A, N, sA, B, N, sB, C, N, NN, EA, EB, status_d);
        return ozaki_zgemm(st, true, conj_a, fa, fb, batch, N, N, N, A, N, sA, B, N, sB, C, N, NN, EA, EB);
    };
    int rc;
    // 1. FP32 eigenpairs
    if ((rc = eig_batched_f32(st, N, batch, const_cast<zc*>(H), E, X, eigw, eigw_bytes, status_d))) return rc;
    // 2. R = I - X^H X, S = X^H (H X)   (FP64-class, tensor cores)
    if ((rc = hp(true, F32, F32, X, NN, X, NN, bA))) return rc;
    if ((rc = hp(false, F64, F32, H, NN, X, NN, bB))) return rc;
    if ((rc = hp(true, F32, PAIR, X, NN, bB, NN, bC))) return rc;
    {
        KTimer kt(st, "pairs_to_z_kernel");
        pairs_to_z_kernel<<<nblk(batch * NN), 256, 0, st>>>(N, batch, bA, Rz, 1);
        pairs_to_z_kernel<<<nblk(batch * NN), 256, 0, st>>>(N, batch, bC, Sz, 0);
        count_launch(2);
    }
    // 3. Ogita-Aishima update F (into Rz) and refined eigenvalues
    {
        KTimer kt(st, "oa_kernel");
        const size_t smem = sizeof(double) * N + sizeof(int) * N;
        oa_kernel<<<(unsigned)std::min<int64_t>(batch, 152 * 8), 256, smem, st>>>(N, batch, Rz, Sz, E, clusters_d);
        TBG_LAUNCHED("oa_kernel");
    }
    // 4. X' = X + X F  (float pair: hi = X, lo = X F)
    if ((rc = ozaki_zgemm(st, false, false, F32, F64, batch, N, N, N, X, N, NN, Rz, N, NN, bE, N, NN, EA, EB)))
        return rc;
    {
        KTimer kt(st, "xprime_kernel");
        xprime_kernel<<<nblk(batch * NN), 256, 0, st>>>(batch * NN, X, bE, bA);
        TBG_LAUNCHED("xprime_kernel");
    }
    // 5. band-basis velocities B = X'^H V X'
    if ((rc = hp(false, F64, PAIR, Vx, ldV, bA, NN, bB))) return rc;
    if ((rc = hp(false, F64, PAIR, Vy, ldV, bA, NN, bC))) return rc;
    if ((rc = hp(true, PAIR, PAIR, bA, NN, bB, NN, bD))) return rc;
    if ((rc = hp(true, PAIR, PAIR, bA, NN, bC, NN, bE))) return rc;
    // 6. Omega
    {
        KTimer kt(st, "berry_kernel");
        berry_pairs_kernel<<<nblk(batch * N * 32), 256, 0, st>>>(N, batch, bD, bE, E, eta * eta, Om);
        TBG_LAUNCHED("berry_pairs_kernel");
    }
    sort_e_om_kernel<<<(unsigned)std::min<int64_t>(batch, 152 * 8), 256, 2 * sizeof(double) * N, st>>>(N, batch, E,
                                                                                                      Om);
    TBG_LAUNCHED("sort_e_om_kernel");
    return TBG_OK;
}

}  // namespace tbg
