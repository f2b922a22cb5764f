// Mixed path: FP32 eigensolve, one Ogita-Aishima refinement sweep and the
// velocity rotation, with every FP64-class product on the tensor cores
// (exact-slice BF16 GEMM, float-pair results).
//
// For an approximate eigenvector matrix X of the Hermitian H (Ogita & Aishima,
// "Iterative refinement for symmetric eigenvalue decomposition", 2018):
//   R = I - X^H X,  S = X^H H X,
//   lambda_i = Re S_ii / (1 - Re R_ii) = Re S_ii / Re (X^H X)_ii,
//   F_ij = (S_ij + lambda_j R_ij) / (lambda_j - lambda_i)   for separated pairs,
//   F_ij = R_ij / 2                                        inside a cluster,
//   X <- X (I + F).
// Eigenvalues closer than delta = 1e-3 max|lambda| form a cluster; its block
// is resolved by Rayleigh-Ritz: the projected matrix
//   S~ = S_c + (R_c S_c + S_c R_c) / 2
// is diagonalised (complex Jacobi, FP64) and F_c = (I + R_c/2) W - I.
//
// Precision split: lambda (the refined eigenvalues) in FP64 from the float
// pairs; the separated-pair entries of F are a first-order correction of the
// size of the FP32 eigenvector error and are formed in FP32 from the pair sums
// (their own relative accuracy only needs to be ~1e-7); cluster blocks in
// FP64.  Omega is summed in float-pair arithmetic: the FP64 pipe of the part
// is a small fraction of its FP32 rate, and the band-basis velocities carry
// about 2^-43 relative accuracy, which float pairs (~2^-48) preserve.

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include <cstdlib>

#include "tbgpu_internal.cuh"

namespace tbg {

int ozaki_zgemm(cudaStream_t st, bool high, bool conj_a, int fmt_a, int fmt_b, int64_t batch, int M, int Nc, int K,
                const void* A, int64_t lda, int64_t sA, const void* B, int64_t ldb, int64_t sB, float4* C, int64_t ldc,
                int64_t sC, int* EA, int* EB);
int ozaki_zgemm_tc_low(cudaStream_t st, int64_t batch, int M, int Nc, int K, const void* A, int64_t lda, int64_t sA,
                       const void* B, int64_t ldb, int64_t sB, float4* C, int64_t ldc, int64_t sC, int* EA, int* EB,
                       int* err, bool exps_ready = false);
size_t ozaki_exp_bytes(int64_t batch, int M, int Nc);
int ozaki_line_exps(cudaStream_t st, int fmt, bool cols, int64_t batch, int lines, int K, const void* X, int64_t ld,
                    int64_t sX, int* E);

namespace {

constexpr int kMaxCluster = 8;
enum { F64 = 0, F32 = 1, PAIR = 2 };

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

__device__ __forceinline__ zc pair_z(float4 v) { return mk((double)v.x + (double)v.y, (double)v.z + (double)v.w); }
__device__ __forceinline__ zc widen(cc v) { return mk((double)v.re, (double)v.im); }

// Offset (in doubles, even: 16-byte aligned) of the warps' cluster rotations in
// oa_pairs_kernel's shared memory, after lam (N doubles) and four 4-byte arrays.
__host__ __device__ constexpr size_t oa_wslot_off(int N) { return (3 * (size_t)N + 1) & ~(size_t)1; }

// One CTA per matrix.  XX = X^H X and S = X^H H X as float pairs -> refined
// eigenvalues E (FP64) and the update F (FP32 complex).  E is the Rayleigh
// quotient plus its second-order term: with F_tj the first-order coefficient
// of X_t in eigenvector j, lambda_j += sum_t |F_tj|^2 (lambda_j - lambda_t)
// over the separated t (for a cluster member, the same sum over the rotated
// numerators).  The quotient alone is off by |r|^2 / gap for an FP32 residual
// r, 1e-9 of ||H|| for pairs just outside the cluster threshold; the second-
// order term leaves a third-order error.  The Rayleigh-Ritz
// rotations of clusters (entries of order one) are not left in F: a product
// X F whose operand columns hold them would be sliced on those columns'
// exponents and lose the small first-order entries beside them.  They go to
// Fcl in FP64 instead (row i + p, column q of the N x kMaxCluster block of the
// matrix for member p of the cluster starting at i), with cinfo[j] =
// (start << 4) | size for every member column j and -1 elsewhere, and their
// block of F is zero.
__global__ void __launch_bounds__(256, 5) oa_pairs_kernel(int N, int64_t batch, const float4* __restrict__ XX,
                                                       const float4* __restrict__ S, double* __restrict__ E,
                                                       cc* __restrict__ F, int64_t* __restrict__ clusters,
                                                       int* __restrict__ cinfo, zc* __restrict__ Fcl,
                                                       int* __restrict__ Fexp, unsigned long long* __restrict__ clist) {
    extern __shared__ double smem[];
    double* lam = smem;                                   // N
    float* lamf = reinterpret_cast<float*>(lam + N);      // N
    int* cstart = reinterpret_cast<int*>(lamf + N);       // N
    float* corr = reinterpret_cast<float*>(cstart + N);   // N: second-order eigenvalue terms
    float* cmax = corr + N;                               // N: largest |F| entry of each column
    // per warp: the rotation W and Ritz values of the cluster it is working on
    zc* wslot = reinterpret_cast<zc*>(smem + oa_wslot_off(N));
    double* wval = reinterpret_cast<double*>(wslot + (blockDim.x >> 5) * kMaxCluster * kMaxCluster);
    __shared__ double red[32];
    const int NN = N * N;
    for (int64_t b = blockIdx.x; b < batch; b += gridDim.x) {
        const float4* XXb = XX + b * NN;
        const float4* Sb = S + b * NN;
        cc* Fb = F + b * NN;
        double mx = 0.0;
        for (int i = threadIdx.x; i < N; i += blockDim.x) {
            const double l = pair_z(Sb[i * N + i]).re / pair_z(XXb[i * N + i]).re;
            lam[i] = l;
            lamf[i] = (float)l;
            mx = fmax(mx, fabs(l));
        }
        for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
        __syncthreads();
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t = fmax(t, red[w]);
        // clusters: runs of consecutive (sorted) eigenvalues with gaps <= delta.
        // cstart[i] = the last run start at or before i: a block max-scan of
        // (i if a run starts at i), over chunks of blockDim.x indices.
        const double delta = 1e-3 * fmax(t, 1e-300);
        __shared__ int wscan[32];
        __shared__ int carry;
        if (threadIdx.x == 0) carry = 0;
        int ncl = 0;
        for (int i0 = 0; i0 < N; i0 += blockDim.x) {
            const int i = i0 + threadIdx.x;
            const bool start = i < N && (i == 0 || fabs(lam[i] - lam[i - 1]) > delta);
            const bool next_start = i + 1 >= N || fabs(lam[i + 1] - lam[i]) > delta;
            int v = start ? i : 0;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int u = __shfl_up_sync(0xffffffffu, v, o);
                if ((threadIdx.x & 31) >= o) v = max(v, u);
            }
            __syncthreads();
            if ((threadIdx.x & 31) == 31) wscan[threadIdx.x >> 5] = v;
            __syncthreads();
            for (int w = 0; w < (int)(threadIdx.x >> 5); ++w) v = max(v, wscan[w]);
            v = max(v, carry);
            if (i < N) cstart[i] = v;
            // a run of length > 1 starts at i
            ncl += __syncthreads_count(start && i < N && !next_start);
            if (threadIdx.x == blockDim.x - 1) carry = v;
        }
        if (threadIdx.x == 0 && ncl && clusters)
            atomicAdd(reinterpret_cast<unsigned long long*>(clusters), (unsigned long long)ncl);
        __syncthreads();
        // F for separated pairs (FP32); R/2 inside clusters and on the diagonal.
        // Thread (p, j) walks column j over the rows i = p (mod P) and sums the
        // second-order terms of lambda_j in a fixed order (the result must not
        // depend on scheduling: a matrix gives the same bits alone or in a batch).
        const int P = max(1, (int)blockDim.x / N);
        __shared__ float part[256], partm[256];
        for (int cj = threadIdx.x; cj < P * N; cj += blockDim.x) {
            const int p = cj / N, j = cj - p * N;
            const float lj = lamf[j];
            float acc = 0.f, mx = 0.f;
            for (int i = p; i < N; i += P) {
                const int idx = i * N + j;
                const float4 x4 = XXb[idx];
                float fr, fi;
                if (cstart[i] == cstart[j]) {
                    fr = (i == j) ? 0.5f * ((1.f - x4.x) - x4.y) : -0.5f * (x4.x + x4.y);
                    fi = -0.5f * (x4.z + x4.w);
                } else {
                    const float4 s4 = Sb[idx];
                    // |den| > 1e-3 max|lambda|: the fast reciprocal is accurate to a few ulp
                    const float den = (float)(lam[j] - lam[i]);
                    const float rden = __frcp_rn(den);
                    fr = ((s4.x + s4.y) - lj * (x4.x + x4.y)) * rden;
                    fi = ((s4.z + s4.w) - lj * (x4.z + x4.w)) * rden;
                    acc = fmaf(fr * fr + fi * fi, den, acc);
                }
                Fb[idx] = mk(fr, fi);
                mx = fmaxf(mx, f32_mag(fr, fi));
            }
            if (P == 1) {
                corr[j] = acc;
                cmax[j] = mx;
            } else {
                part[cj] = acc;
                partm[cj] = mx;
            }
        }
        if (P > 1) {
            __syncthreads();
            for (int j = threadIdx.x; j < N; j += blockDim.x) {
                float acc = 0.f, mx = 0.f;
                for (int p = 0; p < P; ++p) {
                    acc += part[p * N + j];
                    mx = fmaxf(mx, partm[p * N + j]);
                }
                corr[j] = acc;
                cmax[j] = mx;
            }
        }
        for (int i = threadIdx.x; i < N; i += blockDim.x) cinfo[b * N + i] = -1;
        __syncthreads();
        // Rayleigh-Ritz on clusters, one warp per cluster (dealt to the warps in
        // index order).  Lane 0 diagonalises the projected block (FP64); the lanes
        // then rotate the rows outside the cluster and sum the second-order terms
        // of the Ritz values (a fixed-order warp reduction).
        {
            const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
            zc* Ws = wslot + warp * kMaxCluster * kMaxCluster;
            double* ws = wval + warp * kMaxCluster;
            int k = 0;  // clusters seen so far (the same in every lane)
            for (int base = 0; base < N; base += 32) {
                const int il = base + lane;
                int cl = 0;
                if (il < N && cstart[il] == il) {
                    cl = 1;
                    while (il + cl < N && cstart[il + cl] == il) ++cl;
                }
                unsigned todo = __ballot_sync(0xffffffffu, cl >= 2 && cl <= kMaxCluster);
                while (todo) {
                    const int src = __ffs(todo) - 1;
                    todo &= todo - 1;
                    const int c = __shfl_sync(0xffffffffu, cl, src);
                    if ((k++ % nw) != warp) continue;
                    const int i = base + src;
                    if (lane == 0) {
                        zc A[kMaxCluster * kMaxCluster], W[kMaxCluster * kMaxCluster];
                        double w[kMaxCluster];
                        // S~ = S_c + (R_c S_c + S_c R_c)/2, with R_c = 2 F_c (F_c holds R_c/2 now)
                        for (int p = 0; p < c; ++p)
                            for (int q = 0; q < c; ++q) {
                                zc acc = pair_z(Sb[(i + p) * N + (i + q)]);
                                for (int t = 0; t < c; ++t) {
                                    const zc fpt = widen(Fb[(i + p) * N + (i + t)]);
                                    const zc stq = pair_z(Sb[(i + t) * N + (i + q)]);
                                    const zc spt = pair_z(Sb[(i + p) * N + (i + t)]);
                                    const zc ftq = widen(Fb[(i + t) * N + (i + q)]);
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
                                for (int t = 0; t < c; ++t) acc = acc + widen(Fb[(i + p) * N + (i + t)]) * W[t * c + q];
                                if (p == q) acc.re -= 1.0;
                                Fn[p * c + q] = acc;
                            }
                        for (int p = 0; p < c; ++p) {
                            for (int q = 0; q < c; ++q) {
                                Fb[(i + p) * N + (i + q)] = mk(0.f, 0.f);
                                Fcl[(b * N + i + p) * kMaxCluster + q] = Fn[p * c + q];
                                Ws[p * c + q] = W[p * c + q];
                            }
                            cinfo[b * N + i + p] = (i << 4) | c;
                            ws[p] = w[p];
                            lam[i + p] = w[p];
                        }
                        // the cluster's columns of X' are formed from this list
                        const unsigned long long at = atomicAdd(&clist[0], 1ull);
                        clist[1 + at] = ((unsigned long long)b << 20) | ((unsigned long long)i << 4) | (unsigned)c;
                    }
                    __syncwarp();
                    // rows outside the cluster: F_{t,c} <- F_{t,c} W, and the second-order
                    // terms from the rotated numerators n_tp = sum_q F_tq (lambda_q - lambda_t) W_qp
                    // (lamf is never rewritten)
                    double d2[kMaxCluster];
                    float mq[kMaxCluster];  // the rotated columns' largest entries (the block is zero)
                    for (int p = 0; p < c; ++p) {
                        d2[p] = 0.0;
                        mq[p] = 0.f;
                    }
                    for (int t = lane; t < N; t += 32) {
                        if (t >= i && t < i + c) continue;
                        zc row[kMaxCluster], nrow[kMaxCluster];
                        for (int q = 0; q < c; ++q) {
                            row[q] = widen(Fb[t * N + i + q]);
                            const double g = (double)lamf[i + q] - (double)lamf[t];
                            nrow[q] = mk(row[q].re * g, row[q].im * g);
                        }
                        for (int q = 0; q < c; ++q) {
                            zc acc = mk(0.0, 0.0), nacc = mk(0.0, 0.0);
                            for (int u = 0; u < c; ++u) {
                                acc = acc + row[u] * Ws[u * c + q];
                                nacc = nacc + nrow[u] * Ws[u * c + q];
                            }
                            const float fre = (float)acc.re, fim = (float)acc.im;
                            Fb[t * N + i + q] = mk(fre, fim);
                            mq[q] = fmaxf(mq[q], f32_mag(fre, fim));
                            d2[q] += (nacc.re * nacc.re + nacc.im * nacc.im) / (ws[q] - (double)lamf[t]);
                        }
                    }
                    for (int q = 0; q < c; ++q) {
                        double v = d2[q];
                        float mv = mq[q];
                        for (int o = 16; o > 0; o >>= 1) {
                            v += __shfl_xor_sync(0xffffffffu, v, o);
                            mv = fmaxf(mv, __shfl_xor_sync(0xffffffffu, mv, o));
                        }
                        if (lane == 0) {
                            corr[i + q] = (float)v;
                            cmax[i + q] = mv;
                        }
                    }
                    __syncwarp();
                }
            }
        }
        __syncthreads();
        for (int i = threadIdx.x; i < N; i += blockDim.x) {
            E[b * N + i] = lam[i] + (double)corr[i];
            if (Fexp) Fexp[b * N + i] = line_exp_of(cmax[i]);
        }
        __syncthreads();
    }
}

// Dynamic shared memory of oa_pairs_kernel (256 threads): lam (double),
// lamf, cstart, corr, cmax (4-byte, padded to 8) and each warp's cluster rotation.
size_t oa_smem_bytes(int N) {
    return sizeof(double) * oa_wslot_off(N) + 8 * (sizeof(zc) * kMaxCluster * kMaxCluster + sizeof(double) * kMaxCluster);
}

// X' = X + X F + X_c F_c as a float pair: hi = X (exact FP32 eigenvectors),
// lo = X F (the product of the first-order part of the update).  A column j
// of a cluster also gets the cluster's rotation, sum_p X[r, s + p] Fcl[s + p,
// j - s] in FP64 (cinfo as oa_pairs_kernel writes it), and the pair is formed
// from the FP64 sum.
// One thread per column walks its rows (a warp reads 32 consecutive entries
// of a row), so with xpc the column exponents of X' (the conjugated operand of
// the rotation) come out of the same pass.  Columns of clusters are left to
// xprime_cluster_kernel.
__global__ void __launch_bounds__(128, 16) xprime_kernel(int64_t batch, int N, const cc* __restrict__ X,
                                                         const float4* __restrict__ XF, const int* __restrict__ cinfo,
                                                         float4* __restrict__ Xp, int* __restrict__ xpc) {
    const int nch = (N + 127) / 128;
    const int64_t NN = (int64_t)N * N;
    for (int64_t w = blockIdx.x; w < batch * nch; w += gridDim.x) {
        const int64_t b = w / nch;
        const int j = (int)(w % nch) * 128 + threadIdx.x;
        if (j >= N || cinfo[b * N + j] >= 0) continue;
        const cc* Xb = X + b * NN + j;
        const float4* XFb = XF + b * NN + j;
        float4* Xpb = Xp + b * NN + j;
        float m = 0.f;
#pragma unroll 4
        for (int r = 0; r < N; ++r) {
            const int64_t i = (int64_t)r * N;
            const cc x = Xb[i];
            const float4 f = XFb[i];
            const float4 o = make_float4(x.re, f.x + f.y, x.im, f.z + f.w);
            Xpb[i] = o;
            m = fmaxf(m, pair_mag(o));
        }
        if (xpc) xpc[b * N + j] = line_exp_of(m);
    }
}

// The columns of clusters: X' in FP64 with the cluster's rotation
// sum_p X[r, st + p] Fcl[st + p, j - st], then the pair.  One block per entry
// of clist (count, then (b << 20 | st << 4 | c) per cluster, as
// oa_pairs_kernel appends them), threads over the rows; the column maxima
// are combined in integer order of their bits (the magnitudes are >= 0).
__global__ void __launch_bounds__(128) xprime_cluster_kernel(int N, const cc* __restrict__ X,
                                                             const float4* __restrict__ XF, const zc* __restrict__ Fcl,
                                                             float4* __restrict__ Xp, int* __restrict__ xpc,
                                                             const unsigned long long* __restrict__ clist) {
    __shared__ int wm[4];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned long long n = clist[0];
    const int64_t NN = (int64_t)N * N;
    for (unsigned long long e = blockIdx.x; e < n; e += gridDim.x) {
        const unsigned long long v = clist[1 + e];
        const int64_t b = (int64_t)(v >> 20);
        const int st = (int)((v >> 4) & 0xFFFF), c = (int)(v & 15);
        const cc* Xb = X + b * NN;
        const float4* XFb = XF + b * NN;
        float4* Xpb = Xp + b * NN;
        for (int q = 0; q < c; ++q) {
            const int j = st + q;
            const zc* fc = Fcl + (b * N + st) * kMaxCluster + q;
            float m = 0.f;
            for (int r = threadIdx.x; r < N; r += blockDim.x) {
                const int64_t i = (int64_t)r * N + j;
                const cc x = Xb[i];
                const float4 f = XFb[i];
                const cc* xr = Xb + (int64_t)r * N;  // row r
                double re = ((double)f.x + (double)f.y), im = ((double)f.z + (double)f.w);
                for (int p = 0; p < c; ++p) {
                    const cc a = xr[st + p];
                    const zc wv = fc[p * kMaxCluster];
                    re += (double)a.re * wv.re - (double)a.im * wv.im;
                    im += (double)a.re * wv.im + (double)a.im * wv.re;
                }
                re += (double)x.re;
                im += (double)x.im;
                const float rh = (float)re, ih = (float)im;
                const float4 o = make_float4(rh, (float)(re - (double)rh), ih, (float)(im - (double)ih));
                Xpb[i] = o;
                m = fmaxf(m, pair_mag(o));
            }
            const int wv = __reduce_max_sync(0xffffffffu, __float_as_int(m));
            if (lane == 0) wm[warp] = wv;
            __syncthreads();
            if (threadIdx.x == 0 && xpc) {
                int mx = 0;
                for (int w = 0; w < (int)(blockDim.x >> 5); ++w) mx = max(mx, wm[w]);
                xpc[b * N + j] = line_exp_of(__int_as_float(mx));
            }
            __syncthreads();
        }
    }
}

// Eigenpairs out of the refinement: E ascending (rank by value, ties by index)
// and the columns of X' = hi + lo (FP64) in the same order.  One block per matrix.
__global__ void eigpairs_sorted_kernel(int N, int64_t batch, const float4* __restrict__ Xp, const double* Ein,
                                       double* Eout, zc* __restrict__ U) {  // Ein may be Eout
    extern __shared__ double es[];  // N values, N ranks (as double)
    double* ev = es;
    int* rk = reinterpret_cast<int*>(es + N);
    const int64_t NN = (int64_t)N * N;
    for (int64_t b = blockIdx.x; b < batch; b += gridDim.x) {
        __syncthreads();
        for (int i = threadIdx.x; i < N; i += blockDim.x) ev[i] = Ein[b * N + i];
        __syncthreads();
        for (int i = threadIdx.x; i < N; i += blockDim.x) {
            int r = 0;
            for (int j = 0; j < N; ++j) r += (ev[j] < ev[i]) || (ev[j] == ev[i] && j < i);
            rk[i] = r;
            Eout[b * N + r] = ev[i];
        }
        __syncthreads();
        for (int64_t e = threadIdx.x; e < NN; e += blockDim.x) {
            const int row = (int)(e / N), col = (int)(e % N);
            const float4 x = Xp[b * NN + e];
            U[b * NN + (int64_t)row * N + rk[col]] = mk((double)x.x + (double)x.y, (double)x.z + (double)x.w);
        }
    }
}

__device__ __forceinline__ float2 df_warp_sum(float2 s) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        s = df_add(s, make_float2(__shfl_xor_sync(0xffffffffu, s.x, o), __shfl_xor_sync(0xffffffffu, s.y, o)));
    return s;
}

// Omega_n = sum_{m != n} -2 Im(Bx[n,m] By[m,n]) / ((E_n - E_m)^2 + eta^2)
// (traits.rs:181-195) from float-pair band-basis velocities, in float-pair
// arithmetic.  By is Hermitian, so By[m,n] = conj(By[n,m]) and both operands
// are read along row n.  One warp per row n; E of the matrix as pairs in
// shared memory.
template <bool MET>
__global__ void __launch_bounds__(256) berry_df_kernel(int N, int64_t batch, const float4* __restrict__ Bx,
                                                       const float4* __restrict__ By, const double* __restrict__ E,
                                                       float2 eta2, double* __restrict__ Omega,
                                                       double* __restrict__ Met) {
    extern __shared__ float2 e2s[];  // N
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int NN = N * N;
    for (int64_t b = blockIdx.x; b < batch; b += gridDim.x) {
        __syncthreads();
        for (int i = threadIdx.x; i < N; i += blockDim.x) e2s[i] = df_of(E[b * N + i]);
        __syncthreads();
        for (int n = warp; n < N; n += nw) {
            const float4* bx = Bx + b * NN + n * N;
            const float4* by = By + b * NN + n * N;
            const float2 en = e2s[n];
            float2 s = make_float2(0.f, 0.f), g = make_float2(0.f, 0.f);
            for (int m = lane; m < N; m += 32) {
                if (m == n) continue;
                const float4 x = bx[m];
                const float4 y = by[m];
                // Im(x conj(y)) = x_im y_re - x_re y_im
                const float2 t1 = df_mul(make_float2(x.z, x.w), make_float2(y.x, y.y));
                const float2 t2 = df_mul(make_float2(x.x, x.y), make_float2(y.z, y.w));
                const float2 num = df_add(t1, df_neg(t2));
                const float2 de = df_add(en, df_neg(e2s[m]));
                const float2 den = df_add(df_mul(de, de), eta2);
                const float2 q = df_div(num, den);
                s = df_add(s, make_float2(-2.f * q.x, -2.f * q.y));
                if (MET) {
                    // Re(x conj(y)) = x_re y_re + x_im y_im
                    const float2 r = df_add(df_mul(make_float2(x.x, x.y), make_float2(y.x, y.y)),
                                            df_mul(make_float2(x.z, x.w), make_float2(y.z, y.w)));
                    g = df_add(g, df_div(r, den));
                }
            }
            s = df_warp_sum(s);
            if (MET) g = df_warp_sum(g);
            if (lane == 0) {
                Omega[b * N + n] = df_to_double(s);
                if (MET) Met[b * N + n] = df_to_double(g);
            }
        }
    }
}

// The Berry stage of the hall path in one pass (src/response/traits.rs:181-195
// and src/response/linear/mod.rs:204-223).  With Bx, By Hermitian the term of
// the pair (n, m),
//   T_nm = -2 Im(Bx[n,m] By[m,n]) / ((E_n - E_m)^2 + eta^2) = -2 Im(Bx[n,m] conj(By[n,m])) / (...),
// enters Omega_n as +T_nm and Omega_m as -T_nm, so only the upper triangles
// are read: Omega_n = R_n - C_n with the row sums R_n = sum_{m>n} T_nm and
// the column sums C_m = sum_{n<m} T_nm.  Per k-point, warps take rows n and
// N-1-n together (equal work), lanes the columns m = n+1+lane, n+33+lane, ...
// (consecutive addresses); T in float-pair arithmetic as berry_df_kernel;
// R_n by a warp butterfly, C_m in the lane's registers over the warp's rows and
// then summed over the warps in a fixed order.  Then S_k(mu_j) = sum_n Omega_n
// f(E_n, mu_j) (lanes over n, a fixed butterfly) is Kahan-added into this
// CTA's running sum for mu_j, and the CTA's compensated partials go to part at
// the end.  No per-band Omega is stored and E need not be sorted.  HBM traffic
// per k-point: the upper triangles of the two float-pair band-basis velocity
// matrices (2 x 16 N(N-1)/2 bytes) and E (8 N bytes).  N <= kOccMaxN.
constexpr int kOccMaxN = 256;
constexpr int kOccSlots = kOccMaxN / 32;
__global__ void __launch_bounds__(256) berry_occ_df_kernel(int N, int64_t batch, const float4* __restrict__ Bx,
                                                           const float4* __restrict__ By, const double* __restrict__ E,
                                                           float2 eta2, int nmu, const double* __restrict__ mu,
                                                           double width, double* __restrict__ part) {
    extern __shared__ double occ_sm[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    double* ed = occ_sm;                                 // N
    double* om = ed + N;                                 // N: R_n, then Omega_n
    double* colp = om + N;                               // nw x N column sums
    double* rs = colp + (size_t)nw * N;                  // nmu running sums
    double* rc = rs + nmu;                               // nmu compensations
    float2* e2s = reinterpret_cast<float2*>(rc + nmu);   // N
    const int64_t NN = (int64_t)N * N;
    for (int j = threadIdx.x; j < nmu; j += blockDim.x) {
        rs[j] = 0.0;
        rc[j] = 0.0;
    }
    const int npair = (N + 1) >> 1;  // rows n and N-1-n
    for (int64_t b = blockIdx.x; b < batch; b += gridDim.x) {
        __syncthreads();
        for (int i = threadIdx.x; i < N; i += blockDim.x) {
            const double e = E[b * N + i];
            ed[i] = e;
            e2s[i] = df_of(e);
        }
        __syncthreads();
        float2 cs[kOccSlots];  // column sums of m = 32 q + lane over this warp's rows
#pragma unroll
        for (int q = 0; q < kOccSlots; ++q) cs[q] = make_float2(0.f, 0.f);
        for (int p = warp; p < npair; p += nw) {
            for (int half = 0; half < 2; ++half) {
                const int n = half ? N - 1 - p : p;
                if (half && n == p) break;  // the middle row of an odd N
                const float4* bx = Bx + b * NN + (int64_t)n * N;
                const float4* by = By + b * NN + (int64_t)n * N;
                const float2 en = e2s[n];
                float2 racc = make_float2(0.f, 0.f);
#pragma unroll
                for (int q = 0; q < kOccSlots; ++q) {
                    const int m = 32 * q + lane;
                    if (m > n && m < N) {
                        const float4 x = bx[m];
                        const float4 y = by[m];
                        // Im(x conj(y)) = x_im y_re - x_re y_im
                        const float2 t1 = df_mul(make_float2(x.z, x.w), make_float2(y.x, y.y));
                        const float2 t2 = df_mul(make_float2(x.x, x.y), make_float2(y.z, y.w));
                        const float2 num = df_add(t1, df_neg(t2));
                        const float2 de = df_add(en, df_neg(e2s[m]));
                        const float2 den = df_add(df_mul(de, de), eta2);
                        const float2 qv = df_div(num, den);
                        const float2 t = make_float2(-2.f * qv.x, -2.f * qv.y);
                        racc = df_add(racc, t);
                        cs[q] = df_add(cs[q], t);
                    }
                }
                racc = df_warp_sum(racc);
                if (lane == 0) om[n] = df_to_double(racc);
            }
        }
#pragma unroll
        for (int q = 0; q < kOccSlots; ++q) {
            const int m = 32 * q + lane;
            if (m < N) colp[(size_t)warp * N + m] = df_to_double(cs[q]);
        }
        __syncthreads();
        for (int n = threadIdx.x; n < N; n += blockDim.x) {
            double c = 0.0;
            for (int w = 0; w < nw; ++w) c += colp[(size_t)w * N + n];
            om[n] -= c;
        }
        __syncthreads();
        for (int j = warp; j < nmu; j += nw) {
            const double mj = mu[j];
            double t = 0.0;
            for (int n = lane; n < N; n += 32) t += om[n] * occupation_f(ed[n], mj, width);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
            if (lane == 0) kahan_step(rs[j], rc[j], t);
        }
    }
    __syncthreads();
    for (int j = threadIdx.x; j < nmu; j += blockDim.x) {
        part[((int64_t)blockIdx.x * nmu + j) * 2] = rs[j];
        part[((int64_t)blockIdx.x * nmu + j) * 2 + 1] = rc[j];
    }
}

// acc[2 j], acc[2 j + 1] += the partials of every block: one CTA per mu, each
// thread Kahan-sums a contiguous range of blocks, and the ranges are combined
// along a fixed tree (deterministic).
__global__ void occ_partials_kernel(int blocks, int nmu, const double* __restrict__ part, double* __restrict__ acc) {
    __shared__ double ps[256], pc[256];
    const int j = blockIdx.x;
    const int seg = (blocks + blockDim.x - 1) / blockDim.x;
    const int t0 = threadIdx.x * seg, t1 = min(blocks, t0 + seg);
    double sm = 0.0, c = 0.0;
    for (int t = t0; t < t1; ++t) {
        kahan_step(sm, c, part[((int64_t)t * nmu + j) * 2]);
        kahan_step(sm, c, -part[((int64_t)t * nmu + j) * 2 + 1]);
    }
    ps[threadIdx.x] = sm;  // the value is sm - c
    pc[threadIdx.x] = -c;
    dd_block_sum(ps, pc);
    if (threadIdx.x == 0) {
        double tot = acc[2 * j], comp = acc[2 * j + 1];
        kahan_step(tot, comp, ps[0]);
        kahan_step(tot, comp, pc[0]);
        acc[2 * j] = tot;
        acc[2 * j + 1] = comp;
    }
}

// Keep E ascending (with Omega and the metric when given) after refinement;
// a no-op when already sorted.
__global__ void sort_e_om_kernel(int N, int64_t batch, double* __restrict__ E, double* __restrict__ Om,
                                 double* __restrict__ Met) {
    extern __shared__ double sm3[];
    double* e = sm3;
    double* o = sm3 + N;
    double* g = sm3 + 2 * N;
    __shared__ int s_sorted;
    for (int64_t b = blockIdx.x; b < batch; b += gridDim.x) {
        if (threadIdx.x == 0) s_sorted = 1;
        __syncthreads();
        for (int i = threadIdx.x; i < N; i += blockDim.x) {
            e[i] = E[b * N + i];
            if (Om) o[i] = Om[b * N + i];
            if (Met) g[i] = Met[b * N + i];
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
                if (Om) Om[b * N + rank] = o[i];
                if (Met) Met[b * N + rank] = g[i];
            }
        }
        __syncthreads();
    }
}

inline unsigned nblk(int64_t total) {
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>((total + 255) / 256, 152LL * 64));
}

}  // namespace

int occ_sums_blocks(int64_t batch) { return (int)std::max<int64_t>(1, std::min<int64_t>(batch, 152 * 8)); }

// Dynamic shared memory of berry_occ_df_kernel (256 threads).
size_t occ_smem_bytes(int N, int nmu) {
    return (2 + 8) * sizeof(double) * (size_t)N + 2 * sizeof(double) * (size_t)nmu + sizeof(float2) * (size_t)N;
}
bool occ_fused_ok(int N, int nmu) { return N <= kOccMaxN && occ_smem_bytes(N, nmu) <= 48 * 1024; }

int occ_partials_add(cudaStream_t st, const OccSums& o, double* acc) {
    KTimer kt(st, "occ_partials_kernel");
    occ_partials_kernel<<<o.nmu, 256, 0, st>>>(o.blocks, o.nmu, o.part, acc);
    TBG_LAUNCHED("occ_partials_kernel");
    return TBG_OK;
}

// Class of the rotation products B = X'^H V X': MID unless TBG_ROTATION_HIGH=1.
bool rotation_mid() {
    static const bool mid = [] {
        const char* e = std::getenv("TBG_ROTATION_HIGH");
        return !(e && e[0] == '1');
    }();
    return mid;
}

size_t mixed_berry_workspace_bytes(int N, int64_t batch) {
    const size_t NN = (size_t)N * N;
    // X and F (cc) + 5 pair buffers + line exponents (10 operand sides) + FP32 solver workspace
    return (size_t)batch * NN * (2 * sizeof(cc) + 5 * sizeof(float4)) + sizeof(int) * 10 * (size_t)batch * N +
           ozaki_exp_bytes(batch, N, N) + eig_workspace_bytes(N, batch, 1) +
           (size_t)batch * N * (sizeof(int) + kMaxCluster * sizeof(zc)) +
           sizeof(unsigned long long) * ((size_t)batch * N / 2 + 1) + 4096 + 768;
}

// H, Vx, Vy as float pairs (batch stride N*N) -> E (refined, ascending), Omega and, when Met is
// not null, the quantum metric.
int mixed_berry(cudaStream_t st, int N, int64_t batch, const float4* H, const float4* Vx, const float4* Vy,
                double eta, double* E, double* Om, void* work, size_t work_bytes, int* status_d,
                int64_t* clusters_d, double* Met, zc* Uout, const OccSums* occ, const int* h_rexp,
                const int* v_rexp) {
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
    cc* F = static_cast<cc*>(take(sizeof(cc) * batch * NN));
    float4* bA = static_cast<float4*>(take(sizeof(float4) * batch * NN));
    float4* bB = static_cast<float4*>(take(sizeof(float4) * batch * NN));
    float4* bC = static_cast<float4*>(take(sizeof(float4) * batch * NN));
    float4* bD = static_cast<float4*>(take(sizeof(float4) * batch * NN));
    float4* bE = static_cast<float4*>(take(sizeof(float4) * batch * NN));
    int* EA = static_cast<int*>(take(ozaki_exp_bytes(batch, N, N)));
    int* EB = EA + batch * N;
    // tcgen05 form: the exponents of each operand side are scanned once and
    // shared by the products that use it
    int* ex = static_cast<int*>(take(sizeof(int) * 10 * (size_t)batch * N));
    int* cinfo = static_cast<int*>(take(sizeof(int) * (size_t)batch * N));
    zc* Fcl = static_cast<zc*>(take(sizeof(zc) * kMaxCluster * (size_t)batch * N));
    // clusters found by the refinement: a count, then one entry per cluster
    unsigned long long* clist =
        static_cast<unsigned long long*>(take(sizeof(unsigned long long) * ((size_t)batch * N / 2 + 1)));
    enum { XC, HR, HXC, XR, FC, XPC, VXR, VYR, BXC, BYC, NSLOT };
    // slots whose exponents a kernel writing the operand has already produced
    // (the caller's for H, Vx, Vy; the refinement kernel's for F; the X' pass's)
    int* given[NSLOT] = {};
    bool ready[NSLOT] = {};
    auto slot = [&](int i) { return given[i] ? given[i] : ex + (size_t)i * batch * N; };
    const bool tc = ozaki_use_tc();
    if (tc) {
        given[HR] = const_cast<int*>(h_rexp);
        given[VXR] = const_cast<int*>(v_rexp);
        given[VYR] = v_rexp ? const_cast<int*>(v_rexp) + batch * N : nullptr;
        ready[HR] = h_rexp != nullptr;
        ready[VXR] = ready[VYR] = v_rexp != nullptr;
    }
    auto exps = [&](int fmt, bool cols, const void* M, int s) -> int {
        if (!tc || ready[s]) return TBG_OK;
        return ozaki_line_exps(st, fmt, cols, batch, N, N, M, N, NN, slot(s));
    };
    const size_t eigw_bytes = eig_workspace_bytes(N, batch, 1);
    void* eigw = take(eigw_bytes);
    // FP64-class products: tcgen05 form unless the mma.sync form is selected
    // (mid: the MID class, for the rotation into the eigenbasis)
    auto hp = [&](bool conj_a, int fa, int fb, const void* A, const void* B, float4* C, int sa, int sb,
                  bool mid = false) -> int {
        if (tc)
            return ozaki_zgemm_tc(st, conj_a, fa, fb, batch, N, N, N, A, N, NN, B, N, NN, C, N, NN, slot(sa),
                                  slot(sb), status_d, true, nullptr, mid);
        return ozaki_zgemm(st, true, conj_a, fa, fb, batch, N, N, N, A, N, NN, B, N, NN, C, N, NN, EA, EB);
    };
    // the same with the column exponents of the output into slot sc: fused into
    // the product's epilogue when one tile holds every row (N <= 128)
    auto hpe = [&](bool conj_a, int fa, int fb, const void* A, const void* B, float4* C, int sa, int sb, int sc,
                   bool mid = false) -> int {
        if (tc && N <= 128)
            return ozaki_zgemm_tc(st, conj_a, fa, fb, batch, N, N, N, A, N, NN, B, N, NN, C, N, NN, slot(sa),
                                  slot(sb), status_d, true, slot(sc), mid);
        const int r = hp(conj_a, fa, fb, A, B, C, sa, sb, mid);
        return r ? r : exps(PAIR, true, C, sc);
    };
    int rc;
    // 1. FP32 eigenpairs of H
    {
        bool xe = false;
        if ((rc = eig_batched_f32(st, N, batch, nullptr, E, X, eigw, eigw_bytes, status_d, H, tc ? slot(XR) : nullptr,
                                  tc ? slot(XC) : nullptr, &xe)))
            return rc;
        ready[XR] = ready[XC] = xe;
    }
    // 2. X^H X and S = X^H (H X)   (FP64-class, tensor cores)
    if ((rc = exps(F32, true, X, XC)) || (rc = exps(PAIR, false, H, HR))) return rc;
    if ((rc = hp(true, F32, F32, X, X, bA, XC, XC))) return rc;
    if ((rc = hpe(false, PAIR, F32, H, X, bB, HR, XC, HXC))) return rc;
    if ((rc = hp(true, F32, PAIR, X, bB, bC, XC, HXC))) return rc;
    // 3. Ogita-Aishima update F and refined eigenvalues
    {
        KTimer kt(st, "oa_kernel");
        const size_t smem = oa_smem_bytes(N);
        cudaError_t ea = cudaFuncSetAttribute(oa_pairs_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (ea != cudaSuccess) return cuda_error(ea, "cudaFuncSetAttribute(oa_kernel)");
        TBG_CUDA(cudaMemsetAsync(clist, 0, sizeof(unsigned long long), st));
        oa_pairs_kernel<<<(unsigned)std::min<int64_t>(batch, 152 * 8), 256, smem, st>>>(
            N, batch, bA, bC, E, F, clusters_d, cinfo, Fcl, tc ? slot(FC) : nullptr, clist);
        TBG_LAUNCHED("oa_kernel");
        ready[FC] = tc;
    }
    auto energies_out = [&]() -> int {
        sort_e_om_kernel<<<(unsigned)std::min<int64_t>(batch, 152 * 8), 256, 3 * sizeof(double) * N, st>>>(
            N, batch, E, nullptr, nullptr);
        TBG_LAUNCHED("sort_e_om_kernel");
        return (int)TBG_OK;
    };
    if (!Om && !Uout && !occ) return energies_out();  // band energies only
    // 4. X' = X + X F + X_c F_c  (float pair: hi = X, lo = the rest).  F holds
    // only first-order entries (the cluster rotations F_c are applied in FP64
    // by xprime_kernel), so the LOW class's 2^-21 of each column's largest
    // entry stays far below the refinement's accuracy; above kHighCorrN bands
    // X F is a HIGH product.
    if ((rc = exps(F32, false, X, XR)) || (rc = exps(F32, true, F, FC))) return rc;
    if (tc && N > kHighCorrN)
        rc = ozaki_zgemm_tc(st, false, F32, F32, batch, N, N, N, X, N, NN, F, N, NN, bE, N, NN, slot(XR), slot(FC),
                            status_d, true);
    else
        rc = tc ? ozaki_zgemm_tc_low(st, batch, N, N, N, X, N, NN, F, N, NN, bE, N, NN, slot(XR), slot(FC), status_d,
                                     true)
                : ozaki_zgemm(st, false, false, F32, F32, batch, N, N, N, X, N, NN, F, N, NN, bE, N, NN, EA, EB);
    if (rc) return rc;
    {
        KTimer kt(st, "xprime_kernel");
        const int64_t work = batch * ((N + 127) / 128);
        const unsigned g = (unsigned)std::min<int64_t>(work, 152 * 64);
        xprime_kernel<<<g, 128, 0, st>>>(batch, N, X, bE, cinfo, bA, tc ? slot(XPC) : nullptr);
        TBG_LAUNCHED("xprime_kernel");
        xprime_cluster_kernel<<<152 * 4, 128, 0, st>>>(N, X, bE, Fcl, bA, tc ? slot(XPC) : nullptr, clist);
        TBG_LAUNCHED("xprime_cluster_kernel");
        ready[XPC] = tc;
    }
    if (Uout) {  // eigenpairs only: refined E and X' in ascending order, no velocities
        const size_t smem = (sizeof(double) + sizeof(int)) * (size_t)N;
        eigpairs_sorted_kernel<<<(unsigned)std::min<int64_t>(batch, 152 * 8), 256, smem, st>>>(N, batch, bA, E, E,
                                                                                             Uout);
        TBG_LAUNCHED("eigpairs_sorted_kernel");
        return TBG_OK;
    }
    // 5. band-basis velocities B = X'^H V X'
    if ((rc = exps(PAIR, true, bA, XPC)) || (rc = exps(PAIR, false, Vx, VXR)) || (rc = exps(PAIR, false, Vy, VYR)))
        return rc;
    //    in the MID class (about 2^-35 of each product's scale): Omega and its
    //    k-sum need about 1e-9, where the refinement above needs FP64 class
    const bool rmid = rotation_mid();
    if ((rc = hpe(false, PAIR, PAIR, Vx, bA, bB, VXR, XPC, BXC, rmid))) return rc;
    if ((rc = hpe(false, PAIR, PAIR, Vy, bA, bC, VYR, XPC, BYC, rmid))) return rc;
    if ((rc = hp(true, PAIR, PAIR, bA, bB, bD, XPC, BXC, rmid))) return rc;
    if ((rc = hp(true, PAIR, PAIR, bA, bC, bE, XPC, BYC, rmid))) return rc;
    // 6. Omega (with the occupation k-sum when the caller wants only sums)
    if (occ) {
        if (Om || Met || occ->blocks != occ_sums_blocks(batch))
            return set_error(TBG_E_INVALID_ARGUMENT, "mixed_berry: fused sums take no per-band outputs");
        KTimer kt(st, "berry_occ_kernel");
        const double e2 = eta * eta;
        const float hi = (float)e2;
        const float2 eta2 = make_float2(hi, (float)(e2 - (double)hi));
        const size_t smem = occ_smem_bytes(N, occ->nmu);
        if (N > kOccMaxN || smem > 48 * 1024)
            return set_error(TBG_E_UNSUPPORTED, "mixed_berry: fused sums beyond 256 bands or too many potentials");
        berry_occ_df_kernel<<<(unsigned)occ->blocks, 256, smem, st>>>(N, batch, bD, bE, E, eta2, occ->nmu, occ->mu,
                                                                     occ->width, occ->part);
        TBG_LAUNCHED("berry_occ_df_kernel");
        return TBG_OK;
    }
    {
        KTimer kt(st, "berry_kernel");
        const double e2 = eta * eta;
        const float hi = (float)e2;
        const float2 eta2 = make_float2(hi, (float)(e2 - (double)hi));
        const unsigned g = (unsigned)std::min<int64_t>(batch, 152 * 8);
        if (Met)
            berry_df_kernel<true><<<g, 256, sizeof(float2) * N, st>>>(N, batch, bD, bE, E, eta2, Om, Met);
        else
            berry_df_kernel<false><<<g, 256, sizeof(float2) * N, st>>>(N, batch, bD, bE, E, eta2, Om, nullptr);
        TBG_LAUNCHED("berry_df_kernel");
    }
    sort_e_om_kernel<<<(unsigned)std::min<int64_t>(batch, 152 * 8), 256, 3 * sizeof(double) * N, st>>>(N, batch, E,
                                                                                                      Om, Met);
    TBG_LAUNCHED("sort_e_om_kernel");
    return TBG_OK;
}

}  // namespace tbg
