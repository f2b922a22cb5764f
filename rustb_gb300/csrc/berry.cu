// Velocity rotation into the eigenbasis, band-resolved Berry curvature, the
// occupation-weighted k-sum and its deterministic compensated reduction.
//
// Replaces src/response/traits.rs:170-195 (spin dressing, U^T V U*, the
// Omega_n loop) and the Direct-integration sum of
// src/response/linear/mod.rs:204-223 with src/thermodynamics.rs:100-118.

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "tbgpu_internal.cuh"

namespace tbg {

namespace {

// C[b] = op(A[b]) * B[b] for square N x N row-major complex matrices,
// op = identity or conjugate transpose.  64x64 output tile per CTA,
// 4x4 outputs per thread, K staged 8 at a time.  FP64 (plain path).
template <bool CONJ_A>
__global__ void __launch_bounds__(256) zgemm_batched_kernel(int N, const zc* __restrict__ A, int64_t sA,
                                                            const zc* __restrict__ B, int64_t sB,
                                                            zc* __restrict__ C, int64_t sC) {
    constexpr int BT = 64, KT = 8;
    __shared__ zc tA[BT][KT + 1];
    __shared__ zc tB[KT][BT];
    const int64_t b = blockIdx.z;
    const zc* Ab = A + b * sA;
    const zc* Bb = B + b * sB;
    zc* Cb = C + b * sC;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int row0 = blockIdx.y * BT, col0 = blockIdx.x * BT;
    zc acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = mk(0.0, 0.0);
    for (int l0 = 0; l0 < N; l0 += KT) {
        for (int idx = threadIdx.x; idx < BT * KT; idx += 256) {
            int r, l;
            zc a = mk(0.0, 0.0);
            if (CONJ_A) {
                r = idx % BT;
                l = idx / BT;
                if (row0 + r < N && l0 + l < N) a = conj(Ab[(int64_t)(l0 + l) * N + row0 + r]);
            } else {
                l = idx % KT;
                r = idx / KT;
                if (row0 + r < N && l0 + l < N) a = Ab[(int64_t)(row0 + r) * N + l0 + l];
            }
            tA[r][l] = a;
        }
        for (int idx = threadIdx.x; idx < BT * KT; idx += 256) {
            const int c = idx % BT, l = idx / BT;
            zc v = mk(0.0, 0.0);
            if (col0 + c < N && l0 + l < N) v = Bb[(int64_t)(l0 + l) * N + col0 + c];
            tB[l][c] = v;
        }
        __syncthreads();
#pragma unroll
        for (int l = 0; l < KT; ++l) {
            zc a[4], bv[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = tA[ty + 16 * i][l];
#pragma unroll
            for (int j = 0; j < 4; ++j) bv[j] = tB[l][tx + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) fma_cx(acc[i][j], a[i], bv[j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int r = row0 + ty + 16 * i;
        if (r >= N) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int c = col0 + tx + 16 * j;
            if (c < N) Cb[(int64_t)r * N + c] = acc[i][j];
        }
    }
}

// Small matrices (N <= 16): one thread per output element, 256 / N^2 matrices
// per block, operands read through L1.  C[b] = op(A[b]) B[b].
template <bool CONJ_A>
__global__ void __launch_bounds__(256) zgemm_small_kernel(int N, int64_t batch, const zc* __restrict__ A, int64_t sA,
                                                          const zc* __restrict__ B, int64_t sB, zc* __restrict__ C,
                                                          int64_t sC) {
    const int NN = N * N;
    const int per = blockDim.x / NN;
    const int local = threadIdx.x / NN, e = threadIdx.x % NN;
    if (local >= per) return;
    const int i = e / N, j = e % N;
    for (int64_t b = (int64_t)blockIdx.x * per + local; b < batch; b += (int64_t)gridDim.x * per) {
        const zc* Ab = A + b * sA;
        const zc* Bb = B + b * sB;
        zc acc = mk(0.0, 0.0);
        for (int l = 0; l < N; ++l) {
            if (CONJ_A)
                fma_cjx(acc, Ab[(int64_t)l * N + i], Bb[(int64_t)l * N + j]);
            else
                fma_cx(acc, Ab[(int64_t)i * N + l], Bb[(int64_t)l * N + j]);
        }
        C[b * sC + e] = acc;
    }
}

// Omega_n = sum_{m != n} -2 Im(Bx[n,m] By[m,n]) / ((E_n - E_m)^2 + eta^2), one warp per row n.
// With MET, also the quantum metric g_n = sum_{m != n} Re(Bx[n,m] By[m,n]) / ((E_n - E_m)^2 + eta^2)
// (src/quantum_geometry.rs:160-187: the real part of the same tensor).
template <bool MET>
__global__ void berry_kernel(int N, int64_t batch, const zc* __restrict__ Bx, const zc* __restrict__ By,
                             int64_t ldB, const double* __restrict__ E, double eta2,
                             double* __restrict__ Omega, double* __restrict__ Met) {
    const int lane = threadIdx.x & 31;
    const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t w = gw; w < batch * N; w += nw) {
        const int64_t b = w / N;
        const int n = (int)(w % N);
        const zc* bx = Bx + b * ldB + (int64_t)n * N;
        const zc* by = By + b * ldB;
        const double* Eb = E + b * N;
        const double en = Eb[n];
        double s = 0.0, g = 0.0;
        for (int m = lane; m < N; m += 32) {
            if (m == n) continue;
            const zc kx = bx[m];
            const zc ky = by[(int64_t)m * N + n];
            const double im = kx.re * ky.im + kx.im * ky.re;
            const double de = en - Eb[m];
            const double den = de * de + eta2;
            s += -2.0 * im / den;
            if (MET) g += (kx.re * ky.re - kx.im * ky.im) / den;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            s += __shfl_xor_sync(0xffffffffu, s, o);
            if (MET) g += __shfl_xor_sync(0xffffffffu, g, o);
        }
        if (lane == 0) {
            Omega[b * N + n] = s;
            if (MET) Met[b * N + n] = g;
        }
    }
}

// J = 1/2 (S V + V S), S = sigma_d (x) I_norb / 2 (src/response/helpers.rs:11-40,
// src/math.rs anti_comm).  S has one non-zero per row: S[i][pi(i)] = s_i.
__device__ __forceinline__ void spin_entry(int spin, int norb, int i, int& pi, zc& s) {
    const bool up = i < norb;
    if (spin == TBG_SPIN_X) {
        pi = up ? i + norb : i - norb;
        s = mk(0.5, 0.0);
    } else if (spin == TBG_SPIN_Y) {
        pi = up ? i + norb : i - norb;
        s = up ? mk(0.0, -0.5) : mk(0.0, 0.5);
    } else {
        pi = i;
        s = up ? mk(0.5, 0.0) : mk(-0.5, 0.0);
    }
}

__global__ void spin_dress_kernel(int N, int norb, int64_t batch, int spin, const zc* __restrict__ V, int64_t ldV,
                                  zc* __restrict__ J) {
    const int64_t NN = (int64_t)N * N;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < batch * NN;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t b = idx / NN;
        const int e = (int)(idx % NN), i = e / N, j = e % N;
        int pi, pj, ppj;
        zc si, sj;
        spin_entry(spin, norb, i, pi, si);
        spin_entry(spin, norb, j, pj, sj);
        // (V S)[i][j] = V[i][pi(j)] S[pi(j)][j]: the weight belongs to row pi(j)
        spin_entry(spin, norb, pj, ppj, sj);
        const zc* Vb = V + b * ldV;
        const zc a = si * Vb[(int64_t)pi * N + j];
        const zc c = Vb[(int64_t)i * N + pj] * sj;
        J[b * NN + e] = mk(0.5 * (a.re + c.re), 0.5 * (a.im + c.im));
    }
}

// s (one of +-1/2, +-i/2) times a float-pair complex {re_hi, re_lo, im_hi, im_lo}: exact
__device__ __forceinline__ float4 spin_scale(float4 v, zc s) {
    if (s.im == 0.0) {
        const float f = (float)s.re;
        return make_float4(v.x * f, v.y * f, v.z * f, v.w * f);
    }
    const float f = (float)s.im;  // i f (re + i im) = -f im + i f re
    return make_float4(-v.z * f, -v.w * f, v.x * f, v.y * f);
}

// J = 1/2 (S V + V S) on float pairs, same index algebra as spin_dress_kernel.
__global__ void spin_dress_pairs_kernel(int N, int norb, int64_t batch, int spin, const float4* __restrict__ V,
                                        int64_t ldV, float4* __restrict__ J) {
    const int NN = N * N;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= NN) return;
    const int i = e / N, j = e - i * N;
    int pi, pj, ppj;
    zc si, sj;
    spin_entry(spin, norb, i, pi, si);
    spin_entry(spin, norb, j, pj, sj);
    spin_entry(spin, norb, pj, ppj, sj);
    for (int64_t b = blockIdx.y; b < batch; b += gridDim.y) {
        const float4* Vb = V + b * ldV;
        const float4 a = spin_scale(Vb[(int64_t)pi * N + j], si);
        const float4 c = spin_scale(Vb[(int64_t)i * N + pj], sj);
        const float2 re = df_add(make_float2(a.x, a.y), make_float2(c.x, c.y));
        const float2 im = df_add(make_float2(a.z, a.w), make_float2(c.z, c.w));
        J[b * NN + e] = make_float4(0.5f * re.x, 0.5f * re.y, 0.5f * im.x, 0.5f * im.y);
    }
}

__global__ void z_to_pairs_kernel(int64_t nb, int64_t N2, const zc* __restrict__ in, int64_t ld_in,
                                  float4* __restrict__ out) {
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < nb * N2;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t b = idx / N2, e = idx - b * N2;
        const zc v = in[b * ld_in + e];
        const float2 r = df_of(v.re), q = df_of(v.im);
        out[idx] = make_float4(r.x, r.y, q.x, q.y);
    }
}

__device__ __forceinline__ double fermi(double e, double mu, double width) { return occupation_f(e, mu, width); }

__global__ void occupation_kernel(int N, int64_t batch, const double* __restrict__ Om, const double* __restrict__ E,
                                  int nmu, const double* __restrict__ mu, double width, double* __restrict__ S) {
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < batch * nmu;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t b = idx / nmu;
        const int j = (int)(idx % nmu);
        const double m = mu[j];
        double s = 0.0;
        for (int n = 0; n < N; ++n) s += Om[b * N + n] * fermi(E[b * N + n], m, width);
        S[idx] = s;
    }
}

__device__ __forceinline__ void kahan_add(double& sum, double& c, double x) { kahan_step(sum, c, x); }

// One block per mu: each thread Kahan-sums a contiguous k segment, then the
// segments are combined along a fixed tree of double-double sums
// (deterministic).
__global__ void kahan_kernel(int64_t nk, int nmu, const double* __restrict__ S, double* __restrict__ acc) {
    __shared__ double ps[256], pc[256];
    const int j = blockIdx.x;
    const int64_t seg = (nk + blockDim.x - 1) / blockDim.x;
    const int64_t b0 = threadIdx.x * seg, b1 = std::min<int64_t>(nk, b0 + seg);
    double s = 0.0, c = 0.0;
    for (int64_t b = b0; b < b1; ++b) kahan_add(s, c, S[b * nmu + j]);
    ps[threadIdx.x] = s;  // the value is s - c
    pc[threadIdx.x] = -c;
    dd_block_sum(ps, pc);
    if (threadIdx.x == 0) {
        double tot = acc[2 * j], comp = acc[2 * j + 1];
        kahan_add(tot, comp, ps[0]);
        kahan_add(tot, comp, pc[0]);
        acc[2 * j] = tot;
        acc[2 * j + 1] = comp;
    }
}

inline unsigned grid_for(int64_t total, int threads) {
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>((total + threads - 1) / threads, 152LL * 64));
}

}  // namespace

int zgemm_batched(cudaStream_t st, int N, int64_t batch, bool conj_a, const zc* A, int64_t sA, const zc* B,
                  int64_t sB, zc* C, int64_t sC) {
    KTimer kt(st, "zgemm_batched_kernel", 8.0 * (double)N * N * N * batch);
    if (N <= 16) {
        const int per = 256 / (N * N);
        const unsigned g = (unsigned)std::max<int64_t>(1, std::min<int64_t>((batch + per - 1) / per, 152LL * 64));
        if (conj_a)
            zgemm_small_kernel<true><<<g, 256, 0, st>>>(N, batch, A, sA, B, sB, C, sC);
        else
            zgemm_small_kernel<false><<<g, 256, 0, st>>>(N, batch, A, sA, B, sB, C, sC);
        TBG_LAUNCHED("zgemm_small_kernel");
        return TBG_OK;
    }
    for (int64_t b0 = 0; b0 < batch; b0 += 65535) {
        const int64_t nb = std::min<int64_t>(65535, batch - b0);
        dim3 grid((N + 63) / 64, (N + 63) / 64, (unsigned)nb);
        if (conj_a)
            zgemm_batched_kernel<true><<<grid, 256, 0, st>>>(N, A + b0 * sA, sA, B + b0 * sB, sB, C + b0 * sC, sC);
        else
            zgemm_batched_kernel<false><<<grid, 256, 0, st>>>(N, A + b0 * sA, sA, B + b0 * sB, sB, C + b0 * sC, sC);
        TBG_LAUNCHED("zgemm_batched_kernel");
    }
    return TBG_OK;
}

int spin_dress(cudaStream_t st, int N, int64_t norb, int64_t batch, int spin, zc* V, int64_t ldV, zc* scratch) {
    const int64_t NN = (int64_t)N * N;
    KTimer kt(st, "spin_dress_kernel");
    spin_dress_kernel<<<grid_for(batch * NN, 256), 256, 0, st>>>(N, (int)norb, batch, spin, V, ldV, scratch);
    TBG_LAUNCHED("spin_dress_kernel");
    // copy J back into the V_0 slots
    TBG_CUDA(cudaMemcpy2DAsync(V, sizeof(zc) * ldV, scratch, sizeof(zc) * NN, sizeof(zc) * NN, batch,
                               cudaMemcpyDeviceToDevice, st));
    return TBG_OK;
}

int spin_dress_pairs(cudaStream_t st, int N, int64_t norb, int64_t batch, int spin, float4* V, int64_t ldV,
                     float4* scratch) {
    const int64_t NN = (int64_t)N * N;
    KTimer kt(st, "spin_dress_kernel");
    dim3 grid((unsigned)((NN + 255) / 256), (unsigned)std::min<int64_t>(batch, 65535));
    spin_dress_pairs_kernel<<<grid, 256, 0, st>>>(N, (int)norb, batch, spin, V, ldV, scratch);
    TBG_LAUNCHED("spin_dress_pairs_kernel");
    TBG_CUDA(cudaMemcpy2DAsync(V, sizeof(float4) * ldV, scratch, sizeof(float4) * NN, sizeof(float4) * NN, batch,
                               cudaMemcpyDeviceToDevice, st));
    return TBG_OK;
}

int z_to_pairs(cudaStream_t st, int64_t nb, int64_t N2, const zc* in, int64_t ld_in, float4* out) {
    z_to_pairs_kernel<<<grid_for(nb * N2, 256), 256, 0, st>>>(nb, N2, in, ld_in, out);
    TBG_LAUNCHED("z_to_pairs_kernel");
    return TBG_OK;
}

static int launch_berry(cudaStream_t st, int N, int64_t batch, const zc* Bx, const zc* By, int64_t ldB, const double* E,
                  double eta, double* Omega, double* Met) {
    KTimer kt(st, "berry_kernel");
    const unsigned g = grid_for(batch * N * 32, 256);
    if (Met)
        berry_kernel<true><<<g, 256, 0, st>>>(N, batch, Bx, By, ldB, E, eta * eta, Omega, Met);
    else
        berry_kernel<false><<<g, 256, 0, st>>>(N, batch, Bx, By, ldB, E, eta * eta, Omega, nullptr);
    TBG_LAUNCHED("berry_kernel");
    return TBG_OK;
}

// Bx = U^H (Vx U), By = U^H (Vy U) written over Vx / Vy, then Omega (and the metric when Met is given).
int berry_rotate(cudaStream_t st, int N, int64_t batch, const zc* U, const zc* Vx, const zc* Vy, int64_t ldV,
                 const double* E, double eta, double* Omega, zc* scratch, double* Met) {
    const int64_t NN = (int64_t)N * N;
    zc* Vxm = const_cast<zc*>(Vx);
    zc* Vym = const_cast<zc*>(Vy);
    int rc;
    rc = zgemm_batched(st, N, batch, false, Vx, ldV, U, NN, scratch, NN);
    if (rc) return rc;
    rc = zgemm_batched(st, N, batch, true, U, NN, scratch, NN, Vxm, ldV);
    if (rc) return rc;
    rc = zgemm_batched(st, N, batch, false, Vy, ldV, U, NN, scratch, NN);
    if (rc) return rc;
    rc = zgemm_batched(st, N, batch, true, U, NN, scratch, NN, Vym, ldV);
    if (rc) return rc;
    return launch_berry(st, N, batch, Vx, Vy, ldV, E, eta, Omega, Met);
}

int berry_from_bands(cudaStream_t st, int N, int64_t batch, const zc* Bx, const zc* By, int64_t ldB,
                     const double* E, double eta, double* Omega) {
    return launch_berry(st, N, batch, Bx, By, ldB, E, eta, Omega, nullptr);
}

int occupation_sums(cudaStream_t st, int N, int64_t batch, const double* Omega, const double* E, int nmu,
                    const double* mu_d, double width, double* S) {
    KTimer kt(st, "occupation_kernel");
    occupation_kernel<<<grid_for(batch * nmu, 256), 256, 0, st>>>(N, batch, Omega, E, nmu, mu_d, width, S);
    TBG_LAUNCHED("occupation_kernel");
    return TBG_OK;
}

int kahan_column_sums(cudaStream_t st, int64_t nk, int nmu, const double* S, double* acc) {
    KTimer kt(st, "kahan_kernel");
    kahan_kernel<<<nmu, 256, 0, st>>>(nk, nmu, S, acc);
    TBG_LAUNCHED("kahan_kernel");
    return TBG_OK;
}

}  // namespace tbg
