// Bloch Fourier sum H(k) and direction-projected velocities, direct form.
//
// Replaces the zaxpy loops of Model::gen_ham (src/model_physics.rs:92-96) and
// Model::gen_v_projected (src/velocity.rs:538-541, 581-613):
//
//   H_lat(k)[e] = sum_R u(k,R) ham[R][e],                u = e^{2 pi i k.R}
//   V_p(k)[e]   = i sum_R (w_p . R_cart) u(k,R) ham[R][e]
//   Atom gauge:   H[m,n] = conj(phi_m) H_lat[m,n] phi_n,       phi = e^{2 pi i k.tau}
//                 V_p[m,n] = (V_p[m,n] + i (w_p.tau_n - w_p.tau_m) H_lat[m,n]) conj(phi_m) phi_n
//
// As a contraction this is phase[nk x nR] . hop[nR x N^2] for H and the same
// with the phase column scaled by w_p.R_cart for each V_p.  The kernel stages
// tiles of the hop table and of the phases in shared memory and keeps one
// complex accumulator per output in registers; the gauge / tau epilogue is
// fused.  FP64 throughout (plain path).

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cmath>
#include <mutex>
#include <vector>

#include "tbgpu_internal.cuh"

namespace tbg {
namespace {

constexpr double kTwoPi = 6.283185307179586476925286766559;

// u(k,R) = exp(2 pi i k.R) for R rows [0, nR); phi(k,s) = exp(2 pi i k.tau_s).
__global__ void phases_kernel(int64_t nk, int dim, const double* __restrict__ k, int nR,
                              const int* __restrict__ hamR, int nsta, const double* __restrict__ tau,
                              zc* __restrict__ ph, zc* __restrict__ orbph) {
    const int64_t total = nk * (int64_t)(nR + nsta);
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t kk = idx / (nR + nsta);
        const int j = (int)(idx % (nR + nsta));
        const double* kv = k + kk * dim;
        double s = 0.0;
        if (j < nR) {
            const int* r = hamR + 3 * j;
            // same operation order as the reference: r0*k0 + r1*k1 + r2*k2
            s = (double)r[0] * kv[0];
            if (dim > 1) s += (double)r[1] * kv[1];
            if (dim > 2) s += (double)r[2] * kv[2];
            double sn, cs;
            sincos(kTwoPi * s, &sn, &cs);
            ph[kk * nR + j] = mk(cs, sn);
        } else {
            const double* t = tau + 3 * (j - nR);
            s = t[0] * kv[0];
            if (dim > 1) s += t[1] * kv[1];
            if (dim > 2) s += t[2] * kv[2];
            double sn, cs;
            sincos(kTwoPi * s, &sn, &cs);
            orbph[kk * nsta + (j - nR)] = mk(cs, sn);
        }
    }
}

constexpr int TK = 32;   // k-points per tile
constexpr int TE = 64;   // matrix elements per tile
constexpr int RC = 8;    // R rows per shared-memory stage

// NP velocity projections (0..3).  coef: (NP, nR) = w_p . R_cart.
// taup: (NP, N) = w_p . tau_cart (Atom gauge only).
template <int NP>
__global__ void __launch_bounds__(256) fourier_gemm_kernel(
    int64_t nk, int nR, int ldph, int N, const zc* __restrict__ ph, const zc* __restrict__ hop,
    const double* __restrict__ coef, const zc* __restrict__ orbph, const double* __restrict__ taup,
    int gauge, zc* __restrict__ H, int64_t ldH, zc* __restrict__ V, int64_t ldV) {
    __shared__ zc s_hop[RC][TE];
    __shared__ zc s_ph[RC][TK];
    __shared__ double s_coef[NP > 0 ? NP : 1][RC];
    const int tid = threadIdx.x;
    const int te = tid & 15;  // element lane: e = te + 16 j
    const int tk = tid >> 4;  // k lane: k = tk + 16 i
    const int64_t NN = (int64_t)N * N;
    const int64_t e0 = (int64_t)blockIdx.x * TE;
    const int64_t k0 = (int64_t)blockIdx.y * TK;

    zc accH[2][4];
    zc accV[NP > 0 ? NP : 1][2][4];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            accH[i][j] = mk(0.0, 0.0);
#pragma unroll
            for (int p = 0; p < NP; ++p) accV[p][i][j] = mk(0.0, 0.0);
        }

    for (int r0 = 0; r0 < nR; r0 += RC) {
        for (int idx = tid; idx < RC * TE; idx += 256) {
            const int r = idx / TE, e = idx % TE;
            zc h = mk(0.0, 0.0);
            if (r0 + r < nR && e0 + e < NN) h = hop[(int64_t)(r0 + r) * NN + e0 + e];
            s_hop[r][e] = h;
        }
        {
            const int r = tid / TK, kk = tid % TK;  // 256 == RC*TK
            zc u = mk(0.0, 0.0);
            if (r0 + r < nR && k0 + kk < nk) u = ph[(k0 + kk) * ldph + r0 + r];
            s_ph[r][kk] = u;
        }
        if (NP > 0 && tid < NP * RC) {
            const int p = tid / RC, r = tid % RC;
            s_coef[p][r] = (r0 + r < nR) ? coef[(int64_t)p * nR + r0 + r] : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < RC; ++r) {
            zc h[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) h[j] = s_hop[r][te + 16 * j];
            double c[NP > 0 ? NP : 1];
#pragma unroll
            for (int p = 0; p < NP; ++p) c[p] = s_coef[p][r];
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                const zc u = s_ph[r][tk + 16 * i];
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const zc t = u * h[j];
                    accH[i][j].re += t.re;
                    accH[i][j].im += t.im;
#pragma unroll
                    for (int p = 0; p < NP; ++p) {
                        accV[p][i][j].re = fma(c[p], t.re, accV[p][i][j].re);
                        accV[p][i][j].im = fma(c[p], t.im, accV[p][i][j].im);
                    }
                }
            }
        }
        __syncthreads();
    }

#pragma unroll
    for (int i = 0; i < 2; ++i) {
        const int64_t kk = k0 + tk + 16 * i;
        if (kk >= nk) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int64_t e = e0 + te + 16 * j;
            if (e >= NN) continue;
            const int mrow = (int)(e / N), ncol = (int)(e % N);
            const zc hl = accH[i][j];
            zc g = mk(1.0, 0.0);
            if (gauge == TBG_GAUGE_ATOM) g = cmul(orbph[kk * N + mrow], orbph[kk * N + ncol]);
            if (H) H[kk * ldH + e] = hl * g;
#pragma unroll
            for (int p = 0; p < NP; ++p) {
                // i * acc
                zc v = mk(-accV[p][i][j].im, accV[p][i][j].re);
                if (gauge == TBG_GAUGE_ATOM) {
                    const double diff = taup[p * N + ncol] - taup[p * N + mrow];
                    v.re -= diff * hl.im;
                    v.im += diff * hl.re;
                    v = v * g;
                }
                V[kk * ldV + p * NN + e] = v;
            }
        }
    }
}

// coef[p][r] = w_p . R_cart[r];  taup[p][s] = w_p . tau_cart[s]
__global__ void proj_coef_kernel(int nproj, int dim, const double* __restrict__ dirs, int nR,
                                 const double* __restrict__ Rcart, int nsta, const double* __restrict__ taucart,
                                 double* __restrict__ coef, double* __restrict__ taup) {
    const int total = nproj * (nR + nsta);
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += gridDim.x * blockDim.x) {
        const int p = idx / (nR + nsta), j = idx % (nR + nsta);
        const double* w = dirs + p * dim;
        if (j < nR) {
            const double* r = Rcart + 3 * j;
            double s = w[0] * r[0];
            if (dim > 1) s += w[1] * r[1];
            if (dim > 2) s += w[2] * r[2];
            coef[p * nR + j] = s;
        } else {
            const double* t = taucart + 3 * (j - nR);
            double s = w[0] * t[0];
            if (dim > 1) s += w[1] * t[1];
            if (dim > 2) s += w[2] * t[2];
            taup[p * nsta + (j - nR)] = s;
        }
    }
}

template <int NP>
int launch_gemm(cudaStream_t st, int64_t nk, int nR, int ldph, int N, const zc* ph, const zc* hop,
                const double* coef, const zc* orbph, const double* taup, int gauge, zc* H, int64_t ldH,
                zc* V, int64_t ldV) {
    const int64_t NN = (int64_t)N * N;
    KTimer kt(st, "fourier_gemm_kernel", 8.0 * nR * (double)NN * nk * ((H ? 1 : 0) + NP));
    for (int64_t kb = 0; kb < nk; kb += (int64_t)TK * 65535) {
        const int64_t nkb = std::min<int64_t>(nk - kb, (int64_t)TK * 65535);
        dim3 grid((unsigned)((NN + TE - 1) / TE), (unsigned)((nkb + TK - 1) / TK));
        fourier_gemm_kernel<NP><<<grid, 256, 0, st>>>(nkb, nR, ldph, N, ph + kb * ldph, hop, coef,
                                                        orbph + kb * N, taup, gauge,
                                                        H ? H + kb * ldH : nullptr, ldH,
                                                        V ? V + kb * ldV : nullptr, ldV);
        TBG_LAUNCHED("fourier_gemm_kernel");
    }
    return TBG_OK;
}

int dispatch_gemm(cudaStream_t st, int np, int64_t nk, int nR, int ldph, int N, const zc* ph, const zc* hop,
                  const double* coef, const zc* orbph, const double* taup, int gauge, zc* H, int64_t ldH,
                  zc* V, int64_t ldV) {
    switch (np) {
        case 0: return launch_gemm<0>(st, nk, nR, ldph, N, ph, hop, coef, orbph, taup, gauge, H, ldH, V, ldV);
        case 1: return launch_gemm<1>(st, nk, nR, ldph, N, ph, hop, coef, orbph, taup, gauge, H, ldH, V, ldV);
        case 2: return launch_gemm<2>(st, nk, nR, ldph, N, ph, hop, coef, orbph, taup, gauge, H, ldH, V, ldV);
        default: return launch_gemm<3>(st, nk, nR, ldph, N, ph, hop, coef, orbph, taup, gauge, H, ldH, V, ldV);
    }
}

// Fourier sums from the +-R paired table (FP64; rows 2q, 2q + 1 of T are A_q,
// B_q, pair 0 is R = 0 with A_0 = t(0), B_0 = 0): with (c, s) = (cos, sin) of
// 2 pi k . R_q,
//   H += c A_q + s B_q,   V_p += c_p(R_q) (c B_q - s A_q)   (c_p(R_0) = 0),
// 8 + 2 NP FMAs per pair and element for two R (10 + 2 NP per R unpaired).
// Same tiling and epilogue as fourier_gemm_kernel; the velocity accumulators
// already hold V_p (no factor i).
template <int NP>
__global__ void __launch_bounds__(256) fourier_pair_kernel(
    int64_t nk, int Kc, int N, const zc* __restrict__ cs, const zc* __restrict__ T, const int* __restrict__ pair,
    int nR, const double* __restrict__ coef, const zc* __restrict__ orbph, const double* __restrict__ taup,
    int gauge, zc* __restrict__ H, int64_t ldH, zc* __restrict__ V, int64_t ldV) {
    __shared__ zc s_A[RC][TE], s_B[RC][TE];
    __shared__ zc s_cs[RC][TK];
    __shared__ double s_coef[NP > 0 ? NP : 1][RC];
    const int tid = threadIdx.x;
    const int te = tid & 15;  // element lane: e = te + 16 j
    const int tk = tid >> 4;  // k lane: k = tk + 16 i
    const int64_t NN = (int64_t)N * N;
    const int64_t e0 = (int64_t)blockIdx.x * TE;
    const int64_t k0 = (int64_t)blockIdx.y * TK;

    zc accH[2][4];
    zc accV[NP > 0 ? NP : 1][2][4];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            accH[i][j] = mk(0.0, 0.0);
#pragma unroll
            for (int p = 0; p < NP; ++p) accV[p][i][j] = mk(0.0, 0.0);
        }

    for (int q0 = 0; q0 < Kc; q0 += RC) {
        for (int idx = tid; idx < RC * TE; idx += 256) {
            const int r = idx / TE, e = idx % TE;
            zc a = mk(0.0, 0.0), b = mk(0.0, 0.0);
            if (q0 + r < Kc && e0 + e < NN) {
                a = T[(int64_t)(2 * (q0 + r)) * NN + e0 + e];
                b = T[(int64_t)(2 * (q0 + r) + 1) * NN + e0 + e];
            }
            s_A[r][e] = a;
            s_B[r][e] = b;
        }
        {
            const int r = tid / TK, kk = tid % TK;  // 256 == RC*TK
            zc u = mk(0.0, 0.0);
            if (q0 + r < Kc && k0 + kk < nk) u = cs[(k0 + kk) * Kc + q0 + r];
            s_cs[r][kk] = u;
        }
        if (NP > 0 && tid < NP * RC) {
            const int p = tid / RC, r = tid % RC, q = q0 + r;
            s_coef[p][r] = (q > 0 && q < Kc) ? coef[(int64_t)p * nR + pair[q - 1]] : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < RC; ++r) {
            zc a[4], b[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                a[j] = s_A[r][te + 16 * j];
                b[j] = s_B[r][te + 16 * j];
            }
            double cp[NP > 0 ? NP : 1];
#pragma unroll
            for (int p = 0; p < NP; ++p) cp[p] = s_coef[p][r];
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                const zc u = s_cs[r][tk + 16 * i];  // (cos, sin)
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    accH[i][j].re = fma(u.re, a[j].re, accH[i][j].re);
                    accH[i][j].re = fma(u.im, b[j].re, accH[i][j].re);
                    accH[i][j].im = fma(u.re, a[j].im, accH[i][j].im);
                    accH[i][j].im = fma(u.im, b[j].im, accH[i][j].im);
                    if (NP > 0) {
                        const double wr = fma(u.re, b[j].re, -u.im * a[j].re);
                        const double wi = fma(u.re, b[j].im, -u.im * a[j].im);
#pragma unroll
                        for (int p = 0; p < NP; ++p) {
                            accV[p][i][j].re = fma(cp[p], wr, accV[p][i][j].re);
                            accV[p][i][j].im = fma(cp[p], wi, accV[p][i][j].im);
                        }
                    }
                }
            }
        }
        __syncthreads();
    }

#pragma unroll
    for (int i = 0; i < 2; ++i) {
        const int64_t kk = k0 + tk + 16 * i;
        if (kk >= nk) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int64_t e = e0 + te + 16 * j;
            if (e >= NN) continue;
            const int mrow = (int)(e / N), ncol = (int)(e % N);
            const zc hl = accH[i][j];
            zc g = mk(1.0, 0.0);
            if (gauge == TBG_GAUGE_ATOM) g = cmul(orbph[kk * N + mrow], orbph[kk * N + ncol]);
            if (H) H[kk * ldH + e] = hl * g;
#pragma unroll
            for (int p = 0; p < NP; ++p) {
                zc v = accV[p][i][j];
                if (gauge == TBG_GAUGE_ATOM) {
                    const double diff = taup[p * N + ncol] - taup[p * N + mrow];
                    v.re -= diff * hl.im;
                    v.im += diff * hl.re;
                    v = v * g;
                }
                V[kk * ldV + p * NN + e] = v;
            }
        }
    }
}

// (cos, sin) of 2 pi k . R_q per k-point and pair (pair 0: R = 0), from the
// same operation order as phases_kernel.
__global__ void phases_pair_kernel(int64_t nk, int dim, const double* __restrict__ k, int np,
                                   const int* __restrict__ pair, const int* __restrict__ hamR, zc* __restrict__ cs) {
    const int Kc = np + 1;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < nk * Kc;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t kk = idx / Kc;
        const int q = (int)(idx % Kc);
        if (q == 0) {
            cs[idx] = mk(1.0, 0.0);
            continue;
        }
        const int* r = hamR + 3 * pair[q - 1];
        const double* kv = k + kk * dim;
        double s = (double)r[0] * kv[0];
        if (dim > 1) s += (double)r[1] * kv[1];
        if (dim > 2) s += (double)r[2] * kv[2];
        double sn, c;
        sincos(kTwoPi * s, &sn, &c);
        cs[idx] = mk(c, sn);
    }
}

template <int NP>
int launch_pair(cudaStream_t st, int64_t nk, int Kc, int N, const zc* cs, const zc* T, const int* pair, int nR,
                const double* coef, const zc* orbph, const double* taup, int gauge, zc* H, int64_t ldH, zc* V,
                int64_t ldV) {
    const int64_t NN = (int64_t)N * N;
    // algorithmic work as for the unpaired sum (8 nR N^2 per output matrix)
    KTimer kt(st, "fourier_gemm_kernel", 8.0 * nR * (double)NN * nk * ((H ? 1 : 0) + NP));
    for (int64_t kb = 0; kb < nk; kb += (int64_t)TK * 65535) {
        const int64_t nkb = std::min<int64_t>(nk - kb, (int64_t)TK * 65535);
        dim3 grid((unsigned)((NN + TE - 1) / TE), (unsigned)((nkb + TK - 1) / TK));
        fourier_pair_kernel<NP><<<grid, 256, 0, st>>>(nkb, Kc, N, cs + kb * Kc, T, pair, nR, coef, orbph + kb * N,
                                                        taup, gauge, H ? H + kb * ldH : nullptr, ldH,
                                                        V ? V + kb * ldV : nullptr, ldV);
        TBG_LAUNCHED("fourier_pair_kernel");
    }
    return TBG_OK;
}

int dispatch_pair(cudaStream_t st, int np, int64_t nk, int Kc, int N, const zc* cs, const zc* T, const int* pair,
                  int nR, const double* coef, const zc* orbph, const double* taup, int gauge, zc* H, int64_t ldH,
                  zc* V, int64_t ldV) {
    switch (np) {
        case 0: return launch_pair<0>(st, nk, Kc, N, cs, T, pair, nR, coef, orbph, taup, gauge, H, ldH, V, ldV);
        case 1: return launch_pair<1>(st, nk, Kc, N, cs, T, pair, nR, coef, orbph, taup, gauge, H, ldH, V, ldV);
        case 2: return launch_pair<2>(st, nk, Kc, N, cs, T, pair, nR, coef, orbph, taup, gauge, H, ldH, V, ldV);
        default: return launch_pair<3>(st, nk, Kc, N, cs, T, pair, nR, coef, orbph, taup, gauge, H, ldH, V, ldV);
    }
}

// Gauge transform + zeroed diagonal of the rmatrix Fourier sum (Atom gauge),
// velocity.rs:646-656.
__global__ void rmat_gauge_kernel(int64_t nk, int N, const zc* __restrict__ orbph, zc* __restrict__ A) {
    const int64_t NN = (int64_t)N * N;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < nk * NN;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t kk = idx / NN;
        const int e = (int)(idx % NN), m = e / N, n = e % N;
        zc a = A[idx];
        if (m == n) {
            a = mk(0.0, 0.0);
        } else {
            a = a * cmul(orbph[kk * N + m], orbph[kk * N + n]);
        }
        A[idx] = a;
    }
}

// V[k] += i (H A - A H) for one k per block row tile; simple tiled FP64 GEMM.
__global__ void __launch_bounds__(256) commutator_kernel(int N, const zc* __restrict__ H, int64_t ldH,
                                                         const zc* __restrict__ A, zc* __restrict__ V,
                                                         int64_t ldV) {
    const int64_t kk = blockIdx.z;
    const zc* Hk = H + kk * ldH;
    const zc* Ak = A + kk * (int64_t)N * N;
    zc* Vk = V + kk * ldV;
    __shared__ zc sH[16][17], sA[16][17], sA2[16][17], sH2[16][17];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int row = blockIdx.y * 16 + ty, col = blockIdx.x * 16 + tx;
    zc acc = mk(0.0, 0.0);
    for (int t0 = 0; t0 < N; t0 += 16) {
        // (H A)[row][col] = sum_l H[row][l] A[l][col];  (A H)[row][col] = sum_l A[row][l] H[l][col]
        sH[ty][tx] = (row < N && t0 + tx < N) ? Hk[(int64_t)row * N + t0 + tx] : mk(0.0, 0.0);
        sA2[ty][tx] = (row < N && t0 + tx < N) ? Ak[(int64_t)row * N + t0 + tx] : mk(0.0, 0.0);
        sA[ty][tx] = (t0 + ty < N && col < N) ? Ak[(int64_t)(t0 + ty) * N + col] : mk(0.0, 0.0);
        sH2[ty][tx] = (t0 + ty < N && col < N) ? Hk[(int64_t)(t0 + ty) * N + col] : mk(0.0, 0.0);
        __syncthreads();
#pragma unroll
        for (int l = 0; l < 16; ++l) {
            fma_cx(acc, sH[ty][l], sA[l][tx]);
            const zc t = sA2[ty][l] * sH2[l][tx];
            acc.re -= t.re;
            acc.im -= t.im;
        }
        __syncthreads();
    }
    if (row < N && col < N) {
        zc v = Vk[(int64_t)row * N + col];
        v.re -= acc.im;
        v.im += acc.re;
        Vk[(int64_t)row * N + col] = v;
    }
}

// combined rmatrix table for projection p: rm_p[r][e] = sum_d w_pd rmatrix[r][d][e]
__global__ void rmat_combine_kernel(int64_t n_rmat, int dim, int N, const double* __restrict__ w,
                                    const zc* __restrict__ rm, zc* __restrict__ out) {
    const int64_t NN = (int64_t)N * N;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < n_rmat * NN;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = idx / NN, e = idx % NN;
        zc s = mk(0.0, 0.0);
        for (int d = 0; d < dim; ++d) {
            const zc a = rm[(r * dim + d) * NN + e];
            s.re += w[d] * a.re;
            s.im += w[d] * a.im;
        }
        out[idx] = s;
    }
}

// ph3 rows: [0, nk) = u(k,R); [nk, 2nk) = i c_0(R) u; [2nk, 3nk) = i c_1(R) u.
__global__ void phases3_kernel(int64_t nk, int dim, const double* __restrict__ k, int nR,
                               const int* __restrict__ hamR, const double* __restrict__ coef,
                               zc* __restrict__ ph3) {
    const int64_t total = nk * (int64_t)nR;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t kk = idx / nR;
        const int j = (int)(idx % nR);
        const double* kv = k + kk * dim;
        const int* r = hamR + 3 * j;
        double s = (double)r[0] * kv[0];
        if (dim > 1) s += (double)r[1] * kv[1];
        if (dim > 2) s += (double)r[2] * kv[2];
        double sn, cs;
        sincos(kTwoPi * s, &sn, &cs);
        ph3[idx] = mk(cs, sn);
        const double c0 = coef[j], c1 = coef[nR + j];
        ph3[total + idx] = mk(-c0 * sn, c0 * cs);      // i c0 u
        ph3[2 * total + idx] = mk(-c1 * sn, c1 * cs);  // i c1 u
    }
}

// Atom gauge and tau term from the lattice-gauge float-pair sums:
//   H = conj(phi_m) H_l phi_n,  V_p = (V_l,p + i (tau_p,n - tau_p,m) H_l) conj(phi_m) phi_n
// Contraction output C, component c (0: H, 1, 2: V_p) of k-point kk, element
// (m, n): full N x N columns, or only the upper triangle (packed row by row);
// then the lower triangle is the conjugate of its mirror (H and V_p are Hermitian).
__host__ __device__ __forceinline__ int64_t upper_index(int N, int m, int n) {
    return (int64_t)m * N - (int64_t)m * (m - 1) / 2 + (n - m);
}
__device__ __forceinline__ float4 c_elem(const float4* __restrict__ C, bool packed, int64_t nk, int N, int c,
                                         int64_t kk, int m, int n) {
    if (!packed) return C[(c * nk + kk) * (int64_t)N * N + (int64_t)m * N + n];
    const int64_t np = (int64_t)N * (N + 1) / 2;
    if (m <= n) return C[(c * nk + kk) * np + upper_index(N, m, n)];
    const float4 v = C[(c * nk + kk) * np + upper_index(N, n, m)];
    return make_float4(v.x, v.y, -v.z, -v.w);
}

__global__ void gauge_pairs_kernel(int64_t nk, int N, const float4* __restrict__ C, bool packed,
                                   const zc* __restrict__ orbph, const double* __restrict__ taup, zc* __restrict__ H,
                                   zc* __restrict__ V) {
    const int64_t NN = (int64_t)N * N;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < nk * NN;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t kk = idx / NN;
        const int e = (int)(idx % NN), mrow = e / N, ncol = e % N;
        const float4 h4 = c_elem(C, packed, nk, N, 0, kk, mrow, ncol);
        const zc hl = mk((double)h4.x + (double)h4.y, (double)h4.z + (double)h4.w);
        const zc g = cmul(orbph[kk * N + mrow], orbph[kk * N + ncol]);
        H[idx] = hl * g;
#pragma unroll
        for (int p = 0; p < 2; ++p) {
            const float4 v4 = c_elem(C, packed, nk, N, 1 + p, kk, mrow, ncol);
            zc v = mk((double)v4.x + (double)v4.y, (double)v4.z + (double)v4.w);
            const double diff = taup[p * N + ncol] - taup[p * N + mrow];
            v.re -= diff * hl.im;
            v.im += diff * hl.re;
            V[kk * 2 * NN + p * NN + e] = v * g;
        }
    }
}

// taup (FP64) -> float pairs
__global__ void tau_split_kernel(int n, const double* __restrict__ taup, float2* __restrict__ tau2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) tau2[i] = df_of(taup[i]);
}

// Lattice gauge, float-pair arithmetic, in place on the contraction output:
//   V_p += i (tau_p,n - tau_p,m) H_l   (velocity.rs:602-610 before the phase).
// The Atom-gauge phase conj(phi_m) phi_n is a diagonal unitary similarity
// (H_atom = P^H H_l P, V_atom = P^H V_l P), so energies and band-basis
// velocities, hence Omega, do not depend on it; the mixed path skips it.
__global__ void tau_pairs_kernel(int64_t nk, int N, float4* __restrict__ C, const float2* __restrict__ tau2) {
    const int64_t NN = (int64_t)N * N;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= NN) return;
    const int mrow = e / N, ncol = e - mrow * N;
    float2 d[2];
#pragma unroll
    for (int p = 0; p < 2; ++p) d[p] = df_add(tau2[p * N + ncol], df_neg(tau2[p * N + mrow]));
    for (int64_t kk = blockIdx.y; kk < nk; kk += gridDim.y) {
        const int64_t idx = kk * NN + e;
        const float4 h = C[idx];
        const float2 hr = make_float2(h.x, h.y), hi = make_float2(h.z, h.w);
#pragma unroll
        for (int p = 0; p < 2; ++p) {
            float4* vp = C + (1 + p) * nk * NN + idx;
            const float4 v = *vp;
            const float2 vr = df_add(make_float2(v.x, v.y), df_neg(df_mul(d[p], hi)));
            const float2 vi = df_add(make_float2(v.z, v.w), df_mul(d[p], hr));
            *vp = make_float4(vr.x, vr.y, vi.x, vi.y);
        }
    }
}

// Packed upper-triangle contraction output -> full float-pair H, V_0, V_1
// (P: three blocks of nk N^2 elements, blk elements apart) with the
// orbital-position term V_p += i (tau_p,n - tau_p,m) H, in float-pair arithmetic.
// With rexp (three blocks of nk N ints) the row exponents of the three written
// matrices come out too: when a block of 256 threads holds whole rows (N a
// multiple of 32 dividing 256) each warp's maximum goes through shared memory
// and the row's exponent is stored; otherwise rexp is preset below every
// exponent and the maxima are folded in by atomicMax, one per warp when N is
// a multiple of 32 (a warp then lies in one row), else per lane.
constexpr int kUnpackThreads = 256;
__host__ __device__ constexpr bool unpack_block_rows(int N) { return (N & 31) == 0 && kUnpackThreads % N == 0; }

__global__ void __launch_bounds__(kUnpackThreads) unpack_tau_kernel(int64_t nk, int N, const float4* __restrict__ Cp,
                                                                   const float2* __restrict__ tau2,
                                                                   float4* __restrict__ P, int64_t blk,
                                                                   int* __restrict__ rexp) {
    const int64_t NN = (int64_t)N * N;
    const int e = blockIdx.x * kUnpackThreads + threadIdx.x;
    const bool valid = e < NN;
    const int mrow = valid ? e / N : 0, ncol = valid ? e - mrow * N : 0;
    const bool warp_row = (N & 31) == 0, block_rows = unpack_block_rows(N);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __shared__ int wmax[2][3][kUnpackThreads / 32];
    float2 d[2];
#pragma unroll
    for (int p = 0; p < 2; ++p) d[p] = df_add(tau2[p * N + ncol], df_neg(tau2[p * N + mrow]));
    int par = 0;  // alternates per k-point of this block
    for (int64_t kk = blockIdx.y; kk < nk; kk += gridDim.y, par ^= 1) {
        float mag[3] = {0.f, 0.f, 0.f};
        if (valid) {
            const float4 h = c_elem(Cp, true, nk, N, 0, kk, mrow, ncol);
            P[kk * NN + e] = h;
            mag[0] = pair_mag(h);
            const float2 hr = make_float2(h.x, h.y), hi = make_float2(h.z, h.w);
#pragma unroll
            for (int p = 0; p < 2; ++p) {
                const float4 v = c_elem(Cp, true, nk, N, 1 + p, kk, mrow, ncol);
                const float2 vr = df_add(make_float2(v.x, v.y), df_neg(df_mul(d[p], hi)));
                const float2 vi = df_add(make_float2(v.z, v.w), df_mul(d[p], hr));
                const float4 o = make_float4(vr.x, vr.y, vi.x, vi.y);
                P[(1 + p) * blk + kk * NN + e] = o;
                mag[1 + p] = pair_mag(o);
            }
        }
        if (rexp) {
            // magnitudes are >= 0 (NaN counts as 0, as fmaxf over a row would
            // skip it), so their bit patterns order as integers
#pragma unroll
            for (int c = 0; c < 3; ++c) mag[c] = (mag[c] == mag[c]) ? mag[c] : 0.f;
            if (block_rows) {
                // every thread is valid (NN is a multiple of 256); the buffer
                // alternates per k-point, so one barrier per k-point suffices
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const int v = __reduce_max_sync(0xffffffffu, __float_as_int(mag[c]));
                    if (lane == 0) wmax[par][c][warp] = v;
                }
                __syncthreads();
                const int rows = kUnpackThreads / N, wpr = N / 32;
                if (threadIdx.x < 3 * rows) {
                    const int c = threadIdx.x / rows, rr = threadIdx.x - c * rows;
                    int v = 0;
                    for (int w = rr * wpr; w < (rr + 1) * wpr; ++w) v = max(v, wmax[par][c][w]);
                    rexp[(c * nk + kk) * N + blockIdx.x * rows + rr] = line_exp_of(__int_as_float(v));
                }
            } else if (warp_row) {  // NN and the warps' starts are multiples of 32: all lanes valid or none
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const int v = __reduce_max_sync(0xffffffffu, __float_as_int(mag[c]));
                    if (valid && lane == 0) atomicMax(&rexp[(c * nk + kk) * N + mrow], line_exp_of(__int_as_float(v)));
                }
            } else if (valid) {
#pragma unroll
                for (int c = 0; c < 3; ++c) atomicMax(&rexp[(c * nk + kk) * N + mrow], line_exp_of(mag[c]));
            }
        }
    }
}

std::mutex g_hop_mu;

}  // namespace

int ozaki_fourier_max_k();
size_t ozaki_hop_slices_bytes(int K, int64_t Nc);
int ozaki_build_hop_slices_real(cudaStream_t st, int Kc, int64_t Nc, const zc* T, int* EB, void* Bs,
                                const int* colmap, int64_t ncols);
int ozaki_build_hop_slices(cudaStream_t st, int K, int64_t Nc, const zc* ham, int* EB, void* Bs, const int* colmap,
                           int64_t ncols);
int ozaki_fourier(cudaStream_t st, int64_t M, int64_t Nc, int K, const zc* A, int* EA, const int* EB,
                  const void* Bs, float4* C, int* err, int64_t high_rows, void* aimg);
size_t ozaki_fourier_img_bytes(int64_t M, int K);

// Class of the velocity rows of the exact-slice Fourier sum: MID (five digits,
// about 2^-35 of the row scale; the velocities only enter the rotation, which
// is a MID product itself) unless TBG_FOURIER_V_HIGH=1.  The Hamiltonian rows
// stay HIGH.
static bool fourier_v_mid() {
    static const bool mid = [] {
        const char* e = std::getenv("TBG_FOURIER_V_HIGH");
        return !(e && e[0] == '1');
    }();
    return mid;
}

bool fourier_mixed_ok(const ModelDev& m) { return m.nR <= ozaki_fourier_max_k(); }

size_t fourier_mixed_scratch_bytes(const ModelDev& m, int64_t nk) {
    const size_t N = (size_t)m.nsta, nR = (size_t)m.nR;
    // phases, orbital phases, exponents; the packed (upper-triangle) contraction
    // output; the phases' stage images
    return (size_t)nk * (3 * (nR + 1) * sizeof(zc) + N * sizeof(zc) + 3 * sizeof(int) +
                         3 * (N * (N + 1) / 2) * sizeof(float4)) +
           ozaki_fourier_img_bytes(3 * nk, (int)nR + 1) + 2 * nR * sizeof(double) + 2 * N * sizeof(double) +
           2 * N * sizeof(float2) + 11 * 256;
}

namespace {

// Phases and the tensor-core contraction: C (3 nk N^2 float pairs) = lattice-
// gauge H, V_0, V_1 without the orbital-position term.  orbph (nk, N) and
// taup (2, N) are left in the scratch for the gauge step.
// With the tcgen05 kernels the contraction covers only the upper-triangle
// elements (m <= n) of H and V_p, which are Hermitian: N(N+1)/2 columns, written
// packed to *Cg in the scratch; otherwise all N^2 columns are written to C.
__global__ void gather_exps_kernel(int64_t n, const int* __restrict__ idx, const int* __restrict__ src,
                                   int* __restrict__ dst) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        dst[i] = src[idx[i]];
}

// The table paired over +-R for real coefficients: with theta = 2 pi k . R,
//   t(R) e^{i theta} + t(-R) e^{-i theta} = A cos(theta) + B sin(theta),
//   A = t(R) + t(-R),  B = i (t(R) - t(-R))
// (an R without its -R partner takes t(-R) = 0).  Rows: 0 = t(0), 1 = 0,
// 2 + 2p = A_p, 3 + 2p = B_p.  pi[p] is the pair's R, pj[p] its -R or -1.
// A non-finite entry sets *nonfinite (the exact-slice digits of the
// tensor-core form cannot carry NaN or Inf, so the mixed path refuses such a
// table up front).
__global__ void pair_table_kernel(int np, const int* __restrict__ pi, const int* __restrict__ pj, int z, int64_t NN,
                                  const zc* __restrict__ ham, zc* __restrict__ T, int* __restrict__ nonfinite) {
    const int64_t total = (int64_t)(np + 1) * NN;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t p = idx / NN - 1, e = idx % NN;
        zc a, b;
        if (p < 0) {
            a = (z >= 0) ? ham[(int64_t)z * NN + e] : mk(0.0, 0.0);
            b = mk(0.0, 0.0);
            T[e] = a;
            T[NN + e] = b;
        } else {
            a = ham[(int64_t)pi[p] * NN + e];
            b = (pj[p] >= 0) ? ham[(int64_t)pj[p] * NN + e] : mk(0.0, 0.0);
            T[(2 + 2 * p) * NN + e] = mk(a.re + b.re, a.im + b.im);
            T[(3 + 2 * p) * NN + e] = mk(-(a.im - b.im), a.re - b.re);
        }
        if (!(isfinite(a.re) && isfinite(a.im) && isfinite(b.re) && isfinite(b.im))) atomicOr(nonfinite, 1);
    }
}

// Real coefficients of the paired table, as complex numbers whose real and
// imaginary parts are consecutive rows (Phi (3, nk, Kc), Kc = 1 + np): H row
// (1, 0 | cos, sin ...), V_p rows (0, 0 | -c_p(R) sin, c_p(R) cos ...), from
//   i c_p(R) (t(R) e^{i theta} - t(-R) e^{-i theta}) = c_p(R) (B cos - A sin).
__global__ void phases_real_kernel(int64_t nk, int dim, const double* __restrict__ k, int np,
                                   const int* __restrict__ pair, const int* __restrict__ hamR, int nR,
                                   const double* __restrict__ coef, zc* __restrict__ Phi) {
    const int Kc = np + 1;
    const int64_t total = nk * (int64_t)Kc;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t kk = idx / Kc;
        const int c = (int)(idx % Kc);
        zc h = mk(1.0, 0.0), vx = mk(0.0, 0.0), vy = mk(0.0, 0.0);
        if (c > 0) {
            const int j = pair[c - 1];
            const int* r = hamR + 3 * j;
            const double* kv = k + kk * dim;
            // same operation order as the reference: r0*k0 + r1*k1 + r2*k2
            double s = (double)r[0] * kv[0];
            if (dim > 1) s += (double)r[1] * kv[1];
            if (dim > 2) s += (double)r[2] * kv[2];
            double sn, cs;
            sincos(kTwoPi * s, &sn, &cs);
            const double c0 = coef[j], c1 = coef[nR + j];
            h = mk(cs, sn);
            vx = mk(-c0 * sn, c0 * cs);
            vy = mk(-c1 * sn, c1 * cs);
        }
        Phi[idx] = h;
        Phi[total + idx] = vx;
        Phi[2 * total + idx] = vy;
    }
}

// The +-R paired table (pair_table_kernel) and the index of each pair's R,
// built once per model for both Fourier forms; the caller holds g_hop_mu.
int ensure_pair_table(ModelDev& m, cudaStream_t st) {
    if (m.pair_T) return TBG_OK;
    const int nR = (int)m.nR;
    const int64_t NN = (int64_t)m.nsta * m.nsta;
    int z = -1;
    std::vector<int> pi, pj;
    std::vector<char> used((size_t)nR, 0);
    auto rvec = [&](int i, int d) { return d < m.dim ? m.hamR[(size_t)i * m.dim + d] : (int64_t)0; };
    for (int i = 0; i < nR; ++i) {
        if (used[i]) continue;
        used[i] = 1;
        if (rvec(i, 0) == 0 && rvec(i, 1) == 0 && rvec(i, 2) == 0 && z < 0) {
            z = i;  // a repeated R = 0 entry is paired below as a singleton (theta = 0)
            continue;
        }
        int partner = -1;
        for (int j = i + 1; j < nR && partner < 0; ++j)
            if (!used[j] && rvec(j, 0) == -rvec(i, 0) && rvec(j, 1) == -rvec(i, 1) && rvec(j, 2) == -rvec(i, 2))
                partner = j;
        if (partner >= 0) used[partner] = 1;
        pi.push_back(i);
        pj.push_back(partner);
    }
    const int np = (int)pi.size(), Kc = np + 1;
    int *pair_d = nullptr, *pj_d = nullptr;
    zc* T = nullptr;
    int rc = TBG_OK;
    if (cudaMalloc(&T, sizeof(zc) * 2 * (size_t)Kc * NN) != cudaSuccess ||
        cudaMalloc(&pair_d, sizeof(int) * std::max(np, 1)) != cudaSuccess ||
        cudaMalloc(&pj_d, sizeof(int) * (std::max(np, 1) + 1)) != cudaSuccess)
        rc = set_error(TBG_E_OOM, "paired hop table");
    int* nonfinite_d = pj_d + std::max(np, 1);
    if (!rc && cudaMemsetAsync(nonfinite_d, 0, sizeof(int), st) != cudaSuccess)
        rc = set_error(TBG_E_CUDA, "paired hop table flag");
    if (!rc && np > 0 &&
        (cudaMemcpy(pair_d, pi.data(), sizeof(int) * np, cudaMemcpyHostToDevice) != cudaSuccess ||
         cudaMemcpy(pj_d, pj.data(), sizeof(int) * np, cudaMemcpyHostToDevice) != cudaSuccess))
        rc = set_error(TBG_E_CUDA, "paired hop table indices");
    if (!rc) {
        pair_table_kernel<<<(unsigned)std::min<int64_t>(((int64_t)Kc * NN + 255) / 256, 152 * 64), 256, 0, st>>>(
            np, pair_d, pj_d, z, NN, m.ham, T, nonfinite_d);
        count_launch();
        int nf = 0;
        cudaError_t e = cudaMemcpyAsync(&nf, nonfinite_d, sizeof(int), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // other streams use the table next
        if (e != cudaSuccess) rc = cuda_error(e, "paired hop table");
        m.nonfinite = nf != 0;
    }
    cudaFree(pj_d);
    if (rc) {
        cudaFree(T);
        cudaFree(pair_d);
        return rc;
    }
    m.pair_T = T;
    m.hop_pair_d = pair_d;
    m.hop_np = np;
    m.hop_K = Kc;
    return TBG_OK;
}

int build_hop_table(ModelDev& m, cudaStream_t st) {
    const int N = (int)m.nsta, nR = (int)m.nR;
    const int64_t NN = (int64_t)N * N, NP = (int64_t)N * (N + 1) / 2;
    const bool packed = ozaki_use_tc();
    const int64_t ncols = packed ? NP : NN;
    if (packed) {
        int rc = ensure_pair_table(m, st);
        if (rc) return rc;
    }
    const int Kc = packed ? m.hop_K : nR;
    const zc* T = m.pair_T;
    void* bs = nullptr;
    int *eb_full = nullptr, *eb = nullptr, *colmap = nullptr;
    int rc = TBG_OK;
    if (cudaMalloc(&bs, ozaki_hop_slices_bytes(Kc, ncols)) != cudaSuccess) return set_error(TBG_E_OOM, "hop table digit planes");
    if (cudaMalloc(&eb_full, sizeof(int) * NN) != cudaSuccess ||
        (packed && (cudaMalloc(&eb, sizeof(int) * NP) != cudaSuccess ||
                    cudaMalloc(&colmap, sizeof(int) * NP) != cudaSuccess)))
        rc = set_error(TBG_E_OOM, "hop table digit planes");
    if (!rc && packed) {
        std::vector<int> cm((size_t)NP);
        for (int a = 0; a < N; ++a)
            for (int b = a; b < N; ++b) cm[(size_t)upper_index(N, a, b)] = a * N + b;
        if (cudaMemcpy(colmap, cm.data(), sizeof(int) * NP, cudaMemcpyHostToDevice) != cudaSuccess)
            rc = set_error(TBG_E_CUDA, "hop table column map");
    }
    if (!rc)
        rc = packed ? ozaki_build_hop_slices_real(st, Kc, NN, T, eb_full, bs, colmap, ncols)
                    : ozaki_build_hop_slices(st, nR, NN, m.ham, eb_full, bs, nullptr, ncols);
    if (!rc && packed) {
        gather_exps_kernel<<<(unsigned)std::min<int64_t>((NP + 255) / 256, 1024), 256, 0, st>>>(NP, colmap, eb_full,
                                                                                                  eb);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) rc = cuda_error(e, "hop table exponents");
    }
    if (!rc) {
        cudaError_t e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) rc = cuda_error(e, "hop table digit planes");
    }
    cudaFree(colmap);
    if (rc) {
        cudaFree(bs);
        cudaFree(eb_full);
        cudaFree(eb);
        return rc;
    }
    if (packed) cudaFree(eb_full);
    m.hop_slices = bs;
    m.hop_EB = packed ? eb : eb_full;
    m.hop_packed = packed;
    return TBG_OK;
}

int fourier_mixed_gemm(ModelDev& m, cudaStream_t st, int64_t nk, const double* k_d, const double* dirs_d, float4* C,
                       void* scratch, zc** orbph_out, double** taup_out, float2** tau2_out, float4** Cg_out) {
    const int N = (int)m.nsta, nR = (int)m.nR;
    const int64_t NN = (int64_t)N * N, NP = (int64_t)N * (N + 1) / 2;
    {
        std::lock_guard<std::mutex> lk(g_hop_mu);
        if (!m.hop_slices) {
            int rc = build_hop_table(m, st);
            if (rc) return rc;
        }
    }
    if (m.nonfinite) return set_error(TBG_E_NOCONV, "the hopping table contains NaN or Inf");
    unsigned char* p = static_cast<unsigned char*>(scratch);
    auto take = [&](size_t bytes) {
        void* q = p;
        p += (bytes + 255) & ~size_t(255);
        return q;
    };
    zc* ph3 = static_cast<zc*>(take(sizeof(zc) * 3 * nk * (nR + 1)));  // Phi (3 nk x hop_K <= nR + 1) when packed
    zc* orbph = static_cast<zc*>(take(sizeof(zc) * nk * N));
    double* coef = static_cast<double*>(take(sizeof(double) * 2 * nR));
    double* taup = static_cast<double*>(take(sizeof(double) * 2 * N));
    float2* tau2 = static_cast<float2*>(take(sizeof(float2) * 2 * N));
    int* EA = static_cast<int*>(take(sizeof(int) * 3 * nk));
    int* err = static_cast<int*>(take(sizeof(int)));
    float4* Cpk = static_cast<float4*>(take(sizeof(float4) * 3 * nk * NP));
    void* aimg = take(ozaki_fourier_img_bytes(3 * nk, m.hop_packed ? m.hop_K : nR));
    float4* Cg = m.hop_packed ? Cpk : C;
    {
        KTimer kt(st, "phases_kernel");
        const int total = 2 * (nR + N);
        proj_coef_kernel<<<(total + 255) / 256, 256, 0, st>>>(2, m.dim, dirs_d, nR, m.Rcart_d, N, m.taucart_d, coef,
                                                              taup);
        if (m.hop_packed) {
            // orbital phases only, then the real coefficients of the paired table
            const int64_t t1 = nk * (int64_t)N;
            phases_kernel<<<(unsigned)std::min<int64_t>((t1 + 255) / 256, 65535 * 8), 256, 0, st>>>(
                nk, m.dim, k_d, 0, m.hamR_d, N, m.tau_d, ph3, orbph);
            const int64_t t2 = nk * (int64_t)m.hop_K;
            phases_real_kernel<<<(unsigned)std::min<int64_t>((t2 + 255) / 256, 65535 * 8), 256, 0, st>>>(
                nk, m.dim, k_d, m.hop_np, m.hop_pair_d, m.hamR_d, nR, coef, ph3);
        } else {
            const int64_t t1 = nk * (int64_t)(nR + N);
            phases_kernel<<<(unsigned)std::min<int64_t>((t1 + 255) / 256, 65535 * 8), 256, 0, st>>>(
                nk, m.dim, k_d, nR, m.hamR_d, N, m.tau_d, ph3, orbph);  // ph3[0 .. nk*nR) reused below
            const int64_t t2 = nk * (int64_t)nR;
            phases3_kernel<<<(unsigned)std::min<int64_t>((t2 + 255) / 256, 65535 * 8), 256, 0, st>>>(
                nk, m.dim, k_d, nR, m.hamR_d, coef, ph3);
        }
        tau_split_kernel<<<(2 * N + 255) / 256, 256, 0, st>>>(2 * N, taup, tau2);
        count_launch(4);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return cuda_error(e, "phases");
    }
    int rc = cudaMemsetAsync(err, 0, sizeof(int), st) == cudaSuccess ? TBG_OK : set_error(TBG_E_CUDA, "memset");
    if (rc) return rc;
    // rows [H | Vx | Vy] (nk each): H in the HIGH class, the velocities in MID
    rc = ozaki_fourier(st, 3 * nk, m.hop_packed ? NP : NN, m.hop_packed ? m.hop_K : nR, ph3, EA, m.hop_EB,
                       m.hop_slices, Cg, err, fourier_v_mid() ? nk : -1, aimg);
    if (rc) return rc;
    *Cg_out = Cg;
    *orbph_out = orbph;
    *taup_out = taup;
    *tau2_out = tau2;
    return TBG_OK;
}

}  // namespace

int fourier_mixed(ModelDev& m, cudaStream_t st, int64_t nk, const double* k_d, const double* dirs_d, zc* H, zc* V,
                  float4* C, void* scratch, size_t scratch_bytes) {
    if (nk <= 0) return TBG_OK;
    const int N = (int)m.nsta;
    const int64_t NN = (int64_t)N * N;
    if (!fourier_mixed_ok(m) || !C || scratch_bytes < fourier_mixed_scratch_bytes(m, nk))
        return fourier_direct(m, st, nk, k_d, TBG_GAUGE_ATOM, 2, dirs_d, H, V, NN, 2 * NN);
    zc* orbph;
    double* taup;
    float2* tau2;
    float4* Cg;
    int rc = fourier_mixed_gemm(m, st, nk, k_d, dirs_d, C, scratch, &orbph, &taup, &tau2, &Cg);
    if (rc) return rc;
    KTimer kt(st, "gauge_pairs_kernel");
    gauge_pairs_kernel<<<(unsigned)std::min<int64_t>((nk * NN + 255) / 256, 152 * 64), 256, 0, st>>>(
        nk, N, Cg, m.hop_packed, orbph, taup, H, V);
    TBG_LAUNCHED("gauge_pairs_kernel");
    return TBG_OK;
}

int fourier_mixed_packed(ModelDev& m, cudaStream_t st, bool* packed) {
    std::lock_guard<std::mutex> lk(g_hop_mu);
    if (!m.hop_slices) {
        int rc = build_hop_table(m, st);
        if (rc) return rc;
    }
    *packed = m.hop_packed;
    return TBG_OK;
}

int fourier_mixed_pairs(ModelDev& m, cudaStream_t st, int64_t nk, const double* k_d, const double* dirs_d,
                        float4* C, void* scratch, size_t scratch_bytes, float4* out, int64_t blk, int* rexp,
                        bool* rexp_filled) {
    if (rexp_filled) *rexp_filled = false;
    if (nk <= 0) return TBG_OK;
    if (!fourier_mixed_ok(m) || scratch_bytes < fourier_mixed_scratch_bytes(m, nk))
        return set_error(TBG_E_UNSUPPORTED, "fourier_mixed_pairs: nR beyond the exact contraction length");
    const int N = (int)m.nsta;
    const int64_t NN = (int64_t)N * N;
    if (!out) {
        out = C;
        blk = nk * NN;
    }
    zc* orbph;
    double* taup;
    float2* tau2;
    float4* Cg;
    int rc = fourier_mixed_gemm(m, st, nk, k_d, dirs_d, C, scratch, &orbph, &taup, &tau2, &Cg);
    if (rc) return rc;
    KTimer kt(st, "tau_pairs_kernel");
    dim3 grid((unsigned)((NN + 255) / 256), (unsigned)std::min<int64_t>(nk, 65535));
    if (m.hop_packed) {
        if (rexp) {
            // below every exponent (0x80808080), so each row's first atomicMax sets it
            if (!unpack_block_rows(N))
                TBG_CUDA(cudaMemsetAsync(rexp, 0x80, sizeof(int) * 3 * (size_t)nk * N, st));
            if (rexp_filled) *rexp_filled = true;
        }
        unpack_tau_kernel<<<grid, kUnpackThreads, 0, st>>>(nk, N, Cg, tau2, out, blk, rexp);
        TBG_LAUNCHED("unpack_tau_kernel");
    } else {
        tau_pairs_kernel<<<grid, 256, 0, st>>>(nk, N, C, tau2);
        TBG_LAUNCHED("tau_pairs_kernel");
        if (out != C)
            for (int p = 0; p < 3; ++p)
                TBG_CUDA(cudaMemcpyAsync(out + p * blk, C + p * nk * NN, sizeof(float4) * nk * NN,
                                         cudaMemcpyDeviceToDevice, st));
    }
    return TBG_OK;
}

int fourier_direct(const ModelDev& m, cudaStream_t st, int64_t nk, const double* k_d, int gauge, int nproj,
                   const double* dirs_d, zc* H, zc* V, int64_t ldH, int64_t ldV) {
    if (nk <= 0) return TBG_OK;
    const int N = (int)m.nsta, nR = (int)m.nR;
    {
        // the +-R paired table, built once per model (a cache: logically const)
        std::lock_guard<std::mutex> lk(g_hop_mu);
        int rc = ensure_pair_table(const_cast<ModelDev&>(m), st);
        if (rc) return rc;
    }
    const int Kc = m.hop_K;
    zc *cs = nullptr, *orbph = nullptr;
    double *coef = nullptr, *taup = nullptr;
    TBG_CUDA(cudaMallocAsync(&cs, sizeof(zc) * nk * Kc, st));
    TBG_CUDA(cudaMallocAsync(&orbph, sizeof(zc) * nk * N, st));
    const int npc = std::max(nproj, 1);
    TBG_CUDA(cudaMallocAsync(&coef, sizeof(double) * npc * nR, st));
    TBG_CUDA(cudaMallocAsync(&taup, sizeof(double) * npc * N, st));
    int rc = TBG_OK;
    {
        KTimer kt(st, "phases_kernel");
        const int64_t t1 = nk * (int64_t)N;  // orbital phases only
        phases_kernel<<<(unsigned)std::min<int64_t>((t1 + 255) / 256, 65535 * 8), 256, 0, st>>>(
            nk, m.dim, k_d, 0, m.hamR_d, N, m.tau_d, cs, orbph);
        const int64_t t2 = nk * (int64_t)Kc;
        phases_pair_kernel<<<(unsigned)std::min<int64_t>((t2 + 255) / 256, 65535 * 8), 256, 0, st>>>(
            nk, m.dim, k_d, m.hop_np, m.hop_pair_d, m.hamR_d, cs);
        count_launch(2);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) rc = cuda_error(e, "phases_kernel");
    }
    if (rc == TBG_OK && nproj > 0) {
        const int total = nproj * (nR + N);
        proj_coef_kernel<<<(total + 255) / 256, 256, 0, st>>>(nproj, m.dim, dirs_d, nR, m.Rcart_d, N,
                                                              m.taucart_d, coef, taup);
        count_launch();
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) rc = cuda_error(e, "proj_coef_kernel");
    }
    // H together with up to 3 projections per pass
    for (int p0 = 0; rc == TBG_OK && (p0 < nproj || (p0 == 0 && nproj == 0)); p0 += 3) {
        const int np = std::min(3, std::max(0, nproj - p0));
        zc* Hout = (p0 == 0) ? H : nullptr;
        if (!Hout && np == 0) break;
        rc = dispatch_pair(st, np, nk, Kc, N, cs, m.pair_T, m.hop_pair_d, nR, coef + (int64_t)p0 * nR, orbph,
                           taup + (int64_t)p0 * N, gauge, Hout, ldH, V ? V + (int64_t)p0 * N * N : nullptr, ldV);
        if (nproj == 0) break;
    }
    cudaFreeAsync(cs, st);
    cudaFreeAsync(orbph, st);
    cudaFreeAsync(coef, st);
    cudaFreeAsync(taup, st);
    return rc;
}

int rmatrix_term(const ModelDev& m, cudaStream_t st, int64_t nk, const double* k_d, int gauge, int nproj,
                 const double* dirs_d, const zc* H, zc* V, zc* /*scratch*/) {
    if (m.n_rmat <= 0 || nk <= 0 || nproj <= 0) return TBG_OK;
    KTimer kt(st, "rmatrix_term");
    const int N = (int)m.nsta, nR = (int)m.nR;
    const int64_t NN = (int64_t)N * N;
    zc *ph = nullptr, *orbph = nullptr, *tab = nullptr, *A = nullptr;
    TBG_CUDA(cudaMallocAsync(&ph, sizeof(zc) * nk * nR, st));
    TBG_CUDA(cudaMallocAsync(&orbph, sizeof(zc) * nk * N, st));
    TBG_CUDA(cudaMallocAsync(&tab, sizeof(zc) * m.n_rmat * NN, st));
    TBG_CUDA(cudaMallocAsync(&A, sizeof(zc) * nk * NN, st));
    int rc = TBG_OK;
    {
        const int64_t total = nk * (int64_t)(nR + N);
        const unsigned blocks = (unsigned)std::min<int64_t>((total + 255) / 256, 65535 * 8);
        phases_kernel<<<blocks, 256, 0, st>>>(nk, m.dim, k_d, nR, m.hamR_d, N, m.tau_d, ph, orbph);
        count_launch();
    }
    std::vector<double> dirs_h((size_t)nproj * m.dim);
    if (cudaMemcpyAsync(dirs_h.data(), dirs_d, sizeof(double) * dirs_h.size(), cudaMemcpyDeviceToHost, st) !=
            cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        rc = cuda_error(cudaGetLastError(), "rmatrix_term: copy directions");
    double* w_d = nullptr;
    if (rc == TBG_OK) {
        TBG_CUDA(cudaMallocAsync(&w_d, sizeof(double) * m.dim, st));
    }
    for (int p = 0; rc == TBG_OK && p < nproj; ++p) {
        TBG_CUDA(cudaMemcpyAsync(w_d, dirs_d + (int64_t)p * m.dim, sizeof(double) * m.dim,
                                 cudaMemcpyDeviceToDevice, st));
        const int64_t tot = m.n_rmat * NN;
        rmat_combine_kernel<<<(unsigned)std::min<int64_t>((tot + 255) / 256, 65535 * 8), 256, 0, st>>>(
            m.n_rmat, m.dim, N, w_d, m.rmatrix, tab);
        count_launch();
        // A = sum_{r < n_rmat} u(k,r) rm_p[r]   (H-only contraction, lattice gauge)
        rc = dispatch_gemm(st, 0, nk, (int)m.n_rmat, nR, N, ph, tab, nullptr, orbph, nullptr,
                           TBG_GAUGE_LATTICE, A, NN, nullptr, 0);
        if (rc != TBG_OK) break;
        if (gauge == TBG_GAUGE_ATOM) {
            const int64_t t2 = nk * NN;
            rmat_gauge_kernel<<<(unsigned)std::min<int64_t>((t2 + 255) / 256, 65535 * 8), 256, 0, st>>>(
                nk, N, orbph, A);
            count_launch();
        }
        dim3 grid((N + 15) / 16, (N + 15) / 16, (unsigned)nk);
        commutator_kernel<<<grid, 256, 0, st>>>(N, H, NN, A, V + (int64_t)p * NN, (int64_t)nproj * NN);
        count_launch();
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) rc = cuda_error(e, "rmatrix_term kernels");
    }
    if (w_d) cudaFreeAsync(w_d, st);
    cudaFreeAsync(ph, st);
    cudaFreeAsync(orbph, st);
    cudaFreeAsync(tab, st);
    cudaFreeAsync(A, st);
    return rc;
}

}  // namespace tbg
