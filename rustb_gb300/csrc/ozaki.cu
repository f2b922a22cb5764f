// Batched complex GEMM with FP64-class accuracy on the BF16 tensor cores.
//
//   C[b] (M x Nc) = op(A[b]) (M x K) . B[b] (K x Nc),   op = identity or ^H
//
// Exact-slice scheme (after Ozaki, Ogita, Oishi & Rump, "Error-free
// transformations of matrix multiplication", 2012, restated for BF16):
//   * every row i of op(A) is scaled by 2^-EA_i and every column j of B by
//     2^-EB_j (powers of two, |x| < 2^E), so entries lie in (-1, 1);
//   * each scaled entry is written with 42 fractional bits and cut into S
//     signed digits of 7 bits by rounding: x = 2^-7 sum_s q_s 2^-7s with
//     |q_0| <= 128 and |q_s| <= 64 (s >= 1); the slice q_s 2^-7s is exact in BF16;
//   * slice products are summed by BF16 MMA with FP32 accumulation.  Pairs with
//     s + t = 0, 1 and 2 each go to their own accumulator, whose partial sums
//     stay below 2^24 units for K <= 256, so they are exact; the pairs with
//     s + t in [3, LMAX] share a fourth accumulator (relative weight <= 2^-21);
//   * the accumulators are combined into an unevaluated float pair (hi, lo) by
//     error-free TwoSums and scaled by 2^(EA_i + EB_j - 14).
// Complex operands use the real embedding
//   [Re C | Im C] = [Re A | Im A] . [[Re B, Im B], [-Im B, Re B]].
// The slicing works on the integer bits of the inputs (no FP64 arithmetic).
//
// Operand formats: complex double, complex float, or complex float pair
// {re_hi, re_lo, im_hi, im_lo}.  The output is always a complex float pair.
//
// This version issues mma.sync.m16n8k16 (BF16 -> FP32) from ldmatrix-loaded
// fragments.

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <vector>

#include "tbgpu_internal.cuh"

namespace tbg {

namespace {

constexpr int OZ_TM = 64;      // output rows per CTA
constexpr int OZ_TN = 64;      // complex output columns per CTA (128 real)
constexpr int OZ_TK = 16;      // complex k per stage (32 real)
constexpr int OZ_PAD = 40;     // bf16 per smem row (32 + 8 pad, 80 bytes)
constexpr int OZ_ZERO_EXP = kLineZeroExp;

__device__ __forceinline__ int exp_of_max(float m) { return line_exp_of(m); }  // m < 2^E

// Signed fixed-point value trunc(x * 2^(42 - E)) of a double, |x| < 2^E.
__device__ __forceinline__ long long fixed_f64(double x, int E) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int ex = (int)((b >> 52) & 0x7ff);
    if (ex == 0) return 0;
    const unsigned long long M = (b & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    const int sh = 10 + E - (ex - 1023);  // >= 11 when |x| < 2^E
    const long long F = (sh >= 64) ? 0 : (long long)(M >> sh);
    return (b >> 63) ? -F : F;
}

// Same for a float: |x| < 2^E.
__device__ __forceinline__ long long fixed_f32(float x, int E) {
    const unsigned b = __float_as_uint(x);
    const int ex = (int)((b >> 23) & 0xff);
    if (ex == 0) return 0;
    const unsigned long long M = (unsigned long long)((b & 0x7FFFFFu) | 0x800000u);
    const int sh = (ex - 127) - 23 + 42 - E;  // F = M * 2^sh
    long long F;
    if (sh >= 0)
        F = (sh >= 40) ? 0 : (long long)(M << sh);  // sh <= 18 when |x| < 2^E
    else
        F = (-sh >= 64) ? 0 : (long long)(M >> (-sh));
    return (b >> 31) ? -F : F;
}

// Signed 7-bit digits of F (42 fractional bits) by rounding, pre-scaled:
// slice s = q_s 2^-7s with |q_0| <= 128, |q_s| <= 64 for s >= 1.
template <int S>
__device__ __forceinline__ void slices_of(long long F, __nv_bfloat16* out, int stride) {
#pragma unroll
    for (int s = 0; s < S; ++s) {
        const int sh = 35 - 7 * s;
        long long q;
        if (s == S - 1 && sh == 0) {
            q = F;
        } else {
            q = (F + (1ll << (sh - 1))) >> sh;  // round half up (arithmetic shift)
            F -= q << sh;
        }
        const float v = (float)(int)q * __int_as_float((127 - 7 * s) << 23);  // q * 2^-7s, exact
        out[s * stride] = __float2bfloat16_rn(v);
    }
}

enum { FMT_F64 = 0, FMT_F32 = 1, FMT_PAIR = 2, FMT_PRESLICED = 3 };

template <int FMT>
__device__ __forceinline__ void load_fixed(const void* base, int64_t idx, int E, long long& re, long long& im) {
    if (E == OZ_ZERO_EXP) {
        re = im = 0;
        return;
    }
    if (FMT == FMT_F64) {
        const double2 v = reinterpret_cast<const double2*>(base)[idx];
        re = fixed_f64(v.x, E);
        im = fixed_f64(v.y, E);
    } else if (FMT == FMT_F32) {
        const float2 v = reinterpret_cast<const float2*>(base)[idx];
        re = fixed_f32(v.x, E);
        im = fixed_f32(v.y, E);
    } else if (FMT == FMT_PAIR) {
        const float4 v = reinterpret_cast<const float4*>(base)[idx];
        re = fixed_f32(v.x, E) + fixed_f32(v.y, E);
        im = fixed_f32(v.z, E) + fixed_f32(v.w, E);
    } else {
        re = im = 0;
    }
}

template <int FMT>
__device__ __forceinline__ float mag_of(const void* base, int64_t idx) {
    if (FMT == FMT_F64) {
        const double2 v = reinterpret_cast<const double2*>(base)[idx];
        return (float)fmax(fabs(v.x), fabs(v.y)) * 1.0000002f;
    } else if (FMT == FMT_F32) {
        const float2 v = reinterpret_cast<const float2*>(base)[idx];
        return f32_mag(v.x, v.y);
    } else if (FMT == FMT_PAIR) {
        return pair_mag(reinterpret_cast<const float4*>(base)[idx]);
    }
    return 0.f;
}

// Row exponents of a row-major operand (one warp per row, lanes along the row)
// and column exponents (one thread per column, rows walked in order, so a
// warp reads 32 consecutive elements of a row at a time).
template <int FMT>
__global__ void row_exps_kernel(int64_t batch, int M, int K, const void* A, int64_t lda, int64_t sA, int* E) {
    const int lane = threadIdx.x & 31;
    const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t w = gw; w < batch * M; w += nw) {
        const int64_t b = w / M;
        const int r = (int)(w % M);
        float m = 0.f;
        for (int k = lane; k < K; k += 32) m = fmaxf(m, mag_of<FMT>(A, b * sA + (int64_t)r * lda + k));
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (lane == 0) E[w] = exp_of_max(m);
    }
}
template <int FMT>
__global__ void col_exps_kernel(int64_t batch, int Ncols, int K, const void* B, int64_t ldb, int64_t sB, int* E) {
    const int64_t nchunk = (Ncols + blockDim.x - 1) / blockDim.x;
    for (int64_t w = blockIdx.x; w < batch * nchunk; w += gridDim.x) {
        const int64_t b = w / nchunk;
        const int j = (int)(w % nchunk) * blockDim.x + threadIdx.x;
        if (j >= Ncols) continue;
        float m0 = 0.f, m1 = 0.f;
        int k = 0;
        for (; k + 1 < K; k += 2) {
            m0 = fmaxf(m0, mag_of<FMT>(B, b * sB + (int64_t)k * ldb + j));
            m1 = fmaxf(m1, mag_of<FMT>(B, b * sB + (int64_t)(k + 1) * ldb + j));
        }
        if (k < K) m0 = fmaxf(m0, mag_of<FMT>(B, b * sB + (int64_t)k * ldb + j));
        E[b * Ncols + j] = exp_of_max(fmaxf(m0, m1));
    }
}

template <int FMT>
int line_exps(cudaStream_t st, bool cols, int64_t batch, int lines, int K, const void* X, int64_t ld, int64_t sX,
              int* E) {
    if (cols) {
        const int64_t work = batch * ((lines + 127) / 128);
        col_exps_kernel<FMT><<<(unsigned)std::max<int64_t>(1, std::min<int64_t>(work, 152 * 16)), 128, 0, st>>>(
            batch, lines, K, X, ld, sX, E);
    } else {
        const int64_t warps = batch * lines;
        row_exps_kernel<FMT><<<(unsigned)std::max<int64_t>(1, std::min<int64_t>((warps * 32 + 255) / 256, 152 * 64)),
                                256, 0, st>>>(batch, lines, K, X, ld, sX, E);
    }
    TBG_LAUNCHED("oz_exp_kernel");
    return TBG_OK;
}

int exps_of(cudaStream_t st, int fmt, bool cols, int64_t batch, int lines, int K, const void* X, int64_t ld,
            int64_t sX, int* E) {
    switch (fmt) {
        case FMT_F64: return line_exps<FMT_F64>(st, cols, batch, lines, K, X, ld, sX, E);
        case FMT_F32: return line_exps<FMT_F32>(st, cols, batch, lines, K, X, ld, sX, E);
        case FMT_PAIR: return line_exps<FMT_PAIR>(st, cols, batch, lines, K, X, ld, sX, E);
        default: return set_error(TBG_E_UNSUPPORTED, "exponents: operand format");
    }
}

__device__ __forceinline__ void ldsm_x4(unsigned addr, unsigned& r0, unsigned& r1, unsigned& r2, unsigned& r3) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(addr));
}

__device__ __forceinline__ void mma_bf16(float* c, const unsigned* a, unsigned b0, unsigned b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// smem: sA[SA][OZ_TM][OZ_PAD], sB[SB][2*OZ_TN][OZ_PAD] (bf16)
template <int SA, int SB, int LMAX, bool CONJ_A, int FMTA, int FMTB>
__global__ void __launch_bounds__(256, 1) oz_gemm_kernel(int M, int Nc, int K, const void* __restrict__ A,
                                                         int64_t lda, int64_t sA_, const void* __restrict__ B,
                                                         int64_t ldb, int64_t sB_, const int* __restrict__ EA,
                                                         const int* __restrict__ EB, float4* __restrict__ C,
                                                         int64_t ldc, int64_t sC) {
    extern __shared__ __align__(16) unsigned char oz_smem[];
    __nv_bfloat16* sA = reinterpret_cast<__nv_bfloat16*>(oz_smem);
    __nv_bfloat16* sB = sA + SA * OZ_TM * OZ_PAD;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int warp_m = warp & 1, warp_n = warp >> 1;
    const int64_t b = blockIdx.z;
    const int row0 = blockIdx.y * OZ_TM, col0 = blockIdx.x * OZ_TN;

    float acc[4][2][4][4];
#pragma unroll
    for (int l = 0; l < 4; ++l)
#pragma unroll
        for (int i = 0; i < 2; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j)
#pragma unroll
                for (int c = 0; c < 4; ++c) acc[l][i][j][c] = 0.f;

    for (int k0 = 0; k0 < K; k0 += OZ_TK) {
        // ---- stage A: 64 rows x 16 complex k -> sA[s][row][k (re) | 16 + k (im)]
#pragma unroll
        for (int rep = 0; rep < 4; ++rep) {
            const int e = tid + 256 * rep;
            int r, kk;
            if (CONJ_A) {
                r = e & 63;
                kk = e >> 6;
            } else {
                kk = e & 15;
                r = e >> 4;
            }
            const int gi = row0 + r, gk = k0 + kk;
            long long fre = 0, fim = 0;
            if (gi < M && gk < K) {
                const int E = EA[b * M + gi];
                const int64_t idx = CONJ_A ? (b * sA_ + (int64_t)gk * lda + gi) : (b * sA_ + (int64_t)gi * lda + gk);
                load_fixed<FMTA>(A, idx, E, fre, fim);
                if (CONJ_A) fim = -fim;
            }
            __nv_bfloat16* dst = sA + r * OZ_PAD;
            slices_of<SA>(fre, dst + kk, OZ_TM * OZ_PAD);
            slices_of<SA>(fim, dst + 16 + kk, OZ_TM * OZ_PAD);
        }
        // ---- stage B: 16 complex k x 64 complex columns
        if (FMTB == FMT_PRESLICED) {
            // B points at digit planes laid out [col tile][k chunk][slice][re|im][16 k][64 cols]
            const int kc = k0 / OZ_TK;
            const int nkc = (K + OZ_TK - 1) / OZ_TK;
            const __nv_bfloat16* src = static_cast<const __nv_bfloat16*>(B) +
                                       ((int64_t)blockIdx.x * nkc + kc) * (int64_t)SB * 2 * OZ_TK * OZ_TN;
#pragma unroll
            for (int rep = 0; rep < 4; ++rep) {
                const int e = tid + 256 * rep;
                const int j = e & 63, kk = e >> 6;
#pragma unroll
                for (int t = 0; t < SB; ++t) {
                    const __nv_bfloat16 re = src[((t * 2 + 0) * OZ_TK + kk) * OZ_TN + j];
                    const __nv_bfloat16 im = src[((t * 2 + 1) * OZ_TK + kk) * OZ_TN + j];
                    __nv_bfloat16* d0 = sB + t * 2 * OZ_TN * OZ_PAD + j * OZ_PAD;
                    __nv_bfloat16* d1 = sB + t * 2 * OZ_TN * OZ_PAD + (OZ_TN + j) * OZ_PAD;
                    d0[kk] = re;
                    d0[16 + kk] = __hneg(im);
                    d1[kk] = im;
                    d1[16 + kk] = re;
                }
            }
        } else
#pragma unroll
        for (int rep = 0; rep < 4; ++rep) {
            const int e = tid + 256 * rep;
            const int j = e & 63, kk = e >> 6;
            const int gj = col0 + j, gk = k0 + kk;
            long long fre = 0, fim = 0;
            if (gj < Nc && gk < K) {
                const int E = EB[b * Nc + gj];
                load_fixed<FMTB>(B, b * sB_ + (int64_t)gk * ldb + gj, E, fre, fim);
            }
            // real output column j:    rows k -> Re B, rows 16+k -> -Im B
            // imag output column 64+j: rows k -> Im B, rows 16+k ->  Re B
            __nv_bfloat16* d0 = sB + j * OZ_PAD;
            __nv_bfloat16* d1 = sB + (OZ_TN + j) * OZ_PAD;
            slices_of<SB>(fre, d0 + kk, 2 * OZ_TN * OZ_PAD);
            slices_of<SB>(-fim, d0 + 16 + kk, 2 * OZ_TN * OZ_PAD);
            slices_of<SB>(fim, d1 + kk, 2 * OZ_TN * OZ_PAD);
            slices_of<SB>(fre, d1 + 16 + kk, 2 * OZ_TN * OZ_PAD);
        }
        __syncthreads();
        // ---- tensor-core products over the 32 real k of this stage
#pragma unroll
        for (int ks = 0; ks < 2; ++ks) {
            unsigned af[SA][2][4];
#pragma unroll
            for (int s = 0; s < SA; ++s)
#pragma unroll
                for (int mt = 0; mt < 2; ++mt) {
                    const __nv_bfloat16* p = sA + s * OZ_TM * OZ_PAD +
                                             (warp_m * 32 + mt * 16 + (lane & 15)) * OZ_PAD + ks * 16 + (lane >> 4) * 8;
                    ldsm_x4((unsigned)__cvta_generic_to_shared(p), af[s][mt][0], af[s][mt][1], af[s][mt][2],
                            af[s][mt][3]);
                }
#pragma unroll
            for (int t = 0; t < SB; ++t) {
                unsigned bf[4][2];
#pragma unroll
                for (int np = 0; np < 2; ++np) {
                    // lanes 0-7: n 0-7 k 0; 8-15: n 0-7 k 8; 16-23: n 8-15 k 0; 24-31: n 8-15 k 8
                    const int nrow = warp_n * 32 + np * 16 + (lane & 7) + ((lane >> 4) << 3);
                    const int kof = ks * 16 + ((lane >> 3) & 1) * 8;
                    const __nv_bfloat16* p = sB + t * 2 * OZ_TN * OZ_PAD + nrow * OZ_PAD + kof;
                    ldsm_x4((unsigned)__cvta_generic_to_shared(p), bf[2 * np][0], bf[2 * np][1], bf[2 * np + 1][0],
                            bf[2 * np + 1][1]);
                }
#pragma unroll
                for (int s = 0; s < SA; ++s) {
                    if (s + t > LMAX) continue;
                    const int lv = (s + t) < 3 ? (s + t) : 3;
#pragma unroll
                    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
                        for (int nt = 0; nt < 4; ++nt) mma_bf16(acc[lv][mt][nt], af[s][mt], bf[nt][0], bf[nt][1]);
                }
            }
        }
        __syncthreads();
    }

    // ---- epilogue: exact TwoSum of the exact levels, scaled float pair out
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int nt = 0; nt < 4; ++nt)
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const int r = row0 + warp_m * 32 + mt * 16 + (lane >> 2) + ((c >> 1) << 3);
                const int cn = warp_n * 32 + nt * 8 + (lane & 3) * 2 + (c & 1);
                const bool im = cn >= OZ_TN;
                const int j = col0 + (im ? cn - OZ_TN : cn);
                if (r >= M || j >= Nc) continue;
                const float a0 = acc[0][mt][nt][c], a1 = acc[1][mt][nt][c];
                const float a2 = acc[2][mt][nt][c], a3 = acc[3][mt][nt][c];
                // exact levels a0 + a1 + a2 -> (hi, e1 + e2), inexact level a3 into lo
                const float s1 = a0 + a1;
                const float t1 = s1 - a0;
                const float e1 = (a0 - (s1 - t1)) + (a1 - t1);
                const float hi = s1 + a2;
                const float t2 = hi - s1;
                const float e2 = (s1 - (hi - t2)) + (a2 - t2);
                const float lo = (e1 + e2) + a3;
                const int ea = EA[b * M + r], eb = EB[b * Nc + j];
                float2 out = make_float2(0.f, 0.f);
                if (ea != OZ_ZERO_EXP && eb != OZ_ZERO_EXP) {
                    int n = ea + eb - 14;
                    n = max(-126, min(127, n));
                    const float sc = __int_as_float((127 + n) << 23);
                    out = make_float2(hi * sc, lo * sc);
                }
                float* dst = reinterpret_cast<float*>(C + b * sC + (int64_t)r * ldc + j) + (im ? 2 : 0);
                *reinterpret_cast<float2*>(dst) = out;
            }
}

template <int SA, int SB, int LMAX, bool CONJ_A, int FMTA, int FMTB>
int launch_oz(cudaStream_t st, int64_t batch, int M, int Nc, int K, const void* A, int64_t lda, int64_t sA,
              const void* B, int64_t ldb, int64_t sB, float4* C, int64_t ldc, int64_t sC, int* EA, int* EB) {
    if (int rc = exps_of(st, FMTA, CONJ_A, batch, M, K, A, lda, sA, EA)) return rc;
    if (int rc = exps_of(st, FMTB, true, batch, Nc, K, B, ldb, sB, EB)) return rc;
    const size_t smem = sizeof(__nv_bfloat16) * OZ_PAD * (SA * OZ_TM + SB * 2 * OZ_TN);
    auto kern = oz_gemm_kernel<SA, SB, LMAX, CONJ_A, FMTA, FMTB>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_error(e, "cudaFuncSetAttribute(oz_gemm)");
    int pairs = 0;
    for (int s = 0; s < SA; ++s)
        for (int t = 0; t < SB; ++t) pairs += (s + t <= LMAX);
    // algorithmic flops of the complex product, counted once (8 M Nc K); the
    // tensor pipe executes `pairs` times that
    KTimer kt(st, pairs >= 10 ? "ozaki_gemm_kernel<high>" : "ozaki_gemm_kernel<low>",
              8.0 * (double)M * Nc * K * batch);
    for (int64_t b0 = 0; b0 < batch; b0 += 65535) {
        const int64_t nb = std::min<int64_t>(65535, batch - b0);
        dim3 grid((Nc + OZ_TN - 1) / OZ_TN, (M + OZ_TM - 1) / OZ_TM, (unsigned)nb);
        const size_t ea = FMTA == FMT_F64 ? 16 : (FMTA == FMT_F32 ? 8 : 16);
        const size_t eb = FMTB == FMT_F64 ? 16 : (FMTB == FMT_F32 ? 8 : 16);
        kern<<<grid, 256, smem, st>>>(M, Nc, K, static_cast<const char*>(A) + b0 * sA * ea, lda, sA,
                                      static_cast<const char*>(B) + b0 * sB * eb, ldb, sB, EA + b0 * M, EB + b0 * Nc,
                                      C + b0 * sC, ldc, sC);
        TBG_LAUNCHED("ozaki_gemm_kernel");
    }
    return TBG_OK;
}

}  // namespace

size_t ozaki_exp_bytes(int64_t batch, int M, int Nc) { return sizeof(int) * (size_t)batch * (M + Nc) + 256; }

// Exponents of the rows (cols = false: rows of a row-major X with leading
// dimension ld) or columns (cols = true) of `batch` operands of `lines` lines
// and K elements each, in the given format.
int ozaki_line_exps(cudaStream_t st, int fmt, bool cols, int64_t batch, int lines, int K, const void* X, int64_t ld,
                    int64_t sX, int* E) {
    return exps_of(st, fmt, cols, batch, lines, K, X, ld, sX, E);
}

// Row / column exponents for any operand format combination (shared by the
// mma.sync and tcgen05 forms).
int ozaki_exp_launch(cudaStream_t st, bool conj_a, int fmt_a, int fmt_b, int64_t batch, int M, int Nc, int K,
                     const void* A, int64_t lda, int64_t sA, const void* B, int64_t ldb, int64_t sB, int* EA, int* EB) {
    // rows of op(A): rows of A, or (conj) columns of A; columns of B
    int rc = exps_of(st, fmt_a, conj_a, batch, M, K, A, lda, sA, EA);
    if (rc) return rc;
    return exps_of(st, fmt_b, true, batch, Nc, K, B, ldb, sB, EB);
}

int ozaki_fourier_tc(cudaStream_t st, int64_t M, int64_t Nc, int K, const zc* A, const int* EA, const int* EB,
                     const void* Bs, float4* C, int* err, int64_t high_rows, void* aimg);
int ozaki_zgemm_tc_low(cudaStream_t st, int64_t batch, int M, int Nc, int K, const void* A, int64_t lda, int64_t sA,
                       const void* B, int64_t ldb, int64_t sB, float4* C, int64_t ldc, int64_t sC, int* EA, int* EB,
                       int* err, bool exps_ready = false);

// tcgen05 kernels are used unless TBG_OZAKI_MMA_SYNC=1 (the mma.sync form).
bool ozaki_use_tc() {
    static int v = -1;
    if (v < 0) {
        const char* e = std::getenv("TBG_OZAKI_MMA_SYNC");
        v = (e && e[0] == '1') ? 0 : 1;
    }
    return v == 1;
}

namespace {

// Column exponents of the hop table: EB[e] over R (one warp per column e).
__global__ void hop_exp_kernel(int K, int64_t Nc, const zc* __restrict__ ham, int* __restrict__ EB) {
    const int lane = threadIdx.x & 31;
    const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t e = gw; e < Nc; e += nw) {
        float m = 0.f;
        for (int r = lane; r < K; r += 32) m = fmaxf(m, mag_of<FMT_F64>(ham, (int64_t)r * Nc + e));
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (lane == 0) EB[e] = exp_of_max(m);
    }
}

// Digit planes of the hop table: [col tile][k chunk][slice][re|im][16 k][64 cols].
template <int S>
__global__ void hop_slice_kernel(int K, int64_t Nc, const zc* __restrict__ ham, const int* __restrict__ EB,
                                 __nv_bfloat16* __restrict__ Bs) {
    const int nkc = (K + OZ_TK - 1) / OZ_TK;
    const int64_t nct = (Nc + OZ_TN - 1) / OZ_TN;
    const int64_t total = nct * nkc * OZ_TK * OZ_TN;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int j = (int)(idx % OZ_TN);
        const int kk = (int)((idx / OZ_TN) % OZ_TK);
        const int64_t blk = idx / (OZ_TN * OZ_TK);  // = ct * nkc + kc
        const int kc = (int)(blk % nkc);
        const int64_t ct = blk / nkc;
        const int64_t e = ct * OZ_TN + j;
        const int r = kc * OZ_TK + kk;
        long long fre = 0, fim = 0;
        if (e < Nc && r < K) load_fixed<FMT_F64>(ham, (int64_t)r * Nc + e, EB[e], fre, fim);
        __nv_bfloat16* dst = Bs + blk * (int64_t)S * 2 * OZ_TK * OZ_TN + kk * OZ_TN + j;
        slices_of<S>(fre, dst, 2 * OZ_TK * OZ_TN);
        slices_of<S>(fim, dst + OZ_TK * OZ_TN, 2 * OZ_TK * OZ_TN);
    }
}

// Row exponents of a plain complex-double A (M x K): one warp per row.
__global__ void row_exp_kernel(int64_t M, int K, const zc* __restrict__ A, int64_t lda, int* __restrict__ EA) {
    const int lane = threadIdx.x & 31;
    const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t r = gw; r < M; r += nw) {
        float m = 0.f;
        for (int k = lane; k < K; k += 32) m = fmaxf(m, mag_of<FMT_F64>(A, r * lda + k));
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (lane == 0) EA[r] = exp_of_max(m);
    }
}

}  // namespace

// Largest contraction length for which levels 0-2 stay exact.
int ozaki_fourier_max_k() { return 408; }

size_t ozaki_hop_image_bytes(int K, int64_t Nc);
int ozaki_hop_image_launch(cudaStream_t st, int K, int64_t Nc, const zc* ham, const int* EB, void* img,
                          const int* colmap, int64_t ldh);

// Bytes of the hop table's digit planes in the layout of the selected kernel
// (tcgen05 stage images, or the mma.sync slice layout).
size_t ozaki_hop_slices_bytes(int K, int64_t Nc) {
    if (ozaki_use_tc()) return ozaki_hop_image_bytes(K, Nc);
    const int64_t nkc = (K + OZ_TK - 1) / OZ_TK, nct = (Nc + OZ_TN - 1) / OZ_TN;
    return sizeof(__nv_bfloat16) * (size_t)nct * nkc * 6 * 2 * OZ_TK * OZ_TN;
}

// Build the digit planes of the hop table (K = nR rows of Nc = N^2 elements);
// EB gets the exponent of every table element.  The tcgen05 images cover the
// ncols elements listed in colmap (all Nc when colmap is null).
int ozaki_build_hop_slices(cudaStream_t st, int K, int64_t Nc, const zc* ham, int* EB, void* Bs, const int* colmap,
                           int64_t ncols) {
    KTimer kt(st, "hop_slice_kernel");
    hop_exp_kernel<<<(unsigned)std::min<int64_t>((Nc * 32 + 255) / 256, 152 * 64), 256, 0, st>>>(K, Nc, ham, EB);
    TBG_LAUNCHED("hop_exp_kernel");
    if (ozaki_use_tc()) return ozaki_hop_image_launch(st, K, colmap ? ncols : Nc, ham, EB, Bs, colmap, Nc);
    const int64_t total = ((Nc + OZ_TN - 1) / OZ_TN) * ((K + OZ_TK - 1) / OZ_TK) * OZ_TK * OZ_TN;
    hop_slice_kernel<6><<<(unsigned)std::min<int64_t>((total + 255) / 256, 152 * 64), 256, 0, st>>>(
        K, Nc, ham, EB, static_cast<__nv_bfloat16*>(Bs));
    TBG_LAUNCHED("hop_slice_kernel");
    return TBG_OK;
}

int ozaki_hop_image_real_launch(cudaStream_t st, int Kc, int64_t Nc, const zc* T, const int* EB, void* img,
                                const int* colmap, int64_t ldh);
// Stage images of a table T with 2 Kc rows contracted against real
// coefficients (tcgen05 form only); EB over all 2 Kc rows of each element.
int ozaki_build_hop_slices_real(cudaStream_t st, int Kc, int64_t Nc, const zc* T, int* EB, void* Bs,
                                const int* colmap, int64_t ncols) {
    if (!ozaki_use_tc()) return set_error(TBG_E_UNSUPPORTED, "real-coefficient hop images need the tcgen05 kernels");
    KTimer kt(st, "hop_slice_kernel");
    hop_exp_kernel<<<(unsigned)std::min<int64_t>((Nc * 32 + 255) / 256, 152 * 64), 256, 0, st>>>(2 * Kc, Nc, T, EB);
    TBG_LAUNCHED("hop_exp_kernel");
    return ozaki_hop_image_real_launch(st, Kc, colmap ? ncols : Nc, T, EB, Bs, colmap, Nc);
}

// C (M x Nc, float pairs) = A (M x K, complex double) . hop (digit planes).
int ozaki_fourier(cudaStream_t st, int64_t M, int64_t Nc, int K, const zc* A, int* EA, const int* EB,
                  const void* Bs, float4* C, int* err, int64_t high_rows, void* aimg) {
    if (K > ozaki_fourier_max_k()) return set_error(TBG_E_UNSUPPORTED, "ozaki_fourier: nR > 408");
    row_exp_kernel<<<(unsigned)std::min<int64_t>((M * 32 + 255) / 256, 152 * 64), 256, 0, st>>>(M, K, A, K, EA);
    TBG_LAUNCHED("row_exp_kernel");
    if (ozaki_use_tc() && err && aimg) return ozaki_fourier_tc(st, M, Nc, K, A, EA, EB, Bs, C, err, high_rows, aimg);
    constexpr int SA = 6, SB = 6, LMAX = 5;
    const size_t smem = sizeof(__nv_bfloat16) * OZ_PAD * (SA * OZ_TM + SB * 2 * OZ_TN);
    auto kern = oz_gemm_kernel<SA, SB, LMAX, false, FMT_F64, FMT_PRESLICED>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_error(e, "cudaFuncSetAttribute(oz_fourier)");
    KTimer kt(st, "ozaki_fourier_kernel", 8.0 * (double)M * Nc * K);
    for (int64_t m0 = 0; m0 < M; m0 += (int64_t)OZ_TM * 65535) {
        const int64_t mb = std::min<int64_t>(M - m0, (int64_t)OZ_TM * 65535);
        dim3 grid((unsigned)((Nc + OZ_TN - 1) / OZ_TN), (unsigned)((mb + OZ_TM - 1) / OZ_TM), 1);
        kern<<<grid, 256, smem, st>>>((int)mb, (int)Nc, K, A + m0 * K, K, 0, Bs, Nc, 0, EA + m0, EB, C + m0 * Nc, Nc,
                                      0);
        TBG_LAUNCHED("ozaki_fourier_kernel");
    }
    return TBG_OK;
}

// Precision classes used by the mixed path:
//   HIGH: 6 x 6 slices, levels s + t <= 5  (about 2^-43 of the product scale)
//   LOW : 3 x 3 slices, levels s + t <= 2  (about 2^-22; corrections that are
//         themselves ~1e-7 of the result)
int ozaki_zgemm(cudaStream_t st, bool high, bool conj_a, int fmt_a, int fmt_b, int64_t batch, int M, int Nc, int K,
                const void* A, int64_t lda, int64_t sA, const void* B, int64_t ldb, int64_t sB, float4* C, int64_t ldc,
                int64_t sC, int* EA, int* EB) {
    if (K > 256) return set_error(TBG_E_UNSUPPORTED, "ozaki_zgemm: K > 256");
#define OZ_CASE(H, CJ, FA, FB)                                                                                   \
    if (high == H && conj_a == CJ && fmt_a == FA && fmt_b == FB)                                                 \
        return H ? launch_oz<6, 6, 5, CJ, FA, FB>(st, batch, M, Nc, K, A, lda, sA, B, ldb, sB, C, ldc, sC, EA, EB) \
                 : launch_oz<3, 3, 2, CJ, FA, FB>(st, batch, M, Nc, K, A, lda, sA, B, ldb, sB, C, ldc, sC, EA, EB);
    // combinations used by the mixed path and by the unit test
    OZ_CASE(true, false, FMT_F64, FMT_F64)
    OZ_CASE(true, true, FMT_F64, FMT_F64)
    OZ_CASE(true, true, FMT_F32, FMT_F32)    // X^H X
    OZ_CASE(true, false, FMT_PAIR, FMT_F32)  // H X
    OZ_CASE(true, true, FMT_F32, FMT_PAIR)   // X^H (H X)
    OZ_CASE(true, false, FMT_PAIR, FMT_PAIR) // V X'
    OZ_CASE(true, true, FMT_PAIR, FMT_PAIR)  // X'^H (V X')
    OZ_CASE(false, false, FMT_F32, FMT_F32)  // X F
    OZ_CASE(false, false, FMT_F64, FMT_F64)
#undef OZ_CASE
    return set_error(TBG_E_UNSUPPORTED, "ozaki_zgemm: operand format combination not instantiated");
}

}  // namespace tbg

// Internal test hook (not part of the public header): C = op(A) B for host
// complex-double inputs, result as complex double (hi + lo).  high: 1 HIGH
// class, 0 LOW, 2 MID (tcgen05 only).
extern "C" int tbg_internal_ozaki_zgemm(int high, int conj_a, int64_t batch, int M, int Nc, int K, const double* A,
                                        const double* B, double* C, int use_tc) {
    using namespace tbg;
    const int64_t ar = conj_a ? K : M, ac = conj_a ? M : K;
    const size_t abytes = sizeof(double) * 2 * ar * ac * batch, bbytes = sizeof(double) * 2 * (size_t)K * Nc * batch;
    const size_t cbytes = sizeof(float4) * (size_t)M * Nc * batch;
    void *dA = nullptr, *dB = nullptr, *dC = nullptr, *dE = nullptr;
    cudaStream_t st = nullptr;
    cudaStreamCreate(&st);
    int rc = TBG_OK;
    if (cudaMalloc(&dA, abytes) || cudaMalloc(&dB, bbytes) || cudaMalloc(&dC, cbytes) ||
        cudaMalloc(&dE, ozaki_exp_bytes(batch, M, Nc)))
        rc = set_error(TBG_E_OOM, "ozaki test alloc");
    if (!rc) {
        cudaMemcpy(dA, A, abytes, cudaMemcpyHostToDevice);
        cudaMemcpy(dB, B, bbytes, cudaMemcpyHostToDevice);
        int* EA = static_cast<int*>(dE);
        int* derr = nullptr;
        cudaMalloc(&derr, sizeof(int));
        cudaMemset(derr, 0, sizeof(int));
        if (use_tc && !high && !conj_a) {
            // LOW class on tcgen05 takes FP32 operands: round the inputs once
            std::vector<float> a32((size_t)2 * ar * ac * batch), b32((size_t)2 * K * Nc * batch);
            for (size_t i = 0; i < a32.size(); ++i) a32[i] = (float)A[i];
            for (size_t i = 0; i < b32.size(); ++i) b32[i] = (float)B[i];
            cudaMemcpy(dA, a32.data(), sizeof(float) * a32.size(), cudaMemcpyHostToDevice);
            cudaMemcpy(dB, b32.data(), sizeof(float) * b32.size(), cudaMemcpyHostToDevice);
            rc = ozaki_zgemm_tc_low(st, batch, M, Nc, K, dA, ac, ar * ac, dB, Nc, (int64_t)K * Nc,
                                    static_cast<float4*>(dC), Nc, (int64_t)M * Nc, EA, EA + batch * M, derr);
        } else if (use_tc && high)  // high = 2: the MID class
            rc = ozaki_zgemm_tc(st, conj_a != 0, 0, 0, batch, M, Nc, K, dA, ac, ar * ac, dB, Nc, (int64_t)K * Nc,
                                static_cast<float4*>(dC), Nc, (int64_t)M * Nc, EA, EA + batch * M, derr, false,
                                nullptr, high == 2);
        else
            rc = ozaki_zgemm(st, high != 0, conj_a != 0, 0, 0, batch, M, Nc, K, dA, ac, ar * ac, dB, Nc,
                             (int64_t)K * Nc, static_cast<float4*>(dC), Nc, (int64_t)M * Nc, EA, EA + batch * M);
        int herr = 0;
        cudaStreamSynchronize(st);
        cudaMemcpy(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost);
        cudaFree(derr);
        if (!rc && (herr & 2)) rc = set_error(TBG_E_TIMEOUT, "ozaki tcgen05 kernel: a bounded wait ran out");
        cudaError_t e = cudaStreamSynchronize(st);
        if (!rc && e != cudaSuccess) rc = cuda_error(e, "ozaki test");
        if (!rc) {
            std::vector<float4> h((size_t)M * Nc * batch);
            cudaMemcpy(h.data(), dC, cbytes, cudaMemcpyDeviceToHost);
            for (size_t i = 0; i < h.size(); ++i) {
                C[2 * i] = (double)h[i].x + (double)h[i].y;
                C[2 * i + 1] = (double)h[i].z + (double)h[i].w;
            }
        }
    }
    cudaFree(dA);
    cudaFree(dB);
    cudaFree(dC);
    cudaFree(dE);
    cudaStreamDestroy(st);
    return rc;
}
