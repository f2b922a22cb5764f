// Exact-slice complex GEMM on the 5th-generation tensor cores (tcgen05, TMEM).
//
// Same arithmetic as ozaki.cu (6 signed 7-bit digits per value, levels
// s + t = 0, 1, 2 exact, 3..5 together, float-pair output), issued as
// tcgen05.mma.cta_group::1.kind::f16 (BF16 x BF16 -> FP32, M = 128, N = 128,
// K = 16) from shared-memory descriptors.  The four accumulation levels live
// in tensor memory: 4 x 128 FP32 columns = the whole 512-column allocation.
//
// CTA = 8 warps, one output tile of 128 rows x 64 complex columns:
//   warp 0      allocates TMEM; lane 0 issues the MMAs and commits them;
//   warps 1..7  digit producers: read the FP64 / FP32 / pair / pre-sliced
//               operands, write digit planes (K-major, no-swizzle core
//               matrices of 8 rows x 16 bytes) into one of two stage buffers;
//   warps 4..7  after the K loop: read the four levels from TMEM
//               (tcgen05.ld 32x32b, one TMEM lane = one output row), combine
//               them with error-free TwoSums and write the float pairs.
// Stage hand-off uses mbarriers: full[b] (224 producer arrivals) and empty[b]
// (tcgen05.commit of the MMAs that read buffer b).  Every wait is bounded;
// on a time-out the CTA records an error, drains its committed MMAs (bounded),
// frees TMEM and returns.

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "tbgpu_internal.cuh"

namespace tbg {

namespace {

constexpr int TC_TM = 128;        // output rows
constexpr int TC_TN = 64;         // complex output columns (128 real)
constexpr int TC_TK = 16;         // complex k per stage (32 real)
constexpr int TC_S = 6;           // digits per value
constexpr int TC_LMAX = 5;
constexpr int PLANE = 128 * 32 * 2;             // bytes of one digit plane (128 rows x 32 k bf16)
constexpr int STAGE_BYTES = 2 * TC_S * PLANE;   // A and B planes of one stage
constexpr int TC_SMEM = 2 * STAGE_BYTES + 1024; // two stages + barriers / scratch
constexpr int N_PRODUCERS = 224;
constexpr int ZERO_EXP = -100000;

enum { FMT_F64 = 0, FMT_F32 = 1, FMT_PAIR = 2, FMT_PRESLICED = 3 };

// instruction descriptor, kind::f16: D = F32, A = B = BF16, K-major, N = 128, M = 128
constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((128u >> 3) << 17) | ((128u >> 4) << 24);

__device__ __forceinline__ uint32_t su32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(su32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(su32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait without abort check (used to drain committed MMAs before freeing TMEM).
__device__ __forceinline__ bool mbar_wait_plain(uint64_t* bar, uint32_t parity) {
    for (int it = 0; it < (1 << 20); ++it)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}
// Bounded wait: false on time-out or when another warp has flagged an abort.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, volatile int* abort_flag) {
    for (int it = 0; it < (1 << 20); ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if (*abort_flag) return false;
    }
    return false;
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;  // descriptor version for sm_100-class tensor cores; no swizzle
    return d;
}

__device__ __forceinline__ void umma(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\ttcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(
            d_tmem),
        "l"(adesc), "l"(bdesc), "r"(IDESC), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(su32(bar))
                 : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,"
        "%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
          "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// ---- digit extraction (identical arithmetic to ozaki.cu) ----
__device__ __forceinline__ long long fx64(double x, int E) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int ex = (int)((b >> 52) & 0x7ff);
    if (ex == 0) return 0;
    const unsigned long long M = (b & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    const int sh = 10 + E - (ex - 1023);
    const long long F = (sh >= 64) ? 0 : (long long)(M >> sh);
    return (b >> 63) ? -F : F;
}
__device__ __forceinline__ long long fx32(float x, int E) {
    const unsigned b = __float_as_uint(x);
    const int ex = (int)((b >> 23) & 0xff);
    if (ex == 0) return 0;
    const unsigned long long M = (unsigned long long)((b & 0x7FFFFFu) | 0x800000u);
    const int sh = (ex - 127) - 23 + 42 - E;
    long long F;
    if (sh >= 0)
        F = (sh >= 40) ? 0 : (long long)(M << sh);
    else
        F = (-sh >= 64) ? 0 : (long long)(M >> (-sh));
    return (b >> 31) ? -F : F;
}
template <int FMT>
__device__ __forceinline__ void load_fx(const void* base, int64_t idx, int E, long long& re, long long& im) {
    if (E == ZERO_EXP) {
        re = im = 0;
        return;
    }
    if (FMT == FMT_F64) {
        const double2 v = reinterpret_cast<const double2*>(base)[idx];
        re = fx64(v.x, E);
        im = fx64(v.y, E);
    } else if (FMT == FMT_F32) {
        const float2 v = reinterpret_cast<const float2*>(base)[idx];
        re = fx32(v.x, E);
        im = fx32(v.y, E);
    } else {
        const float4 v = reinterpret_cast<const float4*>(base)[idx];
        re = fx32(v.x, E) + fx32(v.y, E);
        im = fx32(v.z, E) + fx32(v.w, E);
    }
}
// Raw 16-byte (or 8-byte) element of an operand, loaded ahead of the digit work.
template <int FMT>
struct Raw {
    int4 v;
};
template <int FMT>
__device__ __forceinline__ Raw<FMT> load_raw(const void* base, int64_t idx) {
    Raw<FMT> r;
    if (FMT == FMT_F32) {
        const int2 t = reinterpret_cast<const int2*>(base)[idx];
        r.v = make_int4(t.x, t.y, 0, 0);
    } else {
        r.v = reinterpret_cast<const int4*>(base)[idx];
    }
    return r;
}
template <int FMT>
__device__ __forceinline__ void raw_fx(const Raw<FMT>& r, int E, long long& re, long long& im) {
    if (E == ZERO_EXP) {
        re = im = 0;
        return;
    }
    if (FMT == FMT_F64) {
        re = fx64(__hiloint2double(r.v.y, r.v.x), E);
        im = fx64(__hiloint2double(r.v.w, r.v.z), E);
    } else if (FMT == FMT_F32) {
        re = fx32(__int_as_float(r.v.x), E);
        im = fx32(__int_as_float(r.v.y), E);
    } else {
        re = fx32(__int_as_float(r.v.x), E) + fx32(__int_as_float(r.v.y), E);
        im = fx32(__int_as_float(r.v.z), E) + fx32(__int_as_float(r.v.w), E);
    }
}

// digits of F (42 fractional bits), rounded, pre-scaled by 2^-7s
__device__ __forceinline__ void digits(long long F, __nv_bfloat16* d) {
#pragma unroll
    for (int s = 0; s < TC_S; ++s) {
        const int sh = 35 - 7 * s;
        long long q;
        if (sh == 0) {
            q = F;
        } else {
            q = (F + (1ll << (sh - 1))) >> sh;
            F -= q << sh;
        }
        d[s] = __float2bfloat16_rn((float)(int)q * __int_as_float((127 - 7 * s) << 23));
    }
}
// byte offset of element (row, k') inside one digit plane (K-major core matrices)
__device__ __forceinline__ int plane_off(int row, int kp) {
    return (((row >> 3) * 4 + (kp >> 3)) << 7) + ((row & 7) << 4) + ((kp & 7) << 1);
}

template <bool CONJ_A, int FMTA, int FMTB>
__global__ void __launch_bounds__(256, 1) oz_tc_kernel(int M, int Nc, int K, const void* __restrict__ A, int64_t lda,
                                                       int64_t sA, const void* __restrict__ B, int64_t ldb, int64_t sB,
                                                       const int* __restrict__ EA, const int* __restrict__ EB,
                                                       float4* __restrict__ C, int64_t ldc, int64_t sC,
                                                       int* __restrict__ err) {
    extern __shared__ __align__(1024) unsigned char tc_smem[];
    unsigned char* base = reinterpret_cast<unsigned char*>(((uintptr_t)tc_smem + 1023) & ~(uintptr_t)1023);
    unsigned char* stage[2] = {base, base + STAGE_BYTES};
    __shared__ __align__(8) uint64_t bar_full[2], bar_empty[2], bar_done;
    __shared__ uint32_t tmem_base_sh;
    __shared__ volatile int abort_sh;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int64_t b = blockIdx.z;
    const int row0 = blockIdx.y * TC_TM, col0 = blockIdx.x * TC_TN;
    const int nstages = (K + TC_TK - 1) / TC_TK;

    if (tid == 0) {
        mbar_init(&bar_full[0], N_PRODUCERS);
        mbar_init(&bar_full[1], N_PRODUCERS);
        mbar_init(&bar_empty[0], 1);
        mbar_init(&bar_empty[1], 1);
        mbar_init(&bar_done, 1);
        abort_sh = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(su32(&tmem_base_sh))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base_sh;

    if (warp == 0) {
        // ------------------------------------------------ MMA issuer (lane 0)
        if (lane == 0) {
            int issued_any = 0;
            for (int it = 0; it < nstages; ++it) {
                const int bi = it & 1;
                if (!mbar_wait(&bar_full[bi], (it >> 1) & 1, &abort_sh)) {
                    abort_sh = 1;
                    break;
                }
                tc_fence_after();
                const uint32_t sa = su32(stage[bi]);
                const uint32_t sb = sa + TC_S * PLANE;
#pragma unroll
                for (int ks = 0; ks < 2; ++ks) {
#pragma unroll
                    for (int t = 0; t < TC_S; ++t) {
#pragma unroll
                        for (int s = 0; s < TC_S; ++s) {
                            if (s + t > TC_LMAX) continue;
                            const int lv = (s + t) < 3 ? (s + t) : 3;
                            const uint64_t ad = smem_desc(sa + s * PLANE + ks * 256, 128, 512);
                            const uint64_t bd = smem_desc(sb + t * PLANE + ks * 256, 128, 512);
                            const uint32_t acc = (it == 0 && ks == 0 && t == 0 && s <= 3) ? 0u : 1u;
                            umma(tmem + (uint32_t)(lv * 128), ad, bd, acc);
                        }
                    }
                }
                issued_any = 1;
                umma_commit(&bar_empty[bi]);
            }
            (void)issued_any;
            umma_commit(&bar_done);  // tracks every MMA issued above
        }
        __syncwarp();
    } else {
        // ----------------------------------------------- digit producers
        const int p = tid - 32;  // 0 .. 223
        for (int it = 0; it < nstages && !abort_sh; ++it) {
            const int bi = it & 1;
            if (it >= 2 && !mbar_wait(&bar_empty[bi], ((it >> 1) - 1) & 1, &abort_sh)) {
                abort_sh = 1;
                break;
            }
            unsigned char* sa = stage[bi];
            unsigned char* sb = sa + TC_S * PLANE;
            const int k0 = it * TC_TK;
            // A: 128 rows x 16 complex k.  All loads of the stage are issued first.
            constexpr int PA = (TC_TM * TC_TK + N_PRODUCERS - 1) / N_PRODUCERS;
            Raw<FMTA> ra[PA];
            int ea_[PA];
#pragma unroll
            for (int q = 0; q < PA; ++q) {
                const int e = p + q * N_PRODUCERS;
                ea_[q] = ZERO_EXP;
                ra[q].v = make_int4(0, 0, 0, 0);
                if (e < TC_TM * TC_TK) {
                    const int r = CONJ_A ? (e & 127) : (e >> 4);
                    const int kk = CONJ_A ? (e >> 7) : (e & 15);
                    const int gi = row0 + r, gk = k0 + kk;
                    if (gi < M && gk < K) {
                        ea_[q] = EA[b * M + gi];
                        const int64_t idx =
                            CONJ_A ? (b * sA + (int64_t)gk * lda + gi) : (b * sA + (int64_t)gi * lda + gk);
                        ra[q] = load_raw<FMTA>(A, idx);
                    }
                }
            }
#pragma unroll
            for (int q = 0; q < PA; ++q) {
                const int e = p + q * N_PRODUCERS;
                if (e >= TC_TM * TC_TK) continue;
                const int r = CONJ_A ? (e & 127) : (e >> 4);
                const int kk = CONJ_A ? (e >> 7) : (e & 15);
                long long fre, fim;
                raw_fx<FMTA>(ra[q], ea_[q], fre, fim);
                if (CONJ_A) fim = -fim;
                __nv_bfloat16 dre[TC_S], dim_[TC_S];
                digits(fre, dre);
                digits(fim, dim_);
                const int ore = plane_off(r, kk), oim = plane_off(r, 16 + kk);
#pragma unroll
                for (int s = 0; s < TC_S; ++s) {
                    *reinterpret_cast<__nv_bfloat16*>(sa + s * PLANE + ore) = dre[s];
                    *reinterpret_cast<__nv_bfloat16*>(sa + s * PLANE + oim) = dim_[s];
                }
            }
            // B: 16 complex k x 64 complex columns -> rows n (re: j, im: 64 + j)
            constexpr int PB = (TC_TK * TC_TN + N_PRODUCERS - 1) / N_PRODUCERS;
            Raw<FMTB == FMT_PRESLICED ? FMT_F64 : FMTB> rb[PB];
            int eb_[PB];
            if (FMTB != FMT_PRESLICED) {
#pragma unroll
                for (int q = 0; q < PB; ++q) {
                    const int e = p + q * N_PRODUCERS;
                    eb_[q] = ZERO_EXP;
                    rb[q].v = make_int4(0, 0, 0, 0);
                    if (e < TC_TK * TC_TN) {
                        const int j = e & 63, kk = e >> 6;
                        const int gj = col0 + j, gk = k0 + kk;
                        if (gj < Nc && gk < K) {
                            eb_[q] = EB[b * Nc + gj];
                            rb[q] = load_raw<FMTB == FMT_PRESLICED ? FMT_F64 : FMTB>(B, b * sB + (int64_t)gk * ldb + gj);
                        }
                    }
                }
            }
#pragma unroll
            for (int q = 0; q < PB; ++q) {
                const int e = p + q * N_PRODUCERS;
                if (e >= TC_TK * TC_TN) continue;
                const int j = e & 63, kk = e >> 6;
                __nv_bfloat16 dre[TC_S], dim_[TC_S];
                if (FMTB == FMT_PRESLICED) {
                    const int nkc = (K + TC_TK - 1) / TC_TK;
                    const __nv_bfloat16* src = static_cast<const __nv_bfloat16*>(B) +
                                               ((int64_t)blockIdx.x * nkc + it) * (int64_t)TC_S * 2 * TC_TK * TC_TN;
#pragma unroll
                    for (int t = 0; t < TC_S; ++t) {
                        dre[t] = src[((t * 2 + 0) * TC_TK + kk) * TC_TN + j];
                        dim_[t] = src[((t * 2 + 1) * TC_TK + kk) * TC_TN + j];
                    }
                } else {
                    long long fre, fim;
                    raw_fx<FMTB == FMT_PRESLICED ? FMT_F64 : FMTB>(rb[q], eb_[q], fre, fim);
                    digits(fre, dre);
                    digits(fim, dim_);
                }
                const int o00 = plane_off(j, kk), o01 = plane_off(j, 16 + kk);
                const int o10 = plane_off(64 + j, kk), o11 = plane_off(64 + j, 16 + kk);
#pragma unroll
                for (int t = 0; t < TC_S; ++t) {
                    unsigned char* pl = sb + t * PLANE;
                    *reinterpret_cast<__nv_bfloat16*>(pl + o00) = dre[t];
                    *reinterpret_cast<__nv_bfloat16*>(pl + o01) = __hneg(dim_[t]);
                    *reinterpret_cast<__nv_bfloat16*>(pl + o10) = dim_[t];
                    *reinterpret_cast<__nv_bfloat16*>(pl + o11) = dre[t];
                }
            }
            fence_async_smem();  // make the generic-proxy writes visible to the tensor core
            mbar_arrive(&bar_full[bi]);
        }
    }

    // ---------------------------------------------------------- epilogue
    if (warp >= 4) {
        bool ok = mbar_wait(&bar_done, 0, &abort_sh) && !abort_sh;
        ok = __all_sync(0xffffffffu, ok);  // tcgen05.ld is warp-collective
        tc_fence_after();
        const int q = warp - 4;  // TMEM lanes 32q .. 32q+31
        const int r = row0 + 32 * q + lane;
        const uint32_t lane_addr = tmem + ((uint32_t)(32 * q) << 16);
        if (ok) {
            const int ea = (r < M) ? EA[b * M + r] : ZERO_EXP;
            for (int cb = 0; cb < 4; ++cb) {  // 32 real columns at a time
                float a0[32], a1[32], a2[32], a3[32];
                tmem_ld32(lane_addr + 0 * 128 + cb * 32, a0);
                tmem_ld32(lane_addr + 1 * 128 + cb * 32, a1);
                tmem_ld32(lane_addr + 2 * 128 + cb * 32, a2);
                tmem_ld32(lane_addr + 3 * 128 + cb * 32, a3);
                if (r < M) {
#pragma unroll
                    for (int c = 0; c < 32; ++c) {
                        const int cn = cb * 32 + c;
                        const bool im = cn >= TC_TN;
                        const int j = col0 + (im ? cn - TC_TN : cn);
                        if (j >= Nc) continue;
                        const float s1 = a0[c] + a1[c];
                        const float t1 = s1 - a0[c];
                        const float e1 = (a0[c] - (s1 - t1)) + (a1[c] - t1);
                        const float hi = s1 + a2[c];
                        const float t2 = hi - s1;
                        const float e2 = (s1 - (hi - t2)) + (a2[c] - t2);
                        const float lo = (e1 + e2) + a3[c];
                        const int eb = EB[b * Nc + j];
                        float2 out = make_float2(0.f, 0.f);
                        if (ea != ZERO_EXP && eb != ZERO_EXP) {
                            int n = ea + eb - 14;
                            n = max(-126, min(127, n));
                            const float sc = __int_as_float((127 + n) << 23);
                            out = make_float2(hi * sc, lo * sc);
                        }
                        float* dst = reinterpret_cast<float*>(C + b * sC + (int64_t)r * ldc + j) + (im ? 2 : 0);
                        *reinterpret_cast<float2*>(dst) = out;
                    }
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (abort_sh && tid == 0) atomicOr(err, 2);  // bit 1: a bounded wait ran out
    if (warp == 0) {
        if (lane == 0) mbar_wait_plain(&bar_done, 0);  // every committed MMA has finished
        __syncwarp();
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem) : "memory");
    }
}

}  // namespace

int ozaki_exp_launch(cudaStream_t st, bool conj_a, int fmt_a, int fmt_b, int64_t batch, int M, int Nc, int K,
                     const void* A, int64_t lda, int64_t sA, const void* B, int64_t ldb, int64_t sB, int* EA, int* EB);

// tcgen05 form of ozaki_zgemm for the HIGH precision class.
template <bool CJ, int FA, int FB>
static int launch_tc(cudaStream_t st, int64_t batch, int M, int Nc, int K, const void* A, int64_t lda, int64_t sA,
                     const void* B, int64_t ldb, int64_t sB, float4* C, int64_t ldc, int64_t sC, int* EA, int* EB,
                     int* err, const char* name, double work) {
    auto kern = oz_tc_kernel<CJ, FA, FB>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM);
    if (e != cudaSuccess) return cuda_error(e, "cudaFuncSetAttribute(oz_tc)");
    KTimer kt(st, name, work);
    for (int64_t b0 = 0; b0 < batch; b0 += 65535) {
        const int64_t nb = std::min<int64_t>(65535, batch - b0);
        dim3 grid((Nc + TC_TN - 1) / TC_TN, (M + TC_TM - 1) / TC_TM, (unsigned)nb);
        const size_t ea = FA == FMT_F32 ? 8 : 16;
        const size_t eb = FB == FMT_F32 ? 8 : (FB == FMT_PRESLICED ? 0 : 16);
        kern<<<grid, 256, TC_SMEM, st>>>(M, Nc, K, static_cast<const char*>(A) + b0 * sA * ea, lda, sA,
                                         static_cast<const char*>(B) + b0 * sB * eb, ldb, sB, EA + b0 * M,
                                         EB + (FB == FMT_PRESLICED ? 0 : b0 * Nc), C + b0 * sC, ldc, sC, err);
        TBG_LAUNCHED(name);
    }
    return TBG_OK;
}

int ozaki_zgemm_tc(cudaStream_t st, bool conj_a, int fmt_a, int fmt_b, int64_t batch, int M, int Nc, int K,
                   const void* A, int64_t lda, int64_t sA, const void* B, int64_t ldb, int64_t sB, float4* C,
                   int64_t ldc, int64_t sC, int* EA, int* EB, int* err) {
    if (K > 256) return set_error(TBG_E_UNSUPPORTED, "ozaki_zgemm_tc: K > 256");
    int rc = ozaki_exp_launch(st, conj_a, fmt_a, fmt_b, batch, M, Nc, K, A, lda, sA, B, ldb, sB, EA, EB);
    if (rc) return rc;
    const double work = 8.0 * (double)M * Nc * K * batch;
#define TC_CASE(CJ, FA, FB)                                                                                          \
    if (conj_a == CJ && fmt_a == FA && fmt_b == FB)                                                                  \
        return launch_tc<CJ, FA, FB>(st, batch, M, Nc, K, A, lda, sA, B, ldb, sB, C, ldc, sC, EA, EB, err,          \
                                     "ozaki_tc_kernel<high>", work);
    TC_CASE(false, FMT_F64, FMT_F64)
    TC_CASE(true, FMT_F64, FMT_F64)
    TC_CASE(true, FMT_F32, FMT_F32)
    TC_CASE(false, FMT_F64, FMT_F32)
    TC_CASE(true, FMT_F32, FMT_PAIR)
    TC_CASE(false, FMT_F64, FMT_PAIR)
    TC_CASE(true, FMT_PAIR, FMT_PAIR)
#undef TC_CASE
    return set_error(TBG_E_UNSUPPORTED, "ozaki_zgemm_tc: operand format combination not instantiated");
}

// Fourier contraction on tcgen05: C (M x Nc) = A (M x K FP64) . hop digit planes; EA filled by the caller.
int ozaki_fourier_tc(cudaStream_t st, int64_t M, int64_t Nc, int K, const zc* A, const int* EA, const int* EB,
                     const void* Bs, float4* C, int* err) {
    auto kern = oz_tc_kernel<false, FMT_F64, FMT_PRESLICED>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM);
    if (e != cudaSuccess) return cuda_error(e, "cudaFuncSetAttribute(oz_tc fourier)");
    KTimer kt(st, "ozaki_tc_fourier_kernel", 8.0 * (double)M * Nc * K);
    for (int64_t m0 = 0; m0 < M; m0 += (int64_t)TC_TM * 65535) {
        const int64_t mb = std::min<int64_t>(M - m0, (int64_t)TC_TM * 65535);
        dim3 grid((unsigned)((Nc + TC_TN - 1) / TC_TN), (unsigned)((mb + TC_TM - 1) / TC_TM), 1);
        kern<<<grid, 256, TC_SMEM, st>>>((int)mb, (int)Nc, K, A + m0 * K, K, 0, Bs, Nc, 0, EA + m0, EB, C + m0 * Nc,
                                         Nc, 0, err);
        TBG_LAUNCHED("ozaki_tc_fourier_kernel");
    }
    return TBG_OK;
}

}  // namespace tbg
