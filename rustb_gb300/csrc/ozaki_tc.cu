// Exact-slice complex GEMM on the 5th-generation tensor cores (tcgen05, TMEM).
//
// Same number format as ozaki.cu: every value of a row (column) of an operand
// is written on the fixed-point grid 2^(E-42) of that row's exponent E and cut
// into six signed 7-bit digits, stored pre-scaled as BF16 planes q_s 2^(-7s);
// digit products of level s + t = 0, 1, 2 are accumulated exactly in separate
// FP32 accumulators, levels 3..5 together, and the four are combined into a
// float pair.  Issued as tcgen05.mma.cta_group::1.kind::f16 (BF16 x BF16 ->
// FP32, M = 128, N = 128, K = 16) from shared-memory descriptors; the four
// accumulation levels are 4 x 128 FP32 columns of tensor memory.
//
// CTA = 13 warps, one output tile of 128 rows x 64 complex columns:
//   warps 0..7   A digit producers: thread = (row, 8 consecutive k); load the
//                8 elements of the next stage into registers while converting
//                the current one, write each digit plane as one 16-byte store
//                (K-major core matrices of 8 rows x 16 bytes, no swizzle);
//   warps 8..11  B digit producers, same per (column, 8 consecutive k), or,
//                for a pre-sliced operand, one thread that copies the stage
//                image with cp.async.bulk (completion on an mbarrier);
//   warp 12      allocates TMEM; lane 0 issues the MMAs and commits them;
//   warps 0..7   after the K loop: read the four levels from TMEM (tcgen05.ld
//                32x32b, one TMEM lane = one output row), combine them with
//                error-free sums and write the float pairs.
// Stage hand-off uses mbarriers: full[b] (producer arrivals), bcopy[b] (bulk
// copy bytes), empty[b] (tcgen05.commit of the MMAs that read buffer b).
// Every wait is bounded; on a time-out the CTA records an error, waits
// (bounded) for its own bulk copies and committed MMAs, frees TMEM and returns.

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdint>

#include "tbgpu_internal.cuh"
#include "tc_ptx.cuh"

namespace tbg {

namespace {

constexpr int TC_TM = 128;        // output rows
constexpr int TC_TN = 64;         // complex output columns (128 real)
constexpr int TC_TK = 16;         // complex k per stage (32 real)
constexpr int TC_S = 6;           // digits per value (HIGH precision class)
constexpr int PLANE = 128 * 32 * 2;             // bytes of one digit plane (128 rows x 32 k bf16)
constexpr int HALF_STAGE = TC_S * PLANE;        // the six planes of one operand (49152 bytes)
// Precision classes: S digits per value, digit pairs s + t <= LMAX, NLEV TMEM
// accumulators (levels below NLEV - 1 each exact in their own, the rest merged).
//   HIGH: S = 6, LMAX = 5, NLEV = 4  (about 2^-43 of the product scale)
//   LOW : S = 3, LMAX = 2, NLEV = 1  (about 2^-21; for small corrections)
template <int S> struct Class;
template <> struct Class<6> { static constexpr int LMAX = 5, NLEV = 4, MIN_CTAS = 1; };
//   MID : S = 5, LMAX = 4, NLEV = 4  (about 2^-35; the rotation into the eigenbasis)
template <> struct Class<5> { static constexpr int LMAX = 4, NLEV = 4, MIN_CTAS = 1; };
template <> struct Class<3> { static constexpr int LMAX = 2, NLEV = 1, MIN_CTAS = 2; };
constexpr int tc_smem_bytes(int S) { return 2 * 2 * S * PLANE + 1024; }  // two stages of A and B planes + slack
constexpr int TC_SMEM = tc_smem_bytes(TC_S);
// whether a class's two stage buffers can hold the 128 x 65 float-pair output tile
constexpr bool tc_staged(int S) { return 2 * 2 * S * PLANE >= 128 * 65 * 16; }
constexpr int TC_THREADS = 416;                 // 13 warps
constexpr int MMA_WARP = 12;
constexpr int A_PRODUCERS = 256;
constexpr int B_PRODUCERS = 128;
constexpr int ZERO_EXP = kLineZeroExp;
// Longest contraction one launch keeps exact: 2K real terms of digit products
// below 2^15 per level stay within FP32's 24-bit significand.
constexpr int kTcMaxK = 256;

enum { FMT_F64 = 0, FMT_F32 = 1, FMT_PAIR = 2, FMT_PRESLICED = 3 };

// instruction descriptor, kind::f16: D = F32, A = B = BF16, K-major, N = 128, M = 128
constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((128u >> 3) << 17) | ((128u >> 4) << 24);

using namespace tc;

std::atomic<int> g_tc_wait_limit{kTcWaitPolls};

// 1-D bulk copy global -> shared, completion counted in bytes on `bar`.
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(su32(bar))
                 : "memory");
}

// One MMA; COL selects the use of the A collector buffer across consecutive
// MMAs with the same A: 0 none, 1 fill, 2 use, 3 last use.
template <int COL>
__device__ __forceinline__ void umma(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
#define TBG_UMMA(Q)                                                                                             \
    asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\ttcgen05.mma.cta_group::1.kind::f16" Q        \
                 " [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),                                                     \
                 "l"(adesc), "l"(bdesc), "r"(IDESC), "r"(accumulate)                                            \
                 : "memory")
    if constexpr (COL == 1)
        TBG_UMMA(".collector::a::fill");
    else if constexpr (COL == 2)
        TBG_UMMA(".collector::a::use");
    else if constexpr (COL == 3)
        TBG_UMMA(".collector::a::lastuse");
    else
        TBG_UMMA("");
#undef TBG_UMMA
}
// ---- digit extraction ----
// Fixed-point value trunc(x * 2^(42 - E)) of a double with |x| < 2^E.
__device__ __forceinline__ long long fx64(double x, int E) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int ex = (int)((b >> 52) & 0x7ff);
    if (ex == 0) return 0;
    const unsigned long long M = (b & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    const int sh = 10 + E - (ex - 1023);
    const long long F = (sh >= 64) ? 0 : (long long)(M >> sh);
    return (b >> 63) ? -F : F;
}
// Fixed-point value trunc(x * 2^(42 - E)) of a float with |x| < 2^E.
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

// r rounded to the nearest multiple of 2^k (ties to even) by adding and
// subtracting 1.5 * 2^(23 + k); exact for |r| < 2^(22 + k).
constexpr double pow2c(int e) { return e == 0 ? 1.0 : (e > 0 ? 2.0 * pow2c(e - 1) : 0.5 * pow2c(e + 1)); }
template <int K>
__device__ __forceinline__ float round_to_pow2(float r) {
    constexpr float C = (float)(1.5 * pow2c(23 + K));
    return __fsub_rn(__fadd_rn(r, C), C);
}

// Six pre-scaled digits P_s = q_s 2^(-7s) of a fixed-point F (|F| < 2^42),
// F = sum_s q_s 2^(35 - 7s).  F is split as hi 2^21 + lo (lo in [0, 2^21)),
// each half is exact in FP32 and is cut by rounding to the nearest multiple
// of the digit weight; every step is exact.  |q_0| <= 128, |q_1|, |q_2|,
// |q_4|, |q_5| <= 64, q_3 in [0, 128].
__device__ __forceinline__ void digits_fixed(long long F, float* P) {
    const int hi = (int)(F >> 21);
    const int lo = (int)(F & 0x1FFFFF);
    const float a = (float)hi * 0x1p-14f;  // [-128, 128)
    P[0] = round_to_pow2<0>(a);
    const float r = __fsub_rn(a, P[0]);    // a multiple of 2^-14, |r| <= 1/2
    P[1] = round_to_pow2<-7>(r);
    P[2] = __fsub_rn(r, P[1]);              // q_2 2^-14
    const float c = (float)lo * 0x1p-35f;  // [0, 2^-14)
    P[3] = round_to_pow2<-21>(c);
    const float r2 = __fsub_rn(c, P[3]);
    P[4] = round_to_pow2<-28>(r2);
    P[5] = __fsub_rn(r2, P[4]);             // q_5 2^-35
}
// Six pre-scaled digits of u = x 2^(7 - E) in (-128, 128) for an FP32 x:
// P_s = u_s rounded to a multiple of 2^(-7s), u_{s+1} = u_s - P_s, every step
// exact; the sum equals x rounded to the grid 2^(E-42).  |q_0| <= 128,
// |q_s| <= 64.
__device__ __forceinline__ void digits_float(float u, float* P) {
    P[0] = round_to_pow2<0>(u);
    float r = __fsub_rn(u, P[0]);
    P[1] = round_to_pow2<-7>(r);
    r = __fsub_rn(r, P[1]);
    P[2] = round_to_pow2<-14>(r);
    r = __fsub_rn(r, P[2]);
    P[3] = round_to_pow2<-21>(r);
    r = __fsub_rn(r, P[3]);
    P[4] = round_to_pow2<-28>(r);
    r = __fsub_rn(r, P[4]);
    P[5] = round_to_pow2<-35>(r);
}
// Six pre-scaled digits of u = (hi + lo) 2^(7 - E) in (-128, 128] for a
// float pair, in FP32 arithmetic only.  The pair is first renormalised by an
// error-free two-sum (the producers' pairs need not have |lo| <= ulp(hi) / 2);
// digits 0..2 then come from the leading part, whose remainder r (|r| <=
// 2^-15, a subset of its bits) is exact; t = r + lo then needs the bits from
// 2^-15 down to the grid 2^-35 (21 bits), so its rounding stays below the
// grid, and digits 3..5 come from t.  The sum of the digits is u on the grid
// 2^-35 up to half a grid step plus t's rounding (the integer form truncates
// each part: up to two grid steps).  |q_0| <= 128, |q_1|, |q_2|, |q_4|,
// |q_5| <= 64, |q_3| <= 72.
__device__ __forceinline__ void digits_pair(float uh, float ul, float* P) {
    {
        const float sm = __fadd_rn(uh, ul);
        const float v = __fsub_rn(sm, uh);
        ul = __fadd_rn(__fsub_rn(uh, __fsub_rn(sm, v)), __fsub_rn(ul, v));
        uh = sm;
    }
    P[0] = round_to_pow2<0>(uh);
    float r = __fsub_rn(uh, P[0]);
    P[1] = round_to_pow2<-7>(r);
    r = __fsub_rn(r, P[1]);
    P[2] = round_to_pow2<-14>(r);
    r = __fsub_rn(r, P[2]);
    float t = __fadd_rn(r, ul);
    P[3] = round_to_pow2<-21>(t);
    t = __fsub_rn(t, P[3]);
    P[4] = round_to_pow2<-28>(t);
    t = __fsub_rn(t, P[4]);
    P[5] = round_to_pow2<-35>(t);
}
__device__ __forceinline__ float pow2f(int n) { return __int_as_float((127 + n) << 23); }  // n in [-126, 127]
// 2^(7 - E) as s1 * s2 (each a normal float) for FP32 operands; 0 for a zero line.
__device__ __forceinline__ void f32_scales(int E, float& s1, float& s2) {
    if (E == ZERO_EXP) {
        s1 = s2 = 0.f;
        return;
    }
    const int sh = 7 - E;  // in [-122, 155] for finite floats
    const int a = min(sh, 127);
    s1 = pow2f(max(a, -126));
    s2 = pow2f(sh - a);
}

// One element as raw bits: F64 {re, im} doubles, F32 {re, im} floats in .x/.y,
// PAIR {re_hi, re_lo, im_hi, im_lo} floats.
template <int FMT>
__device__ __forceinline__ int4 ld_elem(const void* base, int64_t idx) {
    if (FMT == FMT_F32) {
        const int2 t = __ldg(reinterpret_cast<const int2*>(base) + idx);
        return make_int4(t.x, t.y, 0, 0);
    }
    return __ldg(reinterpret_cast<const int4*>(base) + idx);
}
template <int FMT>
__device__ __forceinline__ void load8(const void* base, int64_t idx0, int64_t stride, int nvalid, int4 (&r)[8]) {
#pragma unroll
    for (int i = 0; i < 8; ++i) r[i] = (i < nvalid) ? ld_elem<FMT>(base, idx0 + (int64_t)i * stride) : make_int4(0, 0, 0, 0);
}
// Digits of the real (part 0) or imaginary (part 1) component of one element.
template <int FMT, int PART>
__device__ __forceinline__ void elem_digits(const int4& r, int E, float s1, float s2, float* P) {
    if (FMT == FMT_F32) {
        const float x = __int_as_float(PART ? r.y : r.x);
        digits_float((x * s1) * s2, P);
    } else if (FMT == FMT_PAIR) {
        const float hi = __int_as_float(PART ? r.z : r.x), lo = __int_as_float(PART ? r.w : r.y);
        digits_pair(__fmul_rn(__fmul_rn(hi, s1), s2), __fmul_rn(__fmul_rn(lo, s1), s2), P);
    } else {
        long long F = 0;
        if (E != ZERO_EXP) {
            if (FMT == FMT_F64)
                F = PART ? fx64(__hiloint2double(r.w, r.z), E) : fx64(__hiloint2double(r.y, r.x), E);
            else
                F = PART ? fx32(__int_as_float(r.z), E) + fx32(__int_as_float(r.w), E)
                         : fx32(__int_as_float(r.x), E) + fx32(__int_as_float(r.y), E);
        }
        digits_fixed(F, P);
    }
}
// (ah + al) + (bh + bl) as a float pair: two-sum of the leading parts, the
// trailing parts and the rounding error added, then renormalised.
__device__ __forceinline__ float2 pair_add(float ah, float al, float bh, float bl) {
    const float s = __fadd_rn(ah, bh);
    const float v = __fsub_rn(s, ah);
    const float e = __fadd_rn(__fadd_rn(__fsub_rn(ah, __fsub_rn(s, v)), __fsub_rn(bh, v)), __fadd_rn(al, bl));
    const float h = __fadd_rn(s, e);
    return make_float2(h, __fsub_rn(e, __fsub_rn(h, s)));
}
__device__ __forceinline__ uint32_t pack_bf16x2(float lo_k, float hi_k) {
    __nv_bfloat162 h = __floats2bfloat162_rn(lo_k, hi_k);
    return *reinterpret_cast<uint32_t*>(&h);
}
// The six digit planes of one component of 8 consecutive-k elements: out[s]
// holds 8 BF16 (k ascending) = one 16-byte row segment of a core matrix.
// The leading S of the six digits are kept (S = 3: the value truncated to 21 bits).
template <int FMT, int PART, int S>
__device__ __forceinline__ void item_planes(const int4 (&r)[8], int E, float s1, float s2, uint4 (&out)[S]) {
    uint32_t pk[S][4];
#pragma unroll
    for (int i = 0; i < 8; i += 2) {
        float P0[TC_S], P1[TC_S];
        elem_digits<FMT, PART>(r[i], E, s1, s2, P0);
        elem_digits<FMT, PART>(r[i + 1], E, s1, s2, P1);
#pragma unroll
        for (int s = 0; s < S; ++s) pk[s][i >> 1] = pack_bf16x2(P0[s], P1[s]);
    }
#pragma unroll
    for (int s = 0; s < S; ++s) out[s] = make_uint4(pk[s][0], pk[s][1], pk[s][2], pk[s][3]);
}
__device__ __forceinline__ uint4 neg_bf16x8(uint4 v) {
    const uint32_t m = 0x80008000u;
    return make_uint4(v.x ^ m, v.y ^ m, v.z ^ m, v.w ^ m);
}
// byte offset of element (row, k') inside one digit plane (K-major core matrices)
__host__ __device__ __forceinline__ int plane_off(int row, int kp) {
    return (((row >> 3) * 4 + (kp >> 3)) << 7) + ((row & 7) << 4) + ((kp & 7) << 1);
}
__device__ __forceinline__ int n_valid(int K, int kfirst) { return max(0, min(8, K - kfirst)); }

// One tile = 128 rows x 64 complex columns of one matrix.  Tiles are numbered
// as the blocks of a (gx, gy, batch) grid, x fastest: x = row tile when
// rows_fast, else column tile.
struct TileId {
    int rt, ct;
    int64_t b;
};
__device__ __forceinline__ TileId tile_of(int64_t L, int gx, int gy, int rows_fast) {
    const int x = (int)(L % gx);
    const int64_t r = L / gx;
    const int y = (int)(r % gy);
    TileId t;
    t.b = r / gy;
    t.rt = rows_fast ? x : y;
    t.ct = rows_fast ? y : x;
    return t;
}

// OR of v over the eight epilogue warps (named barrier 1, 256 threads): every
// participating thread gets the same verdict.
__device__ __forceinline__ bool epilogue_any(bool v) {
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\tsetp.ne.u32 q, %1, 0;\n\tbar.red.or.pred p, 1, 256, q;\n\tselp.u32 %0, 1, 0, "
        "p;\n\t}"
        : "=r"(r)
        : "r"((uint32_t)v)
        : "memory");
    return r != 0;
}

// Persistent CTAs: each walks the tiles blockIdx.x, blockIdx.x + gridDim.x, ...
// Every role keeps the same tile order; a stage's buffer and barrier phase come
// from the CTA's running stage count gs = (tiles before) * nstages + it.  The
// epilogue warps (the A producers) drain the tile's accumulators from TMEM
// (bar_tmem frees them for the next tile's MMAs), stage the tile of float
// pairs in the idle stage buffers and write it out row by row, coalesced;
// bar_stage then hands the buffers to the next tile's B stages.  The next
// tile's first A and B stages are loaded into registers before the drain.
template <bool CONJ_A, int FMTA, int FMTB, int S>
__global__ void __launch_bounds__(TC_THREADS, Class<S>::MIN_CTAS)
    oz_tc_kernel(int M, int Nc, int K, const void* __restrict__ A, int64_t lda, int64_t sA, const void* __restrict__ B,
                 int64_t ldb, int64_t sB, const int* __restrict__ EA, const int* __restrict__ EB,
                 float4* __restrict__ C, int64_t ldc, int64_t sC, int rows_fast, int* __restrict__ err,
                 int accumulate, int* __restrict__ Ecol, int wait_limit, int gx, int gy, int64_t ntiles) {
    constexpr bool PRE = FMTB == FMT_PRESLICED;
    // A pre-sliced too (stage images of S planes per row tile, the Fourier
    // sum's phases): the copy thread brings both operands, the A warps only run
    // the epilogue
    constexpr bool PRE_A = FMTA == FMT_PRESLICED;
    static_assert(!PRE_A || (PRE && !CONJ_A), "pre-sliced A goes with pre-sliced B, not conjugated");
    constexpr int LMAX = Class<S>::LMAX, NLEV = Class<S>::NLEV;
    constexpr int HS = S * PLANE;             // planes of one operand in a stage
    constexpr int SB = 2 * HS;                // stage bytes
    constexpr uint32_t TMEM_COLS = NLEV * 128;
    extern __shared__ __align__(1024) unsigned char tc_smem[];
    unsigned char* base = reinterpret_cast<unsigned char*>(((uintptr_t)tc_smem + 1023) & ~(uintptr_t)1023);
    __shared__ __align__(8) uint64_t bar_full[2], bar_bcopy[2], bar_empty[2], bar_done, bar_tmem, bar_stage;
    __shared__ uint32_t tmem_base_sh;
    __shared__ volatile int abort_sh;
    __shared__ int emax[2][4][TC_TN];  // column maxima of a tile (float bits) by lane quarter
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nstages = (K + TC_TK - 1) / TC_TK;
    const uint32_t sbase = su32(base);
    // With room in the stage buffers the 128 x 64 output tile is staged there
    // (rows padded to 65 entries: no bank conflicts either way).
    constexpr int TROW = TC_TN + 1;
    constexpr bool STAGE = 2 * SB >= TC_TM * TROW * 16;
    float4* tile = reinterpret_cast<float4*>(base);

    if (tid == 0) {
        const uint32_t nfull = PRE ? A_PRODUCERS : A_PRODUCERS + B_PRODUCERS;
        mbar_init(&bar_full[0], nfull);
        mbar_init(&bar_full[1], nfull);
        mbar_init(&bar_bcopy[0], 1);
        mbar_init(&bar_bcopy[1], 1);
        mbar_init(&bar_empty[0], 1);
        mbar_init(&bar_empty[1], 1);
        mbar_init(&bar_done, 1);
        mbar_init(&bar_tmem, 8);  // one arrival per epilogue warp
        mbar_init(&bar_stage, 1);
        abort_sh = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == MMA_WARP) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(&tmem_base_sh)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base_sh;
    int ndone = 0;  // MMA thread: tiles committed to bar_done

    if (warp == MMA_WARP) {
        // ------------------------------------------------ MMA issuer (lane 0)
        if (lane == 0) {
            int tn = 0;
            for (int64_t L = blockIdx.x; L < ntiles; L += gridDim.x, ++tn) {
                // the previous tile's accumulators have been read out
                if (tn > 0 && !mbar_wait(&bar_tmem, (tn - 1) & 1, &abort_sh, wait_limit)) {
                    abort_sh = 1;
                    break;
                }
                tc_fence_after();
                bool stop = false;
                for (int it = 0; it < nstages; ++it) {
                    const int64_t gs = (int64_t)tn * nstages + it;
                    const int bi = (int)(gs & 1);
                    const uint32_t ph = (uint32_t)((gs >> 1) & 1);
                    if ((!PRE_A && !mbar_wait(&bar_full[bi], ph, &abort_sh, wait_limit)) ||
                        (PRE && !mbar_wait(&bar_bcopy[bi], ph, &abort_sh, wait_limit))) {
                        abort_sh = 1;
                        stop = true;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t sa = sbase + bi * SB;
                    const uint32_t sb = sa + HS;
                    // A digit s outer, B digit t inner: the A tile of a group of
                    // products stays in the collector buffer
#pragma unroll
                    for (int ks = 0; ks < 2; ++ks) {
#pragma unroll
                        for (int s = 0; s < S; ++s) {
                            const int tmax = LMAX - s < S - 1 ? LMAX - s : S - 1;
#pragma unroll
                            for (int t = 0; t <= tmax; ++t) {
                                const int lv = (s + t) < NLEV - 1 ? (s + t) : NLEV - 1;
                                const uint64_t ad = smem_desc(sa + s * PLANE + ks * 256, 128, 512);
                                const uint64_t bd = smem_desc(sb + t * PLANE + ks * 256, 128, 512);
                                // the first product into each accumulator overwrites it
                                // (level l first gets digit pair (0, l); levels >= NLEV - 1 (0, NLEV - 1))
                                const uint32_t acc = (it == 0 && ks == 0 && s == 0 && t <= NLEV - 1) ? 0u : 1u;
                                const uint32_t dst = tmem + (uint32_t)(lv * 128);
                                if (tmax == 0)
                                    umma<0>(dst, ad, bd, acc);
                                else if (t == 0)
                                    umma<1>(dst, ad, bd, acc);
                                else if (t == tmax)
                                    umma<3>(dst, ad, bd, acc);
                                else
                                    umma<2>(dst, ad, bd, acc);
                            }
                        }
                    }
                    umma_commit(&bar_empty[bi]);
                }
                umma_commit(&bar_done);  // this tile's MMAs (all issued so far)
                ++ndone;
                if (stop) break;
            }
        }
        __syncwarp();
    } else if (tid < A_PRODUCERS) {
        // -------------------- A digit producers (row, 8 k), then the epilogue
        const int r = CONJ_A ? (tid & 127) : (tid >> 1);
        const int g = CONJ_A ? (tid >> 7) : (tid & 1);
        const int64_t kstride = CONJ_A ? lda : 1;
        const uint32_t o_re = plane_off(r, 8 * g), o_im = plane_off(r, 16 + 8 * g);
        const int q = warp & 3, h = warp >> 2;  // epilogue: TMEM lanes 32q .. 32q+31; complex columns 32h .. 32h+31
        const uint32_t lane_addr = tmem + ((uint32_t)(32 * q) << 16);
        // element index of (row gi of op(A), k = 0) for tile L, and whether the row exists
        auto row_base = [&](int64_t L, bool& rv) -> int64_t {
            const TileId t = tile_of(L, gx, gy, rows_fast);
            const int gi = t.rt * TC_TM + r;
            rv = gi < M;
            return CONJ_A ? (t.b * sA + gi) : (t.b * sA + (int64_t)gi * lda);
        };
        int4 nxt[8];
        if constexpr (!PRE_A) {
            bool rv0;
            const int64_t i0 = row_base(blockIdx.x, rv0);
            if (blockIdx.x < ntiles)
                load8<FMTA>(A, i0 + (int64_t)(8 * g) * kstride, kstride, rv0 ? n_valid(K, 8 * g) : 0, nxt);
        }
        int tn = 0;
        for (int64_t L = blockIdx.x; L < ntiles; L += gridDim.x, ++tn) {
            const TileId t = tile_of(L, gx, gy, rows_fast);
            const int row0 = t.rt * TC_TM, col0 = t.ct * TC_TN;
            const int gi = row0 + r;
            const bool rv = gi < M;
            const int E = rv ? EA[t.b * M + gi] : ZERO_EXP;
            float s1, s2;
            f32_scales(E, s1, s2);
            const int64_t idx0 = CONJ_A ? (t.b * sA + gi) : (t.b * sA + (int64_t)gi * lda);
            if constexpr (!PRE_A) for (int it = 0; it < nstages; ++it) {
                const int64_t gs = (int64_t)tn * nstages + it;
                const int bi = (int)(gs & 1);
                int4 cur[8];
#pragma unroll
                for (int i = 0; i < 8; ++i) cur[i] = nxt[i];
                if (it + 1 < nstages) {
                    const int kf = (it + 1) * TC_TK + 8 * g;
                    load8<FMTA>(A, idx0 + (int64_t)kf * kstride, kstride, rv ? n_valid(K, kf) : 0, nxt);
                } else if (L + gridDim.x < ntiles) {
                    // the next tile's first stage, in flight during this tile's epilogue
                    bool rvn;
                    const int64_t in = row_base(L + gridDim.x, rvn);
                    load8<FMTA>(A, in + (int64_t)(8 * g) * kstride, kstride, rvn ? n_valid(K, 8 * g) : 0, nxt);
                }
                // slice this stage while the MMAs of the two stages before it run; then
                // wait only for the buffer and store
                uint4 dre[S], dim[S];
                item_planes<FMTA, 0, S>(cur, E, s1, s2, dre);
                item_planes<FMTA, 1, S>(cur, E, s1, s2, dim);
                if (gs >= 2 && !mbar_wait(&bar_empty[bi], (uint32_t)(((gs >> 1) - 1) & 1), &abort_sh, wait_limit)) {
                    abort_sh = 1;
                    break;
                }
                if (abort_sh) break;
                const uint32_t sa = sbase + bi * SB;
#pragma unroll
                for (int s = 0; s < S; ++s) st_shared_v4(sa + s * PLANE + o_re, dre[s]);
#pragma unroll
                for (int s = 0; s < S; ++s) st_shared_v4(sa + s * PLANE + o_im, CONJ_A ? neg_bf16x8(dim[s]) : dim[s]);
                fence_async_smem();  // make the generic-proxy writes visible to the tensor core
                mbar_arrive(&bar_full[bi]);
            }
            // ------------------------------------------------------ epilogue
            // A time-out here is an abort too; either the whole tile is written
            // or none of it
            // (the verdict is one barrier reduction: roles still running may set
            // abort_sh at any time, and the eight warps must agree)
            bool bad = abort_sh != 0;
            if (!bad && !mbar_wait(&bar_done, tn & 1, &abort_sh, wait_limit)) {
                abort_sh = 1;
                bad = true;
            }
            if (epilogue_any(bad)) break;
            tc_fence_after();
            const int re_ = row0 + 32 * q + lane;
            const int ea = (re_ < M) ? EA[t.b * M + re_] : ZERO_EXP;
            const int par = tn & 1;
            for (int cc = 0; cc < 4; ++cc) {
                const int c0 = 32 * h + 8 * cc;
                uint32_t v[2 * NLEV][8];  // [2 * level + (0 re, 1 im)][column]
#pragma unroll
                for (int Lv = 0; Lv < NLEV; ++Lv) {
                    tmem_ld8(lane_addr + (uint32_t)(Lv * 128 + c0), v[2 * Lv]);
                    tmem_ld8(lane_addr + (uint32_t)(Lv * 128 + TC_TN + c0), v[2 * Lv + 1]);
                }
                tmem_wait_ld();
                if (cc == 3) {
                    // every accumulator of this warp's lanes and columns is in registers
                    tc_fence_before();
                    __syncwarp();
                    if (lane == 0) mbar_arrive(&bar_tmem);
                }
#pragma unroll
                for (int c = 0; c < 8; ++c) {
                    const int j = col0 + c0 + c;
                    float hl[4];
#pragma unroll
                    for (int part = 0; part < 2; ++part) {
                        if (NLEV == 1) {
                            hl[2 * part] = __uint_as_float(v[part][c]);
                            hl[2 * part + 1] = 0.f;
                            continue;
                        }
                        const float a0 = __uint_as_float(v[0 + part][c]), a1 = __uint_as_float(v[2 + part][c]);
                        const float a2 = __uint_as_float(v[4 + part][c]), a3 = __uint_as_float(v[6 + part][c]);
                        const float s1_ = a0 + a1;
                        const float t1 = s1_ - a0;
                        const float e1 = (a0 - (s1_ - t1)) + (a1 - t1);
                        const float hi = s1_ + a2;
                        const float t2 = hi - s1_;
                        const float e2 = (s1_ - (hi - t2)) + (a2 - t2);
                        hl[2 * part] = hi;
                        hl[2 * part + 1] = (e1 + e2) + a3;
                    }
                    const int eb = (j < Nc) ? EB[t.b * Nc + j] : ZERO_EXP;
                    float4 out = make_float4(0.f, 0.f, 0.f, 0.f);
                    if (ea != ZERO_EXP && eb != ZERO_EXP) {
                        const int n = max(-126, min(127, ea + eb - 14));
                        const float sc = pow2f(n);
                        out = make_float4(hl[0] * sc, hl[1] * sc, hl[2] * sc, hl[3] * sc);
                    }
                    if (STAGE) {
                        tile[(32 * q + lane) * TROW + c0 + c] = out;
                        continue;
                    }
                    const bool in = re_ < M && j < Nc;
                    if (in) {
                        float4* cp = C + t.b * sC + (int64_t)re_ * ldc + j;
                        if (accumulate) {  // a later K chunk: add to the stored pair
                            const float4 prev = *cp;
                            const float2 pre = pair_add(prev.x, prev.y, out.x, out.y);
                            const float2 pim = pair_add(prev.z, prev.w, out.z, out.w);
                            out = make_float4(pre.x, pre.y, pim.x, pim.y);
                        }
                        *cp = out;
                    }
                    if (Ecol) {
                        // the column's largest magnitude over this warp's rows (>= 0,
                        // NaN as 0: ordered as integers)
                        float mg = in ? pair_mag(out) : 0.f;
                        mg = (mg == mg) ? mg : 0.f;
                        const int mv = __reduce_max_sync(0xffffffffu, __float_as_int(mg));
                        if (lane == 0) emax[par][q][c0 + c] = mv;
                    }
                }
            }
            if (STAGE) {
                asm volatile("bar.sync 1, 256;" ::: "memory");  // the tile is staged
                if (Ecol) {
                    // exponents of the output's columns, as the line scan would take
                    // them (one row tile holds all rows): warp w, columns w, w + 8, ...
                    for (int cl = warp; cl < TC_TN; cl += 8) {
                        float m = 0.f;
                        for (int rl = lane; rl < TC_TM; rl += 32) m = fmaxf(m, pair_mag(tile[rl * TROW + cl]));
#pragma unroll
                        for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
                        if (lane == 0 && col0 + cl < Nc) Ecol[t.b * Nc + col0 + cl] = line_exp_of(m);
                    }
                }
                // warp w writes rows w, w + 8, ...; lanes over the 64 columns
                for (int rl = warp; rl < TC_TM; rl += 8) {
                    const int rr = row0 + rl;
                    if (rr >= M) break;
#pragma unroll
                    for (int half = 0; half < 2; ++half) {
                        const int jl = lane + 32 * half, j = col0 + jl;
                        if (j >= Nc) continue;
                        float4 out = tile[rl * TROW + jl];
                        float4* cp = C + t.b * sC + (int64_t)rr * ldc + j;
                        if (accumulate) {  // a later K chunk: add to the stored pair
                            const float4 prev = *cp;
                            const float2 pre = pair_add(prev.x, prev.y, out.x, out.y);
                            const float2 pim = pair_add(prev.z, prev.w, out.z, out.w);
                            out = make_float4(pre.x, pre.y, pim.x, pim.y);
                        }
                        *cp = out;
                    }
                }
                asm volatile("bar.sync 1, 256;" ::: "memory");  // every read of the staged tile done
                if (tid == 0) mbar_arrive(&bar_stage);
            } else if (Ecol) {
                // one row tile holds every row: the tile's column maxima are the columns'
                asm volatile("bar.sync 1, 256;" ::: "memory");
                if (tid < TC_TN && col0 + tid < Nc) {
                    const int mx = max(max(emax[par][0][tid], emax[par][1][tid]), max(emax[par][2][tid], emax[par][3][tid]));
                    Ecol[t.b * Nc + col0 + tid] = line_exp_of(__int_as_float(mx));
                }
            }
        }
    } else if (tid < A_PRODUCERS + B_PRODUCERS) {
        const int qb = tid - A_PRODUCERS;
        if (PRE) {
            // ------------------------- pre-sliced B: bulk copy of stage images
            if (qb == 0) {
                int64_t last[2] = {-1, -1};
                int tn = 0;
                bool stop = false;
                for (int64_t L = blockIdx.x; L < ntiles && !stop; L += gridDim.x, ++tn) {
                    const TileId t = tile_of(L, gx, gy, rows_fast);
                    // stage images hold TC_S planes; a class with fewer digits copies the leading S
                    const unsigned char* src =
                        static_cast<const unsigned char*>(B) + (int64_t)t.ct * nstages * HALF_STAGE;
                    // the A images of this row tile (S planes per stage)
                    const unsigned char* srca =
                        PRE_A ? static_cast<const unsigned char*>(A) + (int64_t)t.rt * nstages * HS : nullptr;
                    for (int it = 0; it < nstages; ++it) {
                        const int64_t gs = (int64_t)tn * nstages + it;
                        const int bi = (int)(gs & 1);
                        if ((gs >= 2 &&
                             !mbar_wait(&bar_empty[bi], (uint32_t)(((gs >> 1) - 1) & 1), &abort_sh, wait_limit)) ||
                            (STAGE && tn > 0 && it < 2 &&
                             !mbar_wait(&bar_stage, (uint32_t)((tn - 1) & 1), &abort_sh, wait_limit))) {
                            abort_sh = 1;
                            stop = true;
                            break;
                        }
                        if (abort_sh) {
                            stop = true;
                            break;
                        }
                        mbar_arrive_tx(&bar_bcopy[bi], PRE_A ? 2 * HS : HS);
                        if (PRE_A) bulk_g2s(sbase + bi * SB, srca + (int64_t)it * HS, HS, &bar_bcopy[bi]);
                        bulk_g2s(sbase + bi * SB + HS, src + (int64_t)it * HALF_STAGE, HS, &bar_bcopy[bi]);
                        last[bi] = gs;
                    }
                }
                // every copy issued has landed before the CTA can leave
                for (int bi = 0; bi < 2; ++bi)
                    if (last[bi] >= 0) mbar_wait_plain(&bar_bcopy[bi], (uint32_t)((last[bi] >> 1) & 1));
            }
        } else {
            // ---------------------------------- B digit producers (col, 8 k)
            // real embedding: row j = [Re B | -Im B], row 64 + j = [Im B | Re B]
            const int j = qb & 63, g = qb >> 6;
            const uint32_t o_jre = plane_off(j, 8 * g), o_jim = plane_off(j, 16 + 8 * g);
            const uint32_t o_kre = plane_off(64 + j, 8 * g), o_kim = plane_off(64 + j, 16 + 8 * g);
            constexpr int FB = PRE ? FMT_F64 : FMTB;
            auto col_base = [&](int64_t L, bool& cv) -> int64_t {
                const TileId t = tile_of(L, gx, gy, rows_fast);
                const int gj = t.ct * TC_TN + j;
                cv = gj < Nc;
                return t.b * sB + gj;
            };
            int4 nxt[8];
            {
                bool cv0;
                const int64_t i0 = col_base(blockIdx.x, cv0);
                if (blockIdx.x < ntiles) load8<FB>(B, i0 + (int64_t)(8 * g) * ldb, ldb, cv0 ? n_valid(K, 8 * g) : 0, nxt);
            }
            int tn = 0;
            bool stop = false;
            for (int64_t L = blockIdx.x; L < ntiles && !stop; L += gridDim.x, ++tn) {
                const TileId t = tile_of(L, gx, gy, rows_fast);
                const int gj = t.ct * TC_TN + j;
                const bool cv = gj < Nc;
                const int E = cv ? EB[t.b * Nc + gj] : ZERO_EXP;
                float s1, s2;
                f32_scales(E, s1, s2);
                const int64_t idx0 = t.b * sB + gj;
                for (int it = 0; it < nstages; ++it) {
                    const int64_t gs = (int64_t)tn * nstages + it;
                    const int bi = (int)(gs & 1);
                    int4 cur[8];
#pragma unroll
                    for (int i = 0; i < 8; ++i) cur[i] = nxt[i];
                    if (it + 1 < nstages) {
                        const int kf = (it + 1) * TC_TK + 8 * g;
                        load8<FB>(B, idx0 + (int64_t)kf * ldb, ldb, cv ? n_valid(K, kf) : 0, nxt);
                    } else if (L + gridDim.x < ntiles) {
                        bool cvn;
                        const int64_t in = col_base(L + gridDim.x, cvn);
                        load8<FB>(B, in + (int64_t)(8 * g) * ldb, ldb, cvn ? n_valid(K, 8 * g) : 0, nxt);
                    }
                    uint4 dre[S], dim[S];
                    item_planes<FB, 0, S>(cur, E, s1, s2, dre);
                    item_planes<FB, 1, S>(cur, E, s1, s2, dim);
                    if ((gs >= 2 &&
                         !mbar_wait(&bar_empty[bi], (uint32_t)(((gs >> 1) - 1) & 1), &abort_sh, wait_limit)) ||
                        (STAGE && tn > 0 && it < 2 &&
                         !mbar_wait(&bar_stage, (uint32_t)((tn - 1) & 1), &abort_sh, wait_limit))) {
                        abort_sh = 1;
                        stop = true;
                        break;
                    }
                    if (abort_sh) {
                        stop = true;
                        break;
                    }
                    const uint32_t sb = sbase + bi * SB + HS;
#pragma unroll
                    for (int s = 0; s < S; ++s) {
                        st_shared_v4(sb + s * PLANE + o_jre, dre[s]);
                        st_shared_v4(sb + s * PLANE + o_kim, dre[s]);
                    }
#pragma unroll
                    for (int s = 0; s < S; ++s) {
                        st_shared_v4(sb + s * PLANE + o_kre, dim[s]);
                        st_shared_v4(sb + s * PLANE + o_jim, neg_bf16x8(dim[s]));
                    }
                    fence_async_smem();
                    mbar_arrive(&bar_full[bi]);
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (abort_sh && tid == 0) atomicOr(err, 2);  // bit 1: a bounded wait ran out
    if (warp == MMA_WARP) {
        // every committed MMA has finished (the last commit tracks all of them)
        if (lane == 0 && ndone > 0) mbar_wait_plain(&bar_done, (uint32_t)((ndone - 1) & 1));
        __syncwarp();
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
    }
}

// Stage images of the hop table for the Fourier contraction: for column tile
// ct and stage it, the six B digit planes exactly as oz_tc_kernel's shared
// stage holds them (HALF_STAGE bytes at (ct * nstages + it) * HALF_STAGE).
// One thread per (column, 8 consecutive R).
// Column gj of the contraction is matrix element colmap[gj] of the hop table
// (identity when colmap is null); rows of the table are ldh elements apart.
__global__ void hop_image_kernel(int K, int64_t Nc, const zc* __restrict__ ham, const int* __restrict__ EB,
                                 unsigned char* __restrict__ img, const int* __restrict__ colmap, int64_t ldh) {
    const int nst = (K + TC_TK - 1) / TC_TK;
    const int64_t nct = (Nc + TC_TN - 1) / TC_TN;
    const int64_t total = nct * nst * B_PRODUCERS;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int q = (int)(idx % B_PRODUCERS);
        const int64_t blk = idx / B_PRODUCERS;  // ct * nst + it
        const int it = (int)(blk % nst);
        const int64_t ct = blk / nst;
        const int j = q & 63, g = q >> 6;
        const int64_t gj = ct * TC_TN + j;
        const bool cv = gj < Nc;
        const int64_t el = cv ? (colmap ? (int64_t)colmap[gj] : gj) : 0;
        const int E = cv ? EB[el] : ZERO_EXP;
        const int kf = it * TC_TK + 8 * g;
        int4 r[8];
        load8<FMT_F64>(ham, (int64_t)kf * ldh + el, ldh, cv ? n_valid(K, kf) : 0, r);
        unsigned char* dst = img + blk * HALF_STAGE;
        uint4 d[TC_S];
        item_planes<FMT_F64, 0, TC_S>(r, E, 0.f, 0.f, d);
#pragma unroll
        for (int s = 0; s < TC_S; ++s) {
            *reinterpret_cast<uint4*>(dst + s * PLANE + plane_off(j, 8 * g)) = d[s];
            *reinterpret_cast<uint4*>(dst + s * PLANE + plane_off(64 + j, 16 + 8 * g)) = d[s];
        }
        item_planes<FMT_F64, 1, TC_S>(r, E, 0.f, 0.f, d);
#pragma unroll
        for (int s = 0; s < TC_S; ++s) {
            *reinterpret_cast<uint4*>(dst + s * PLANE + plane_off(64 + j, 8 * g)) = d[s];
            *reinterpret_cast<uint4*>(dst + s * PLANE + plane_off(j, 16 + 8 * g)) = neg_bf16x8(d[s]);
        }
    }
}

// Stage images for a contraction with real coefficients: A' = Phi as complex
// numbers whose real and imaginary parts are consecutive coefficients
// (A'_kappa = Phi_{2 kappa} + i Phi_{2 kappa + 1}), B = table T with 2 Kc rows.
// With B rows j = [Re T_{2 kappa} | Re T_{2 kappa + 1}] and 64 + j =
// [Im T_{2 kappa} | Im T_{2 kappa + 1}] over the stage's 16 + 16 k slots, the
// unchanged kernel yields column j = Re(sum_k Phi_k T_k), 64 + j = its
// imaginary part: half the stages of the complex-coefficient form.
__global__ void hop_image_real_kernel(int Kc, int64_t Nc, const zc* __restrict__ T, const int* __restrict__ EB,
                                      unsigned char* __restrict__ img, const int* __restrict__ colmap, int64_t ldh) {
    const int nst = (Kc + TC_TK - 1) / TC_TK;
    const int64_t nct = (Nc + TC_TN - 1) / TC_TN;
    const int64_t total = nct * nst * B_PRODUCERS;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int q = (int)(idx % B_PRODUCERS);
        const int64_t blk = idx / B_PRODUCERS;  // ct * nst + it
        const int it = (int)(blk % nst);
        const int64_t ct = blk / nst;
        const int j = q & 63, g = q >> 6;
        const int64_t gj = ct * TC_TN + j;
        const bool cv = gj < Nc;
        const int64_t el = cv ? (colmap ? (int64_t)colmap[gj] : gj) : 0;
        const int E = cv ? EB[el] : ZERO_EXP;
        const int kf = it * TC_TK + 8 * g;  // first kappa of this thread
        const int nv = cv ? n_valid(Kc, kf) : 0;
        int4 re[8], ro[8];                   // rows 2 kappa and 2 kappa + 1
        load8<FMT_F64>(T, (int64_t)(2 * kf) * ldh + el, 2 * ldh, nv, re);
        load8<FMT_F64>(T, (int64_t)(2 * kf + 1) * ldh + el, 2 * ldh, nv, ro);
        unsigned char* dst = img + blk * HALF_STAGE;
        uint4 d[TC_S];
        item_planes<FMT_F64, 0, TC_S>(re, E, 0.f, 0.f, d);
#pragma unroll
        for (int s = 0; s < TC_S; ++s) *reinterpret_cast<uint4*>(dst + s * PLANE + plane_off(j, 8 * g)) = d[s];
        item_planes<FMT_F64, 0, TC_S>(ro, E, 0.f, 0.f, d);
#pragma unroll
        for (int s = 0; s < TC_S; ++s) *reinterpret_cast<uint4*>(dst + s * PLANE + plane_off(j, 16 + 8 * g)) = d[s];
        item_planes<FMT_F64, 1, TC_S>(re, E, 0.f, 0.f, d);
#pragma unroll
        for (int s = 0; s < TC_S; ++s) *reinterpret_cast<uint4*>(dst + s * PLANE + plane_off(64 + j, 8 * g)) = d[s];
        item_planes<FMT_F64, 1, TC_S>(ro, E, 0.f, 0.f, d);
#pragma unroll
        for (int s = 0; s < TC_S; ++s)
            *reinterpret_cast<uint4*>(dst + s * PLANE + plane_off(64 + j, 16 + 8 * g)) = d[s];
    }
}

}  // namespace

int tc_wait_limit() { return g_tc_wait_limit.load(std::memory_order_relaxed); }

// Multiprocessors of the current device (the persistent kernels' grid).
static int sm_count() {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n < 1) {
        cudaGetLastError();
        n = 1;
    }
    return n;
}

int ozaki_exp_launch(cudaStream_t st, bool conj_a, int fmt_a, int fmt_b, int64_t batch, int M, int Nc, int K,
                     const void* A, int64_t lda, int64_t sA, const void* B, int64_t ldb, int64_t sB, int* EA, int* EB);

// tcgen05 form of ozaki_zgemm for the HIGH precision class.
template <bool CJ, int FA, int FB, int S>
static int launch_tc(cudaStream_t st, int64_t batch, int M, int Nc, int K, const void* A, int64_t lda, int64_t sA,
                     const void* B, int64_t ldb, int64_t sB, float4* C, int64_t ldc, int64_t sC, int* EA, int* EB,
                     int* err, const char* name, double work, int accumulate = 0, int* Ecol = nullptr) {
    auto kern = oz_tc_kernel<CJ, FA, FB, S>;
    constexpr int smem = tc_smem_bytes(S);
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return cuda_error(e, "cudaFuncSetAttribute(oz_tc)");
    KTimer kt(st, name, work);
    // tiles (column tile, row tile, matrix), column tiles fastest; persistent
    // CTAs where the output is staged in shared memory (HIGH, MID: the
    // per-CTA set-up and launch gap were ~12 % of a 128^3 tile), one tile per
    // CTA for the LOW class (two CTAs per SM already overlap its epilogues)
    const int gx = (Nc + TC_TN - 1) / TC_TN, gy = (M + TC_TM - 1) / TC_TM;
    const int64_t ntiles = (int64_t)gx * gy * batch;
    if (ntiles <= 0) return TBG_OK;  // nothing to compute
    if (K <= 0) return set_error(TBG_E_INVALID_ARGUMENT, "ozaki_zgemm_tc: empty contraction");
    const int64_t grid = tc_staged(S) ? std::min<int64_t>(ntiles, (int64_t)sm_count() * Class<S>::MIN_CTAS)
                                      : std::min<int64_t>(ntiles, 0x7fffffff);
    kern<<<(unsigned)grid, TC_THREADS, smem, st>>>(M, Nc, K, A, lda, sA, B, ldb, sB, EA, EB, C, ldc, sC, 0, err,
                                                   accumulate, Ecol, tc_wait_limit(), gx, gy, ntiles);
    TBG_LAUNCHED(name);
    return TBG_OK;
}

static int ozaki_zgemm_tc_chunk(cudaStream_t st, bool conj_a, int fmt_a, int fmt_b, int64_t batch, int M, int Nc,
                                int K, const void* A, int64_t lda, int64_t sA, const void* B, int64_t ldb, int64_t sB,
                                float4* C, int64_t ldc, int64_t sC, int* EA, int* EB, int* err, bool accumulate,
                                int* Ecol, bool mid);

// With exps_ready the caller has filled EA (rows of op(A)) and EB (columns of
// B) already, e.g. once for an operand shared by several products.  With
// Ecol (only for M <= 128 and K <= 256: one row tile, one launch) the
// epilogue also writes the exponents of C's columns.
int ozaki_zgemm_tc(cudaStream_t st, bool conj_a, int fmt_a, int fmt_b, int64_t batch, int M, int Nc, int K,
                   const void* A, int64_t lda, int64_t sA, const void* B, int64_t ldb, int64_t sB, float4* C,
                   int64_t ldc, int64_t sC, int* EA, int* EB, int* err, bool exps_ready, int* Ecol, bool mid) {
    if (Ecol && (M > TC_TM || K > kTcMaxK))
        return set_error(TBG_E_UNSUPPORTED, "ozaki_zgemm_tc: fused column exponents need M <= 128 and K <= 256");
    if (!exps_ready) {
        int rc = ozaki_exp_launch(st, conj_a, fmt_a, fmt_b, batch, M, Nc, K, A, lda, sA, B, ldb, sB, EA, EB);
        if (rc) return rc;
    }
    // Contractions longer than kTcMaxK run in chunks of kTcMaxK (each exact in
    // its level accumulators); later chunks add their float pairs to C.  The
    // exponents stay those of the whole rows and columns.
    if (K > kTcMaxK) {
        const size_t ea = fmt_a == FMT_F32 ? 8 : 16, eb = fmt_b == FMT_F32 ? 8 : 16;
        for (int k0 = 0; k0 < K; k0 += kTcMaxK) {
            const int kc = std::min(kTcMaxK, K - k0);
            const char* Ak = static_cast<const char*>(A) + (conj_a ? (int64_t)k0 * lda : (int64_t)k0) * ea;
            const char* Bk = static_cast<const char*>(B) + (int64_t)k0 * ldb * eb;
            const int rc = ozaki_zgemm_tc_chunk(st, conj_a, fmt_a, fmt_b, batch, M, Nc, kc, Ak, lda, sA, Bk, ldb, sB, C,
                                                ldc, sC, EA, EB, err, k0 > 0, nullptr, mid);
            if (rc) return rc;
        }
        return TBG_OK;
    }
    return ozaki_zgemm_tc_chunk(st, conj_a, fmt_a, fmt_b, batch, M, Nc, K, A, lda, sA, B, ldb, sB, C, ldc, sC, EA, EB,
                                err, false, Ecol, mid);
}

static int ozaki_zgemm_tc_chunk(cudaStream_t st, bool conj_a, int fmt_a, int fmt_b, int64_t batch, int M, int Nc,
                                int K, const void* A, int64_t lda, int64_t sA, const void* B, int64_t ldb, int64_t sB,
                                float4* C, int64_t ldc, int64_t sC, int* EA, int* EB, int* err, bool accumulate,
                                int* Ecol, bool mid) {
    const double work = 8.0 * (double)M * Nc * K * batch;
#define TC_CASE(CJ, FA, FB, S, NAME)                                                                                 \
    if (conj_a == CJ && fmt_a == FA && fmt_b == FB)                                                                  \
        return launch_tc<CJ, FA, FB, S>(st, batch, M, Nc, K, A, lda, sA, B, ldb, sB, C, ldc, sC, EA, EB, err, NAME,  \
                                        work, accumulate ? 1 : 0, Ecol);
    if (mid) {
        TC_CASE(false, FMT_F64, FMT_F64, 5, "ozaki_tc_kernel<mid>")   // unit test
        TC_CASE(true, FMT_F64, FMT_F64, 5, "ozaki_tc_kernel<mid>")    // unit test
        TC_CASE(false, FMT_PAIR, FMT_PAIR, 5, "ozaki_tc_kernel<mid>") // V X'
        TC_CASE(true, FMT_PAIR, FMT_PAIR, 5, "ozaki_tc_kernel<mid>")  // X'^H (V X')
        return set_error(TBG_E_UNSUPPORTED, "ozaki_zgemm_tc: operand format combination not instantiated (MID)");
    }
    TC_CASE(false, FMT_F64, FMT_F64, TC_S, "ozaki_tc_kernel<high>")   // unit test
    TC_CASE(true, FMT_F64, FMT_F64, TC_S, "ozaki_tc_kernel<high>")    // unit test
    TC_CASE(true, FMT_F32, FMT_F32, TC_S, "ozaki_tc_kernel<high>")    // X^H X
    TC_CASE(false, FMT_F32, FMT_F32, TC_S, "ozaki_tc_kernel<high>")   // X F (HIGH above kHighCorrN bands)
    TC_CASE(false, FMT_PAIR, FMT_F32, TC_S, "ozaki_tc_kernel<high>")  // H X
    TC_CASE(true, FMT_F32, FMT_PAIR, TC_S, "ozaki_tc_kernel<high>")   // X^H (H X)
    TC_CASE(false, FMT_PAIR, FMT_PAIR, TC_S, "ozaki_tc_kernel<high>") // V X'
    TC_CASE(true, FMT_PAIR, FMT_PAIR, TC_S, "ozaki_tc_kernel<high>")  // X'^H (V X')
#undef TC_CASE
    return set_error(TBG_E_UNSUPPORTED, "ozaki_zgemm_tc: operand format combination not instantiated");
}

// tcgen05 form of the LOW precision class (3 x 3 digits, one FP32 accumulator):
// C = A B for FP32 A and B, e.g. the correction X F of the refinement.
int ozaki_zgemm_tc_low(cudaStream_t st, int64_t batch, int M, int Nc, int K, const void* A, int64_t lda, int64_t sA,
                       const void* B, int64_t ldb, int64_t sB, float4* C, int64_t ldc, int64_t sC, int* EA, int* EB,
                       int* err, bool exps_ready) {
    if (!exps_ready) {
        int rc = ozaki_exp_launch(st, false, FMT_F32, FMT_F32, batch, M, Nc, K, A, lda, sA, B, ldb, sB, EA, EB);
        if (rc) return rc;
    }
    for (int k0 = 0; k0 < K; k0 += kTcMaxK) {  // chunks of kTcMaxK, as in ozaki_zgemm_tc
        const int kc = std::min(kTcMaxK, K - k0);
        const int rc = launch_tc<false, FMT_F32, FMT_F32, 3>(
            st, batch, M, Nc, kc, static_cast<const char*>(A) + (int64_t)k0 * 8, lda, sA,
            static_cast<const char*>(B) + (int64_t)k0 * ldb * 8, ldb, sB, C, ldc, sC, EA, EB, err,
            "ozaki_tc_kernel<low>", 8.0 * (double)M * Nc * kc * batch, k0 > 0);
        if (rc) return rc;
    }
    return TBG_OK;
}

// Bytes of the hop-table stage images (K = nR rows of Nc = N^2 elements).
size_t ozaki_hop_image_bytes(int K, int64_t Nc) {
    const int64_t nst = (K + TC_TK - 1) / TC_TK, nct = (Nc + TC_TN - 1) / TC_TN;
    return (size_t)nct * nst * HALF_STAGE;
}
// Build the stage images from the hop table and its column exponents EB.
// Nc columns (matrix elements colmap[0 .. Nc) of a table with ldh elements per row,
// or the first Nc elements when colmap is null); EB per table element.
int ozaki_hop_image_launch(cudaStream_t st, int K, int64_t Nc, const zc* ham, const int* EB, void* img,
                          const int* colmap, int64_t ldh) {
    const int64_t nst = (K + TC_TK - 1) / TC_TK, nct = (Nc + TC_TN - 1) / TC_TN;
    const int64_t total = nct * nst * B_PRODUCERS;
    hop_image_kernel<<<(unsigned)std::min<int64_t>((total + 255) / 256, 152 * 64), 256, 0, st>>>(
        K, Nc, ham, EB, static_cast<unsigned char*>(img), colmap, ldh);
    TBG_LAUNCHED("hop_image_kernel");
    return TBG_OK;
}

// Stage images of a real-coefficient table (2 Kc rows; hop_image_real_kernel).
int ozaki_hop_image_real_launch(cudaStream_t st, int Kc, int64_t Nc, const zc* T, const int* EB, void* img,
                                const int* colmap, int64_t ldh) {
    const int64_t nst = (Kc + TC_TK - 1) / TC_TK, nct = (Nc + TC_TN - 1) / TC_TN;
    const int64_t total = nct * nst * B_PRODUCERS;
    hop_image_real_kernel<<<(unsigned)std::min<int64_t>((total + 255) / 256, 152 * 64), 256, 0, st>>>(
        Kc, Nc, T, EB, static_cast<unsigned char*>(img), colmap, ldh);
    TBG_LAUNCHED("hop_image_real_kernel");
    return TBG_OK;
}

// Stage images of the phases (A operand of the Fourier contraction, M x K
// FP64, row exponents EA): for row tile rt and stage it, the S digit planes
// exactly as the A producers would store them in shared memory (S * PLANE
// bytes at (rt * nstages + it) * S * PLANE).  One thread per (row, 8
// consecutive k) of a stage, as the producers.
template <int S>
__global__ void phase_image_kernel(int64_t M, int K, const zc* __restrict__ A, const int* __restrict__ EA,
                                   unsigned char* __restrict__ img) {
    const int nst = (K + TC_TK - 1) / TC_TK;
    const int64_t nrt = (M + TC_TM - 1) / TC_TM;
    const int64_t total = nrt * nst * A_PRODUCERS;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int q = (int)(idx % A_PRODUCERS);
        const int64_t blk = idx / A_PRODUCERS;  // rt * nst + it
        const int it = (int)(blk % nst);
        const int64_t rt = blk / nst;
        const int r = q >> 1, g = q & 1;
        const int64_t gi = rt * TC_TM + r;
        const bool rv = gi < M;
        const int E = rv ? EA[gi] : ZERO_EXP;
        float s1, s2;
        f32_scales(E, s1, s2);
        const int kf = it * TC_TK + 8 * g;
        int4 cur[8];
        load8<FMT_F64>(A, gi * K + kf, 1, rv ? n_valid(K, kf) : 0, cur);
        uint4 dre[S], dim[S];
        item_planes<FMT_F64, 0, S>(cur, E, s1, s2, dre);
        item_planes<FMT_F64, 1, S>(cur, E, s1, s2, dim);
        unsigned char* dst = img + blk * (int64_t)(S * PLANE);
#pragma unroll
        for (int s = 0; s < S; ++s) {
            *reinterpret_cast<uint4*>(dst + s * PLANE + plane_off(r, 8 * g)) = dre[s];
            *reinterpret_cast<uint4*>(dst + s * PLANE + plane_off(r, 16 + 8 * g)) = dim[s];
        }
    }
}

// Fourier contraction on tcgen05: C (M x Nc) = A (M x K FP64 phases) . hop
// table (stage images); EA filled by the caller.  Rows [0, high_rows) use the
// HIGH class, the rest the MID class (five of the images' six digit planes);
// high_rows < 0 keeps every row HIGH.  Row tiles vary fastest so that the CTAs
// resident together share one column tile's images in L2.
template <int S>
static int fourier_tc_launch(cudaStream_t st, int64_t M, int64_t Nc, int K, const zc* A, const int* EA,
                             const int* EB, const void* img, float4* C, int* err, unsigned char* aimg) {
    if (M <= 0) return TBG_OK;
    if (K <= 0) return set_error(TBG_E_INVALID_ARGUMENT, "ozaki_fourier_tc: empty contraction");
    {
        // the phases cut into stage images once, not once per column tile
        const int64_t total = (M + TC_TM - 1) / TC_TM * ((K + TC_TK - 1) / TC_TK) * A_PRODUCERS;
        KTimer kt(st, "phase_image_kernel");
        phase_image_kernel<S><<<(unsigned)std::min<int64_t>((total + 255) / 256, 152 * 64), 256, 0, st>>>(M, K, A, EA,
                                                                                                        aimg);
        TBG_LAUNCHED("phase_image_kernel");
    }
    auto kern = oz_tc_kernel<false, FMT_PRESLICED, FMT_PRESLICED, S>;
    const int smem = tc_smem_bytes(S);
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return cuda_error(e, "cudaFuncSetAttribute(oz_tc fourier)");
    KTimer kt(st, S == TC_S ? "ozaki_tc_fourier_kernel" : "ozaki_tc_fourier_kernel<mid>", 8.0 * (double)M * Nc * K);
    // persistent CTAs over (row tile, column tile), row tiles fastest
    const int gx = (int)((M + TC_TM - 1) / TC_TM), gy = (int)((Nc + TC_TN - 1) / TC_TN);
    const int64_t ntiles = (int64_t)gx * gy;
    if (ntiles <= 0) return TBG_OK;
    if (K <= 0) return set_error(TBG_E_INVALID_ARGUMENT, "ozaki_fourier_tc: empty contraction");
    const int64_t grid = std::min<int64_t>(ntiles, (int64_t)sm_count() * Class<S>::MIN_CTAS);
    kern<<<(unsigned)grid, TC_THREADS, smem, st>>>((int)M, (int)Nc, K, aimg, K, 0, img, Nc, 0, EA, EB, C, Nc, 0, 1,
                                                   err, 0, nullptr, tc_wait_limit(), gx, gy, ntiles);
    TBG_LAUNCHED(S == TC_S ? "ozaki_tc_fourier_kernel" : "ozaki_tc_fourier_kernel<mid>");
    return TBG_OK;
}

// Bytes of the phase images for up to M rows of a K-long contraction (either
// class; the two row ranges of one contraction reuse the buffer in turn).
size_t ozaki_fourier_img_bytes(int64_t M, int K) {
    return (size_t)((M + TC_TM - 1) / TC_TM) * (size_t)((K + TC_TK - 1) / TC_TK) * HALF_STAGE;
}

int ozaki_fourier_tc(cudaStream_t st, int64_t M, int64_t Nc, int K, const zc* A, const int* EA, const int* EB,
                     const void* img, float4* C, int* err, int64_t high_rows, void* aimg) {
    if ((Nc + TC_TN - 1) / TC_TN > 65535 || M > 0x7fffffff)
        return set_error(TBG_E_UNSUPPORTED, "ozaki_fourier_tc: grid too large");
    const int64_t mh = high_rows < 0 ? M : std::min<int64_t>(high_rows, M);
    unsigned char* ai = static_cast<unsigned char*>(aimg);
    int rc = fourier_tc_launch<TC_S>(st, mh, Nc, K, A, EA, EB, img, C, err, ai);
    if (rc) return rc;
    return fourier_tc_launch<5>(st, M - mh, Nc, K, A + mh * K, EA + mh, EB, img, C + mh * Nc, err, ai);
}

}  // namespace tbg

// Internal test hook (not part of the public header): the number of polls a
// tcgen05 stage hand-off wait makes before its CTA gives up and the call
// reports TBG_E_TIMEOUT; polls <= 0 restores the default.  Returns the previous
// value.  Lets a test run the time-out path (drain, TMEM release, status)
// without a fault: the waits that drain in-flight copies and MMAs keep their
// full bound.
extern "C" int tbg_internal_tc_wait_limit(int polls) {
    return tbg::g_tc_wait_limit.exchange(polls > 0 ? polls : tbg::tc::kTcWaitPolls);
}
