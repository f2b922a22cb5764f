// Householder tridiagonalisation of batched Hermitian matrices of up to 128
// bands with the matrix resident in tensor memory and its rank-2 updates on
// the tensor cores: the reduction stage of the FP32 eigensolver of the mixed
// path (LAPACK zhetrd's role inside Rustb's eigh, src/response/traits.rs:168
// and src/ndarray_lapack.rs:412-448).
//
// One CTA (8 warps) per matrix, two CTAs per SM.  The whole matrix A (not
// only a triangle) lives in TMEM as FP32: lane i = row i, column 2 l =
// Re A(i, l), column 2 l + 1 = Im A(i, l); rows and columns past N are zero
// and stay zero.  Step j (trailing block rows/columns j+1 .. N-1):
//
//   1. column j of the current matrix: read from TMEM during step j-1's
//      matrix-vector product (before step j-1's update reached TMEM) and
//      corrected here by that update, a_i -= v_i conj(w_j) + w_i conj(v_j);
//      reflector H_j = I - tau v v^H with H_j^H [alpha; x] = [beta; 0]
//      (beta real, sign opposite to Re alpha), v_{j+1} = 1;
//   2. p = A22 v: the trailing columns in chunks of 8 complex, alternate
//      chunks to the two warps of a lane quarter; each thread reads its row's
//      chunks from TMEM (tcgen05.ld) and multiplies with v in FP32; the two
//      shares meet in shared memory; y = tau p;
//   3. w = y - 1/2 tau (y^H v) v;
//   4. A -= v w^H + w v^H as one tcgen05.mma.kind::tf32 pair accumulating
//      into the TMEM-resident matrix (M = 128 rows, N = the real columns from
//      the first 8-column group the update touches, K = 8): the rank-2
//      complex update in the real embedding is
//        Re dA = [Re v, Im v, Re w, Im w] . [Re w, Im w, Re v, Im v]^T,
//        Im dA = [Re v, Im v, Re w, Im w] . [-Im w, Re w, -Im v, Re v]^T,
//      with each operand split into TF32 hi + lo (3xTF32: hi.hi + lo.hi in
//      one MMA of K = 8 against [b_hi | b_hi], hi.lo in a second against
//      [b_lo | 0]), about FP32 accuracy; the A operand is stored negated.
//      The MMA runs while the next step forms its reflector; the next
//      matrix-vector product waits for it on an mbarrier.
//
// Output, per matrix: the tridiagonal (d, e) for the solver's multisection /
// twisted-factorisation stage, and the reflectors (packed rows) with tau in
// the layout the blocked back-transformation pass reads.  The reflectors and
// tau are the ones the shared-memory reduction forms (the same algorithm; the
// products are rounded differently).
//
// Every wait is bounded; on a time-out the CTA records status bit 2, waits
// (bounded) for its committed MMAs, frees TMEM and stops.

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdlib>

#include "tbgpu_internal.cuh"
#include "tc_ptx.cuh"

namespace tbg {
namespace {

using namespace tc;

constexpr int HT_THREADS = 256;  // warp w: TMEM lanes 32 (w % 4) .. +31 (rows), column half w / 4
constexpr int HT_NC = 128;       // complex columns held per row
constexpr int HT_MAXN = 128;
constexpr uint32_t HT_TMEM_COLS = 2 * HT_NC;
// Dynamic shared memory: operand tiles A (4 KB), B1, B2 (8 KB each), then the
// per-matrix vectors.  80 KB keeps at most two CTAs (512 TMEM columns) per SM.
constexpr size_t HT_SMEM = 80 * 1024;
constexpr int OPA_BYTES = 128 * 32, OPB_BYTES = 2 * HT_NC * 32;

// instruction descriptor, kind::tf32: D = F32, A = B = TF32, both K-major, M = 128; N (bits 17..22, N / 8) per call
constexpr uint32_t IDESC_TF32_M128 = (1u << 4) | (2u << 7) | (2u << 10) | ((128u >> 4) << 24);
__device__ __forceinline__ uint32_t idesc_tf32(uint32_t n) { return IDESC_TF32_M128 | ((n >> 3) << 17); }

// COL: use of the A collector buffer across consecutive MMAs with the same A
// (0 none, 1 fill, 3 last use).
template <int COL = 0>
__device__ __forceinline__ void umma_tf32(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc) {
#define TBG_UMMA32(Q)                                                                                            \
    asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, 1, 0;\n\ttcgen05.mma.cta_group::1.kind::tf32" Q            \
                 " [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),                                                       \
                 "l"(adesc), "l"(bdesc), "r"(idesc)                                                              \
                 : "memory")
    if constexpr (COL == 1)
        TBG_UMMA32(".collector::a::fill");
    else if constexpr (COL == 3)
        TBG_UMMA32(".collector::a::lastuse");
    else
        TBG_UMMA32("");
#undef TBG_UMMA32
}

__device__ __forceinline__ float tf32_rna(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

// Byte offset of row r, K group kc (4 tf32 values) in an operand tile: K-major
// core matrices of 8 rows x 16 bytes; K-adjacent ones 128 bytes apart
// (descriptor LBO), 8-row groups 256 bytes apart (SBO).
__device__ __forceinline__ uint32_t op_off(int r, int kc) {
    return (uint32_t)((r >> 3) * 256 + kc * 128 + (r & 7) * 16);
}

__device__ __forceinline__ float ht_warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ void split4(float a, float b, float c, float d, uint4& hi, uint4& lo) {
    const float h0 = tf32_rna(a), h1 = tf32_rna(b), h2 = tf32_rna(c), h3 = tf32_rna(d);
    hi = make_uint4(__float_as_uint(h0), __float_as_uint(h1), __float_as_uint(h2), __float_as_uint(h3));
    lo = make_uint4(__float_as_uint(tf32_rna(a - h0)), __float_as_uint(tf32_rna(b - h1)),
                    __float_as_uint(tf32_rna(c - h2)), __float_as_uint(tf32_rna(d - h3)));
}

__host__ __device__ __forceinline__ size_t ht_diag_off(int N, int i) {
    return (size_t)i * N - ((size_t)i * (size_t)(i - 1)) / 2;
}
__host__ __device__ __forceinline__ size_t ht_packed_elems(int N) { return ((size_t)N * (N + 1) / 2 + 1) & ~(size_t)1; }

// Hpair: float pairs {re_hi, re_lo, im_hi, im_lo} (batch, N, N), or Hz:
// complex FP64, or Hc: complex FP32.  Vt: (batch, packed + Nbig) reflectors
// (packed rows) and tau; de: (batch, 2 Nbig) d then e.  The matrix may be the
// trailing block (rows and columns off .. off + N - 1) of an Nbig-band one
// whose first off steps another kernel has done: reflectors, tau, d and e
// then go to rows off .. of the big matrix's layouts.
__global__ void __launch_bounds__(HT_THREADS, 2)
    hetrd_tc_kernel(int N, int64_t batch, const float4* __restrict__ Hpair, const zc* __restrict__ Hz,
                    const cc* __restrict__ Hc, cc* __restrict__ Vt, float* __restrict__ de, int* __restrict__ status,
                    int wait_limit, int Nbig, int off) {
    extern __shared__ __align__(1024) unsigned char ht_smem[];
    __shared__ __align__(8) uint64_t bar_mma, bar_ops;
    __shared__ uint32_t tmem_base_sh;
    __shared__ volatile int abort_sh;
    __shared__ cc alpha_sh;
    __shared__ float red[20];
    unsigned char* opA = reinterpret_cast<unsigned char*>(((uintptr_t)ht_smem + 127) & ~(uintptr_t)127);
    unsigned char* opB1 = opA + OPA_BYTES;
    unsigned char* opB2 = opB1 + OPB_BYTES;
    cc* vbuf = reinterpret_cast<cc*>(opB2 + OPB_BYTES);
    cc* wbuf = vbuf + HT_MAXN;
    cc* colbuf = wbuf + HT_MAXN;
    cc* pbuf = colbuf + HT_MAXN;   // half 1's share of p
    cc* p0buf = pbuf + HT_MAXN;    // half 0's share of p
    float* dsm = reinterpret_cast<float*>(p0buf + HT_MAXN);
    float* esm = dsm + HT_MAXN;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int q = warp & 3, h = warp >> 2;
    const int i = 32 * q + lane;  // this thread's row (TMEM lane)
    const size_t NN = (size_t)N * N, pe = ht_packed_elems(Nbig);
    const uint32_t sA = su32(opA), sB1 = su32(opB1), sB2 = su32(opB2);

    if (tid == 0) {
        mbar_init(&bar_mma, 1);
        mbar_init(&bar_ops, 128);
        abort_sh = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(&tmem_base_sh)),
                     "r"(HT_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base_sh;
    const uint32_t trow = tmem + ((uint32_t)(32 * q) << 16);
    // MMA bookkeeping: one operand hand-off (bar_ops, the 128 threads of half 0
    // arrive) and one commit (bar_mma) per issued update, numbered from 0
    // across the CTA's matrices; thread 128 issues, thread 0 waits for them.
    uint32_t base = 0;     // updates issued for earlier matrices
    uint32_t issued = 0;   // updates issued so far (thread 128)

    for (int64_t b = blockIdx.x; b < batch; b += gridDim.x) {
        // ------------------------------------------------ matrix -> TMEM --
        for (int cb = 64 * h; cb < 64 * h + 64; cb += 8) {
            uint32_t r[16];
#pragma unroll
            for (int c = 0; c < 8; ++c) {
                const int col = cb + c;
                float xr = 0.f, xi = 0.f;
                if (i < N && col < N) {
                    if (Hpair) {
                        const float4 p = Hpair[b * NN + (size_t)i * N + col];
                        xr = p.x + p.y;
                        xi = p.z + p.w;
                    } else if (Hc) {
                        const cc z = Hc[b * NN + (size_t)i * N + col];
                        xr = z.re;
                        xi = z.im;
                    } else {
                        const zc z = Hz[b * NN + (size_t)i * N + col];
                        xr = (float)z.re;
                        xi = (float)z.im;
                    }
                }
                if (col == 0) colbuf[i] = mk<float>(xr, xi);
                r[2 * c] = __float_as_uint(xr);
                r[2 * c + 1] = __float_as_uint(xi);
            }
            tmem_st16(trow + (uint32_t)(2 * cb), r);
        }
        tmem_wait_st();
        tc_fence_before();
        __syncthreads();
        tc_fence_after();

        bool aborted = false;
        cc* Vm = Vt + (size_t)b * (pe + Nbig);
        cc wnext = mk<float>(0.f, 0.f);  // w of the previous step at the current column (row j)
        size_t dj = ht_diag_off(Nbig, off);  // packed offset of (big) row off + j's diagonal
        for (int j = 0; j < N - 1; dj += (size_t)(Nbig - off - j), ++j) {
            const int jn = j + 1;
            // ------------------------------------- column j, reflector --
            cc a = mk<float>(0.f, 0.f);
            if (h == 0) {
                a = colbuf[i];
                if (j > 0) {  // step j-1's update of this column (not in the value read from TMEM)
                    fms_mulc(a, vbuf[i], wnext);
                    fms_mulc(a, wbuf[i], vbuf[j]);
                }
                if (i == j) dsm[j] = a.re;
                if (i == jn) alpha_sh = a;
                float x2 = (i > jn && i < N) ? abs2(a) : 0.f;
                x2 = ht_warp_sum(x2);
                if (lane == 0) red[q] = x2;
            }
            __syncthreads();
            // the reflector's scalars (half 0 only: the other half needs none of them)
            cc tau = mk<float>(0.f, 0.f), scal = mk<float>(0.f, 0.f);
            float beta = 0.f;
            const float xnorm2 = (red[0] + red[1]) + (red[2] + red[3]);
            const cc alpha = alpha_sh;
            if (h == 1) {
            } else if (xnorm2 == 0.f && alpha.im == 0.f) {
                tau = mk<float>(0.f, 0.f);
                scal = mk<float>(0.f, 0.f);
                beta = alpha.re;
            } else {
                const float nrm = sqrtf(alpha.re * alpha.re + alpha.im * alpha.im + xnorm2);
                beta = (alpha.re >= 0.f) ? -nrm : nrm;
                const float rb = __frcp_rn(beta);
                tau = mk<float>((beta - alpha.re) * rb, -alpha.im * rb);
                const cc den = mk<float>(alpha.re - beta, alpha.im);
                const float rd = __frcp_rn(den.re * den.re + den.im * den.im);
                scal = mk<float>(den.re * rd, -den.im * rd);
            }
            if (h == 0) {
                const cc v = (i == jn) ? mk<float>(1.f, 0.f) : ((i > jn && i < N) ? a * scal : mk<float>(0.f, 0.f));
                vbuf[i] = v;
                if (i >= jn && i < N) Vm[dj + (size_t)(i - j)] = v;
            }
            if (tid == 0) {
                esm[j] = beta;
                Vm[pe + off + j] = tau;
                // step j-1's update must be in TMEM before the product below reads it
                if (j > 0 && !mbar_wait(&bar_mma, (base + j - 1) & 1u, &abort_sh, wait_limit)) abort_sh = 1;
            }
            __syncthreads();
            tc_fence_after();
            if (abort_sh) {
                aborted = true;
                break;
            }
            // --------------------------- p = A22 v (TMEM), partial v^H p --
            cc acc[4];
#pragma unroll
            for (int g = 0; g < 4; ++g) acc[g] = mk<float>(0.f, 0.f);
            uint32_t sre = 0u, sim = 0u;  // column j+1 of this row, for the next step (half 0)
            if (32 * q + 31 >= jn && 32 * q < N) {  // warp-uniform: some row of this warp is trailing
                if (h == 0) {
                    sre = tmem_ld1(trow + (uint32_t)(2 * jn));
                    sim = tmem_ld1(trow + (uint32_t)(2 * jn + 1));
                }
                // chunks of 8 complex columns cf .. cl; this half takes every other one,
                // up to four per wait (one accumulator each)
                const int cf = jn >> 3, cl = (N - 1) >> 3;
                for (int c = cf + ((cf & 1) != h); c <= cl; c += 8) {
                    uint32_t r[4][16];
#pragma unroll
                    for (int g = 0; g < 4; ++g)
                        if (c + 2 * g <= cl) tmem_ld16(trow + (uint32_t)(16 * (c + 2 * g)), r[g]);
                    tmem_wait_ld();
#pragma unroll
                    for (int g = 0; g < 4; ++g) {
                        if (c + 2 * g > cl) break;
                        const float4* vp = reinterpret_cast<const float4*>(vbuf + 8 * (c + 2 * g));
#pragma unroll
                        for (int u = 0; u < 4; ++u) {
                            const float4 v2 = vp[u];  // v at two consecutive columns
                            const float ar = __uint_as_float(r[g][4 * u]), ai = __uint_as_float(r[g][4 * u + 1]);
                            const float br = __uint_as_float(r[g][4 * u + 2]), bi = __uint_as_float(r[g][4 * u + 3]);
                            acc[g].re = fmaf(ar, v2.x, acc[g].re);
                            acc[g].re = fmaf(-ai, v2.y, acc[g].re);
                            acc[g].re = fmaf(br, v2.z, acc[g].re);
                            acc[g].re = fmaf(-bi, v2.w, acc[g].re);
                            acc[g].im = fmaf(ar, v2.y, acc[g].im);
                            acc[g].im = fmaf(ai, v2.x, acc[g].im);
                            acc[g].im = fmaf(br, v2.w, acc[g].im);
                            acc[g].im = fmaf(bi, v2.z, acc[g].im);
                        }
                    }
                }
                tmem_wait_ld();  // the column j+1 loads, when this half had no chunk to wait for
            }
            if (h == 0) colbuf[i] = mk<float>(__uint_as_float(sre), __uint_as_float(sim));
            const cc accs = (acc[0] + acc[1]) + (acc[2] + acc[3]);
            (h ? pbuf : p0buf)[i] = accs;
            {
                // this half's share of p^H v (v is zero outside the trailing rows)
                const cc vi = vbuf[i];
                float dr = accs.re * vi.re + accs.im * vi.im;
                float di = accs.re * vi.im - accs.im * vi.re;
                dr = ht_warp_sum(dr);
                di = ht_warp_sum(di);
                if (lane == 0) {
                    red[4 + warp] = dr;
                    red[12 + warp] = di;
                }
            }
            tc_fence_before();
            __syncthreads();
            // ------------------ y = tau p, w = y - 1/2 tau (y^H v) v, operands --
            const bool more = jn < N - 1;  // a later product reads this update from TMEM
            if (h == 0) {
                const cc p = accs + pbuf[i];
                const cc y = (i >= jn && i < N) ? tau * p : mk<float>(0.f, 0.f);
                cc s = mk<float>(0.f, 0.f);
#pragma unroll
                for (int k = 0; k < 8; ++k) s = s + mk<float>(red[4 + k], red[12 + k]);
                const cc dp = conj(tau) * s;  // y^H v = conj(tau) p^H v
                const cc alpha2 = -0.5f * (tau * dp);
                const cc vi = vbuf[i];
                const cc w = y + alpha2 * vi;
                wbuf[i] = w;
                // the same value at row j+1 (another thread's row), for the next step's column
                if (jn < N) wnext = tau * (p0buf[jn] + pbuf[jn]) + alpha2 * vbuf[jn];
                if (more) {
                    uint4 ahi, alo, rhi, rlo, ihi, ilo;
                    split4(-vi.re, -vi.im, -w.re, -w.im, ahi, alo);
                    split4(w.re, w.im, vi.re, vi.im, rhi, rlo);
                    split4(-w.im, w.re, -vi.im, vi.re, ihi, ilo);
                    const uint4 z = make_uint4(0u, 0u, 0u, 0u);
                    st_shared_v4(sA + op_off(i, 0), ahi);
                    st_shared_v4(sA + op_off(i, 1), alo);
                    st_shared_v4(sB1 + op_off(2 * i, 0), rhi);
                    st_shared_v4(sB1 + op_off(2 * i, 1), rhi);
                    st_shared_v4(sB1 + op_off(2 * i + 1, 0), ihi);
                    st_shared_v4(sB1 + op_off(2 * i + 1, 1), ihi);
                    st_shared_v4(sB2 + op_off(2 * i, 0), rlo);
                    st_shared_v4(sB2 + op_off(2 * i, 1), z);
                    st_shared_v4(sB2 + op_off(2 * i + 1, 0), ilo);
                    st_shared_v4(sB2 + op_off(2 * i + 1, 1), z);
                    fence_async_smem();
                    mbar_arrive(&bar_ops);
                }
            } else if (tid == 128 && more) {
                // issue the update once half 0 has written its operands
                if (!mbar_wait(&bar_ops, (base + j) & 1u, &abort_sh, wait_limit)) {
                    abort_sh = 1;
                } else {
                    tc_fence_after();
                    // columns below the 8-column group of j+1 are untouched: D and B start there
                    const int c0 = jn & ~7;
                    const uint32_t id = idesc_tf32((uint32_t)(2 * (HT_NC - c0)));
                    const uint64_t ad = smem_desc(sA, 128, 256);
                    umma_tf32<1>(tmem + (uint32_t)(2 * c0), ad, smem_desc(sB1 + 64u * (uint32_t)c0, 128, 256), id);
                    umma_tf32<3>(tmem + (uint32_t)(2 * c0), ad, smem_desc(sB2 + 64u * (uint32_t)c0, 128, 256), id);
                    umma_commit(&bar_mma);
                    ++issued;
                }
            }
        }
        base += (uint32_t)max(N - 2, 0);
        if (aborted) break;
        // last diagonal entry: the stashed column N-1 with the last step's update
        if (h == 0 && i == N - 1) {
            cc a = colbuf[i];
            if (N > 1) {
                fms_mulc(a, vbuf[i], wbuf[i]);
                fms_mulc(a, wbuf[i], vbuf[i]);
            }
            dsm[N - 1] = a.re;
            esm[N - 1] = 0.f;
        }
        __syncthreads();
        float* dout = de + (size_t)b * 2 * Nbig + off;
        for (int k = tid; k < N; k += HT_THREADS) {
            dout[k] = dsm[k];
            dout[Nbig + k] = esm[k];
        }
        if (tid == 0) Vt[(size_t)b * (pe + Nbig) + pe + (Nbig - 1)] = mk<float>(0.f, 0.f);
        __syncthreads();
    }
    tc_fence_before();
    __syncthreads();
    if (abort_sh) {
        if (tid == 0) atomicOr(status, 2);  // bit 1: a bounded wait ran out
        if (tid == 128 && issued > 0) mbar_wait_plain(&bar_mma, (issued - 1) & 1u);  // the last update issued
    }
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(HT_TMEM_COLS)
                     : "memory");
    }
}


// ------------------------------------------------------------------------
// Back-transformation U <- H_0 H_1 ... H_{N-2} U of the FP32 solver for up to
// 128 bands with U resident in tensor memory, transposed: lane c = column c
// of U, columns 2 i / 2 i + 1 = Re / Im U(i, c).  The reflectors are applied
// in blocks of BT8 = 8, last block first: for the block H_j0 ... H_j0+7 =
// I - V T V^H (V: the 8 reflectors as dense zero-masked columns),
//   z = V^H U(:, c)      each thread its column c, from TMEM rows, in FP32
//                        (the two warps of a lane quarter take 4 reflectors
//                        each);
//   y = T z              back-substitution y_l = tau_l (z_l - sum_{m>l}
//                        (v_l^H v_m) y_m) with the block's Gram matrix;
//   U -= V Y             tcgen05.mma.kind::tf32 accumulating into TMEM:
//                        row c of the A operand is -[Re y | Im y] (K = 16),
//                        rows 2 i, 2 i + 1 of B are [Re V(i,:), -Im V(i,:)]
//                        and [Im V(i,:), Re V(i,:)]; 3xTF32 (A_hi B_hi,
//                        A_lo B_hi, A_hi B_lo), N = the rows from j0 on.
// The next block's reflectors are read from global memory while the MMAs of
// this one run.  Rows and columns past N are zero.
constexpr int BT8 = 8;
// Dynamic shared memory: tiles and scratch (61 KB); 80 KB keeps at most two CTAs (512 TMEM columns) per SM.
constexpr size_t BT_SMEM = 80 * 1024;
constexpr int BT_B_BYTES = 256 * 16 * 4, BT_A_BYTES = 128 * 16 * 4;

// operand tiles of K = 16: row r, K group kc (4 values): K-adjacent core matrices 128 bytes apart, 8-row groups 512
__device__ __forceinline__ uint32_t bt_off(int r, int kc) {
    return (uint32_t)((r >> 3) * 512 + kc * 128 + (r & 7) * 16);
}

__global__ void __launch_bounds__(HT_THREADS, 2)
    bt_tc_kernel(int N, int64_t batch, const cc* __restrict__ Vt, cc* __restrict__ Uio, int* __restrict__ status,
                 int wait_limit, int* __restrict__ urow_exp, int* __restrict__ ucol_exp) {
    extern __shared__ __align__(1024) unsigned char bt_smem[];
    __shared__ __align__(8) uint64_t bar_mma, bar_ops;
    __shared__ uint32_t tmem_base_sh;
    __shared__ volatile int abort_sh;
    __shared__ cc G[BT8 * BT8];
    __shared__ cc tau_b[BT8];
    __shared__ int rmax[4][128], cmax[2][128];  // line maxima of U (float bits) by lane quarter / row half
    unsigned char* Bhi = reinterpret_cast<unsigned char*>(((uintptr_t)bt_smem + 127) & ~(uintptr_t)127);
    unsigned char* Blo = Bhi + BT_B_BYTES;
    unsigned char* Ahi = Blo + BT_B_BYTES;
    unsigned char* Alo = Ahi + BT_A_BYTES;
    cc* Vs = reinterpret_cast<cc*>(Alo + BT_A_BYTES);  // (128, 8) the block's reflectors
    cc* zx = Vs + 128 * BT8;                          // (128, 4) half 1's share of z

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int q = warp & 3, h = warp >> 2;
    const int c = 32 * q + lane;  // this thread's column of U (TMEM lane)
    const size_t NN = (size_t)N * N, pe = ht_packed_elems(N);
    const uint32_t sBhi = su32(Bhi), sBlo = su32(Blo), sAhi = su32(Ahi), sAlo = su32(Alo);
    const int nblk = (N - 1 + BT8 - 1) / BT8;  // blocks of reflectors 0 .. N-2

    if (tid == 0) {
        mbar_init(&bar_mma, 1);
        mbar_init(&bar_ops, 128);
        abort_sh = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(&tmem_base_sh)),
                     "r"(HT_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base_sh;
    const uint32_t trow = tmem + ((uint32_t)(32 * q) << 16);
    uint32_t done = 0;    // updates committed and waited for (thread 0)
    uint32_t issued = 0;  // updates issued (thread 128)

    for (int64_t b = blockIdx.x; b < batch; b += gridDim.x) {
        const cc* Vm = Vt + (size_t)b * (pe + N);
        cc* U = Uio + b * NN;
        // ------------------------------------------ U^T -> TMEM (rows 64 h ..) --
        for (int i0 = 64 * h; i0 < 64 * h + 64; i0 += 8) {
            uint32_t r[16];
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                const int i = i0 + k;
                const cc u = (i < N && c < N) ? U[(size_t)i * N + c] : mk<float>(0.f, 0.f);
                r[2 * k] = __float_as_uint(u.re);
                r[2 * k + 1] = __float_as_uint(u.im);
            }
            tmem_st16(trow + (uint32_t)(2 * i0), r);
        }
        tmem_wait_st();
        // this thread's reflector components of the first (last-applied-first) block:
        // row i = tid & 127 of V, reflectors 4 h' .. 4 h' + 3 with h' = tid >> 7
        const int vi = tid & 127, vh = tid >> 7;
        auto load_v = [&](int j0, cc (&vr)[4]) {
#pragma unroll
            for (int t = 0; t < 4; ++t) {
                const int j = j0 + 4 * vh + t;
                vr[t] = (j <= N - 2 && vi > j && vi < N) ? Vm[ht_diag_off(N, j) + (size_t)(vi - j)]
                                                          : mk<float>(0.f, 0.f);
            }
        };
        cc vr[4];
        load_v(BT8 * (nblk - 1), vr);
        tc_fence_before();
        __syncthreads();
        tc_fence_after();

        bool aborted = false;
        for (int blk = nblk - 1; blk >= 0; --blk) {
            const int j0 = BT8 * blk;
            // ---------------- the previous block's update is complete: tiles and TMEM free --
            if (tid == 0 && blk < nblk - 1) {
                if (!mbar_wait(&bar_mma, done & 1u, &abort_sh, wait_limit)) abort_sh = 1;
                ++done;
            }
            __syncthreads();
            tc_fence_after();
            if (abort_sh) {
                aborted = true;
                break;
            }
            // ------------------------------ this block's V: FP32 copy and the B tiles --
            {
#pragma unroll
                for (int t = 0; t < 4; ++t) Vs[vi * BT8 + 4 * vh + t] = vr[t];
                uint4 rhi, rlo, ihi, ilo, jhi, jlo, khi, klo;
                // row 2 i: [Re V(i, 4 vh ..) | ... ] at K group vh, [-Im V(i, 4 vh ..)] at K group 2 + vh
                split4(vr[0].re, vr[1].re, vr[2].re, vr[3].re, rhi, rlo);
                split4(-vr[0].im, -vr[1].im, -vr[2].im, -vr[3].im, ihi, ilo);
                // row 2 i + 1: [Im V] at K group vh, [Re V] at K group 2 + vh
                split4(vr[0].im, vr[1].im, vr[2].im, vr[3].im, jhi, jlo);
                khi = rhi;
                klo = rlo;
                st_shared_v4(sBhi + bt_off(2 * vi, vh), rhi);
                st_shared_v4(sBlo + bt_off(2 * vi, vh), rlo);
                st_shared_v4(sBhi + bt_off(2 * vi, 2 + vh), ihi);
                st_shared_v4(sBlo + bt_off(2 * vi, 2 + vh), ilo);
                st_shared_v4(sBhi + bt_off(2 * vi + 1, vh), jhi);
                st_shared_v4(sBlo + bt_off(2 * vi + 1, vh), jlo);
                st_shared_v4(sBhi + bt_off(2 * vi + 1, 2 + vh), khi);
                st_shared_v4(sBlo + bt_off(2 * vi + 1, 2 + vh), klo);
                if (tid < BT8) tau_b[tid] = (j0 + tid <= N - 2) ? Vm[pe + j0 + tid] : mk<float>(0.f, 0.f);
            }
            __syncthreads();
            // the next block's reflectors, read while this block is applied
            if (blk > 0) load_v(j0 - BT8, vr);
            // ---------------------------------------- Gram matrix G(l, m) = v_l^H v_m, l < m --
            if (tid < 8 * 28) {
                const int e = tid >> 3, p8 = tid & 7;
                int l = 0, m = 1, cnt = e;
                while (cnt >= BT8 - 1 - l) {
                    cnt -= BT8 - 1 - l;
                    ++l;
                }
                m = l + 1 + cnt;
                cc g = mk<float>(0.f, 0.f);
                for (int i = j0 + 1 + p8; i < N; i += 8) fma_cjx(g, Vs[i * BT8 + l], Vs[i * BT8 + m]);
#pragma unroll
                for (int o = 1; o < 8; o <<= 1) {
                    g.re += __shfl_xor_sync(0xffffffffu, g.re, o);
                    g.im += __shfl_xor_sync(0xffffffffu, g.im, o);
                }
                if (p8 == 0) G[l * BT8 + m] = g;
            }
            // ----------------- z = V^H U(:, c) for this half's 4 reflectors, from TMEM rows --
            cc z[4];
#pragma unroll
            for (int t = 0; t < 4; ++t) z[t] = mk<float>(0.f, 0.f);
            {
                // rows j0 + 1 .. N - 1 in chunks of 8 (16 TMEM columns), two chunks per wait
                const int i_first = j0 & ~7, i_end = (N + 7) & ~7;
                for (int i0 = i_first; i0 < i_end; i0 += 16) {
                    const bool two = i0 + 8 < i_end;
                    uint32_t r[2][16];
                    tmem_ld16(trow + (uint32_t)(2 * i0), r[0]);
                    if (two) tmem_ld16(trow + (uint32_t)(2 * i0 + 16), r[1]);
                    tmem_wait_ld();
#pragma unroll
                    for (int g2 = 0; g2 < 2; ++g2) {
                        if (g2 == 1 && !two) break;
#pragma unroll
                        for (int k = 0; k < 8; ++k) {
                            const int i = i0 + 8 * g2 + k;
                            const float ur = __uint_as_float(r[g2][2 * k]), ui = __uint_as_float(r[g2][2 * k + 1]);
                            const float4 va = *reinterpret_cast<const float4*>(Vs + i * BT8 + 4 * h);
                            const float4 vb = *reinterpret_cast<const float4*>(Vs + i * BT8 + 4 * h + 2);
                            // z += conj(V(i, l)) U(i, c)
                            z[0].re = fmaf(va.x, ur, z[0].re); z[0].re = fmaf(va.y, ui, z[0].re);
                            z[0].im = fmaf(va.x, ui, z[0].im); z[0].im = fmaf(-va.y, ur, z[0].im);
                            z[1].re = fmaf(va.z, ur, z[1].re); z[1].re = fmaf(va.w, ui, z[1].re);
                            z[1].im = fmaf(va.z, ui, z[1].im); z[1].im = fmaf(-va.w, ur, z[1].im);
                            z[2].re = fmaf(vb.x, ur, z[2].re); z[2].re = fmaf(vb.y, ui, z[2].re);
                            z[2].im = fmaf(vb.x, ui, z[2].im); z[2].im = fmaf(-vb.y, ur, z[2].im);
                            z[3].re = fmaf(vb.z, ur, z[3].re); z[3].re = fmaf(vb.w, ui, z[3].re);
                            z[3].im = fmaf(vb.z, ui, z[3].im); z[3].im = fmaf(-vb.w, ur, z[3].im);
                        }
                    }
                }
            }
            if (h == 1) {
#pragma unroll
                for (int t = 0; t < 4; ++t) zx[c * 4 + t] = z[t];
            }
            tc_fence_before();
            __syncthreads();
            // --------------------------------- y = T z, A operand row c = -[Re y | Im y] --
            if (h == 0) {
                cc zz[BT8], y[BT8];
#pragma unroll
                for (int t = 0; t < 4; ++t) {
                    zz[t] = z[t];
                    zz[4 + t] = zx[c * 4 + t];
                }
#pragma unroll
                for (int l = BT8 - 1; l >= 0; --l) {
                    cc sv = zz[l];
#pragma unroll
                    for (int m = l + 1; m < BT8; ++m) sv = sv - G[l * BT8 + m] * y[m];
                    y[l] = tau_b[l] * sv;
                }
                uint4 h0, l0, h1, l1, h2, l2, h3, l3;
                split4(-y[0].re, -y[1].re, -y[2].re, -y[3].re, h0, l0);
                split4(-y[4].re, -y[5].re, -y[6].re, -y[7].re, h1, l1);
                split4(-y[0].im, -y[1].im, -y[2].im, -y[3].im, h2, l2);
                split4(-y[4].im, -y[5].im, -y[6].im, -y[7].im, h3, l3);
                st_shared_v4(sAhi + bt_off(c, 0), h0);
                st_shared_v4(sAhi + bt_off(c, 1), h1);
                st_shared_v4(sAhi + bt_off(c, 2), h2);
                st_shared_v4(sAhi + bt_off(c, 3), h3);
                st_shared_v4(sAlo + bt_off(c, 0), l0);
                st_shared_v4(sAlo + bt_off(c, 1), l1);
                st_shared_v4(sAlo + bt_off(c, 2), l2);
                st_shared_v4(sAlo + bt_off(c, 3), l3);
                fence_async_smem();
                mbar_arrive(&bar_ops);
            } else if (tid == 128) {
                if (!mbar_wait(&bar_ops, issued & 1u, &abort_sh, wait_limit)) {
                    abort_sh = 1;
                } else {
                    tc_fence_after();
                    // U rows from j0 on: D columns 2 j0 .., B rows 2 j0 .. (8-row groups of 512 bytes)
                    const uint32_t id = idesc_tf32((uint32_t)(2 * (HT_NC - j0)));
                    const uint32_t d = tmem + (uint32_t)(2 * j0), boff = 128u * (uint32_t)j0;
#pragma unroll
                    for (int kk = 0; kk < 2; ++kk) {
                        const uint64_t ah = smem_desc(sAhi + 256u * kk, 128, 512);
                        const uint64_t al = smem_desc(sAlo + 256u * kk, 128, 512);
                        const uint64_t bh = smem_desc(sBhi + boff + 256u * kk, 128, 512);
                        const uint64_t bl = smem_desc(sBlo + boff + 256u * kk, 128, 512);
                        // the two products with A_hi back to back, A_hi kept in the collector
                        umma_tf32<1>(d, ah, bh, id);
                        umma_tf32<3>(d, ah, bl, id);
                        umma_tf32(d, al, bh, id);
                    }
                    umma_commit(&bar_mma);
                    ++issued;
                }
            }
        }
        if (aborted) break;
        // ------------------------------------------------ TMEM -> U (rows 64 h ..) --
        if (tid == 0) {
            if (!mbar_wait(&bar_mma, done & 1u, &abort_sh, wait_limit)) abort_sh = 1;
            ++done;
        }
        __syncthreads();
        tc_fence_after();
        if (abort_sh) break;
        // with urow_exp / ucol_exp the line exponents of U come out too: the
        // magnitudes (>= 0, NaN as 0) are combined as integers, rows over the
        // lanes of a warp and then the four lane quarters, columns over the
        // two row halves
        const bool lines = urow_exp != nullptr;
        float cm = 0.f;
        for (int i0 = 64 * h; i0 < 64 * h + 64; i0 += 16) {
            uint32_t r[2][16];
            tmem_ld16(trow + (uint32_t)(2 * i0), r[0]);
            tmem_ld16(trow + (uint32_t)(2 * i0 + 16), r[1]);
            tmem_wait_ld();
#pragma unroll
            for (int k = 0; k < 16; ++k) {
                const int i = i0 + k;
                const float ure = __uint_as_float(r[k >> 3][2 * (k & 7)]);
                const float uim = __uint_as_float(r[k >> 3][2 * (k & 7) + 1]);
                const bool in = i < N && c < N;
                if (in) U[(size_t)i * N + c] = mk<float>(ure, uim);
                if (lines) {
                    float mg = in ? f32_mag(ure, uim) : 0.f;
                    mg = (mg == mg) ? mg : 0.f;
                    cm = fmaxf(cm, mg);
                    const int rm = __reduce_max_sync(0xffffffffu, __float_as_int(mg));
                    if (lane == 0) rmax[q][i] = rm;
                }
            }
        }
        if (lines) cmax[h][c] = __float_as_int(cm);
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (lines) {
            if (tid < 128) {
                if (tid < N)
                    urow_exp[b * N + tid] = line_exp_of(__int_as_float(
                        max(max(rmax[0][tid], rmax[1][tid]), max(rmax[2][tid], rmax[3][tid]))));
            } else if (tid - 128 < N) {
                ucol_exp[b * N + (tid - 128)] = line_exp_of(__int_as_float(max(cmax[0][tid - 128], cmax[1][tid - 128])));
            }
            __syncthreads();
        }
    }
    tc_fence_before();
    __syncthreads();
    if (abort_sh) {
        if (tid == 0) atomicOr(status, 2);  // bit 1: a bounded wait ran out
        if (tid == 128 && issued > 0) mbar_wait_plain(&bar_mma, (issued - 1) & 1u);
    }
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(HT_TMEM_COLS)
                     : "memory");
    }
}

}  // namespace

bool eig_tc_enabled() {
    static const bool on = [] {
        const char* s = std::getenv("TBG_EIG_TC");
        return !(s && s[0] == '0');
    }();
    return on;
}

bool hetrd_tc_fits(int N) { return N >= 2 && N <= HT_MAXN; }

// The back-transformation on the tensor cores unless TBG_BT_TC=0 (then the
// shared-memory blocked pass runs after the TMEM-resident reduction).
bool bt_tc_enabled() {
    static const bool on = [] {
        const char* s = std::getenv("TBG_BT_TC");
        return !(s && s[0] == '0');
    }();
    return on;
}

size_t hetrd_tc_de_bytes(int N, int64_t batch) { return sizeof(float) * 2 * (size_t)N * (size_t)batch; }

int hetrd_tc(cudaStream_t st, int N, int64_t batch, const float4* Hpair, const zc* H, cc* Vt, float* de,
             int* status_d, const cc* Hc, int Nbig, int off) {
    if (Nbig <= 0) Nbig = N;
    if (batch <= 0) return TBG_OK;
    if (!hetrd_tc_fits(N)) return set_error(TBG_E_UNSUPPORTED, "hetrd_tc: matrix order beyond 128");
    // a per-function attribute of the current device (set on every call: cheap, and right for every device)
    cudaError_t e = cudaFuncSetAttribute(hetrd_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)HT_SMEM);
    if (e != cudaSuccess) return cuda_error(e, "cudaFuncSetAttribute(hetrd_tc)");
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int64_t grid = std::min<int64_t>((int64_t)nsm * 2, batch);
    KTimer kt(st, "hetrd_tc_kernel", 16.0 / 3.0 * (double)N * N * N * batch);
    hetrd_tc_kernel<<<(unsigned)grid, HT_THREADS, HT_SMEM, st>>>(N, batch, Hpair, H, Hc, Vt, de, status_d,
                                                                 tc_wait_limit(), Nbig, off);
    TBG_LAUNCHED("hetrd_tc_kernel");
    return TBG_OK;
}

int bt_tc(cudaStream_t st, int N, int64_t batch, const cc* Vt, cc* U, int* status_d, int* urow_exp, int* ucol_exp) {
    if (batch <= 0 || N < 2) return TBG_OK;
    if (!hetrd_tc_fits(N)) return set_error(TBG_E_UNSUPPORTED, "bt_tc: matrix order beyond 128");
    cudaError_t e = cudaFuncSetAttribute(bt_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)BT_SMEM);
    if (e != cudaSuccess) return cuda_error(e, "cudaFuncSetAttribute(bt_tc)");
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int64_t grid = std::min<int64_t>((int64_t)nsm * 2, batch);
    KTimer kt(st, "bt_tc_kernel", 8.0 * (double)N * N * N * batch);
    bt_tc_kernel<<<(unsigned)grid, HT_THREADS, BT_SMEM, st>>>(N, batch, Vt, U, status_d, tc_wait_limit(), urow_exp,
                                                              ucol_exp);
    TBG_LAUNCHED("bt_tc_kernel");
    return TBG_OK;
}

}  // namespace tbg
