// Batched Hermitian eigensolver: one CTA per matrix.
//
// Replaces LAPACK zheev as reached from Rustb (src/response/traits.rs:168 via
// ndarray-linalg Eigh; src/ndarray_lapack.rs:412-448).  Algorithm per matrix:
//
//   1. Householder reduction to real symmetric tridiagonal form T = Q^H A Q
//      (unblocked, on the upper triangle: packed rows in shared memory, full
//      rows in global memory).  The reflector H_j = I - tau_j v_j v_j^H is
//      chosen so that H_j^H [alpha; x] = [beta; 0] with real beta of sign
//      opposite to Re(alpha) (no cancellation).  v_j is kept in row j of A.
//   2. Eigenvalues of T by Sturm-count multisection, a few threads per
//      eigenvalue (ascending by construction, absolute accuracy ~ eps ||T||).
//   3. Eigenvectors of T: for eigenvalues farther than 1e-3 ||T|| from their
//      neighbours, the twisted factorisation of T - lambda I (Fernando 1997;
//      one top-down and one bottom-up pivot sweep, no pivoting branches, no
//      iteration); eigenvalues closer than that form a cluster whose vectors
//      are computed by one thread by inverse iteration (tridiagonal LU with
//      partial pivoting) with modified Gram-Schmidt against the earlier
//      members.
//   4. Back-transformation U = H_0 H_1 ... H_{N-2} Z: in compact-WY blocks by
//      a pass of its own (heev_bt_tiled_kernel) when the matrix was in shared
//      memory, else reflector by reflector on column panels in the kernel.
//
// Output: E ascending (double), U with eigenvectors in columns (row-major).
// Precision T = double (plain path; A stays in global memory, L2-resident)
// or float (mixed path; A in shared memory when it fits: two matrices per SM
// up to 148 bands, one up to 215).

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <cstdlib>
#include <vector>

#include "tbgpu_internal.cuh"

namespace tbg {
namespace {

template <typename T>
struct Lim;
template <>
struct Lim<double> {
    static __device__ __forceinline__ double eps() { return DBL_EPSILON; }
    static __device__ __forceinline__ double tiny() { return DBL_MIN; }
    static __device__ __forceinline__ double div(double a, double b) { return a / b; }
};
template <>
struct Lim<float> {
    static __device__ __forceinline__ float eps() { return FLT_EPSILON; }
    static __device__ __forceinline__ float tiny() { return FLT_MIN; }
    static __device__ __forceinline__ float div(float a, float b) { return __fdividef(a, b); }
};

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

template <typename T>
__device__ __forceinline__ T warp_max(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Block-wide sum of one or two values; red must hold 2*32 T.  Ends with a barrier.
template <typename T>
__device__ __forceinline__ void block_sum2(T& a, T& b, T* red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    a = warp_sum(a);
    b = warp_sum(b);
    __syncthreads();
    if (lane == 0) {
        red[warp] = a;
        red[32 + warp] = b;
    }
    __syncthreads();
    T sa = 0, sb = 0;
    for (int w = 0; w < nw; ++w) {
        sa += red[w];
        sb += red[32 + w];
    }
    a = sa;
    b = sb;
    __syncthreads();
}

__device__ __forceinline__ unsigned hash32(unsigned x) {
    x ^= x >> 16;
    x *= 0x7feb352dU;
    x ^= x >> 15;
    x *= 0x846ca68bU;
    x ^= x >> 16;
    return x;
}

// Number of eigenvalues of the tridiagonal (d, e2 = e^2) strictly below x.
template <typename T>
__device__ __forceinline__ int sturm_count(int N, const T* __restrict__ d, const T* __restrict__ e2, T x,
                                           T pivmin) {
    int cnt = 0;
    T q = d[0] - x;
    if (fabs(q) < pivmin) q = -pivmin;
    cnt += (q < 0);
    for (int i = 1; i < N; ++i) {
        q = (d[i] - x) - Lim<T>::div(e2[i - 1], q);
        if (fabs(q) < pivmin) q = -pivmin;
        cnt += (q < 0);
    }
    return cnt;
}

// One inverse-iteration solve (T - lam I) y = x on the tridiagonal (d, e),
// in place on x (stride G in the per-thread scratch).  u0/u1/u2 hold the
// rows of the pivoted U factor.
template <typename T>
__device__ void tri_solve(int N, const T* __restrict__ d, const T* __restrict__ e, T lam, T pert,
                          T* __restrict__ x, T* __restrict__ u0, T* __restrict__ u1, T* __restrict__ u2,
                          int G) {
    // forward elimination with partial pivoting, applied to the RHS on the fly
    T cd = d[0] - lam;   // current row: entry at column i
    T cs = (N > 1) ? e[0] : T(0);  // entry at column i+1
    T cr = x[0];         // current row RHS
    for (int i = 0; i < N - 1; ++i) {
        const T b = e[i];                 // next row, column i
        const T a1 = d[i + 1] - lam;      // next row, column i+1
        const T b1 = (i + 2 < N) ? e[i + 1] : T(0);  // next row, column i+2
        const T xn = x[(i + 1) * G];
        if (fabs(cd) >= fabs(b)) {
            T piv = cd;
            if (fabs(piv) < pert) piv = (piv < 0) ? -pert : pert;
            const T mlt = Lim<T>::div(b, piv);
            u0[i * G] = piv;
            u1[i * G] = cs;
            u2[i * G] = 0;
            x[i * G] = cr;
            cd = a1 - mlt * cs;
            cs = b1;
            cr = xn - mlt * cr;
        } else {
            const T mlt = Lim<T>::div(cd, b);
            u0[i * G] = b;
            u1[i * G] = a1;
            u2[i * G] = b1;
            x[i * G] = xn;
            const T ncd = cs - mlt * a1;
            const T ncs = -mlt * b1;
            cr = cr - mlt * xn;
            cd = ncd;
            cs = ncs;
        }
    }
    if (fabs(cd) < pert) cd = (cd < 0) ? -pert : pert;
    u0[(N - 1) * G] = cd;
    x[(N - 1) * G] = cr;
    // back substitution
    T y2 = 0, y1 = 0;
    for (int i = N - 1; i >= 0; --i) {
        T r = x[i * G];
        if (i + 1 < N) r -= u1[i * G] * y1;
        if (i + 2 < N) r -= u2[i * G] * y2;
        const T yi = Lim<T>::div(r, u0[i * G]);
        x[i * G] = yi;
        y2 = y1;
        y1 = yi;
    }
}

// Eigenvector of the symmetric tridiagonal (d, e) for an isolated eigenvalue
// lam by the twisted factorisation of T - lam I (Fernando, "On computing an
// eigenvector of a tridiagonal matrix", 1997): stationary (top-down) pivots
// D+ and progressive (bottom-up) pivots D-, twist index r at the smallest
// |gamma_k| = |D+_k + D-_k - (d_k - lam)|, then z_r = 1 and
//   z_i = -e_i z_{i+1} / D+_i (i < r),   z_{i+1} = -e_i z_i / D-_{i+1} (i >= r).
// Pivots smaller than pert are replaced by -pert.  X holds N values with
// stride S: D+ first; once the twist index is known, D- is recomputed into
// the slots above it (D+ is needed only below it), and the vector overwrites
// both.  Writes the normalised (real) vector to u[i * ldu]; returns false if
// it is not finite.
template <typename T>
__device__ bool twisted_vector(int N, const T* __restrict__ d, const T* __restrict__ e, const T* __restrict__ e2,
                               T lam, T pert, T* __restrict__ X, int S, cx<T>* __restrict__ u, int ldu) {
    T p = d[0] - lam;
    if (fabs(p) < pert) p = -pert;
    X[0] = p;
    for (int i = 0; i < N - 1; ++i) {
        p = (d[i + 1] - lam) - Lim<T>::div(e2[i], p);
        if (fabs(p) < pert) p = -pert;
        X[(size_t)(i + 1) * S] = p;
    }
    T q = d[N - 1] - lam;
    if (fabs(q) < pert) q = -pert;
    const T q_last = q;
    int r = N - 1;
    T best = fabs(p + q - (d[N - 1] - lam));
    for (int i = N - 1; i >= 1; --i) {
        q = (d[i - 1] - lam) - Lim<T>::div(e2[i - 1], q);
        if (fabs(q) < pert) q = -pert;
        const T g = fabs(X[(size_t)(i - 1) * S] + q - (d[i - 1] - lam));
        if (g < best) {
            best = g;
            r = i - 1;
        }
    }
    // D-_i for i > r (the same operations as above, so the same values)
    q = q_last;
    if (r < N - 1) X[(size_t)(N - 1) * S] = q;
    for (int i = N - 1; i >= r + 2; --i) {
        q = (d[i - 1] - lam) - Lim<T>::div(e2[i - 1], q);
        if (fabs(q) < pert) q = -pert;
        X[(size_t)(i - 1) * S] = q;
    }
    // the vector, in place: z_i (i < r) over D+, z_i (i > r) over D-
    T z = 1, amax = 1;
#pragma unroll 4
    for (int i = r - 1; i >= 0; --i) {
        const T ratio = Lim<T>::div(e[i], X[(size_t)i * S]);
        z = -ratio * z;
        X[(size_t)i * S] = z;
        amax = max(amax, fabs(z));
    }
    z = 1;
#pragma unroll 4
    for (int i = r; i < N - 1; ++i) {
        const T ratio = Lim<T>::div(e[i], X[(size_t)(i + 1) * S]);
        z = -ratio * z;
        X[(size_t)(i + 1) * S] = z;
        amax = max(amax, fabs(z));
    }
    if (!(amax < T(INFINITY))) return false;  // also NaN
    const T sc = T(1) / amax;
    T nrm = 0;
    for (int i = 0; i < N; ++i) {
        const T v = (i == r ? T(1) : X[(size_t)i * S]) * sc;
        nrm += v * v;
    }
    if (!(nrm > T(0))) return false;
    const T inv = sc / sqrt(nrm);
    for (int i = 0; i < N; ++i) {
        const T v = (i == r ? T(1) : X[(size_t)i * S]) * inv;
        u[(size_t)i * ldu] = mk<T>(v, T(0));
    }
    return true;
}

template <typename T>
struct EigShared {
    cx<T>* A;   // N*N (shared or global)
    T* d;       // N
    T* e;       // N
    T* e2;      // N
    T* lam;     // N
    cx<T>* tau; // N
    cx<T>* v;   // N  (reflector of even steps)
    cx<T>* v2;  // N  (reflector of odd steps)
    cx<T>* w;   // N
    T* red;     // 64
    T* scratch; // inverse iteration: 4*N*G ; back-transform panel: N*PB complex
    int* flags; // 4 + N: status flags, then per-eigenvalue "left to inverse iteration" marks
};

constexpr int BT_NB = 16;  // reflectors per block of the blocked back-transformation

// Offset of A(i, i) in the working matrix.  In shared memory the upper
// triangle is packed row by row (row i holds columns i .. N-1, so two
// matrices of 128 bands fit one SM); in global memory rows are LDA apart.
// A(i, l) for l >= i is at diag_off(i) + (l - i).
template <bool PACKED>
__host__ __device__ __forceinline__ size_t diag_off(int N, int LDA, int i) {
    return PACKED ? (size_t)i * N - ((size_t)i * (size_t)(i - 1)) / 2 : (size_t)i * LDA + i;
}
template <bool PACKED>
__host__ __device__ inline size_t packed_elems(int N) {  // rounded to 16 bytes for the next buffers
    return PACKED ? (((size_t)N * (N + 1) / 2 + 1) & ~(size_t)1) : (size_t)N * N;
}

// First packed element of the rows kept in shared memory in the hybrid layout
// (rows below r0 in global memory), rounded down to an even index so the
// buffers after the matrix stay 16-byte aligned; 0 without it.
__host__ __device__ inline size_t hyb_smem_start(int N, int r0) {
    return r0 > 0 ? diag_off<true>(N, 0, r0) & ~(size_t)1 : 0;
}

template <typename T>
__host__ __device__ inline size_t eig_smem_bytes(int N, bool a_smem, int G, int PB, int r0 = 0) {
    size_t b = 0;
    if (a_smem) b += sizeof(cx<T>) * (packed_elems<true>(N) - hyb_smem_start(N, r0));  // packed upper triangle
    b += sizeof(T) * 4 * (size_t)N;
    b += sizeof(cx<T>) * 4 * (size_t)N;  // tau, v, v2, w
    b += sizeof(T) * 64;
    // inverse-iteration scratch; with the matrix in shared memory it lives in
    // the matrix's storage, free once the reflectors have gone out
    size_t s1 = a_smem ? 0 : sizeof(T) * 4 * (size_t)N * G;
    // back-transform in the kernel (matrix in global memory): a column-major
    // panel with stride N + 4; with the matrix in shared memory it is a pass
    // of its own (heev_bt_tiled_kernel)
    size_t s2 = a_smem ? 0 : sizeof(cx<T>) * (size_t)(N + 4) * PB;
    b += std::max(s1, s2);
    b += sizeof(int) * (4 + (size_t)N);  // flags + per-eigenvalue redo marks
    return b;
}


// Main kernel.  Hin: (batch, N, N) FP64.  For T = double and !A_SMEM the
// input matrix is reduced in place (destroyed).  U: (batch, N, N) cx<T>.
// MINB = CTAs per SM the launch bounds are set for: 3 (320 threads) for the
// packed matrices of up to about 130 bands, else 2 or 1 (512 threads).
// HYB (with A_SMEM): the hybrid layout for matrices whose packed triangle
// exceeds shared memory: rows below r0 (the longest, and the ones the first
// r0 steps finish) in global memory, Aglob (per CTA, packed as in shared
// memory), the rest in shared memory.
template <typename T, bool A_SMEM, int MINB = (A_SMEM ? 2 : 1), bool HYB = false>
__global__ void __launch_bounds__(MINB == 3 ? 320 : 512, MINB) heev_kernel(int N, int64_t batch, zc* __restrict__ Hin,
                                                   const float4* __restrict__ Hpair, double* __restrict__ Eout,
                                                   cx<T>* __restrict__ Uout, cx<T>* __restrict__ Awork,
                                                   int* __restrict__ status, int G, int PB,
                                                   const float* __restrict__ tri_de, cx<T>* __restrict__ Aglob,
                                                   int r0, int stop, cx<T>* __restrict__ Tout,
                                                   float* __restrict__ de_out) {
    static_assert(!HYB || A_SMEM, "the hybrid layout extends the shared-memory one");
    if (!HYB) r0 = 0;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    EigShared<T> sh;
    {
        unsigned char* p = smem_raw;
        if (A_SMEM) {
            sh.A = reinterpret_cast<cx<T>*>(p);
            p += sizeof(cx<T>) * (packed_elems<true>(N) - hyb_smem_start(N, r0));
        }
        sh.tau = reinterpret_cast<cx<T>*>(p);
        p += sizeof(cx<T>) * N;
        sh.v = reinterpret_cast<cx<T>*>(p);
        p += sizeof(cx<T>) * N;
        sh.v2 = reinterpret_cast<cx<T>*>(p);
        p += sizeof(cx<T>) * N;
        sh.w = reinterpret_cast<cx<T>*>(p);
        p += sizeof(cx<T>) * N;
        sh.d = reinterpret_cast<T*>(p);
        p += sizeof(T) * N;
        sh.e = reinterpret_cast<T*>(p);
        p += sizeof(T) * N;
        sh.e2 = reinterpret_cast<T*>(p);
        p += sizeof(T) * N;
        sh.lam = reinterpret_cast<T*>(p);
        p += sizeof(T) * N;
        sh.red = reinterpret_cast<T*>(p);
        p += sizeof(T) * 64;
        sh.scratch = A_SMEM ? reinterpret_cast<T*>(sh.A) : reinterpret_cast<T*>(p);
        // flags close the layout that eig_smem_bytes sizes
        sh.flags =
            reinterpret_cast<int*>(smem_raw + eig_smem_bytes<T>(N, A_SMEM, G, PB, r0) - sizeof(int) * (4 + (size_t)N));
    }
    const int tid = threadIdx.x, nthr = blockDim.x;
    const int lane = tid & 31, warp = tid >> 5, nwarps = nthr >> 5;
    const size_t NN = (size_t)N * N;
    const int LDA = N;  // row stride of the working matrix in global memory
    auto doff = [&](int i) { return diag_off<A_SMEM>(N, LDA, i); };
    const size_t e0s = hyb_smem_start(N, r0), e0 = HYB ? diag_off<true>(N, 0, r0) : 0;
    cx<T>* Ag = HYB ? Aglob + (size_t)blockIdx.x * e0 : nullptr;

    for (int64_t b = blockIdx.x; b < batch; b += gridDim.x) {
        cx<T>* A;
        if (A_SMEM) {
            A = sh.A;  // (hybrid: the shared-memory rows, element doff(r) at A[doff(r) - e0s])
        } else if (sizeof(T) == sizeof(double)) {
            A = reinterpret_cast<cx<T>*>(Hin + b * NN);
        } else {
            A = Awork + (size_t)blockIdx.x * NN;
        }
        // A(r, r): row r of the working matrix from its diagonal on
        auto rowp = [&](int r) -> cx<T>* {
            if constexpr (HYB) return (r < r0) ? Ag + doff(r) : A + (doff(r) - e0s);
            return A + doff(r);
        };
        if (tri_de) {
            // tridiagonal form given (TMEM-resident reduction): d then e
            const float* src = tri_de + (size_t)b * 2 * N;
            for (int i = tid; i < N; i += nthr) {
                sh.d[i] = (T)src[i];
                sh.e[i] = (T)src[N + i];
            }
            if (tid == 0) sh.flags[0] = 0;
            __syncthreads();
        } else {
        // ---------------------------------------------------------- load --
        if (Hpair) {
            // float-pair input {re_hi, re_lo, im_hi, im_lo} (FP32 solver only)
            const float4* src = Hpair + b * NN;
            for (size_t idx = tid; idx < NN; idx += nthr) {
                const int r = (int)(idx / N), c = (int)(idx % N);
                if (A_SMEM && c < r) continue;  // upper triangle only
                const float4 h = src[idx];
                rowp(r)[c - r] = mk<T>((T)(h.x + h.y), (T)(h.z + h.w));
            }
        } else if (A_SMEM || sizeof(T) != sizeof(double)) {
            const zc* src = Hin + b * NN;
            for (size_t idx = tid; idx < NN; idx += nthr) {
                const int r = (int)(idx / N), c = (int)(idx % N);
                if (A_SMEM && c < r) continue;
                zc h = src[idx];
                rowp(r)[c - r] = mk<T>((T)h.re, (T)h.im);
            }
        }
        if (tid == 0) sh.flags[0] = 0;
        __syncthreads();

        // ------------------------------------------------- tridiagonalise --
        // Only the upper triangle is kept (row i from column i on): A22 v reads
        // row i right of the diagonal and column i above it.  Warp 0 updates
        // row j+1 first and forms the reflector of step j+1 from it while the
        // other warps update the rest of the trailing matrix; reflectors of
        // consecutive steps alternate between two buffers.
        // reflector by warp 0 from row jr: H^H [alpha; x] = [beta; 0]
        auto make_reflector = [&](int jr, cx<T>* vout) {
            const int mr = N - 1 - jr;
            cx<T>* rowj = rowp(jr) + 1;  // row jr, columns jr+1.. = conj(column jr)
            T part = 0;
            for (int i = 1 + lane; i < mr; i += 32) part += abs2(rowj[i]);
            const T xnorm2 = warp_sum(part);
            const cx<T> alpha = conj(rowj[0]);
            cx<T> tau, scal;
            T beta;
            if (xnorm2 == T(0) && alpha.im == T(0)) {
                tau = mk<T>(0, 0);
                scal = mk<T>(0, 0);
                beta = alpha.re;
            } else {
                const T nrm = sqrt(alpha.re * alpha.re + alpha.im * alpha.im + xnorm2);
                beta = (alpha.re >= T(0)) ? -nrm : nrm;
                tau = mk<T>((beta - alpha.re) / beta, -alpha.im / beta);
                const cx<T> den = mk<T>(alpha.re - beta, alpha.im);
                const T dd = den.re * den.re + den.im * den.im;
                scal = mk<T>(den.re / dd, -den.im / dd);
            }
            for (int i = lane; i < mr; i += 32) {
                const cx<T> vi = (i == 0) ? mk<T>(1, 0) : conj(rowj[i]) * scal;
                vout[i] = vi;
                rowj[i] = vi;  // keep v_jr in row jr for the back-transformation
            }
            if (lane == 0) {
                sh.tau[jr] = tau;
                sh.e[jr] = beta;
                sh.d[jr] = rowp(jr)[0].re;
            }
        };
        // stop > 0 (shared-memory layouts): only the first `stop` steps; the trailing
        // block, the tridiagonal so far and the reflectors then go to global memory
        // for the TMEM-resident reduction to finish
        const int jend = (A_SMEM && stop > 0 && stop < N - 1) ? stop : N - 1;
        if (N > 1 && warp == 0) make_reflector(0, sh.v);
        __syncthreads();
        for (int j = 0; j < jend; ++j) {
            const int m = N - 1 - j;
            const cx<T>* v = (j & 1) ? sh.v2 : sh.v;
            const cx<T> tau = sh.tau[j];
            // A22(i, l) = A(j+1+i, j+1+l); row22(i)[l] = A22(i, l) for l >= i
            auto row22 = [&](int i) { return rowp(j + 1 + i) - i; };
            // w = tau * A22 v: four threads per row, two-level butterfly; partial of w^H v
            cx<T> dpart = mk<T>(0, 0);
            {
                const int q = tid & 3;
                const unsigned gm = 0xFu << (lane & 28);
                for (int i = tid >> 2; i < m; i += nthr >> 2) {
                    const cx<T>* row = row22(i);
                    // two partial sums per part: independent load/FMA chains
                    cx<T> acc = mk<T>(0, 0), acc2 = mk<T>(0, 0);
                    int l = i + q;
                    for (; l + 4 < m; l += 8) {
                        fma_cx(acc, row[l], v[l]);
                        fma_cx(acc2, row[l + 4], v[l + 4]);
                    }
                    if (l < m) fma_cx(acc, row[l], v[l]);
                    // conj(A22(l, i)) from the column above the diagonal, l = q, q + 4, ...:
                    // element offsets advance by doff(r + 4) - doff(r) - 4 per 4 rows
                    // (4 LDA for full rows; 4 N - 4 r - 10 packed, r the global row)
                    l = q;
                    if constexpr (HYB) {
                        // row by row (the rows below r0 are in global memory)
                        const int col = j + 1 + i;
                        for (; l + 4 < i; l += 8) {
                            fma_cjx(acc, rowp(j + 1 + l)[col - (j + 1 + l)], v[l]);
                            fma_cjx(acc2, rowp(j + 5 + l)[col - (j + 5 + l)], v[l + 4]);
                        }
                        if (l < i) fma_cjx(acc, rowp(j + 1 + l)[col - (j + 1 + l)], v[l]);
                    } else {
                        int r = j + 1 + q;
                        int a = (int)doff(r) + (j + 1 + i) - r;
                        int s4 = A_SMEM ? 4 * N - 4 * r - 10 : 4 * LDA;
                        for (; l + 4 < i; l += 8) {
                            fma_cjx(acc, A[a], v[l]);
                            fma_cjx(acc2, A[a + s4], v[l + 4]);
                            a += A_SMEM ? 2 * s4 - 16 : 2 * s4;  // doff(r + 8) - doff(r) - 8
                            if (A_SMEM) s4 -= 32;
                        }
                        if (l < i) fma_cjx(acc, A[a], v[l]);
                    }
                    acc = acc + acc2;
                    acc.re += __shfl_xor_sync(gm, acc.re, 1);
                    acc.im += __shfl_xor_sync(gm, acc.im, 1);
                    acc.re += __shfl_xor_sync(gm, acc.re, 2);
                    acc.im += __shfl_xor_sync(gm, acc.im, 2);
                    if (q == 0) {
                        const cx<T> wi = tau * acc;
                        sh.w[i] = wi;
                        fma_cjx(dpart, wi, v[i]);
                    }
                }
                dpart.re = warp_sum(dpart.re);
                dpart.im = warp_sum(dpart.im);
            }
            if (lane == 0) {
                sh.red[warp] = dpart.re;
                sh.red[32 + warp] = dpart.im;
            }
            __syncthreads();
            // w^H v: lane k holds warp k's partial, then a fixed butterfly (same order everywhere)
            cx<T> dp = (lane < nwarps) ? mk<T>(sh.red[lane], sh.red[32 + lane]) : mk<T>(0, 0);
            dp.re = warp_sum(dp.re);
            dp.im = warp_sum(dp.im);
            // alpha2 = -1/2 tau (w^H v); w' = w + alpha2 v;  A22 -= v w'^H + w' v^H (upper triangle):
            // A22(i, l) -= v_i conj(w_l) + c_i conj(v_l),  c_i = v_i conj(alpha2) + w'_i
            const cx<T> alpha2 = T(-0.5) * (tau * dp);
            auto update_row = [&](int i) {
                cx<T>* row = row22(i);
                const cx<T> vi = v[i];
                const cx<T> ci = mulc(vi, alpha2) + (sh.w[i] + alpha2 * vi);
                for (int l = i + lane; l < m; l += 32) {
                    cx<T> x = row[l];
                    fms_mulc(x, vi, sh.w[l]);
                    fms_mulc(x, ci, v[l]);
                    row[l] = x;
                }
            };
            if (warp == 0) {
                update_row(0);
                if (nwarps == 1)
                    for (int i = 1; i < m; ++i) update_row(i);
                __syncwarp();
                if (m >= 2 && j + 1 < jend) make_reflector(j + 1, (j & 1) ? sh.v : sh.v2);
            } else {
                for (int i = warp; i < m; i += nwarps - 1) update_row(i);  // rows 1 .. m-1 over warps 1 ..

            }
            __syncthreads();
        }
        if (jend < N - 1) {
            const int M = N - jend;
            cx<T>* Tb = Tout + (size_t)b * M * M;
            for (int idx = tid; idx < M * M; idx += nthr) {
                const int i = idx / M, l = idx - i * M;
                Tb[idx] = (i <= l) ? rowp(jend + i)[l - i] : conj(rowp(jend + l)[i - l]);
            }
            float* dd = de_out + (size_t)b * 2 * N;
            for (int i = tid; i < jend; i += nthr) {
                dd[i] = (float)sh.d[i];
                dd[N + i] = (float)sh.e[i];
            }
            const size_t pe = packed_elems<true>(N);
            cx<T>* dst = Awork + (size_t)b * (pe + N);  // rows from jend on are overwritten by the finish
            for (size_t i = tid; i < pe; i += nthr) dst[i] = (HYB && i < e0) ? Ag[i] : A[i - e0s];
            for (int i = tid; i < jend; i += nthr) dst[pe + i] = sh.tau[i];
            __syncthreads();
            continue;
        }
        if (tid == 0) {
            sh.d[N - 1] = rowp(N - 1)[0].re;
            sh.e[N - 1] = 0;
        }
        __syncthreads();
        }  // reduction
        // deflation: off-diagonals below eps (|d_i| + |d_i+1|) are set to zero,
        // as QR-type solvers do, so decoupled 1x1 blocks give d_i exactly
        for (int i = tid; i < N; i += nthr) {
            T ei = sh.e[i];
            if (i < N - 1 && fabs(ei) <= Lim<T>::eps() * (fabs(sh.d[i]) + fabs(sh.d[i + 1]))) ei = 0;
            sh.e[i] = ei;
        }
        __syncthreads();
        for (int i = tid; i < N; i += nthr) sh.e2[i] = sh.e[i] * sh.e[i];
        if constexpr (A_SMEM) {
            // reflectors (packed rows) and tau to the back-transformation pass;
            // the matrix's shared memory then serves the eigenvector scratch
            if (Uout && !tri_de) {
                const size_t pe = packed_elems<true>(N);
                cx<T>* dst = Awork + (size_t)b * (pe + N);
                for (size_t i = tid; i < pe; i += nthr) dst[i] = (HYB && i < e0) ? Ag[i] : A[i - e0s];
                for (int i = tid; i < N; i += nthr) dst[pe + i] = sh.tau[i];
            }
        }
        __syncthreads();

        // ------------------------------------------------------ bisection --
        T lo_g, hi_g, tnorm, pivmin;
        {
            T lo = INFINITY, hi = -INFINITY, em = 0;
            bool bad = false;  // min/max skip NaN, so non-finite entries are looked for as such
            for (int i = tid; i < N; i += nthr) {
                const T r = ((i > 0) ? fabs(sh.e[i - 1]) : T(0)) + ((i < N - 1) ? fabs(sh.e[i]) : T(0));
                lo = min(lo, sh.d[i] - r);
                hi = max(hi, sh.d[i] + r);
                em = max(em, sh.e2[i]);
                bad = bad || !isfinite(sh.d[i]) || !isfinite(sh.e[i]);
            }
            if (__any_sync(0xffffffffu, bad) && lane == 0) sh.flags[0] = 1;  // NaN/Inf input
            lo = -warp_max(-lo);
            hi = warp_max(hi);
            em = warp_max(em);
            if (lane == 0) {
                sh.red[warp] = lo;
                sh.red[32 + warp] = hi;
            }
            if (lane == 0) sh.scratch[warp] = em;
            __syncthreads();
            lo = INFINITY;
            hi = -INFINITY;
            em = 0;
            for (int w2 = 0; w2 < nwarps; ++w2) {
                lo = min(lo, sh.red[w2]);
                hi = max(hi, sh.red[32 + w2]);
                em = max(em, sh.scratch[w2]);
            }
            __syncthreads();
            tnorm = max(fabs(lo), fabs(hi));
            if (!(tnorm == tnorm) || isinf(tnorm)) {
                if (tid == 0) sh.flags[0] = 1;  // NaN/Inf input
                tnorm = 1;
                lo = -1;
                hi = 1;
            }
            pivmin = Lim<T>::tiny() * max(T(1), em);
            const T pad = T(2) * Lim<T>::eps() * tnorm + T(4) * pivmin;
            lo_g = lo - pad - T(2) * Lim<T>::eps() * tnorm;
            hi_g = hi + pad + T(2) * Lim<T>::eps() * tnorm;
            if (tnorm == T(0)) {
                lo_g = -pivmin;
                hi_g = pivmin;
            }
        }
        const T atol = T(2) * Lim<T>::eps() * tnorm + T(2) * pivmin;
        // Multisection: S threads (a power of two, S N <= threads) share one
        // eigenvalue; each round they evaluate the Sturm count at the S inner
        // points of S + 1 equal subintervals and keep the one holding it.
        {
            int S = 1;
            while (S < 8 && 2 * S * N <= nthr) S *= 2;
            const int passes = (N * S + nthr - 1) / nthr;  // uniform over the CTA
            for (int ps = 0; ps < passes; ++ps) {
                const int idx = ps * nthr + tid;
                const int i = idx / S, q = idx - (idx / S) * S;
                const int gbase = (lane / S) * S;
                const unsigned gmask = (S == 32) ? 0xffffffffu : ((1u << S) - 1u);
                T a = lo_g, c = hi_g;
                bool done = i >= N;
                for (int it = 0; it < 200; ++it) {
                    done = done || (c - a <= atol + T(2) * Lim<T>::eps() * max(fabs(a), fabs(c)));
                    if (__all_sync(0xffffffffu, done)) break;
                    const T h = (c - a) / T(S + 1);
                    const T x = a + T(q + 1) * h;
                    const bool above = !done && sturm_count<T>(N, sh.d, sh.e2, x, pivmin) > i;
                    const unsigned g = (__ballot_sync(0xffffffffu, above) >> gbase) & gmask;
                    if (!done) {
                        const int qs = g ? __ffs(g) - 1 : S;  // first inner point above the eigenvalue
                        const T na = (qs == 0) ? a : a + T(qs) * h;
                        const T nc = (qs == S) ? c : a + T(qs + 1) * h;
                        a = na;
                        c = nc;
                    }
                }
                if (i < N && q == 0) {
                    T lam = T(0.5) * (a + c);
                    // an isolated diagonal entry inside the final bracket is the exact eigenvalue
                    for (int j = 0; j < N; ++j) {
                        const bool iso = (j == 0 || sh.e[j - 1] == T(0)) && (j == N - 1 || sh.e[j] == T(0));
                        if (iso && sh.d[j] >= a && sh.d[j] <= c) {
                            lam = sh.d[j];
                            break;
                        }
                    }
                    sh.lam[i] = lam;
                }
            }
        }
        __syncthreads();
        // non-finite input (found while bounding the spectrum) is reported for
        // eigenvalue-only calls as well as for eigenpairs
        if (tid == 0 && sh.flags[0] && status) atomicOr(status, 1);
        if (Eout) {
            for (int i = tid; i < N; i += nthr) Eout[b * N + i] = (double)sh.lam[i];
        }
        if (Uout == nullptr) {
            __syncthreads();
            continue;
        }

        // ------------------------------------------ eigenvectors of T --
        cx<T>* U = Uout + b * NN;
        const T ctol = T(1e-3) * max(tnorm, Lim<T>::tiny());
        const T pert = max(Lim<T>::eps() * tnorm, pivmin);
        int* redo = sh.flags + 4;
        // (1) isolated eigenvalues: twisted factorisation, N scratch values
        //     each, at most one per thread at a time: all N in the freed matrix
        //     storage (N (N + 1) values) when it is in shared memory, else 4G
        // (hybrid: the shared-memory rows hold 4 N G values, as in the global layout)
        const int tw = (A_SMEM && !HYB) ? min(N, nthr) : min(4 * G, nthr);
        T* twx = A_SMEM ? reinterpret_cast<T*>(A) : sh.scratch;
        for (int g0 = 0; g0 < N; g0 += tw) {
            if (tid < tw && g0 + tid < N) {
                const int i = g0 + tid;
                const bool iso = (i == 0 || sh.lam[i] - sh.lam[i - 1] > ctol) &&
                                 (i == N - 1 || sh.lam[i + 1] - sh.lam[i] > ctol);
                redo[i] = iso ? !twisted_vector<T>(N, sh.d, sh.e, sh.e2, sh.lam[i], pert, twx + tid, tw, U + i, N)
                              : 1;
            }
            __syncthreads();
        }
        // (2) clusters (and any vector the twisted pass could not form): inverse
        //     iteration with Gram-Schmidt against the earlier cluster members
        for (int g0 = 0; g0 < N; g0 += G) {
            const int t = tid;
            if (t < G && g0 + t < N) {
                const int i = g0 + t;
                const bool first = (i == 0) || (sh.lam[i] - sh.lam[i - 1] > ctol);
                if (first && redo[i]) {
                    int c1 = i;
                    while (c1 + 1 < N && sh.lam[c1 + 1] - sh.lam[c1] <= ctol) ++c1;
                    T* x = sh.scratch + t;
                    T* u0 = x + (size_t)N * G;
                    T* u1 = u0 + (size_t)N * G;
                    T* u2 = u1 + (size_t)N * G;
                    T shift_prev = -INFINITY;
                    for (int jj = i; jj <= c1; ++jj) {
                        T shift = sh.lam[jj];
                        // separate coincident shifts inside a cluster
                        const T pertol = T(10) * Lim<T>::eps() * max(fabs(shift), tnorm * T(1e-3));
                        if (jj > i && shift - shift_prev < pertol) shift = shift_prev + pertol;
                        shift_prev = shift;
                        for (int r = 0; r < N; ++r) {
                            const unsigned h = hash32((unsigned)(r * 7919 + jj * 104729 + 12345));
                            x[(size_t)r * G] = T(1) + T(0.5) * ((T)(h & 0xffff) / T(65535) - T(0.5));
                        }
                        for (int iter = 0; iter < (sizeof(T) == sizeof(float) ? 2 : 3); ++iter) {
                            tri_solve<T>(N, sh.d, sh.e, shift, pert, x, u0, u1, u2, G);
                            // Gram-Schmidt against earlier cluster members (stored in U, real parts)
                            for (int pp = i; pp < jj; ++pp) {
                                T dot = 0;
                                for (int r = 0; r < N; ++r) dot += U[(size_t)r * N + pp].re * x[(size_t)r * G];
                                for (int r = 0; r < N; ++r) x[(size_t)r * G] -= dot * U[(size_t)r * N + pp].re;
                            }
                            T nrm = 0, amax = 0;
                            for (int r = 0; r < N; ++r) amax = max(amax, fabs(x[(size_t)r * G]));
                            if (!(amax > T(0)) || isinf(amax)) {
                                for (int r = 0; r < N; ++r) x[(size_t)r * G] = (r == (jj % N)) ? T(1) : T(0);
                                amax = 1;
                            }
                            const T sc = T(1) / amax;
                            for (int r = 0; r < N; ++r) {
                                const T xv = x[(size_t)r * G] * sc;
                                x[(size_t)r * G] = xv;
                                nrm += xv * xv;
                            }
                            const T inv = T(1) / sqrt(nrm);
                            for (int r = 0; r < N; ++r) x[(size_t)r * G] *= inv;
                        }
                        for (int r = 0; r < N; ++r) U[(size_t)r * N + jj] = mk<T>(x[(size_t)r * G], T(0));
                    }
                }
            }
            __syncthreads();
        }
        __threadfence_block();
        __syncthreads();

        // ----------------------------------------------- back-transform --
        if constexpr (A_SMEM) {
            // the reflectors went out after the reduction
            __syncthreads();
            continue;
        }
        // Panel P holds PB columns of U, column-major with stride N + 4.  Column
        // c belongs to the 8 threads 8c .. 8c+7 (rows interleaved), which apply
        // every reflector to it without block barriers.
        cx<T>* P = reinterpret_cast<cx<T>*>(sh.scratch);
        const int PS = N + 4;
        for (int c0 = 0; c0 < N; c0 += PB) {
            const int pw = min(PB, N - c0);
            for (int idx = tid; idx < N * pw; idx += nthr) {
                const int r = idx / pw, c = idx % pw;
                P[(size_t)c * PS + r] = U[(size_t)r * N + c0 + c];
            }
            __syncthreads();
            const int ngroups = nthr >> 3;
            const int q8 = tid & 7;
            const unsigned gm = 0xFFu << (lane & 24);
            for (int c = tid >> 3; c < pw; c += ngroups) {
                cx<T>* pc = P + (size_t)c * PS;
                for (int j = N - 2; j >= 0; --j) {
                    const cx<T> tau = sh.tau[j];
                    if (tau.re == T(0) && tau.im == T(0)) continue;
                    const int m = N - 1 - j;
                    const cx<T>* vj = A + doff(j) + 1;
                    cx<T> acc = mk<T>(0, 0);
                    for (int i = q8; i < m; i += 8) fma_cjx(acc, vj[i], pc[j + 1 + i]);
#pragma unroll
                    for (int o = 1; o < 8; o <<= 1) {
                        acc.re += __shfl_xor_sync(gm, acc.re, o);
                        acc.im += __shfl_xor_sync(gm, acc.im, o);
                    }
                    const cx<T> sc = tau * acc;
                    for (int i = q8; i < m; i += 8) pc[j + 1 + i] = pc[j + 1 + i] - vj[i] * sc;
                    __syncwarp(gm);
                }
            }
            __syncthreads();
            for (int idx = tid; idx < N * pw; idx += nthr) {
                const int r = idx / pw, c = idx % pw;
                U[(size_t)r * N + c0 + c] = P[(size_t)c * PS + r];
            }
            __syncthreads();
        }
        __syncthreads();
    }
}

// Back-transformation pass of the FP32 solver (matrix in shared memory during
// the reduction): U <- H_0 H_1 ... H_{N-2} U with H_j = I - tau_j v_j v_j^H,
// in compact-WY blocks of BT_NB reflectors, H_{j0} ... H_{j1-1} = I - V T V^H
// with T^{-1} = diag(1/tau) + striu(V^H V) (Joffrain, Low, Quintana-Orti,
// van de Geijn, Van Zee, "Accumulating Householder transformations,
// revisited", 2006), applied last-first.  One CTA per matrix; U in column
// panels of PB (a multiple of 4; all of U up to 144 bands) held in shared
// memory with N4 = N rounded up to 4 rows (zero padded), and each block of
// reflectors staged as a dense zero-masked BT_NB x N4 tile Vb (Vb[i][k] =
// v_{j0+i}[k] for k > j0 + i, else 0), so no product needs masks:
//   Gram G(l, i) = Vb[l]^H Vb[i] for l < i, four lanes per entry;
//   Y = Vb^H P: a thread holds rows i and i + 8 by four columns over a
//       quarter of the rows k (k = k0 + q (mod 4)); quarters are summed by
//       shuffles between lanes 8 and 16 apart;
//   Y <- T Y by back-substitution, per column: y_i = tau_i (y_i - sum_{l>i} G_il y_l);
//   P <- P - Vb^T Y in 4 x 4 register tiles (rows k..k+3).
// A thread's four columns are 2c, 2c + 1 and the same two W / 2 further on (W
// the panel width), so consecutive lanes read consecutive 16-byte pairs (no
// bank conflicts).  The next block's tile is read from global memory into
// registers while this block's products run and stored into the other of two
// tile buffers.  Vt: (batch, packed + N) = reflectors (packed rows), tau.
__host__ __device__ inline size_t bt_tiled_smem_bytes(int N, int PB) {
    const size_t N4 = (size_t)((N + 3) & ~3);
    return sizeof(cc) * (N4 * PB + 2 * (size_t)BT_NB * N4 + (size_t)BT_NB * PB + (size_t)BT_NB * BT_NB + N4);
}
// Widest panel (a multiple of 4, at most N rounded up to 4) that fits `budget`.
inline int bt_tiled_panel(int N, size_t budget) {
    const int N4 = (N + 3) & ~3;
    const size_t base = bt_tiled_smem_bytes(N, 0);
    if (budget <= base) return 0;
    const size_t pb = (budget - base) / (sizeof(cc) * (size_t)(N4 + BT_NB));
    return (int)std::min<size_t>((size_t)N4, pb & ~(size_t)3);
}

__device__ __forceinline__ cc bt_vb_elem(const cc* __restrict__ Vm, int N, int N4, int j0, int e) {
    const int i = e / N4, k = e - i * N4, j = j0 + i;
    if (j >= N - 1 || k <= j || k >= N) return mk<float>(0.f, 0.f);
    return Vm[diag_off<true>(N, 0, j) + (size_t)(k - j)];
}

template <bool PANELS>
__global__ void __launch_bounds__(512, 1) heev_bt_tiled_kernel(int N, int64_t batch, const cc* __restrict__ Vt,
                                                               cc* __restrict__ Uout, int PB) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int N4 = (N + 3) & ~3;
    const size_t pe = packed_elems<true>(N);
    cc* P = reinterpret_cast<cc*>(smem_raw);  // N4 x W (W <= PB)
    cc* Vbuf = P + (size_t)N4 * PB;             // 2 x BT_NB x N4
    cc* Y = Vbuf + 2 * (size_t)BT_NB * N4;      // BT_NB x W
    cc* G = Y + (size_t)BT_NB * PB;             // BT_NB x BT_NB
    cc* tau = G + BT_NB * BT_NB;                // N4
    const int tid = threadIdx.x, nthr = blockDim.x, lane = tid & 31;
    constexpr int kPre = 8;  // tile elements per thread prefetched: all of BT_NB * N4 up to 256 bands
    if (N < 2) return;
    const int jtop = ((N - 2) / BT_NB) * BT_NB;
    for (int64_t b = blockIdx.x; b < batch; b += gridDim.x) {
        const cc* Vm = Vt + (size_t)b * (pe + N);
        cc* U = Uout + (size_t)b * N * N;
      auto panel = [&](const int c0, const int W) {
        const int CG = W / 4, cgb = (CG + 7) / 8, H = W / 2;
        for (int e = tid; e < N4 * W; e += nthr) {
            const int r = e / W, c = e - r * W;
            P[e] = (r < N && c0 + c < N) ? U[(size_t)r * N + c0 + c] : mk<float>(0.f, 0.f);
        }
        for (int i = tid; i < N4; i += nthr) tau[i] = (i < N) ? Vm[pe + i] : mk<float>(0.f, 0.f);
        for (int e = tid; e < BT_NB * N4; e += nthr) Vbuf[e] = bt_vb_elem(Vm, N, N4, jtop, e);
        __syncthreads();
        int buf = 0;
        for (int j0 = jtop; j0 >= 0; j0 -= BT_NB) {
            const cc* Vb = Vbuf + (size_t)buf * BT_NB * N4;
            const int nb = min(BT_NB, N - 1 - j0);
            const int k0 = j0 + 1;
            cc pre[kPre];
#pragma unroll
            for (int u = 0; u < kPre; ++u) {
                const int e = tid + u * nthr;
                pre[u] = (j0 > 0 && e < BT_NB * N4) ? bt_vb_elem(Vm, N, N4, j0 - BT_NB, e) : mk<float>(0.f, 0.f);
            }
            // Gram: entry p = i (i - 1) / 2 + l, four lanes each
            if (tid < 4 * (BT_NB * (BT_NB - 1) / 2)) {
                const int p = tid >> 2, q = tid & 3;
                int i = 1;
                while ((i + 1) * i / 2 <= p) ++i;
                const int l = p - i * (i - 1) / 2;
                cc g = mk<float>(0.f, 0.f);
                for (int k = k0 + q; k < N; k += 4) fma_cjx(g, Vb[l * N4 + k], Vb[i * N4 + k]);
                g.re += __shfl_xor_sync(0xffffffffu, g.re, 1);
                g.im += __shfl_xor_sync(0xffffffffu, g.im, 1);
                g.re += __shfl_xor_sync(0xffffffffu, g.re, 2);
                g.im += __shfl_xor_sync(0xffffffffu, g.im, 2);
                if (q == 0) G[l * BT_NB + i] = g;
            }
            // Y = Vb^H P
            for (int base = 0; base < 256 * cgb; base += nthr) {
                const int it = base + tid, wt = it >> 5;
                const int qk = lane >> 3, ig = wt / cgb, cg = (wt - ig * cgb) * 8 + (lane & 7);
                const bool valid = it < 256 * cgb && cg < CG;
                float y[2][4][2];
#pragma unroll
                for (int r = 0; r < 2; ++r)
#pragma unroll
                    for (int c = 0; c < 4; ++c) y[r][c][0] = y[r][c][1] = 0.f;
                if (valid) {
                    const cc* va = Vb + ig * N4;
                    const cc* vc = Vb + (ig + 8) * N4;
                    for (int k = k0 + qk; k < N; k += 4) {
                        const cc a0 = va[k], a1 = vc[k];
                        const float4 p01 = *reinterpret_cast<const float4*>(P + (size_t)k * W + 2 * cg);
                        const float4 p23 = *reinterpret_cast<const float4*>(P + (size_t)k * W + 2 * cg + H);
                        const float pr[4] = {p01.x, p01.z, p23.x, p23.z}, pi[4] = {p01.y, p01.w, p23.y, p23.w};
#pragma unroll
                        for (int c = 0; c < 4; ++c) {  // y += conj(a) p
                            y[0][c][0] = fmaf(a0.re, pr[c], y[0][c][0]);
                            y[0][c][0] = fmaf(a0.im, pi[c], y[0][c][0]);
                            y[0][c][1] = fmaf(a0.re, pi[c], y[0][c][1]);
                            y[0][c][1] = fmaf(-a0.im, pr[c], y[0][c][1]);
                            y[1][c][0] = fmaf(a1.re, pr[c], y[1][c][0]);
                            y[1][c][0] = fmaf(a1.im, pi[c], y[1][c][0]);
                            y[1][c][1] = fmaf(a1.re, pi[c], y[1][c][1]);
                            y[1][c][1] = fmaf(-a1.im, pr[c], y[1][c][1]);
                        }
                    }
                }
#pragma unroll
                for (int r = 0; r < 2; ++r)
#pragma unroll
                    for (int c = 0; c < 4; ++c)
#pragma unroll
                        for (int h = 0; h < 2; ++h) {
                            float v = y[r][c][h];
                            v += __shfl_xor_sync(0xffffffffu, v, 8);
                            v += __shfl_xor_sync(0xffffffffu, v, 16);
                            y[r][c][h] = v;
                        }
                if (valid && qk == 0) {
#pragma unroll
                    for (int r = 0; r < 2; ++r) {
                        cc* yr = Y + (ig + 8 * r) * W + 2 * cg;
                        *reinterpret_cast<float4*>(yr) = make_float4(y[r][0][0], y[r][0][1], y[r][1][0], y[r][1][1]);
                        *reinterpret_cast<float4*>(yr + H) =
                            make_float4(y[r][2][0], y[r][2][1], y[r][3][0], y[r][3][1]);
                    }
                }
            }
            __syncthreads();
            // Y <- T Y, per column
            for (int c = tid; c < W; c += nthr) {
                cc yv[BT_NB];
#pragma unroll
                for (int i = 0; i < BT_NB; ++i) yv[i] = Y[i * W + c];
#pragma unroll
                for (int i = BT_NB - 1; i >= 0; --i) {
                    cc sv = yv[i];
#pragma unroll
                    for (int l = i + 1; l < BT_NB; ++l) sv = sv - G[i * BT_NB + l] * yv[l];
                    yv[i] = (i < nb) ? tau[j0 + i] * sv : mk<float>(0.f, 0.f);
                }
#pragma unroll
                for (int i = 0; i < BT_NB; ++i) Y[i * W + c] = yv[i];
            }
            __syncthreads();
            // P <- P - Vb^T Y over row groups from k0 rounded down to 4 (rows
            // above k0 get exact zeros)
            {
                const int ka = k0 & ~3, nrg = (N4 - ka) / 4;
                for (int it = tid; it < nrg * CG; it += nthr) {
                    const int rg = it / CG, cg = it - rg * CG, kb = ka + 4 * rg;
                    float acc[4][4][2];
#pragma unroll
                    for (int a = 0; a < 4; ++a)
#pragma unroll
                        for (int c = 0; c < 4; ++c) acc[a][c][0] = acc[a][c][1] = 0.f;
                    for (int i = 0; i < nb; ++i) {
                        const float4 v01 = *reinterpret_cast<const float4*>(Vb + i * N4 + kb);
                        const float4 v23 = *reinterpret_cast<const float4*>(Vb + i * N4 + kb + 2);
                        const float4 y01 = *reinterpret_cast<const float4*>(Y + i * W + 2 * cg);
                        const float4 y23 = *reinterpret_cast<const float4*>(Y + i * W + 2 * cg + H);
                        const float vr[4] = {v01.x, v01.z, v23.x, v23.z}, vi[4] = {v01.y, v01.w, v23.y, v23.w};
                        const float yr[4] = {y01.x, y01.z, y23.x, y23.z}, yi[4] = {y01.y, y01.w, y23.y, y23.w};
#pragma unroll
                        for (int a = 0; a < 4; ++a)
#pragma unroll
                            for (int c = 0; c < 4; ++c) {
                                acc[a][c][0] = fmaf(vr[a], yr[c], acc[a][c][0]);
                                acc[a][c][0] = fmaf(-vi[a], yi[c], acc[a][c][0]);
                                acc[a][c][1] = fmaf(vr[a], yi[c], acc[a][c][1]);
                                acc[a][c][1] = fmaf(vi[a], yr[c], acc[a][c][1]);
                            }
                    }
#pragma unroll
                    for (int a = 0; a < 4; ++a) {
                        cc* prow = P + (size_t)(kb + a) * W + 2 * cg;
                        float4 p01 = *reinterpret_cast<float4*>(prow), p23 = *reinterpret_cast<float4*>(prow + H);
                        p01.x -= acc[a][0][0];
                        p01.y -= acc[a][0][1];
                        p01.z -= acc[a][1][0];
                        p01.w -= acc[a][1][1];
                        p23.x -= acc[a][2][0];
                        p23.y -= acc[a][2][1];
                        p23.z -= acc[a][3][0];
                        p23.w -= acc[a][3][1];
                        *reinterpret_cast<float4*>(prow) = p01;
                        *reinterpret_cast<float4*>(prow + H) = p23;
                    }
                }
            }
            // the next block's tile into the other buffer (beyond kPre elements per thread,
            // N above 256, the rest is read directly)
            if (j0 > 0) {
                cc* nxt = Vbuf + (size_t)(buf ^ 1) * BT_NB * N4;
#pragma unroll
                for (int u = 0; u < kPre; ++u) {
                    const int e = tid + u * nthr;
                    if (e < BT_NB * N4) nxt[e] = pre[u];
                }
                for (int e = tid + kPre * nthr; e < BT_NB * N4; e += nthr) nxt[e] = bt_vb_elem(Vm, N, N4, j0 - BT_NB, e);
            }
            buf ^= 1;
            __syncthreads();
        }
        for (int e = tid; e < N * W; e += nthr) {
            const int r = e / W, c = e - r * W;
            if (c0 + c < N) U[(size_t)r * N + c0 + c] = P[e];
        }
        __syncthreads();
      };
        if constexpr (PANELS) {
            for (int c0 = 0; c0 < N; c0 += PB) panel(c0, min(PB, N4 - c0));
        } else {
            panel(0, N4);  // all of U in one pass
        }
    }
}

// Shared memory per CTA: one CTA per SM, or two or three sharing the SM's
// 228 KB (1 KB of it reserved per CTA).
constexpr size_t kEigSmemOne = 220 * 1024;
constexpr size_t kEigSmemTwo = 113 * 1024;
constexpr size_t kEigSmemThree = 75 * 1024;

// Threads of the solver's CTA (one matrix per CTA); FP32 with three CTAs per SM: 320.
template <typename T>
inline int eig_threads(int N, int ctas_per_sm = 2) {
    if (N <= 16) return 32;
    if (N <= 48) return 128;
    if (sizeof(T) == sizeof(float)) return ctas_per_sm == 3 ? 320 : 512;
    return 256;
}

// Inverse-iteration group G and back-transform panel PB sized to the shared
// memory left after the matrix (when resident) and the per-matrix vectors.
template <typename T>
inline void choose_g_pb(int N, bool a_smem, int gmax, int pbmax, int& G, int& PB, size_t budget = kEigSmemOne) {
    const size_t fixed = eig_smem_bytes<T>(N, a_smem, 0, 0);
    // with the matrix in shared memory the scratch is the matrix's storage
    const size_t left = a_smem ? sizeof(cx<T>) * packed_elems<true>(N) : (budget > fixed ? budget - fixed : 0);
    G = (int)std::max<size_t>(1, std::min<size_t>(gmax, left / (sizeof(T) * 4 * (size_t)N)));
    if (a_smem) {
        // the back-transformation is a pass of its own (heev_bt_tiled_kernel):
        // its panel is as wide as its shared memory allows (up to all columns)
        PB = bt_tiled_panel(N, kEigSmemOne);
    } else {
        PB = (int)std::max<size_t>(1, std::min<size_t>(pbmax, left / (sizeof(cx<T>) * (size_t)(N + 4))));
    }
}

// The dynamic shared-memory limit is a per-function attribute shared by every
// host thread; it is set once to the device's opt-in maximum (a per-call value
// would race with concurrent calls on other matrix sizes).
template <typename K>
int allow_max_smem(K kern, size_t need) {
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (need > (size_t)optin) return set_error(TBG_E_UNSUPPORTED, "eigensolver: shared memory beyond the device limit");
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
    if (e != cudaSuccess) return cuda_error(e, "cudaFuncSetAttribute(heev)");
    return TBG_OK;
}

template <typename T, bool A_SMEM, int MINB = (A_SMEM ? 2 : 1), bool HYB = false>
int launch_heev(cudaStream_t st, int N, int64_t batch, zc* H, double* E, cx<T>* U, void* work,
                size_t work_bytes, int* status_d, const char* name, int G, int PB, const float4* Hpair = nullptr,
                const float* tri_de = nullptr, bool skip_bt = false, int r0 = 0, int stop = 0,
                cx<T>* Tout = nullptr, float* de_out = nullptr, size_t aglob_off = 0) {
    const size_t smem = eig_smem_bytes<T>(N, A_SMEM, G, PB, HYB ? r0 : 0);
    auto kern = heev_kernel<T, A_SMEM, MINB, HYB>;
    if (int rc = allow_max_smem(kern, smem)) return rc;
    cudaError_t e;
    int dev = 0, nsm = 0, perSM = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int threads = eig_threads<T>(N, MINB);
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, kern, threads, smem);
    if (e != cudaSuccess || perSM < 1) perSM = 1;
    int64_t grid = (int64_t)nsm * perSM;
    const bool needs_work = !A_SMEM && sizeof(T) != sizeof(double);
    if (needs_work) {
        const int64_t per = (int64_t)sizeof(cx<T>) * N * N;
        const int64_t cap = (int64_t)(work_bytes / (size_t)per);
        if (cap < 1) return set_error(TBG_E_OOM, "eigensolver workspace too small");
        grid = std::min(grid, cap);
    }
    const size_t refl = sizeof(cx<T>) * (packed_elems<true>(N) + N) * (size_t)batch;
    if (A_SMEM && U && work_bytes < refl)
        return set_error(TBG_E_OOM, "eigensolver workspace too small for the reflectors");
    grid = std::min<int64_t>(grid, batch);
    if (grid < 1) return TBG_OK;
    // hybrid layout: the global-memory rows of each CTA, after the reflectors (or at aglob_off)
    cx<T>* Aglob = nullptr;
    if (HYB) {
        const size_t e0 = diag_off<true>(N, 0, r0);
        const size_t off = aglob_off ? aglob_off : refl;
        if (work_bytes < off + sizeof(cx<T>) * e0 * (size_t)grid)
            return set_error(TBG_E_OOM, "eigensolver workspace too small for the hybrid layout");
        Aglob = reinterpret_cast<cx<T>*>(static_cast<unsigned char*>(work) + off);
    }
    {
        // flops as LAPACK counts them: 16/3 N^3 (reduction) + 8 N^3 (back-transformation, a
        // separate pass when the matrix is in shared memory) + O(N^2) per matrix
        // (the tridiagonal stage alone, O(N^2) per matrix, is counted as no flops)
        // (the partial reduction: 16/3 (N^3 - (N - stop)^3) flops)
        const double fl = tri_de ? 0.0
                          : stop > 0 ? 16.0 / 3.0 * ((double)N * N * N - (double)(N - stop) * (N - stop) * (N - stop))
                                     : (A_SMEM && U ? 6.0 : 14.0) * (double)N * N * N;
        KTimer kt(st, name, fl * batch);
        kern<<<(unsigned)grid, threads, smem, st>>>(N, batch, H, Hpair, E, U, reinterpret_cast<cx<T>*>(work),
                                                    status_d, G, PB, tri_de, Aglob, HYB ? r0 : 0, stop, Tout, de_out);
        TBG_LAUNCHED(name);
    }
    if constexpr (A_SMEM) {
        if (!U || skip_bt || stop > 0) return TBG_OK;
        static_assert(sizeof(T) == sizeof(float), "the shared-memory solver is the FP32 one");
        const size_t bsm = bt_tiled_smem_bytes(N, PB);
        auto bk = PB >= ((N + 3) & ~3) ? heev_bt_tiled_kernel<false> : heev_bt_tiled_kernel<true>;
        if (int rc = allow_max_smem(bk, bsm)) return rc;
        KTimer kt(st, "heev_bt_kernel", 8.0 * (double)N * N * N * batch);
        bk<<<(unsigned)std::min<int64_t>(nsm, batch), 512, bsm, st>>>(N, batch, reinterpret_cast<const cc*>(work),
                                                                      reinterpret_cast<cc*>(U), PB);
        TBG_LAUNCHED("heev_bt_kernel");
    }
    return TBG_OK;
}

// FP32 solver: matrix in shared memory when it fits, two matrices per SM
// when both fit (up to about 150 bands).
inline bool f32_smem_fits(int N, size_t budget, int& G, int& PB) {
    choose_g_pb<float>(N, true, 32, 64, G, PB, budget);
    return eig_smem_bytes<float>(N, true, G, PB) <= budget && PB >= std::min(16, (N + 3) & ~3) &&
           bt_tiled_smem_bytes(N, PB) <= kEigSmemOne;
}
// CTAs per SM of the shared-memory FP32 solver (3, 2 or 1), 0 when the matrix
// does not fit.  Three (320 threads each) from 49 bands while they fit: the
// reduction is latency-bound, and a third matrix on the SM hides more of it.
inline int f32_smem_ctas(int N, int& G, int& PB) {
    if (N > 48 && f32_smem_fits(N, kEigSmemThree, G, PB)) return 3;
    if (f32_smem_fits(N, kEigSmemTwo, G, PB)) return 2;
    if (f32_smem_fits(N, kEigSmemOne, G, PB)) return 1;
    return 0;
}
inline bool f32_in_smem(int N, int& G, int& PB) { return f32_smem_ctas(N, G, PB) > 0; }
inline bool f32_in_smem(int N) {
    int G, PB;
    return f32_in_smem(N, G, PB);
}

// Hybrid layout for matrices whose packed triangle exceeds one CTA's shared
// memory (from about 229 bands): the smallest r0 whose remaining rows fit with
// room for the inverse-iteration / twisted-factorisation scratch of G >= 8
// groups (4 N G values) and a back-transformation panel of at least 8
// columns.  Up to TBG_F32_HYBRID_MAX bands (default 320; 0 = never).
int f32_hybrid_max_n() {
    static const int v = [] {
        const char* s = std::getenv("TBG_F32_HYBRID_MAX");
        return s ? std::max(0, std::atoi(s)) : 320;
    }();
    return v;
}
inline bool f32_hybrid_plan(int N, int& r0, int& G, int& PB) {
    if (N > f32_hybrid_max_n() || f32_in_smem(N)) return false;
    PB = bt_tiled_panel(N, kEigSmemOne);
    if (PB < 8) return false;
    for (r0 = 1; r0 < N; ++r0) {
        const size_t part = sizeof(cc) * (packed_elems<true>(N) - hyb_smem_start(N, r0));
        G = (int)std::min<size_t>(32, part / (sizeof(float) * 4 * (size_t)N));
        if (G >= 8 && eig_smem_bytes<float>(N, true, G, PB, r0) <= kEigSmemOne) return true;
    }
    return false;
}

// Two-phase FP32 reduction for 129 .. f32_hybrid_max_n() bands: the
// shared-memory (or hybrid) kernel does the first N - 128 steps and hands the
// trailing 128 x 128 block to the TMEM-resident kernel, which finishes it;
// the tridiagonal stage and the back-transformation then run on the whole
// matrix.  Workspace: [reflectors + tau][d, e][trailing blocks][hybrid rows].
struct TwoPhase {
    bool on = false;
    int ctas = 0, r0 = 0, G = 0, PB = 0;
    size_t off_de = 0, off_tb = 0, off_ag = 0, total = 0;
};
inline size_t al256(size_t x) { return (x + 255) & ~(size_t)255; }
TwoPhase two_phase_plan(int N, int64_t batch) {
    TwoPhase t;
    if (!eig_tc_enabled() || N <= 128 || N > f32_hybrid_max_n()) return t;
    int G = 0, PB = 0;
    t.ctas = f32_smem_ctas(N, G, PB);
    if (t.ctas == 0 && !f32_hybrid_plan(N, t.r0, G, PB)) return t;
    t.G = G;
    t.PB = PB;
    const size_t b = (size_t)std::max<int64_t>(batch, 1);
    t.off_de = al256(sizeof(cc) * (packed_elems<true>(N) + N) * b);
    t.off_tb = t.off_de + al256(sizeof(float) * 2 * (size_t)N * b);
    t.off_ag = t.off_tb + al256(sizeof(cc) * 128 * 128 * b);
    size_t ag = 0;
    if (t.r0 > 0) {
        int dev = 0, nsm = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || nsm < 1) nsm = 152;
        ag = sizeof(cc) * diag_off<true>(N, 0, t.r0) * (size_t)std::min<int64_t>((int64_t)b, 2 * (int64_t)nsm);
    }
    t.total = t.off_ag + ag;
    t.on = true;
    return t;
}

}  // namespace

size_t eig_workspace_bytes(int N, int64_t batch, int precision) {
    if (precision == 0) return 0;
    const TwoPhase tp = two_phase_plan(N, batch);
    if (tp.on) return tp.total;
    // reflectors (packed rows) and tau, then the tridiagonal forms of the TMEM-resident reduction
    if (f32_in_smem(N))
        return (sizeof(cc) * (packed_elems<true>(N) + N) + sizeof(float) * 2 * (size_t)N) *
               (size_t)std::max<int64_t>(batch, 1);
    int r0, G, PB;
    if (f32_hybrid_plan(N, r0, G, PB)) {
        // the reflectors, then each resident CTA's global-memory rows (at most two per SM)
        int dev = 0, nsm = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || nsm < 1) nsm = 152;
        const int64_t ctas = std::min<int64_t>(std::max<int64_t>(batch, 1), 2 * (int64_t)nsm);
        return sizeof(cc) * (packed_elems<true>(N) + N) * (size_t)std::max<int64_t>(batch, 1) +
               sizeof(cc) * diag_off<true>(N, 0, r0) * (size_t)ctas;
    }
    return (size_t)sizeof(cc) * N * N * (size_t)std::min<int64_t>(batch, 152 * 4);
}

// Largest band count the FP64 driver sends to the warp-per-matrix Jacobi
// solver: TBG_JACOBI_MAX_N at load, then whatever tbg_set_jacobi_max_n sets
// (the batch autotuner times both solvers per band-count bucket).
std::atomic<int>& jacobi_max_n_ref() {
    static std::atomic<int> v{[] {
        const char* s = std::getenv("TBG_JACOBI_MAX_N");
        return s ? std::max(0, std::min(std::atoi(s), kJacobiMaxN)) : kSmallMaxN;
    }()};
    return v;
}
int jacobi_max_n() { return jacobi_max_n_ref().load(std::memory_order_relaxed); }

// FP64 driver (plain path): A destroyed, U complex<double>.
int eig_batched(cudaStream_t st, int N, int64_t batch, zc* A, double* E, zc* U, void* work,
                size_t work_bytes, int* status_d) {
    if (batch <= 0) return TBG_OK;
    if (N <= kSmallMaxN) return eig_small(st, N, batch, A, E, U, status_d);  // one thread per matrix
    if (N <= jacobi_max_n()) return eig_jacobi(st, N, batch, A, E, U, status_d);  // one warp per matrix
    int G, PB;
    choose_g_pb<double>(N, false, 16, 16, G, PB);
    return launch_heev<double, false>(st, N, batch, A, E, U, work, work_bytes, status_d, "heev_kernel<double>", G,
                                      PB);
}

// Eigenvalues only, FP64, of `batch` matrices held in caller-provided device
// memory `A` (destroyed).  Launches the solver directly: no allocation, no
// events, nothing but the kernel on `st`.
int eig_values_f64_inplace(cudaStream_t st, int N, int64_t batch, zc* A, double* E) {
    if (batch <= 0) return TBG_OK;
    int G, PB;
    choose_g_pb<double>(N, false, 16, 16, G, PB);
    const size_t smem = eig_smem_bytes<double>(N, false, G, PB);
    auto kern = heev_kernel<double, false>;
    if (int rc = allow_max_smem(kern, smem)) return rc;
    cudaError_t e;
    int dev = 0, nsm = 0, perSM = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int threads = (N <= 16) ? 32 : (N <= 48 ? 128 : 256);
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, kern, threads, smem);
    if (e != cudaSuccess || perSM < 1) perSM = 1;
    const int64_t grid = std::min<int64_t>((int64_t)nsm * perSM, batch);
    kern<<<(unsigned)grid, threads, smem, st>>>(N, batch, A, nullptr, E, nullptr, nullptr, nullptr, G, PB, nullptr,
                                                nullptr, 0, 0, nullptr, nullptr);
    TBG_LAUNCHED("heev_kernel<double> (static scratch)");
    return TBG_OK;
}

// FP32 driver (mixed path): H preserved, U complex<float>.
int eig_batched_f32(cudaStream_t st, int N, int64_t batch, zc* H, double* E, cc* U, void* work,
                    size_t work_bytes, int* status_d, const float4* Hpair, int* urow_exp, int* ucol_exp,
                    bool* exps_filled) {
    if (exps_filled) *exps_filled = false;
    if (batch <= 0) return TBG_OK;
    int G, PB;
    const int ctas = f32_smem_ctas(N, G, PB);
    if (ctas == 3 && N > 64 && hetrd_tc_fits(N) && eig_tc_enabled()) {
        // reduction with the matrix in TMEM (tcgen05 rank-2 updates), then the
        // tridiagonal stage and the back-transformation pass
        const size_t vt = sizeof(cc) * (packed_elems<true>(N) + N) * (size_t)batch;
        if (work_bytes < vt + hetrd_tc_de_bytes(N, batch))
            return set_error(TBG_E_OOM, "eigensolver workspace too small for the reduction's output");
        float* de = reinterpret_cast<float*>(static_cast<unsigned char*>(work) + vt);
        if (int rc = hetrd_tc(st, N, batch, Hpair, H, static_cast<cc*>(work), de, status_d)) return rc;
        if (int rc = launch_heev<float, true, 3>(st, N, batch, H, E, U, work, work_bytes, status_d,
                                                 "heev_tri_kernel<float>", G, PB, Hpair, de, bt_tc_enabled()))
            return rc;
        if (!U || !bt_tc_enabled()) return TBG_OK;
        const bool ex = urow_exp && ucol_exp;
        if (int rc = bt_tc(st, N, batch, static_cast<const cc*>(work), U, status_d, ex ? urow_exp : nullptr,
                           ex ? ucol_exp : nullptr))
            return rc;
        if (exps_filled) *exps_filled = ex;
        return TBG_OK;
    }
    const TwoPhase tp = two_phase_plan(N, batch);
    if (tp.on) {
        if (work_bytes < tp.total) return set_error(TBG_E_OOM, "eigensolver workspace too small (two-phase reduction)");
        unsigned char* w = static_cast<unsigned char*>(work);
        float* de = reinterpret_cast<float*>(w + tp.off_de);
        cc* Tb = reinterpret_cast<cc*>(w + tp.off_tb);
        const int stop = N - 128;
        int rc;
        auto finish = [&]() {
            return hetrd_tc(st, 128, batch, nullptr, nullptr, static_cast<cc*>(work), de, status_d, Tb, N, stop);
        };
        if (tp.r0 > 0) {
            rc = launch_heev<float, true, 2, true>(st, N, batch, H, E, U, work, work_bytes, status_d,
                                                   "heev_kernel<float,hybrid>", tp.G, tp.PB, Hpair, nullptr, false,
                                                   tp.r0, stop, Tb, de, tp.off_ag);
            if (!rc) rc = finish();
            if (!rc)
                rc = launch_heev<float, true, 2, true>(st, N, batch, H, E, U, work, work_bytes, status_d,
                                                       "heev_tri_kernel<float>", tp.G, tp.PB, Hpair, de, false, tp.r0,
                                                       0, nullptr, nullptr, tp.off_ag);
        } else if (tp.ctas == 3) {
            rc = launch_heev<float, true, 3>(st, N, batch, H, E, U, work, work_bytes, status_d,
                                             "heev_kernel<float,smem>", tp.G, tp.PB, Hpair, nullptr, false, 0, stop, Tb,
                                             de);
            if (!rc) rc = finish();
            if (!rc)
                rc = launch_heev<float, true, 3>(st, N, batch, H, E, U, work, work_bytes, status_d,
                                                 "heev_tri_kernel<float>", tp.G, tp.PB, Hpair, de);
        } else {
            rc = launch_heev<float, true>(st, N, batch, H, E, U, work, work_bytes, status_d, "heev_kernel<float,smem>",
                                          tp.G, tp.PB, Hpair, nullptr, false, 0, stop, Tb, de);
            if (!rc) rc = finish();
            if (!rc)
                rc = launch_heev<float, true>(st, N, batch, H, E, U, work, work_bytes, status_d,
                                              "heev_tri_kernel<float>", tp.G, tp.PB, Hpair, de);
        }
        return rc;
    }
    if (ctas == 3)
        return launch_heev<float, true, 3>(st, N, batch, H, E, U, work, work_bytes, status_d,
                                           "heev_kernel<float,smem>", G, PB, Hpair);
    if (ctas > 0) {
        return launch_heev<float, true>(st, N, batch, H, E, U, work, work_bytes, status_d, "heev_kernel<float,smem>",
                                        G, PB, Hpair);
    }
    int r0 = 0;
    if (f32_hybrid_plan(N, r0, G, PB))
        return launch_heev<float, true, 2, true>(st, N, batch, H, E, U, work, work_bytes, status_d,
                                                 "heev_kernel<float,hybrid>", G, PB, Hpair, nullptr, false, r0);
    choose_g_pb<float>(N, false, 32, 64, G, PB);
    return launch_heev<float, false>(st, N, batch, H, E, U, work, work_bytes, status_d, "heev_kernel<float,global>",
                                     G, PB, Hpair);
}

}  // namespace tbg

// Internal test hook (not part of the public header): FP64 eigenpairs of nk
// host complex-double matrices by the Householder solver (method 0) or the
// warp-per-matrix Jacobi solver (method 1), run `reps` times on a device copy;
// *ms gets the mean device time of one run (CUDA events around the solver).
extern "C" int tbg_internal_eig_f64(int n, int64_t nk, const double* H, double* E, double* U, int method, int reps,
                                    float* ms) {
    using namespace tbg;
    const size_t NN = (size_t)n * n;
    void *dH = nullptr, *dA = nullptr, *dE = nullptr, *dU = nullptr, *dS = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = TBG_OK;
    if (n < 1 || nk < 1 || reps < 1 || (method == 1 && (n < 2 || n > kJacobiMaxN)))
        return set_error(TBG_E_INVALID_ARGUMENT, "eig test: bad size or method");
    if (cudaMalloc(&dH, 16 * NN * nk) || cudaMalloc(&dA, 16 * NN * nk) || cudaMalloc(&dE, 8 * n * nk) ||
        cudaMalloc(&dU, 16 * NN * nk) || cudaMalloc(&dS, sizeof(int)) || cudaEventCreate(&e0) ||
        cudaEventCreate(&e1))
        rc = set_error(TBG_E_OOM, "eig test alloc");
    float total = 0.0f;
    if (!rc) {
        cudaMemcpy(dH, H, 16 * NN * nk, cudaMemcpyHostToDevice);
        cudaMemset(dS, 0, sizeof(int));
        for (int it = 0; it < reps && !rc; ++it) {
            cudaMemcpyAsync(dA, dH, 16 * NN * nk, cudaMemcpyDeviceToDevice, 0);
            cudaEventRecord(e0, 0);
            if (method == 1)
                rc = eig_jacobi(0, n, nk, static_cast<zc*>(dA), static_cast<double*>(dE), static_cast<zc*>(dU),
                                static_cast<int*>(dS));
            else if (n <= kSmallMaxN)
                rc = eig_small(0, n, nk, static_cast<zc*>(dA), static_cast<double*>(dE), static_cast<zc*>(dU),
                               static_cast<int*>(dS));
            else {
                int G, PB;
                choose_g_pb<double>(n, false, 16, 16, G, PB);
                rc = launch_heev<double, false>(0, n, nk, static_cast<zc*>(dA), static_cast<double*>(dE),
                                                static_cast<zc*>(dU), nullptr, 0, static_cast<int*>(dS),
                                                "heev_kernel<double>", G, PB);
            }
            cudaEventRecord(e1, 0);
            cudaError_t e = cudaEventSynchronize(e1);
            if (!rc && e != cudaSuccess) rc = cuda_error(e, "eig test");
            float t = 0.0f;
            cudaEventElapsedTime(&t, e0, e1);
            total += t;
        }
        int st = 0;
        cudaMemcpy(&st, dS, sizeof(int), cudaMemcpyDeviceToHost);
        if (!rc && st) rc = set_error(TBG_E_NOCONV, "eig test: non-finite eigenvalues");
    }
    if (!rc) {
        if (ms) *ms = total / reps;
        cudaMemcpy(E, dE, 8 * n * nk, cudaMemcpyDeviceToHost);
        cudaMemcpy(U, dU, 16 * NN * nk, cudaMemcpyDeviceToHost);
    }
    cudaFree(dH);
    cudaFree(dA);
    cudaFree(dE);
    cudaFree(dU);
    cudaFree(dS);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    return rc;
}

// Internal test hook (not part of the public header): FP32 eigenpairs of nk
// host complex-double matrices (n x n) -> E (nk, n) and U (nk, n, n) complex
// double (eigenvectors in columns), for checks of the solver's own accuracy.
extern "C" int tbg_internal_eig_f32(int n, int64_t nk, const double* H, double* E, double* U) {
    using namespace tbg;
    const size_t NN = (size_t)n * n;
    void *dH = nullptr, *dE = nullptr, *dU = nullptr, *dW = nullptr, *dS = nullptr;
    const size_t wb = eig_workspace_bytes(n, nk, 1);
    int rc = TBG_OK;
    if (cudaMalloc(&dH, 16 * NN * nk) || cudaMalloc(&dE, 8 * n * nk) || cudaMalloc(&dU, 8 * NN * nk) ||
        cudaMalloc(&dS, sizeof(int)) || (wb && cudaMalloc(&dW, wb)))
        rc = set_error(TBG_E_OOM, "eig test alloc");
    if (!rc) {
        cudaMemcpy(dH, H, 16 * NN * nk, cudaMemcpyHostToDevice);
        cudaMemset(dS, 0, sizeof(int));
        rc = eig_batched_f32(0, n, nk, static_cast<zc*>(dH), static_cast<double*>(dE), static_cast<cc*>(dU), dW, wb,
                             static_cast<int*>(dS));
        cudaError_t e = cudaDeviceSynchronize();
        if (!rc && e != cudaSuccess) rc = cuda_error(e, "eig test");
    }
    if (!rc) {
        std::vector<cc> u(NN * nk);
        cudaMemcpy(E, dE, 8 * n * nk, cudaMemcpyDeviceToHost);
        cudaMemcpy(u.data(), dU, 8 * NN * nk, cudaMemcpyDeviceToHost);
        for (size_t i = 0; i < u.size(); ++i) {
            U[2 * i] = u[i].re;
            U[2 * i + 1] = u[i].im;
        }
    }
    cudaFree(dH);
    cudaFree(dE);
    cudaFree(dU);
    cudaFree(dS);
    cudaFree(dW);
    return rc;
}

// Crossover between the FP64 solvers (see include/tbgpu.h); returns the previous value.
extern "C" int tbg_set_jacobi_max_n(int n) {
    using namespace tbg;
    return jacobi_max_n_ref().exchange(std::max(kSmallMaxN, std::min(n, kJacobiMaxN)));
}
