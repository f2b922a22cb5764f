// Internal declarations shared by the tbgpu CUDA translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/tbgpu.h"

namespace tbg {

// ----------------------------------------------------------------- complex --
// Aligned to its full size, so a complex element moves as one vector load or
// store (LDS.64 / LDG.128) rather than two scalar ones.
template <typename T>
struct alignas(2 * sizeof(T)) cx {
    T re, im;
};

template <typename T>
__host__ __device__ __forceinline__ cx<T> mk(T r, T i) {
    cx<T> z;
    z.re = r;
    z.im = i;
    return z;
}
template <typename T>
__host__ __device__ __forceinline__ cx<T> operator+(cx<T> a, cx<T> b) { return mk(a.re + b.re, a.im + b.im); }
template <typename T>
__host__ __device__ __forceinline__ cx<T> operator-(cx<T> a, cx<T> b) { return mk(a.re - b.re, a.im - b.im); }
template <typename T>
__host__ __device__ __forceinline__ cx<T> operator*(cx<T> a, cx<T> b) {
    return mk(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
template <typename T>
__host__ __device__ __forceinline__ cx<T> operator*(T s, cx<T> a) { return mk(s * a.re, s * a.im); }
template <typename T>
__host__ __device__ __forceinline__ cx<T> conj(cx<T> a) { return mk(a.re, -a.im); }
template <typename T>
__host__ __device__ __forceinline__ T abs2(cx<T> a) { return a.re * a.re + a.im * a.im; }
// a * conj(b)
template <typename T>
__host__ __device__ __forceinline__ cx<T> mulc(cx<T> a, cx<T> b) {
    return mk(a.re * b.re + a.im * b.im, a.im * b.re - a.re * b.im);
}
// conj(a) * b
template <typename T>
__host__ __device__ __forceinline__ cx<T> cmul(cx<T> a, cx<T> b) {
    return mk(a.re * b.re + a.im * b.im, a.re * b.im - a.im * b.re);
}
// acc += a * b
template <typename T>
__host__ __device__ __forceinline__ void fma_cx(cx<T>& acc, cx<T> a, cx<T> b) {
    acc.re = fma(a.re, b.re, acc.re);
    acc.re = fma(-a.im, b.im, acc.re);
    acc.im = fma(a.re, b.im, acc.im);
    acc.im = fma(a.im, b.re, acc.im);
}
// acc -= a * conj(b)
template <typename T>
__host__ __device__ __forceinline__ void fms_mulc(cx<T>& acc, cx<T> a, cx<T> b) {
    acc.re = fma(-a.re, b.re, acc.re);
    acc.re = fma(-a.im, b.im, acc.re);
    acc.im = fma(-a.im, b.re, acc.im);
    acc.im = fma(a.re, b.im, acc.im);
}
// acc += conj(a) * b
template <typename T>
__host__ __device__ __forceinline__ void fma_cjx(cx<T>& acc, cx<T> a, cx<T> b) {
    acc.re = fma(a.re, b.re, acc.re);
    acc.re = fma(a.im, b.im, acc.re);
    acc.im = fma(a.re, b.im, acc.im);
    acc.im = fma(-a.im, b.re, acc.im);
}

typedef cx<double> zc;
typedef cx<float> cc;

// ---------------------------------------------------- float-pair arithmetic --
// Values hi + lo held as two floats (about 48 significant bits).  Error-free
// transformations: TwoSum (Knuth) and TwoProduct through FMA.  Used where the
// FP64 pipe would otherwise bound an elementwise kernel.
__device__ __forceinline__ float2 df_two_sum(float a, float b) {
    const float s = a + b;
    const float bb = s - a;
    return make_float2(s, (a - (s - bb)) + (b - bb));
}
__device__ __forceinline__ float2 df_add(float2 a, float2 b) {
    const float2 s = df_two_sum(a.x, b.x);
    return df_two_sum(s.x, s.y + (a.y + b.y));
}
__device__ __forceinline__ float2 df_neg(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 df_mul(float2 a, float2 b) {
    const float p = a.x * b.x;
    float e = fmaf(a.x, b.x, -p);
    e = fmaf(a.x, b.y, e);
    e = fmaf(a.y, b.x, e);
    return df_two_sum(p, e);
}
// a / b: quotient estimate, one correction step with the exact remainder
__device__ __forceinline__ float2 df_div(float2 a, float2 b) {
    const float q1 = a.x / b.x;
    const float2 r = df_add(a, df_neg(df_mul(make_float2(q1, 0.f), b)));
    const float q2 = (r.x + r.y) / b.x;
    return df_two_sum(q1, q2);
}
__device__ __forceinline__ float2 df_of(double x) {
    const float hi = (float)x;
    return make_float2(hi, (float)(x - (double)hi));
}
__device__ __forceinline__ double df_to_double(float2 a) { return (double)a.x + (double)a.y; }

// Line exponents of the exact-slice products: E with m < 2^E for a line's
// largest magnitude m (kLineZeroExp for an all-zero line).  E is monotone in m,
// so the exponent of a line's maximum is the maximum of its elements'
// exponents: kernels that write an operand fold them in with integer atomicMax
// in any order.  Magnitude of an element: max(|re|, |im|) (FP32 complex) or
// max(|re_hi| + |re_lo|, |im_hi| + |im_lo|) (float pair).
constexpr int kLineZeroExp = -100000;
__device__ __forceinline__ int line_exp_of(float m) { return (m > 0.f) ? ilogbf(m) + 1 : kLineZeroExp; }
__device__ __forceinline__ float f32_mag(float re, float im) { return fmaxf(fabsf(re), fabsf(im)); }
__device__ __forceinline__ float pair_mag(float4 v) {
    return fmaxf(fabsf(v.x) + fabsf(v.y), fabsf(v.z) + fabsf(v.w));
}

// Occupation (src/thermodynamics.rs:100-118): T = 0 step with 1/2 at E == mu,
// else the Fermi function with its +-50 clamp; width = k_B T.
__device__ __forceinline__ double occupation_f(double e, double mu, double width) {
    if (width == 0.0) return (e < mu) ? 1.0 : ((e > mu) ? 0.0 : 0.5);
    const double x = (e - mu) / width;
    if (x > 50.0) return 0.0;
    if (x < -50.0) return 1.0;
    return 1.0 / (1.0 + exp(x));
}
__device__ __forceinline__ void kahan_step(double& sum, double& c, double x) {
    const double y = x - c;
    const double t = sum + y;
    c = (t - sum) - y;
    sum = t;
}
// Double-double sum (hi, lo) + (bh, bl): two-sum of the leading parts, the
// trailing parts added to the error, renormalised.
__device__ __forceinline__ void dd_add(double& hi, double& lo, double bh, double bl) {
    const double s = hi + bh;
    const double v = s - hi;
    double e = (hi - (s - v)) + (bh - v);
    e += lo + bl;
    hi = s + e;
    lo = e - (hi - s);
}
// Block-wide sum of per-thread double-doubles (ph[t], pl[t]) in shared memory
// (blockDim.x a power of two, <= 1024) along a fixed binary tree, so the
// result does not depend on timing; thread 0 gets it in (ph[0], pl[0]).  A
// tree keeps the dependent FP64 chain at log2(threads) steps (FP64 latency is
// long on this part).  Ends with a barrier.
__device__ __forceinline__ void dd_block_sum(double* ph, double* pl) {
    __syncthreads();
    for (int h = blockDim.x >> 1; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h) {
            double a = ph[threadIdx.x], b = pl[threadIdx.x];
            dd_add(a, b, ph[threadIdx.x + h], pl[threadIdx.x + h]);
            ph[threadIdx.x] = a;
            pl[threadIdx.x] = b;
        }
        __syncthreads();
    }
}

// -------------------------------------------------------------- model data --
struct ModelDev {
    int dim = 0, spin = 0;
    int64_t norb = 0, nsta = 0, nR = 0;
    std::vector<int64_t> hamR;   // host copy (nR, dim)
    std::vector<double> orb;     // host (norb, dim)
    std::vector<double> lat;     // host (dim, dim)
    zc* ham = nullptr;           // device (nR, nsta, nsta)
    int* hamR_d = nullptr;       // device (nR, 3), zero padded
    double* Rcart_d = nullptr;   // device (nR, 3) Cartesian R = hamR . lat
    double* tau_d = nullptr;     // device (nsta, 3) fractional, spin-duplicated
    double* taucart_d = nullptr; // device (nsta, 3) Cartesian
    int64_t n_rmat = 0;
    zc* rmatrix = nullptr;       // device (n_rmat, dim, nsta, nsta)
    int device = 0;
    // digit planes of the hop table for the tensor-core Fourier sum (built lazily)
    void* hop_slices = nullptr;
    int* hop_EB = nullptr;         // per contraction column
    bool hop_packed = false;       // columns = upper-triangle elements (m <= n) only
    // tcgen05 form: the table is paired over +-R and contracted against real
    // coefficients (cos, sin): hop_K = 1 + hop_np complex contraction steps,
    // hop_pair_d (hop_np) = the index of each pair's R in hamR
    int hop_K = 0, hop_np = 0;
    int* hop_pair_d = nullptr;
    zc* pair_T = nullptr;          // the paired table (2 hop_K rows, nsta^2 columns)
    bool nonfinite = false;        // the table holds NaN or Inf (found when it is paired)
};

// ------------------------------------------------------------------ errors --
int set_error(int code, const std::string& msg);
int cuda_error(cudaError_t e, const char* where);
void count_launch(int n = 1);

// Scoped per-kernel timer: records CUDA events on `st` around the kernels
// launched in its scope when timing is enabled (tbg_kernel_timing_enable).
bool timing_enabled();
struct KTimer {
    cudaStream_t st;
    const char* name;
    double work;  // algorithmic flops of the launches in scope
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    KTimer(cudaStream_t s, const char* n, double work_flops = 0.0);
    ~KTimer();
};
void timing_flush();  // resolve recorded event pairs (after a stream sync)

#define TBG_CUDA(call)                                   \
    do {                                                 \
        cudaError_t _e = (call);                         \
        if (_e != cudaSuccess) return cuda_error(_e, #call); \
    } while (0)

#define TBG_LAUNCHED(where)                                         \
    do {                                                            \
        count_launch();                                             \
        cudaError_t _e = cudaGetLastError();                        \
        if (_e != cudaSuccess) return cuda_error(_e, where);        \
    } while (0)

// ---------------------------------------------------------- kernel drivers --
// Fourier sum, direct form: for nk k-points (device k, (nk, dim)), outputs
// H (nk, N, N) (may be null) and V (nk, nproj, N, N) (may be null when
// nproj == 0); dirs (nproj, dim) device (Cartesian weights).
int fourier_direct(const ModelDev& m, cudaStream_t st, int64_t nk, const double* k_d, int gauge,
                   int nproj, const double* dirs_d, zc* H, zc* V, int64_t ldH, int64_t ldV);

// Position-matrix commutator term added to V (HasRMatrix models).
int rmatrix_term(const ModelDev& m, cudaStream_t st, int64_t nk, const double* k_d, int gauge,
                 int nproj, const double* dirs_d, const zc* H, zc* V, zc* scratch);

// Separable transform on a uniform mesh: k-points with flat indices
// [k0, k0 + nk) of the mesh kmesh[dim].
int fourier_mesh(ModelDev& m, cudaStream_t st, const int64_t* kmesh, int64_t k0, int64_t nk,
                 int gauge, int nproj, const double* dirs_d, zc* H, zc* V, zc* scratch,
                 size_t scratch_bytes);
size_t fourier_mesh_scratch_bytes(const ModelDev& m, const int64_t* kmesh, int64_t nk_chunk);
bool fourier_mesh_supported(const ModelDev& m);

// Fourier sum for H and two projected velocities on the tensor cores
// (exact-slice BF16 contraction), Atom gauge, FP64 outputs H (nk, N, N) and
// V (nk, 2, N, N).  Falls back to fourier_direct when nR exceeds the exact
// contraction length.
// C (3 nk N^2 float pairs) is the contraction output buffer.
size_t fourier_mixed_scratch_bytes(const ModelDev& m, int64_t nk);
bool fourier_mixed_ok(const ModelDev& m);
int fourier_mixed(ModelDev& m, cudaStream_t st, int64_t nk, const double* k_d, const double* dirs_d, zc* H,
                  zc* V, float4* C, void* scratch, size_t scratch_bytes);
// Same contraction, left in C as float pairs in the lattice gauge with the
// orbital-position term added to V_0, V_1 (blocks [0,nk), [nk,2nk), [2nk,3nk)
// of N^2 elements).  Requires fourier_mixed_ok(m).  With `out` the three
// blocks go there instead, `blk` elements apart (k-points of several models
// stacked in one buffer); C is then only needed when the hop table is not
// packed (fourier_mixed_packed false).  With rexp (3 nk N ints) the row
// exponents of the three blocks (H, V_0, V_1; k-major, as the exact-slice
// products take them) are written there as a by-product when the table is
// packed; *rexp_filled says whether they were.
int fourier_mixed_pairs(ModelDev& m, cudaStream_t st, int64_t nk, const double* k_d, const double* dirs_d,
                        float4* C, void* scratch, size_t scratch_bytes, float4* out = nullptr, int64_t blk = 0,
                        int* rexp = nullptr, bool* rexp_filled = nullptr);
// Builds the model's hop table for the mixed contraction if needed; true when
// its columns are the packed upper triangle (the tcgen05 form).
int fourier_mixed_packed(ModelDev& m, cudaStream_t st, bool* packed);

// Batched Hermitian eigensolver: A (batch, N, N) FP64 input (destroyed),
// E (batch, N) ascending, U (batch, N, N) eigenvectors in columns (may be
// null).  precision: 0 = FP64, 1 = FP32 solve (U32 out, FP32 values) used by
// the mixed path.
size_t eig_workspace_bytes(int N, int64_t batch, int precision);
int eig_batched(cudaStream_t st, int N, int64_t batch, zc* A, double* E, zc* U, void* work,
                size_t work_bytes, int* status_d);

// Spin-current dressing J = 1/2 {S, V} (in place through scratch).
int spin_dress(cudaStream_t st, int N, int64_t norb, int64_t batch, int spin, zc* V, int64_t ldV,
               zc* scratch);

// Rotation into the eigenbasis + band-resolved Berry curvature:
// Omega (batch, N) from U (batch, N, N), Vx/Vy (batch strided), E; the
// quantum metric (batch, N) too when Met is not null.
int berry_rotate(cudaStream_t st, int N, int64_t batch, const zc* U, const zc* Vx, const zc* Vy,
                 int64_t ldV, const double* E, double eta, double* Omega, zc* scratch, double* Met = nullptr);

// Occupation-weighted sums: per k and per mu -> S (batch, nmu).
int occupation_sums(cudaStream_t st, int N, int64_t batch, const double* Omega, const double* E,
                    int nmu, const double* mu_d, double width, double* S);

// Deterministic compensated column sums of S (nk, nmu) -> out (nmu), added
// to a running (sum, compensation) pair held in acc (2*nmu).
int kahan_column_sums(cudaStream_t st, int64_t nk, int nmu, const double* S, double* acc);

// Fused one-thread-per-k path for nsta <= 8 (FP64): Omega, E and/or the
// occupation sums S (nk, nmu).  k from klist_d (nk, dim), or, when klist_d is
// null, the mesh points [k0, k0 + nk) of kmesh.
int small_fused(const ModelDev& m, cudaStream_t st, int64_t nk, const double* klist_d, int64_t k0,
                const int64_t* kmesh, const double* dirs_d, int spin, double eta, int nmu, const double* mu_d,
                double width, double* Om, double* E, double* S, double* Met = nullptr, double* SM = nullptr);
constexpr int kSmallMaxN = 8;
// The one-thread-per-k small-model kernel serves models of up to kSmallMaxN
// states whose hop table has at most small_max_nr() vectors (TBG_SMALL_MAX_NR
// overrides the default); larger tables go through the batched FP64 pipeline,
// whose Fourier sum spreads each k-point's R sum over many threads.
int small_max_nr();
inline bool use_small_fused(const ModelDev& m) {
    return m.nsta <= kSmallMaxN && m.n_rmat == 0 && m.nR <= small_max_nr();
}
// Eigenpairs of N <= kSmallMaxN matrices by per-thread Jacobi (E ascending,
// U columns; U may be null; non-finite input sets bit 0 of *status).
int eig_small(cudaStream_t st, int N, int64_t batch, const zc* H, double* E, zc* U, int* status);
// Eigenpairs of kSmallMaxN < N <= kJacobiMaxN matrices by warp-per-matrix
// cyclic Jacobi (FP64; same outputs as eig_small; H is not modified).
constexpr int kJacobiMaxN = 32;
int eig_jacobi(cudaStream_t st, int N, int64_t batch, const zc* H, double* E, zc* U, int* status);
// Largest N the FP64 driver gives to eig_jacobi (TBG_JACOBI_MAX_N overrides).
int jacobi_max_n();
// Largest model the mixed path takes (FP32 solver with the matrix in global
// memory above 215 bands; tcgen05 products in chunks of 256 along K).
constexpr int kMixedMaxN = 2048;
// Above this many bands the refinement's correction X F is a HIGH product.
constexpr int kHighCorrN = 256;
// tcgen05 form of the exact-slice products (default) or the mma.sync form.
bool ozaki_use_tc();
// Exact-slice complex GEMM on tcgen05 (ozaki_tc.cu): C = op(A) B as float
// pairs.  HIGH class (six BF16 digits per value, about 2^-43 of the product
// scale), or with `mid` the MID class (five digits, about 2^-35).
int ozaki_zgemm_tc(cudaStream_t st, bool conj_a, int fmt_a, int fmt_b, int64_t batch, int M, int Nc, int K,
                   const void* A, int64_t lda, int64_t sA, const void* B, int64_t ldb, int64_t sB, float4* C,
                   int64_t ldc, int64_t sC, int* EA, int* EB, int* err, bool exps_ready = false,
                   int* Ecol = nullptr, bool mid = false);

// Gaussian-smeared DOS: add the terms of count band energies ev (device) to
// the compensated per-bin totals acc (2 E_n: sum, compensation).  part holds
// slices * E_n doubles; slices from dos_slices(E_n, chunk energies).
// Energy-cut Hall integration (see ec.cu).
constexpr int kEcWindow = 8192;  // mu points per integration launch
void ec_track(int dim, const int64_t* kmesh, int N, const double* R, int* perm);
size_t ec_smem_max();
int ec_vertex_data(cudaStream_t st, int N, int64_t batch, const zc* V, int64_t ldV, const double* E, double eta,
                   zc* K, double* Om);
int ec_abs2(cudaStream_t st, int64_t n, const zc* C, double* R);
int ec_integrate(cudaStream_t st, int dim, const int64_t* kmesh, int N, const double* E, const zc* K, const double* Om,
                 const int* perm, int nmu, const double* mu_d, double eta, double* part, double* fpart, int nblocks,
                 int window, double* acc_out, double* full_out);

// Wilson loops from the eigenvectors at the loop points (see wilson.cu).
constexpr int kWilsonMaxOcc = 64;
size_t wilson_workspace_bytes(int N, int64_t n_loops, int n_k, int n_occ);
int wilson_from_vectors(cudaStream_t st, const ModelDev& m, int64_t n_loops, int n_k, const double* kv_d, const zc* U,
                        int n_occ, const int* occ_d, int svd, double* out, void* work, size_t work_bytes,
                        int* status_d);

int dos_slices(int64_t E_n, int64_t count);
int dos_accumulate(cudaStream_t st, int64_t count, const double* ev, int64_t E_n, double E_min, double step,
                   double sigma, double* part, int slices, double* acc);

// ------------------------------------------------------------- mixed path --
// FP32 solver: H (FP64) or, when Hpair is given, float pairs
// {re_hi, re_lo, im_hi, im_lo} (batch stride N*N); U32 eigenvectors in columns.
// With urow_exp / ucol_exp the solver may also write the row and column line
// exponents of U (when its last pass holds them: the TMEM-resident
// back-transformation); *exps_filled says whether it did.
int eig_batched_f32(cudaStream_t st, int N, int64_t batch, zc* H, double* E, cc* U, void* work,
                    size_t work_bytes, int* status_d, const float4* Hpair = nullptr, int* urow_exp = nullptr,
                    int* ucol_exp = nullptr, bool* exps_filled = nullptr);
// Householder reduction of up to 128-band matrices with the matrix resident
// in TMEM and tcgen05 rank-2 updates (eig_tc.cu): Vt (batch, packed + N)
// reflectors and tau, de (batch, 2 N) the tridiagonal d then e.  Used by
// eig_batched_f32 unless TBG_EIG_TC=0.
bool eig_tc_enabled();
bool hetrd_tc_fits(int N);
size_t hetrd_tc_de_bytes(int N, int64_t batch);
int hetrd_tc(cudaStream_t st, int N, int64_t batch, const float4* Hpair, const zc* H, cc* Vt, float* de,
             int* status_d, const cc* Hc = nullptr, int Nbig = 0, int off = 0);
// Back-transformation U <- Q U of the same solver with U (eigenvectors of the
// tridiagonal form, in columns) resident in TMEM and tcgen05 block updates.
// With urow_exp and ucol_exp (batch N ints each) the row and column line
// exponents of the FP32 result come out of the same pass.
int bt_tc(cudaStream_t st, int N, int64_t batch, const cc* Vt, cc* U, int* status_d, int* urow_exp = nullptr,
          int* ucol_exp = nullptr);
bool bt_tc_enabled();
// FP32 eigensolve, refinement and rotation on the tensor cores: H, Vx, Vy as
// float pairs (batch stride N*N) -> refined E (ascending) and Omega.
size_t mixed_berry_workspace_bytes(int N, int64_t batch);
// Occupation-weighted k-sum fused with Omega (hall path): per CTA, the
// compensated partial sums of sum_k sum_n Omega_n f(E_n, mu_j), part[(block
// nmu + j) 2 + {0: sum, 1: compensation}] for `blocks` CTAs.
struct OccSums {
    int nmu = 0;
    const double* mu = nullptr;  // device
    double width = 0.0;          // k_B T (0: step function)
    double* part = nullptr;      // device (blocks, nmu, 2)
    int blocks = 0;
};
int occ_sums_blocks(int64_t batch);
bool occ_fused_ok(int N, int nmu);  // the fused kernel's band and shared-memory limits
// acc[2 j] (sum) and acc[2 j + 1] (compensation) += the blocks' partials, in block order.
int occ_partials_add(cudaStream_t st, const OccSums& o, double* acc);
int mixed_berry(cudaStream_t st, int N, int64_t batch, const float4* H, const float4* Vx, const float4* Vy,
                double eta, double* E, double* Om, void* work, size_t work_bytes, int* status_d,
                int64_t* clusters_d, double* Met = nullptr, zc* Uout = nullptr, const OccSums* occ = nullptr,
                const int* h_rexp = nullptr, const int* v_rexp = nullptr);
// With occ (and Om, Met null) the Berry stage is the fused Omega + occupation +
// compensated k-sum kernel: per-band Omega is not stored and E is not sorted.
// With Uout, mixed_berry stops after the refinement: refined E ascending and the
// refined eigenvectors (columns, FP64) in Uout; Vx, Vy are not read.  With
// neither Om nor Uout it stops after the eigenvalue refinement (refined E
// ascending only).  h_rexp (batch N ints) and v_rexp (2 batch N: Vx then Vy),
// when given, are the row exponents of H and of the velocities as the Fourier
// stage wrote them (line_exp_of over each row), used instead of a scan.
// Spin-current dressing of float-pair velocities (V_0 blocks, batch stride ldV).
int spin_dress_pairs(cudaStream_t st, int N, int64_t norb, int64_t batch, int spin, float4* V, int64_t ldV,
                     float4* scratch);
// FP64 complex -> float pairs: out[b N2 + e] = in[b ld_in + e], b < nb, e < N2.
int z_to_pairs(cudaStream_t st, int64_t nb, int64_t N2, const zc* in, int64_t ld_in, float4* out);

}  // namespace tbg
