// C-ABI entry points of libtbgpu (include/tbgpu.h).
//
// Each call runs on its own CUDA stream, allocates its device workspace from
// the stream-ordered pool, processes the k-points in chunks sized to a device
// memory budget, and synchronises before returning.  Validation mirrors the
// reference's error behaviour (src/response/config.rs:183-303,
// src/response/traits.rs:60-150, src/response/linear/mod.rs:160-188).

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "tbgpu_internal.cuh"

struct tbg_model {
    tbg::ModelDev d;
};

namespace tbg {

static thread_local std::string g_err;
static thread_local int g_code = 0;
static thread_local int64_t g_launches = 0;

int set_error(int code, const std::string& msg) {
    g_code = code;
    g_err = msg;
    return code;
}

int cuda_error(cudaError_t e, const char* where) {
    const int code = (e == cudaErrorMemoryAllocation) ? TBG_E_OOM : TBG_E_CUDA;
    cudaGetLastError();  // clear a non-sticky error
    return set_error(code, std::string(where) + ": " + cudaGetErrorString(e));
}

void count_launch(int n) { g_launches += n; }

int zgemm_batched(cudaStream_t st, int N, int64_t batch, bool conj_a, const zc* A, int64_t sA, const zc* B,
                  int64_t sB, zc* C, int64_t sC);
int berry_from_bands(cudaStream_t st, int N, int64_t batch, const zc* Bx, const zc* By, int64_t ldB,
                     const double* E, double eta, double* Omega);

namespace {

std::once_flag g_pool_once;

void configure_pool() {
    std::call_once(g_pool_once, [] {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess) return;
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
            uint64_t thr = UINT64_MAX;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
        }
    });
}

// Per-call context: stream + stream-ordered allocations released at the end.
struct Ctx {
    cudaStream_t st = nullptr;
    std::vector<void*> bufs;
    int rc = TBG_OK;
    Ctx() {
        configure_pool();
        cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
        if (e != cudaSuccess) rc = cuda_error(e, "cudaStreamCreate");
    }
    template <typename T>
    T* alloc(size_t count) {
        if (rc != TBG_OK) return nullptr;
        void* p = nullptr;
        cudaError_t e = cudaMallocAsync(&p, std::max<size_t>(count, 1) * sizeof(T), st);
        if (e != cudaSuccess) {
            rc = cuda_error(e, "cudaMallocAsync");
            return nullptr;
        }
        bufs.push_back(p);
        return static_cast<T*>(p);
    }
    int sync(const char* where) {
        cudaError_t e = cudaStreamSynchronize(st);
        if (e != cudaSuccess && rc == TBG_OK) rc = cuda_error(e, where);
        timing_flush();
        return rc;
    }
    ~Ctx() {
        if (st) {
            for (void* p : bufs) cudaFreeAsync(p, st);
            cudaStreamSynchronize(st);
            timing_flush();
            cudaStreamDestroy(st);
        }
    }
};

// Device scratch one call sizes its k-point chunks to: a sixth of the free
// device memory, between 6 and 40 GB (so concurrent calls still leave memory
// free).  Larger chunks give each batched kernel more waves over which to
// amortise its last, partly idle one: 8192 k-points of 128 bands took
// 63.1 ms per step in 6 GB chunks, 60.7 in 12 GB and 59.9 in 24 GB (an
// earlier build); with the current kernels 48.3 ms in three chunks, 47.2 in
// two and 46.55 in one (33 GB).
int64_t chunk_budget_bytes() {
    const char* s = std::getenv("TBG_CHUNK_BYTES");
    if (s) {
        const long long v = std::atoll(s);
        if (v > 0) return v;
    }
    int64_t b = 6LL << 30;
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess)
        b = std::max<int64_t>(b, std::min<int64_t>(40LL << 30, (int64_t)(free_b / 6)));
    else
        cudaGetLastError();
    return b;
}

// k-points per chunk: as many as the memory budget allows, then balanced over
// the chunks the call needs and rounded to whole waves of the batched
// per-matrix kernels (two resident matrices per SM), so no chunk ends in a
// nearly empty wave.
int64_t choose_chunk(int64_t nk, int64_t per_k_bytes) {
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || nsm < 1) nsm = 1;
    const int64_t q = 2 * (int64_t)nsm;
    per_k_bytes = std::max<int64_t>(per_k_bytes, 1);
    int64_t budget = chunk_budget_bytes();
    if (!std::getenv("TBG_CHUNK_BYTES") && budget / per_k_bytes < std::min<int64_t>(nk, q)) {
        // large matrices: room for one full wave of the per-matrix kernels
        // (two per SM) when half of the free device memory allows it
        size_t free_b = 0, total_b = 0;
        if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess)
            budget = std::max<int64_t>(budget, std::min<int64_t>(per_k_bytes * std::min<int64_t>(nk, q),
                                                                 (int64_t)(free_b / 2)));
    }
    int64_t c = std::max<int64_t>(1, budget / per_k_bytes);
    c = std::min<int64_t>(c, 65535);
    const char* s = std::getenv("TBG_MAX_CHUNK");
    if (s && std::atoll(s) > 0) c = std::min<int64_t>(c, std::atoll(s));
    if (nk > c) {
        const int64_t n = (nk + c - 1) / c;
        const int64_t bal = (nk + n - 1) / n;
        const int64_t up = (bal + q - 1) / q * q;
        if (up <= c)
            c = up;
        else if (c >= q)
            c = c / q * q;
    }
    return std::max<int64_t>(1, std::min(c, nk));
}

__global__ void kmesh_kernel(int64_t k0, int64_t nk, int dim, int64_t n0, int64_t n1, int64_t n2,
                             double* __restrict__ k) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nk; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t idx = k0 + t;
        // gen_kmesh (src/kpoints.rs:49-87): first dimension outermost
        if (dim == 1) {
            k[t] = (double)idx / (double)n0;
        } else if (dim == 2) {
            k[2 * t] = (double)(idx / n1) / (double)n0;
            k[2 * t + 1] = (double)(idx % n1) / (double)n1;
        } else {
            k[3 * t] = (double)(idx / (n1 * n2)) / (double)n0;
            k[3 * t + 1] = (double)((idx / n2) % n1) / (double)n1;
            k[3 * t + 2] = (double)(idx % n2) / (double)n2;
        }
    }
}

__global__ void transpose_kernel(int N, int64_t batch, const zc* __restrict__ U, zc* __restrict__ Ut) {
    const int64_t NN = (int64_t)N * N;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < batch * NN;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t b = idx / NN;
        const int e = (int)(idx % NN), r = e / N, c = e % N;
        Ut[b * NN + (int64_t)c * N + r] = U[idx];
    }
}

inline unsigned blocks_for(int64_t total) {
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>((total + 255) / 256, 152LL * 64));
}

bool all_finite(const double* p, size_t n) {
    for (size_t i = 0; i < n; ++i)
        if (!std::isfinite(p[i])) return false;
    return true;
}

int check_model(const tbg_model* m) {
    if (!m || !m->d.ham) return set_error(TBG_E_INVALID_ARGUMENT, "null or destroyed model handle");
    if (cudaSetDevice(m->d.device) != cudaSuccess) return set_error(TBG_E_CUDA, "cudaSetDevice failed");
    return TBG_OK;
}

// validate_direction_matrix (config.rs:202-233) for n rows of length dim
int check_dirs(const double* dirs, int64_t rows, int dim, int64_t expect_rows) {
    if (!dirs) return set_error(TBG_E_INVALID_ARGUMENT, "null direction matrix");
    if (expect_rows >= 0 && rows != expect_rows)
        return set_error(TBG_E_DIMENSION_MISMATCH, "direction: expected " + std::to_string(expect_rows) +
                                                       ", found " + std::to_string(rows));
    for (int64_t r = 0; r < rows; ++r) {
        bool nz = false;
        for (int d = 0; d < dim; ++d) {
            const double v = dirs[r * dim + d];
            if (!std::isfinite(v))
                return set_error(TBG_E_INVALID_RESPONSE_PARAMETER, "direction: all components must be finite");
            nz |= (v != 0.0);
        }
        if (!nz)
            return set_error(TBG_E_INVALID_RESPONSE_PARAMETER,
                             "direction: each direction row must not be the zero vector");
    }
    return TBG_OK;
}

int check_k(const double* k, int64_t nk, int dim) {
    if (nk < 0) return set_error(TBG_E_INVALID_ARGUMENT, "negative number of k-points");
    if (nk > 0 && !k) return set_error(TBG_E_INVALID_ARGUMENT, "null k-point array");
    (void)dim;
    return TBG_OK;
}

int check_eta(double eta) {
    if (!std::isfinite(eta) || eta < 0.0)
        return set_error(TBG_E_INVALID_RESPONSE_PARAMETER, "broadening: must be finite and non-negative");
    return TBG_OK;
}

int check_spin(const tbg_model* m, int spin) {
    if (spin < -1 || spin > 2) return set_error(TBG_E_INVALID_ARGUMENT, "spin must be -1 (None), 0, 1 or 2");
    if (spin >= 0 && !m->d.spin)
        return set_error(TBG_E_SPIN_NOT_ALLOWED, "Spin direction is invalid for a model without spin.");
    return TBG_OK;
}

int check_status(int* status_d, cudaStream_t st) {
    int h = 0;
    cudaError_t e = cudaMemcpyAsync(&h, status_d, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_error(e, "status readback");
    // a time-out first: the kernels after it read what the aborted one left
    if (h & 2) return set_error(TBG_E_TIMEOUT, "a bounded device wait ran out in a tensor-core kernel");
    if (h & 1) return set_error(TBG_E_NOCONV, "eigensolver input contains NaN or Inf");
    if (h & 4)
        return set_error(TBG_E_NOCONV,
                         "Wilson loop: an overlap matrix is singular (the occupied bands touch others on the loop)");
    return TBG_OK;
}

double lattice_det(const std::vector<double>& lat, int dim) {
    if (dim == 1) return lat[0];
    if (dim == 2) return lat[0] * lat[3] - lat[1] * lat[2];
    return lat[0] * (lat[4] * lat[8] - lat[5] * lat[7]) - lat[1] * (lat[3] * lat[8] - lat[5] * lat[6]) +
           lat[2] * (lat[3] * lat[7] - lat[4] * lat[6]);
}

// Models of more than kMixedMaxN bands (or of more than 256 with the mma.sync
// products) run the FP64 path (reported in tbg_report).
int effective_precision(const ModelDev& M, int precision) {
    // the tcgen05 products run longer contractions in exact chunks of 256; the
    // mma.sync form (selectable for comparison) stops at 256.  Models of at
    // most kSmallMaxN states run FP64 (the small-model kernel, or the batched
    // FP64 pipeline, which at these sizes is faster than 128-row tensor tiles).
    if (precision == TBG_PREC_MIXED &&
        (M.nsta > kMixedMaxN || (M.nsta > 256 && !ozaki_use_tc()) || M.nsta <= kSmallMaxN))
        return TBG_PREC_FP64;
    return precision;
}

}  // namespace

int small_max_nr() {
    static const int v = [] {
        const char* s = std::getenv("TBG_SMALL_MAX_NR");
        return s ? std::max(0, std::atoi(s)) : 32;
    }();
    return v;
}

namespace {

// Shared per-chunk response pipeline: (k on device) -> Omega, E.
struct BerryJob {
    ModelDev* m;
    int spin;
    double eta;
    int precision;
    const double* dirs_d;  // (2, dim)
    int64_t chunk;
    // buffers
    double* k_d;
    zc *H, *V, *U, *scratch, *Hcopy;
    double *E, *Om;
    int* status_d;
    void* work;
    size_t work_bytes;
    void* fwork;
    size_t fwork_bytes;
    cc* U32;
    float4* pairs;  // mixed: H, V_0, V_1 as float pairs (3 chunk N^2)
    bool want_metric;
    double* Met;  // quantum metric (chunk, N) when want_metric
    const OccSums* occ = nullptr;  // mixed hall path: fused Omega + occupation k-sum
    int* rexp = nullptr;           // mixed: row exponents of H, V_0, V_1 (3 chunk N) from the Fourier stage
    bool rexp_ok = false;          // ... written for the current chunk
};

int alloc_berry(Ctx& ctx, BerryJob& J) {
    const int N = (int)J.m->nsta;
    const int64_t NN = (int64_t)N * N, c = J.chunk;
    J.k_d = ctx.alloc<double>(c * J.m->dim);
    J.H = ctx.alloc<zc>(c * NN);
    J.V = ctx.alloc<zc>(2 * c * NN);
    J.U = ctx.alloc<zc>(c * NN);
    J.scratch = ctx.alloc<zc>(c * NN);
    J.E = ctx.alloc<double>(c * N);
    J.Om = ctx.alloc<double>(c * N);
    J.Met = J.want_metric ? ctx.alloc<double>(c * N) : nullptr;
    J.status_d = ctx.alloc<int>(1);
    J.Hcopy = nullptr;
    J.U32 = nullptr;
    J.work = nullptr;
    J.work_bytes = 0;
    J.fwork = nullptr;
    J.fwork_bytes = 0;
    J.pairs = nullptr;
    if (J.precision == TBG_PREC_MIXED) {
        J.work_bytes = mixed_berry_workspace_bytes(N, c);
        J.work = J.work_bytes ? ctx.alloc<unsigned char>(J.work_bytes) : nullptr;
        J.fwork_bytes = fourier_mixed_scratch_bytes(*J.m, c);
        J.fwork = ctx.alloc<unsigned char>(J.fwork_bytes);
        J.pairs = ctx.alloc<float4>(3 * c * NN);
        J.rexp = ctx.alloc<int>(3 * c * N);
    }
    if (ctx.rc == TBG_OK) {
        cudaError_t e = cudaMemsetAsync(J.status_d, 0, sizeof(int), ctx.st);
        if (e != cudaSuccess) ctx.rc = cuda_error(e, "memset status");
    }
    return ctx.rc;
}

int berry_tail(Ctx& ctx, BerryJob& J, int64_t nkc, int64_t* clusters_d);

int run_berry_chunk(Ctx& ctx, BerryJob& J, int64_t nkc, int64_t* clusters_d) {
    ModelDev& m = *J.m;
    const int N = (int)m.nsta;
    const int64_t NN = (int64_t)N * N;
    int rc;
    if (J.precision == TBG_PREC_MIXED) {
        // H, V_0, V_1 as float pairs: from the tensor-core contraction in the
        // lattice gauge, or (position-matrix models, nR beyond the exact
        // contraction length) Atom-gauge FP64 converted to pairs
        float4* P = J.pairs;
        J.rexp_ok = false;
        if (m.n_rmat == 0 && fourier_mixed_ok(m)) {
            rc = fourier_mixed_pairs(m, ctx.st, nkc, J.k_d, J.dirs_d, P, J.fwork, J.fwork_bytes, nullptr, 0, J.rexp,
                                     &J.rexp_ok);
            if (rc) return rc;
        } else {
            rc = fourier_mixed(m, ctx.st, nkc, J.k_d, J.dirs_d, J.H, J.V, P, J.fwork, J.fwork_bytes);
            if (rc) return rc;
            if (m.n_rmat > 0) {
                rc = rmatrix_term(m, ctx.st, nkc, J.k_d, TBG_GAUGE_ATOM, 2, J.dirs_d, J.H, J.V, J.scratch);
                if (rc) return rc;
            }
            // V is (nkc, 2, N, N); the pairs hold the components as separate blocks
            if ((rc = z_to_pairs(ctx.st, nkc, NN, J.H, NN, P))) return rc;
            if ((rc = z_to_pairs(ctx.st, nkc, NN, J.V, 2 * NN, P + nkc * NN))) return rc;
            if ((rc = z_to_pairs(ctx.st, nkc, NN, J.V + NN, 2 * NN, P + 2 * nkc * NN))) return rc;
        }
        return berry_tail(ctx, J, nkc, clusters_d);
    }
    rc = fourier_direct(m, ctx.st, nkc, J.k_d, TBG_GAUGE_ATOM, 2, J.dirs_d, J.H, J.V, NN, 2 * NN);
    if (rc) return rc;
    if (m.n_rmat > 0) {
        rc = rmatrix_term(m, ctx.st, nkc, J.k_d, TBG_GAUGE_ATOM, 2, J.dirs_d, J.H, J.V, J.scratch);
        if (rc) return rc;
    }
    return berry_tail(ctx, J, nkc, clusters_d);
}

// The part of a chunk after H and the velocities are formed (J.pairs for the
// mixed path, J.H / J.V for FP64): spin dressing, eigensolve, rotation, Omega.
// It depends on the model only through N and norb.
int berry_tail(Ctx& ctx, BerryJob& J, int64_t nkc, int64_t* clusters_d) {
    ModelDev& m = *J.m;
    const int N = (int)m.nsta;
    const int64_t NN = (int64_t)N * N;
    int rc;
    if (J.precision == TBG_PREC_MIXED) {
        float4* P = J.pairs;
        if (J.spin >= 0) {
            rc = spin_dress_pairs(ctx.st, N, m.norb, nkc, J.spin, P + nkc * NN, NN,
                                  reinterpret_cast<float4*>(J.scratch));
            if (rc) return rc;
        }
        // row exponents from the Fourier stage (the velocities' only when no
        // spin dressing has changed them since)
        const int* hr = J.rexp_ok ? J.rexp : nullptr;
        const int* vr = (J.rexp_ok && J.spin < 0) ? J.rexp + nkc * N : nullptr;
        J.rexp_ok = false;
        if (J.occ)
            return mixed_berry(ctx.st, N, nkc, P, P + nkc * NN, P + 2 * nkc * NN, J.eta, J.E, nullptr, J.work,
                               J.work_bytes, J.status_d, clusters_d, nullptr, nullptr, J.occ, hr, vr);
        return mixed_berry(ctx.st, N, nkc, P, P + nkc * NN, P + 2 * nkc * NN, J.eta, J.E, J.Om, J.work, J.work_bytes,
                           J.status_d, clusters_d, J.Met, nullptr, nullptr, hr, vr);
    }
    if (J.spin >= 0) {
        rc = spin_dress(ctx.st, N, m.norb, nkc, J.spin, J.V, 2 * NN, J.scratch);
        if (rc) return rc;
    }
    rc = eig_batched(ctx.st, N, nkc, J.H, J.E, J.U, nullptr, 0, J.status_d);
    if (rc) return rc;
    return berry_rotate(ctx.st, N, nkc, J.U, J.V, J.V + NN, 2 * NN, J.E, J.eta, J.Om, J.scratch, J.Met);
}

// FP64 band energies (ascending) on chunks of the uniform mesh, gen_kmesh
// order: the energies-only fused kernel for nsta <= 8, else the Fourier sum in
// the Atom gauge and the batched eigensolve (values only) -- the path of
// solve_band_all_parallel(gen_kmesh(..)) (src/solve_ham.rs:52-62, 94-107).
struct MeshEnergies {
    const ModelDev* M = nullptr;
    const int64_t* kmesh = nullptr;
    bool small = false;
    int64_t chunk = 0;
    double* k_d = nullptr;
    zc* H = nullptr;
    double* E = nullptr;  // (chunk, nsta)
    double* dirs_d = nullptr;
    int* status_d = nullptr;

    int init(Ctx& ctx, const ModelDev& m, const int64_t* km, int64_t nk, int64_t extra_per_k = 0) {
        M = &m;
        kmesh = km;
        const int N = (int)m.nsta;
        const int64_t NN = (int64_t)N * N;
        small = use_small_fused(m);
        // the fused small-model kernel has no batch limit: one chunk of up to 2^21 k-points
        chunk = small ? std::max<int64_t>(1, std::min<int64_t>({nk, int64_t(1) << 21,
                                                                chunk_budget_bytes() / (16 * N + 64 + extra_per_k)}))
                      : choose_chunk(nk, sizeof(zc) * NN + 16 * N + 64 + extra_per_k);
        k_d = small ? nullptr : ctx.alloc<double>(chunk * m.dim);
        H = small ? nullptr : ctx.alloc<zc>(chunk * NN);
        E = ctx.alloc<double>(chunk * N);
        dirs_d = small ? ctx.alloc<double>(2 * m.dim) : nullptr;
        status_d = ctx.alloc<int>(1);
        if (ctx.rc) return ctx.rc;
        TBG_CUDA(cudaMemsetAsync(status_d, 0, sizeof(int), ctx.st));
        if (dirs_d) TBG_CUDA(cudaMemsetAsync(dirs_d, 0, sizeof(double) * 2 * m.dim, ctx.st));
        return TBG_OK;
    }

    int run(Ctx& ctx, int64_t c0, int64_t nkc) {
        const int N = (int)M->nsta;
        const int64_t NN = (int64_t)N * N;
        if (small)  // energies-only form: no velocities or eigenvectors
            return small_fused(*M, ctx.st, nkc, nullptr, c0, kmesh, dirs_d, -1, 0.0, 0, nullptr, 0.0, nullptr, E,
                               nullptr);
        const int64_t n0 = kmesh[0], n1 = M->dim > 1 ? kmesh[1] : 1, n2 = M->dim > 2 ? kmesh[2] : 1;
        kmesh_kernel<<<blocks_for(nkc), 256, 0, ctx.st>>>(c0, nkc, M->dim, n0, n1, n2, k_d);
        TBG_LAUNCHED("kmesh_kernel");
        int rc = fourier_direct(*M, ctx.st, nkc, k_d, TBG_GAUGE_ATOM, 0, nullptr, H, nullptr, NN, 0);
        if (rc) return rc;
        return eig_batched(ctx.st, N, nkc, H, E, nullptr, nullptr, 0, status_d);
    }
};

int check_kmesh(const ModelDev& M, const int64_t* kmesh, int64_t* nk_out) {
    if (!kmesh) return set_error(TBG_E_INVALID_ARGUMENT, "null k-mesh");
    int64_t nk = 1;
    for (int d = 0; d < M.dim; ++d) {
        if (kmesh[d] <= 0) return set_error(TBG_E_INVALID_KMESH, "Invalid k-point mesh dimensions");
        nk *= kmesh[d];
    }
    *nk_out = nk;
    return TBG_OK;
}

}  // namespace
}  // namespace tbg

using namespace tbg;

extern "C" {

const char* tbg_version(void) { return "tbgpu 0.1.0 sm_103a"; }

int64_t tbg_kernel_launch_count(int reset) {
    const int64_t v = g_launches;
    if (reset) g_launches = 0;
    return v;
}

int tbg_last_error(char* buf, size_t len) {
    if (buf && len) {
        std::strncpy(buf, g_err.c_str(), len - 1);
        buf[len - 1] = '\0';
    }
    return g_code;
}

int tbg_model_create(int dim, int spin, int64_t norb, int64_t nR, const int64_t* hamR, const double* ham,
                     const double* orb, const double* lat, tbg_model** out) {
    if (!out) return set_error(TBG_E_INVALID_ARGUMENT, "null output handle");
    *out = nullptr;
    if (dim < 1 || dim > 3) return set_error(TBG_E_INVALID_DIMENSION, "dim must be 1, 2 or 3");
    if (norb < 1) return set_error(TBG_E_INVALID_MODEL, "model has no orbitals");
    if (nR < 1) return set_error(TBG_E_INVALID_MODEL, "hamR must hold at least the R = 0 block");
    if (!hamR || !ham || !orb || !lat) return set_error(TBG_E_INVALID_ARGUMENT, "null model array");
    const int64_t nsta = spin ? 2 * norb : norb;
    if (nsta > 4096) return set_error(TBG_E_UNSUPPORTED, "nsta > 4096 is not supported");
    if (!all_finite(lat, (size_t)dim * dim) || !all_finite(orb, (size_t)norb * dim))
        return set_error(TBG_E_INVALID_MODEL, "finite_geometry: lattice and orbital positions must be finite");
    // every R needs its Hermitian partner -R (model_build.rs:430-440)
    for (int64_t r = 0; r < nR; ++r) {
        bool found = false;
        for (int64_t q = 0; q < nR && !found; ++q) {
            bool eq = true;
            for (int d = 0; d < dim; ++d) eq &= (hamR[q * dim + d] == -hamR[r * dim + d]);
            found = eq;
        }
        if (!found)
            return set_error(TBG_E_INVALID_MODEL,
                             "Hopping for vector R exists, but its Hermitian conjugate for -R does not");
        for (int d = 0; d < dim; ++d)
            if (std::llabs(hamR[r * dim + d]) > (1LL << 30))
                return set_error(TBG_E_INVALID_MODEL, "R component out of range");
    }
    tbg_model* m = new tbg_model();
    ModelDev& M = m->d;
    cudaGetDevice(&M.device);
    M.dim = dim;
    M.spin = spin ? 1 : 0;
    M.norb = norb;
    M.nsta = nsta;
    M.nR = nR;
    M.hamR.assign(hamR, hamR + nR * dim);
    M.orb.assign(orb, orb + norb * dim);
    M.lat.assign(lat, lat + dim * dim);
    std::vector<int> hr(nR * 3, 0);
    std::vector<double> rc(nR * 3, 0.0), tau(nsta * 3, 0.0), tc(nsta * 3, 0.0);
    for (int64_t r = 0; r < nR; ++r) {
        for (int d = 0; d < dim; ++d) hr[r * 3 + d] = (int)hamR[r * dim + d];
        for (int c = 0; c < dim; ++c) {
            double s = 0.0;  // R_cart = hamR . lat (velocity.rs:530-531)
            for (int d = 0; d < dim; ++d) s += (double)hamR[r * dim + d] * lat[d * dim + c];
            rc[r * 3 + c] = s;
        }
    }
    for (int64_t s = 0; s < nsta; ++s) {
        const int64_t o = s % norb;  // spinful basis duplicates tau (velocity.rs:546-550)
        for (int d = 0; d < dim; ++d) tau[s * 3 + d] = orb[o * dim + d];
        for (int c = 0; c < dim; ++c) {
            double v = 0.0;
            for (int d = 0; d < dim; ++d) v += orb[o * dim + d] * lat[d * dim + c];
            tc[s * 3 + c] = v;
        }
    }
    const size_t hb = sizeof(zc) * (size_t)nR * nsta * nsta;
    cudaError_t e = cudaMalloc(&M.ham, hb);
    if (e == cudaSuccess) e = cudaMemcpy(M.ham, ham, hb, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMalloc(&M.hamR_d, sizeof(int) * hr.size());
    if (e == cudaSuccess) e = cudaMemcpy(M.hamR_d, hr.data(), sizeof(int) * hr.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMalloc(&M.Rcart_d, sizeof(double) * rc.size());
    if (e == cudaSuccess) e = cudaMemcpy(M.Rcart_d, rc.data(), sizeof(double) * rc.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMalloc(&M.tau_d, sizeof(double) * tau.size());
    if (e == cudaSuccess) e = cudaMemcpy(M.tau_d, tau.data(), sizeof(double) * tau.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMalloc(&M.taucart_d, sizeof(double) * tc.size());
    if (e == cudaSuccess) e = cudaMemcpy(M.taucart_d, tc.data(), sizeof(double) * tc.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        const int code = cuda_error(e, "tbg_model_create upload");
        tbg_model_destroy(m);
        return code;
    }
    *out = m;
    return TBG_OK;
}

int tbg_model_set_rmatrix(tbg_model* m, int64_t n_rmat, const double* rmatrix) {
    int rc = check_model(m);
    if (rc) return rc;
    if (n_rmat < 0 || n_rmat > m->d.nR) return set_error(TBG_E_INVALID_MODEL, "n_rmat must be in [0, nR]");
    if (n_rmat > 0 && !rmatrix) return set_error(TBG_E_INVALID_ARGUMENT, "null rmatrix");
    if (m->d.rmatrix) {
        cudaFree(m->d.rmatrix);
        m->d.rmatrix = nullptr;
    }
    m->d.n_rmat = 0;
    if (n_rmat == 0) return TBG_OK;
    const size_t bytes = sizeof(zc) * (size_t)n_rmat * m->d.dim * m->d.nsta * m->d.nsta;
    cudaError_t e = cudaMalloc(&m->d.rmatrix, bytes);
    if (e == cudaSuccess) e = cudaMemcpy(m->d.rmatrix, rmatrix, bytes, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_error(e, "tbg_model_set_rmatrix");
    m->d.n_rmat = n_rmat;
    return TBG_OK;
}

int tbg_model_destroy(tbg_model* m) {
    if (!m) return TBG_OK;
    ModelDev& M = m->d;
    cudaSetDevice(M.device);
    cudaFree(M.ham);
    cudaFree(M.hamR_d);
    cudaFree(M.Rcart_d);
    cudaFree(M.tau_d);
    cudaFree(M.taucart_d);
    cudaFree(M.rmatrix);
    cudaFree(M.hop_slices);
    cudaFree(M.hop_EB);
    cudaFree(M.hop_pair_d);
    cudaFree(M.pair_T);
    M.ham = nullptr;
    delete m;
    return TBG_OK;
}

int tbg_model_info(const tbg_model* m, int* dim, int* spin, int64_t* norb, int64_t* nsta, int64_t* nR) {
    if (!m) return set_error(TBG_E_INVALID_ARGUMENT, "null model handle");
    if (dim) *dim = m->d.dim;
    if (spin) *spin = m->d.spin;
    if (norb) *norb = m->d.norb;
    if (nsta) *nsta = m->d.nsta;
    if (nR) *nR = m->d.nR;
    return TBG_OK;
}

int tbg_gen_v_projected(const tbg_model* m, int64_t nk, const double* k, int gauge, int64_t n_proj,
                        const double* dirs, double* V_out, double* H_out) {
    int rc = check_model(m);
    if (rc) return rc;
    const ModelDev& M = m->d;
    if ((rc = check_k(k, nk, M.dim))) return rc;
    if (gauge != TBG_GAUGE_ATOM && gauge != TBG_GAUGE_LATTICE) return set_error(TBG_E_INVALID_ARGUMENT, "bad gauge");
    if (n_proj < 0 || (n_proj > 0 && (!dirs || !V_out))) return set_error(TBG_E_INVALID_ARGUMENT, "bad projections");
    if (nk == 0) return TBG_OK;
    const int N = (int)M.nsta;
    const int64_t NN = (int64_t)N * N;
    Ctx ctx;
    const int64_t chunk = choose_chunk(nk, sizeof(zc) * NN * (2 + n_proj) + 64);
    double* k_d = ctx.alloc<double>(chunk * M.dim);
    zc* H = ctx.alloc<zc>(chunk * NN);
    zc* V = n_proj ? ctx.alloc<zc>(chunk * n_proj * NN) : nullptr;
    double* dirs_d = n_proj ? ctx.alloc<double>(n_proj * M.dim) : nullptr;
    if (ctx.rc) return ctx.rc;
    if (n_proj) TBG_CUDA(cudaMemcpyAsync(dirs_d, dirs, sizeof(double) * n_proj * M.dim, cudaMemcpyHostToDevice, ctx.st));
    for (int64_t c0 = 0; c0 < nk; c0 += chunk) {
        const int64_t nkc = std::min(chunk, nk - c0);
        TBG_CUDA(cudaMemcpyAsync(k_d, k + c0 * M.dim, sizeof(double) * nkc * M.dim, cudaMemcpyHostToDevice, ctx.st));
        rc = fourier_direct(M, ctx.st, nkc, k_d, gauge, (int)n_proj, dirs_d, H, V, NN, n_proj * NN);
        if (rc) return rc;
        if (M.n_rmat > 0 && n_proj > 0) {
            rc = rmatrix_term(M, ctx.st, nkc, k_d, gauge, (int)n_proj, dirs_d, H, V, nullptr);
            if (rc) return rc;
        }
        if (H_out)
            TBG_CUDA(cudaMemcpyAsync(H_out + c0 * NN * 2, H, sizeof(zc) * nkc * NN, cudaMemcpyDeviceToHost, ctx.st));
        if (n_proj)
            TBG_CUDA(cudaMemcpyAsync(V_out + c0 * n_proj * NN * 2, V, sizeof(zc) * nkc * n_proj * NN,
                                     cudaMemcpyDeviceToHost, ctx.st));
        if (ctx.sync("tbg_gen_v_projected")) return ctx.rc;
    }
    return ctx.sync("tbg_gen_v_projected");
}

int tbg_gen_ham(const tbg_model* m, int64_t nk, const double* k, int gauge, double* H_out) {
    if (!H_out && nk > 0) return set_error(TBG_E_INVALID_ARGUMENT, "null output");
    return tbg_gen_v_projected(m, nk, k, gauge, 0, nullptr, nullptr, H_out);
}

int tbg_gen_v(const tbg_model* m, int64_t nk, const double* k, int gauge, double* V_out, double* H_out) {
    int rc = check_model(m);
    if (rc) return rc;
    const int dim = m->d.dim;
    std::vector<double> eye(dim * dim, 0.0);
    for (int d = 0; d < dim; ++d) eye[d * dim + d] = 1.0;
    return tbg_gen_v_projected(m, nk, k, gauge, dim, eye.data(), V_out, H_out);
}

static int solve_impl(const tbg_model* m, int64_t nk, const double* k, double* E_out, double* U_out, int rows) {
    int rc = check_model(m);
    if (rc) return rc;
    const ModelDev& M = m->d;
    if ((rc = check_k(k, nk, M.dim))) return rc;
    if (nk > 0 && !E_out) return set_error(TBG_E_INVALID_ARGUMENT, "null output");
    if (nk == 0) return TBG_OK;
    const int N = (int)M.nsta;
    const int64_t NN = (int64_t)N * N;
    Ctx ctx;
    const int64_t chunk = choose_chunk(nk, sizeof(zc) * NN * (U_out ? 3 : 1) + 64);
    double* k_d = ctx.alloc<double>(chunk * M.dim);
    zc* H = ctx.alloc<zc>(chunk * NN);
    zc* U = U_out ? ctx.alloc<zc>(chunk * NN) : nullptr;
    zc* Ut = (U_out && rows) ? ctx.alloc<zc>(chunk * NN) : nullptr;
    double* E = ctx.alloc<double>(chunk * N);
    int* status_d = ctx.alloc<int>(1);
    if (ctx.rc) return ctx.rc;
    TBG_CUDA(cudaMemsetAsync(status_d, 0, sizeof(int), ctx.st));
    for (int64_t c0 = 0; c0 < nk; c0 += chunk) {
        const int64_t nkc = std::min(chunk, nk - c0);
        TBG_CUDA(cudaMemcpyAsync(k_d, k + c0 * M.dim, sizeof(double) * nkc * M.dim, cudaMemcpyHostToDevice, ctx.st));
        rc = fourier_direct(M, ctx.st, nkc, k_d, TBG_GAUGE_ATOM, 0, nullptr, H, nullptr, NN, 0);
        if (rc) return rc;
        rc = eig_batched(ctx.st, N, nkc, H, E, U, nullptr, 0, status_d);
        if (rc) return rc;
        TBG_CUDA(cudaMemcpyAsync(E_out + c0 * N, E, sizeof(double) * nkc * N, cudaMemcpyDeviceToHost, ctx.st));
        if (U_out) {
            const zc* src = U;
            if (rows) {
                transpose_kernel<<<blocks_for(nkc * NN), 256, 0, ctx.st>>>(N, nkc, U, Ut);
                TBG_LAUNCHED("transpose_kernel");
                src = Ut;
            }
            TBG_CUDA(cudaMemcpyAsync(U_out + c0 * NN * 2, src, sizeof(zc) * nkc * NN, cudaMemcpyDeviceToHost, ctx.st));
        }
        if (ctx.sync("tbg_solve")) return ctx.rc;
    }
    if ((rc = check_status(status_d, ctx.st))) return rc;
    return ctx.sync("tbg_solve");
}

int tbg_solve_band(const tbg_model* m, int64_t nk, const double* k, double* E_out) {
    return solve_impl(m, nk, k, E_out, nullptr, 0);
}

// Band energies in mixed precision: H as float pairs (tensor-core Fourier sum,
// or the FP64 sum converted when the contraction does not apply), FP32
// eigensolve, FP64-class refinement of the eigenvalues; no eigenvectors out.
static int solve_band_mixed(const tbg_model* m, int64_t nk, const double* k, double* E_out) {
    const ModelDev& M = m->d;
    const int N = (int)M.nsta;
    const int64_t NN = (int64_t)N * N;
    Ctx ctx;
    const int64_t chunk = choose_chunk(nk, sizeof(zc) * NN * 15 + 64 * N + 48 * (int64_t)M.nR);
    const bool tcf = M.n_rmat == 0 && fourier_mixed_ok(M);
    double* k_d = ctx.alloc<double>(chunk * M.dim);
    double* dirs_d = ctx.alloc<double>(2 * M.dim);
    double* E = ctx.alloc<double>(chunk * N);
    int* status_d = ctx.alloc<int>(1);
    int64_t* clusters_d = ctx.alloc<int64_t>(1);
    float4* P = ctx.alloc<float4>((tcf ? 3 : 1) * chunk * NN);
    const size_t fwb = tcf ? fourier_mixed_scratch_bytes(M, chunk) : 0;
    void* fwork = tcf ? static_cast<void*>(ctx.alloc<unsigned char>(fwb)) : nullptr;
    zc* H = tcf ? nullptr : ctx.alloc<zc>(chunk * NN);
    const size_t wb = mixed_berry_workspace_bytes(N, chunk);
    void* work = ctx.alloc<unsigned char>(wb);
    if (ctx.rc) return ctx.rc;
    // velocity directions of the contraction (its V blocks are not used here)
    std::vector<double> dirs(2 * M.dim, 0.0);
    dirs[0] = 1.0;
    dirs[M.dim + (M.dim > 1 ? 1 : 0)] = 1.0;
    TBG_CUDA(cudaMemcpyAsync(dirs_d, dirs.data(), sizeof(double) * 2 * M.dim, cudaMemcpyHostToDevice, ctx.st));
    TBG_CUDA(cudaMemsetAsync(status_d, 0, sizeof(int), ctx.st));
    TBG_CUDA(cudaMemsetAsync(clusters_d, 0, sizeof(int64_t), ctx.st));
    int rc;
    for (int64_t c0 = 0; c0 < nk; c0 += chunk) {
        const int64_t nkc = std::min(chunk, nk - c0);
        TBG_CUDA(cudaMemcpyAsync(k_d, k + c0 * M.dim, sizeof(double) * nkc * M.dim, cudaMemcpyHostToDevice, ctx.st));
        if (tcf) {
            rc = fourier_mixed_pairs(const_cast<ModelDev&>(M), ctx.st, nkc, k_d, dirs_d, P, fwork, fwb);
        } else {
            rc = fourier_direct(M, ctx.st, nkc, k_d, TBG_GAUGE_ATOM, 0, nullptr, H, nullptr, NN, 0);
            if (!rc) rc = z_to_pairs(ctx.st, nkc, NN, H, NN, P);
        }
        if (rc) return rc;
        if ((rc = mixed_berry(ctx.st, N, nkc, P, nullptr, nullptr, 0.0, E, nullptr, work, wb, status_d, clusters_d)))
            return rc;
        TBG_CUDA(cudaMemcpyAsync(E_out + c0 * N, E, sizeof(double) * nkc * N, cudaMemcpyDeviceToHost, ctx.st));
    }
    if (ctx.sync("tbg_solve_band_prec")) return ctx.rc;
    if ((rc = check_status(status_d, ctx.st))) return rc;
    return ctx.sync("tbg_solve_band_prec");
}

int tbg_solve_band_prec(const tbg_model* m, int64_t nk, const double* k, int precision, double* E_out) {
    if (precision != TBG_PREC_FP64 && precision != TBG_PREC_MIXED)
        return set_error(TBG_E_INVALID_ARGUMENT, "precision must be 0 (FP64) or 1 (mixed)");
    int rc = check_model(m);
    if (rc) return rc;
    const ModelDev& M = m->d;
    if (effective_precision(M, precision) != TBG_PREC_MIXED || M.nsta <= kSmallMaxN)
        return solve_impl(m, nk, k, E_out, nullptr, 0);
    if ((rc = check_k(k, nk, M.dim))) return rc;
    if (nk > 0 && !E_out) return set_error(TBG_E_INVALID_ARGUMENT, "null output");
    if (nk == 0) return TBG_OK;
    return solve_band_mixed(m, nk, k, E_out);
}

int tbg_solve(const tbg_model* m, int64_t nk, const double* k, double* E_out, double* U_out, int evec_rows) {
    if (!U_out && nk > 0) return set_error(TBG_E_INVALID_ARGUMENT, "null eigenvector output");
    return solve_impl(m, nk, k, E_out, U_out, evec_rows);
}

static int berry_common(const tbg_model* m, int64_t nk, const double* k, const double* dirs2, int spin, double eta,
                        int precision, double* Omega_out, double* E_out, int nmu, const double* mu, double T,
                        double* occ_out, double* Met_out = nullptr) {
    int rc = check_model(m);
    if (rc) return rc;
    const ModelDev& M = m->d;
    if ((rc = check_k(k, nk, M.dim))) return rc;
    if ((rc = check_dirs(dirs2, 2, M.dim, 2))) return rc;
    if ((rc = check_eta(eta))) return rc;
    if ((rc = check_spin(m, spin))) return rc;
    if (precision != TBG_PREC_FP64 && precision != TBG_PREC_MIXED)
        return set_error(TBG_E_INVALID_ARGUMENT, "precision must be 0 (FP64) or 1 (mixed)");
    if (nk == 0) return TBG_OK;
    precision = effective_precision(M, precision);
    const int N = (int)M.nsta;
    const int64_t NN = (int64_t)N * N;
    Ctx ctx;
    BerryJob J;
    J.m = const_cast<ModelDev*>(&M);
    J.spin = spin;
    J.eta = eta;
    J.precision = precision;
    J.want_metric = Met_out != nullptr;
    J.chunk = choose_chunk(nk, sizeof(zc) * NN * (precision == TBG_PREC_MIXED ? 15 : 5) + 64 * N +
                                   (precision == TBG_PREC_MIXED ? 48 * (int64_t)M.nR : 0));
    double* dirs_d = ctx.alloc<double>(2 * M.dim);
    J.dirs_d = dirs_d;
    double* mu_d = (nmu > 0) ? ctx.alloc<double>(nmu) : nullptr;
    double* S = (nmu > 0) ? ctx.alloc<double>(J.chunk * nmu) : nullptr;
    if (ctx.rc) return ctx.rc;
    if ((rc = alloc_berry(ctx, J))) return rc;
    TBG_CUDA(cudaMemcpyAsync(dirs_d, dirs2, sizeof(double) * 2 * M.dim, cudaMemcpyHostToDevice, ctx.st));
    if (nmu > 0) TBG_CUDA(cudaMemcpyAsync(mu_d, mu, sizeof(double) * nmu, cudaMemcpyHostToDevice, ctx.st));
    const double width = (T <= 0.0) ? 0.0 : T * 8.617333262145e-5;
    const bool small = use_small_fused(M);
    for (int64_t c0 = 0; c0 < nk; c0 += J.chunk) {
        const int64_t nkc = std::min(J.chunk, nk - c0);
        TBG_CUDA(cudaMemcpyAsync(J.k_d, k + c0 * M.dim, sizeof(double) * nkc * M.dim, cudaMemcpyHostToDevice, ctx.st));
        if (small) {
            if ((rc = small_fused(M, ctx.st, nkc, J.k_d, 0, nullptr, dirs_d, spin, eta, occ_out ? nmu : 0, mu_d, width,
                                  J.Om, J.E, occ_out ? S : nullptr, J.Met)))
                return rc;
            if (Met_out)
                TBG_CUDA(cudaMemcpyAsync(Met_out + c0 * N, J.Met, sizeof(double) * nkc * N, cudaMemcpyDeviceToHost,
                                         ctx.st));
            if (Omega_out)
                TBG_CUDA(cudaMemcpyAsync(Omega_out + c0 * N, J.Om, sizeof(double) * nkc * N, cudaMemcpyDeviceToHost,
                                         ctx.st));
            if (E_out)
                TBG_CUDA(cudaMemcpyAsync(E_out + c0 * N, J.E, sizeof(double) * nkc * N, cudaMemcpyDeviceToHost, ctx.st));
            if (occ_out)
                TBG_CUDA(cudaMemcpyAsync(occ_out + c0, S, sizeof(double) * nkc, cudaMemcpyDeviceToHost, ctx.st));
            if (ctx.sync("berry")) return ctx.rc;
            continue;
        }
        if ((rc = run_berry_chunk(ctx, J, nkc, nullptr))) return rc;
        if (Met_out)
            TBG_CUDA(cudaMemcpyAsync(Met_out + c0 * N, J.Met, sizeof(double) * nkc * N, cudaMemcpyDeviceToHost, ctx.st));
        if (Omega_out)
            TBG_CUDA(cudaMemcpyAsync(Omega_out + c0 * N, J.Om, sizeof(double) * nkc * N, cudaMemcpyDeviceToHost, ctx.st));
        if (E_out)
            TBG_CUDA(cudaMemcpyAsync(E_out + c0 * N, J.E, sizeof(double) * nkc * N, cudaMemcpyDeviceToHost, ctx.st));
        if (occ_out) {
            if ((rc = occupation_sums(ctx.st, N, nkc, J.Om, J.E, nmu, mu_d, width, S))) return rc;
            TBG_CUDA(cudaMemcpyAsync(occ_out + c0, S, sizeof(double) * nkc, cudaMemcpyDeviceToHost, ctx.st));
        }
        if (ctx.sync("berry")) return ctx.rc;
    }
    if ((rc = check_status(J.status_d, ctx.st))) return rc;
    return ctx.sync("berry");
}

int tbg_berry_curvature(const tbg_model* m, int64_t nk, const double* k, const double* dirs2, int spin, double eta,
                        int precision, double* Omega_out, double* E_out) {
    return berry_common(m, nk, k, dirs2, spin, eta, precision, Omega_out, E_out, 0, nullptr, 0.0, nullptr);
}

int tbg_occupied_berry_curvature(const tbg_model* m, int64_t nk, const double* k, const double* dirs2, int spin,
                                 double eta, double T, double mu, int precision, double* out) {
    if (!std::isfinite(mu))
        return set_error(TBG_E_INVALID_RESPONSE_PARAMETER, "chemical_potentials: all values must be finite");
    if (!std::isfinite(T) || T < 0.0)
        return set_error(TBG_E_INVALID_RESPONSE_PARAMETER, "T: all values must be finite and non-negative");
    if (!out && nk > 0) return set_error(TBG_E_INVALID_ARGUMENT, "null output");
    return berry_common(m, nk, k, dirs2, spin, eta, precision, nullptr, nullptr, 1, &mu, T, out);
}

int tbg_berry_curvature_multi(int64_t n_models, const tbg_model* const* models, const int64_t* nk, const double* k,
                              const double* dirs2, int spin, double eta, int precision, double* Omega_out,
                              double* E_out) {
    if (n_models < 0) return set_error(TBG_E_INVALID_ARGUMENT, "tbg_berry_curvature_multi: negative model count");
    if (n_models == 0) return TBG_OK;
    if (!models || !nk) return set_error(TBG_E_INVALID_ARGUMENT, "tbg_berry_curvature_multi: null models or k counts");
    int rc;
    for (int64_t i = 0; i < n_models; ++i)
        if ((rc = check_model(models[i]))) return rc;
    const ModelDev& M0 = models[0]->d;
    const int N = (int)M0.nsta, dim = M0.dim;
    int64_t total = 0;
    for (int64_t i = 0; i < n_models; ++i) {
        const ModelDev& Mi = models[i]->d;
        if (Mi.nsta != M0.nsta || Mi.dim != M0.dim)
            return set_error(TBG_E_INVALID_ARGUMENT,
                             "tbg_berry_curvature_multi: the models must have the same number of states and dimension");
        if (nk[i] < 0) return set_error(TBG_E_INVALID_ARGUMENT, "tbg_berry_curvature_multi: negative k count");
        total += nk[i];
    }
    if ((rc = check_k(k, total, dim))) return rc;
    if ((rc = check_dirs(dirs2, 2, dim, 2))) return rc;
    if ((rc = check_eta(eta))) return rc;
    for (int64_t i = 0; i < n_models; ++i)
        if ((rc = check_spin(models[i], spin))) return rc;
    if (precision != TBG_PREC_FP64 && precision != TBG_PREC_MIXED)
        return set_error(TBG_E_INVALID_ARGUMENT, "precision must be 0 (FP64) or 1 (mixed)");
    if (total == 0) return TBG_OK;
    const int prec = effective_precision(M0, precision);  // depends on the number of states only
    const int64_t NN = (int64_t)N * N;
    std::vector<int64_t> off(n_models + 1, 0);
    for (int64_t i = 0; i < n_models; ++i) off[i + 1] = off[i] + nk[i];
    // Models outside the stacked form (the one-thread-per-k small-model kernel,
    // position matrices, tables beyond the exact contraction, another device
    // than the first model's) run alone.
    std::vector<int64_t> sidx;
    int64_t stotal = 0, max_nR = 0;
    for (int64_t i = 0; i < n_models; ++i) {
        const ModelDev& Mi = models[i]->d;
        const bool stack = !use_small_fused(Mi) && Mi.n_rmat == 0 && Mi.device == M0.device &&
                           (prec == TBG_PREC_FP64 || fourier_mixed_ok(Mi));
        if (!stack) {
            if (nk[i] > 0 && (rc = berry_common(models[i], nk[i], k + off[i] * dim, dirs2, spin, eta, precision,
                                                Omega_out ? Omega_out + off[i] * N : nullptr,
                                                E_out ? E_out + off[i] * N : nullptr, 0, nullptr, 0.0, nullptr)))
                return rc;
            continue;
        }
        if (nk[i] == 0) continue;
        sidx.push_back(i);
        stotal += nk[i];
        max_nR = std::max<int64_t>(max_nR, Mi.nR);
    }
    if (stotal == 0) return TBG_OK;
    if (cudaSetDevice(M0.device) != cudaSuccess) return set_error(TBG_E_CUDA, "cudaSetDevice failed");
    // buffers sized for the stacked model with the largest table (the Fourier scratch grows with nR)
    int64_t rep = sidx[0];
    for (int64_t i : sidx)
        if (models[i]->d.nR > models[rep]->d.nR) rep = i;
    Ctx ctx;
    BerryJob J;
    J.m = const_cast<ModelDev*>(&models[rep]->d);
    J.spin = spin;
    J.eta = eta;
    J.precision = prec;
    J.want_metric = false;
    J.chunk = choose_chunk(stotal, sizeof(zc) * NN * (prec == TBG_PREC_MIXED ? 15 : 5) + 64 * N +
                                       (prec == TBG_PREC_MIXED ? 48 * max_nR : 0));
    double* dirs_d = ctx.alloc<double>(2 * dim);
    J.dirs_d = dirs_d;
    if (ctx.rc) return ctx.rc;
    if ((rc = alloc_berry(ctx, J))) return rc;
    // models whose hop table is not packed (the mma.sync form) contract into a
    // buffer of their own and are copied into the stacked one
    bool unpacked = false;
    if (prec == TBG_PREC_MIXED)
        for (int64_t i : sidx) {
            bool packed = true;
            if ((rc = fourier_mixed_packed(const_cast<ModelDev&>(models[i]->d), ctx.st, &packed))) return rc;
            unpacked = unpacked || !packed;
        }
    float4* Ptmp = unpacked ? ctx.alloc<float4>(3 * J.chunk * NN) : nullptr;
    if (ctx.rc) return ctx.rc;
    TBG_CUDA(cudaMemcpyAsync(dirs_d, dirs2, sizeof(double) * 2 * dim, cudaMemcpyHostToDevice, ctx.st));
    struct Seg {
        int64_t model, pos, n, at;  // k-points [pos, pos + n) of the model at chunk position at
    };
    size_t si = 0;
    int64_t spos = 0;
    for (int64_t done = 0; done < stotal;) {
        const int64_t nkc = std::min(J.chunk, stotal - done);
        std::vector<Seg> segs;
        for (int64_t filled = 0; filled < nkc;) {
            const int64_t i = sidx[si];
            const int64_t n = std::min(nk[i] - spos, nkc - filled);
            segs.push_back({i, spos, n, filled});
            filled += n;
            spos += n;
            if (spos == nk[i]) {
                ++si;
                spos = 0;
            }
        }
        // each segment's H and velocities from its own model, into the chunk's stacked buffers
        for (const Seg& g : segs) {
            double* kd = J.k_d + g.at * dim;
            TBG_CUDA(cudaMemcpyAsync(kd, k + (off[g.model] + g.pos) * dim, sizeof(double) * g.n * dim,
                                     cudaMemcpyHostToDevice, ctx.st));
            ModelDev& Mi = const_cast<ModelDev&>(models[g.model]->d);
            rc = (prec == TBG_PREC_MIXED)
                     ? fourier_mixed_pairs(Mi, ctx.st, g.n, kd, dirs_d, Ptmp, J.fwork, J.fwork_bytes,
                                           J.pairs + g.at * NN, nkc * NN)
                     : fourier_direct(Mi, ctx.st, g.n, kd, TBG_GAUGE_ATOM, 2, dirs_d, J.H + g.at * NN,
                                      J.V + g.at * 2 * NN, NN, 2 * NN);
            if (rc) return rc;
        }
        // the rest once for the whole chunk
        if ((rc = berry_tail(ctx, J, nkc, nullptr))) return rc;
        for (const Seg& g : segs) {
            const int64_t o = (off[g.model] + g.pos) * N;
            if (Omega_out)
                TBG_CUDA(cudaMemcpyAsync(Omega_out + o, J.Om + g.at * N, sizeof(double) * g.n * N,
                                         cudaMemcpyDeviceToHost, ctx.st));
            if (E_out)
                TBG_CUDA(cudaMemcpyAsync(E_out + o, J.E + g.at * N, sizeof(double) * g.n * N, cudaMemcpyDeviceToHost,
                                         ctx.st));
        }
        if (ctx.sync("berry multi")) return ctx.rc;
        done += nkc;
    }
    if ((rc = check_status(J.status_d, ctx.st))) return rc;
    return ctx.sync("berry multi");
}

static int hall_impl(const tbg_model* m, const int64_t* kmesh, int64_t k_begin, int64_t k_count, bool whole,
                     const double* dirs2, int64_t nmu, const double* mu, double T, double eta, int spin,
                     int precision, double* out, tbg_report* report, double* metric_out = nullptr) {
    int rc = check_model(m);
    if (rc) return rc;
    const ModelDev& M = m->d;
    // validate_rank2 (config.rs:141-147) order: k-mesh, direction, mu, eta, T
    if (!kmesh) return set_error(TBG_E_INVALID_ARGUMENT, "null k-mesh");
    int64_t nk = 1;
    for (int d = 0; d < M.dim; ++d) {
        if (kmesh[d] <= 0) return set_error(TBG_E_INVALID_KMESH, "Invalid k-point mesh dimensions");
        nk *= kmesh[d];
    }
    if (whole) {
        k_begin = 0;
        k_count = nk;
    } else if (k_begin < 0 || k_count < 0 || k_begin + k_count > nk) {
        return set_error(TBG_E_INVALID_ARGUMENT, "k-range outside the mesh");
    }
    if ((rc = check_dirs(dirs2, 2, M.dim, 2))) return rc;
    if (nmu < 1 || !mu)
        return set_error(TBG_E_INVALID_RESPONSE_PARAMETER, "chemical_potentials: must contain at least one value");
    for (int64_t j = 0; j < nmu; ++j)
        if (!std::isfinite(mu[j]))
            return set_error(TBG_E_INVALID_RESPONSE_PARAMETER, "chemical_potentials: all values must be finite");
    if ((rc = check_eta(eta))) return rc;
    if (!std::isfinite(T) || T < 0.0)
        return set_error(TBG_E_INVALID_RESPONSE_PARAMETER, "T: all values must be finite and non-negative");
    if ((rc = check_spin(m, spin))) return rc;
    if (precision != TBG_PREC_FP64 && precision != TBG_PREC_MIXED)
        return set_error(TBG_E_INVALID_ARGUMENT, "precision must be 0 (FP64) or 1 (mixed)");
    if (!out) return set_error(TBG_E_INVALID_ARGUMENT, "null output");
    const bool met = metric_out != nullptr;
    precision = effective_precision(M, precision);
    const double det = lattice_det(M.lat, M.dim);
    if (whole && (det == 0.0 || !std::isfinite(det)))
        return set_error(TBG_E_LINALG, "Linear algebra operation failed: singular lattice");
    const int N = (int)M.nsta;
    const int64_t NN = (int64_t)N * N;
    const int64_t launches0 = g_launches;
    Ctx ctx;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaEventCreate(&ev0);
    cudaEventCreate(&ev1);
    cudaEventRecord(ev0, ctx.st);
    BerryJob J;
    J.m = const_cast<ModelDev*>(&M);
    J.spin = spin;
    J.eta = eta;
    J.precision = precision;
    J.want_metric = met;
    J.chunk = choose_chunk(std::max<int64_t>(k_count, 1),
                           sizeof(zc) * NN * (precision == TBG_PREC_MIXED ? 15 : 5) + 64 * N + 16 * nmu +
                               (precision == TBG_PREC_MIXED ? 48 * (int64_t)M.nR : 0));
    double* dirs_d = ctx.alloc<double>(2 * M.dim);
    J.dirs_d = dirs_d;
    double* mu_d = ctx.alloc<double>(nmu);
    double* S = ctx.alloc<double>(J.chunk * nmu);
    double* acc = ctx.alloc<double>(2 * nmu);
    // metric: occupation sums and running compensated totals
    double* SG = met ? ctx.alloc<double>(J.chunk * nmu) : nullptr;
    double* accg = met ? ctx.alloc<double>(2 * nmu) : nullptr;
    int64_t* clusters_d = ctx.alloc<int64_t>(1);
    if (ctx.rc) return ctx.rc;
    if ((rc = alloc_berry(ctx, J))) return rc;
    TBG_CUDA(cudaMemcpyAsync(dirs_d, dirs2, sizeof(double) * 2 * M.dim, cudaMemcpyHostToDevice, ctx.st));
    TBG_CUDA(cudaMemcpyAsync(mu_d, mu, sizeof(double) * nmu, cudaMemcpyHostToDevice, ctx.st));
    TBG_CUDA(cudaMemsetAsync(acc, 0, sizeof(double) * 2 * nmu, ctx.st));
    if (met) TBG_CUDA(cudaMemsetAsync(accg, 0, sizeof(double) * 2 * nmu, ctx.st));
    TBG_CUDA(cudaMemsetAsync(clusters_d, 0, sizeof(int64_t), ctx.st));
    const double width = (T <= 0.0) ? 0.0 : T * 8.617333262145e-5;
    const int64_t n0 = kmesh[0], n1 = M.dim > 1 ? kmesh[1] : 1, n2 = M.dim > 2 ? kmesh[2] : 1;
    const bool small = use_small_fused(M);
    // mixed path without the metric: Omega, occupation and the compensated
    // k-sum in one kernel (per-CTA partials, added up in block order)
    OccSums occ;
    const bool fused = !small && !met && precision == TBG_PREC_MIXED && nmu <= (1 << 20) && occ_fused_ok(N, (int)nmu);
    if (fused) {
        occ.nmu = (int)nmu;
        occ.mu = mu_d;
        occ.width = width;
        occ.blocks = occ_sums_blocks(J.chunk);
        occ.part = ctx.alloc<double>((int64_t)occ.blocks * nmu * 2);
        if (ctx.rc) return ctx.rc;
        J.occ = &occ;
    }
    for (int64_t c0 = 0; c0 < k_count; c0 += J.chunk) {
        const int64_t nkc = std::min(J.chunk, k_count - c0);
        if (small) {
            if ((rc = small_fused(M, ctx.st, nkc, nullptr, k_begin + c0, kmesh, dirs_d, spin, eta, (int)nmu, mu_d,
                                  width, nullptr, nullptr, S, nullptr, SG)))
                return rc;
        } else {
            kmesh_kernel<<<blocks_for(nkc), 256, 0, ctx.st>>>(k_begin + c0, nkc, M.dim, n0, n1, n2, J.k_d);
            TBG_LAUNCHED("kmesh_kernel");
            if (fused) occ.blocks = occ_sums_blocks(nkc);
            if ((rc = run_berry_chunk(ctx, J, nkc, clusters_d))) return rc;
            if (fused) {
                if ((rc = occ_partials_add(ctx.st, occ, acc))) return rc;
                continue;
            }
            if ((rc = occupation_sums(ctx.st, N, nkc, J.Om, J.E, (int)nmu, mu_d, width, S))) return rc;
            if (met && (rc = occupation_sums(ctx.st, N, nkc, J.Met, J.E, (int)nmu, mu_d, width, SG))) return rc;
        }
        if ((rc = kahan_column_sums(ctx.st, nkc, (int)nmu, S, acc))) return rc;
        if (met && (rc = kahan_column_sums(ctx.st, nkc, (int)nmu, SG, accg))) return rc;
    }
    std::vector<double> acc_h(2 * nmu), accg_h(met ? 2 * nmu : 0);
    int64_t clusters_h = 0;
    TBG_CUDA(cudaMemcpyAsync(acc_h.data(), acc, sizeof(double) * 2 * nmu, cudaMemcpyDeviceToHost, ctx.st));
    if (met)
        TBG_CUDA(cudaMemcpyAsync(accg_h.data(), accg, sizeof(double) * 2 * nmu, cudaMemcpyDeviceToHost, ctx.st));
    TBG_CUDA(cudaMemcpyAsync(&clusters_h, clusters_d, sizeof(int64_t), cudaMemcpyDeviceToHost, ctx.st));
    cudaEventRecord(ev1, ctx.st);
    if (ctx.sync("tbg_hall_conductivity")) return ctx.rc;
    if ((rc = check_status(J.status_d, ctx.st))) return rc;
    for (int64_t j = 0; j < nmu; ++j) {
        const double s = acc_h[2 * j] - acc_h[2 * j + 1];
        out[j] = whole ? s / (double)nk / det : s;
        if (met) {
            const double g = accg_h[2 * j] - accg_h[2 * j + 1];
            metric_out[j] = whole ? g / (double)nk / det : g;
        }
    }
    if (report) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ev0, ev1);
        report->nk = k_count;
        report->nsta = N;
        report->precision = precision;
        report->fourier_mode = small ? 2 : (precision == TBG_PREC_MIXED ? 1 : 0);
        report->kernel_launches = g_launches - launches0;
        report->device_ms = ms;
        report->eig_ms = 0.0;
        report->refine_clusters = clusters_h;
    }
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);
    return TBG_OK;
}

int64_t tbg_chunk_budget_bytes(void) { return tbg::chunk_budget_bytes(); }

int tbg_hall_conductivity(const tbg_model* m, const int64_t* kmesh, const double* dirs2, int64_t nmu,
                          const double* mu, double T, double eta, int spin, int precision, double* sigma_out,
                          tbg_report* report) {
    return hall_impl(m, kmesh, 0, 0, true, dirs2, nmu, mu, T, eta, spin, precision, sigma_out, report);
}

int tbg_hall_sums_range(const tbg_model* m, const int64_t* kmesh, int64_t k_begin, int64_t k_count,
                        const double* dirs2, int64_t nmu, const double* mu, double T, double eta, int spin,
                        int precision, double* sums_out, tbg_report* report) {
    return hall_impl(m, kmesh, k_begin, k_count, false, dirs2, nmu, mu, T, eta, spin, precision, sums_out,
                     report);
}

int tbg_dos(const tbg_model* m, const int64_t* kmesh, double E_min, double E_max, int64_t E_n, double sigma,
            double* E_out, double* dos_out) {
    int rc = check_model(m);
    if (rc) return rc;
    const ModelDev& M = m->d;
    // model_physics.rs:187-205 order: energy range, bin count, width; then gen_kmesh
    if (E_min >= E_max)
    {
        char msg[96];
        std::snprintf(msg, sizeof(msg), "Invalid energy range: min=%.17g, max=%.17g", E_min, E_max);
        return set_error(TBG_E_INVALID_ENERGY_RANGE, msg);
    }
    if (E_n <= 0)
        return set_error(TBG_E_INVALID_DOS_PARAMETER, "E_n: number of energy bins must be at least 1");
    if (!std::isfinite(sigma) || sigma <= 0.0)
        return set_error(TBG_E_INVALID_DOS_PARAMETER, "sigma: Gaussian smearing width must be finite and positive");
    int64_t nk = 0;
    if ((rc = check_kmesh(M, kmesh, &nk))) return rc;
    if (E_n > (int64_t(1) << 30)) return set_error(TBG_E_UNSUPPORTED, "E_n > 2^30 is not supported");
    if (!dos_out) return set_error(TBG_E_INVALID_ARGUMENT, "null output");
    // ndarray linspace: E_i = E_min + i step, step = (E_max - E_min) / (E_n - 1)
    const double step = E_n > 1 ? (E_max - E_min) / (double)(E_n - 1) : 0.0;
    if (E_out)
        for (int64_t i = 0; i < E_n; ++i) E_out[i] = E_min + step * (double)i;
    const int N = (int)M.nsta;
    Ctx ctx;
    MeshEnergies me;
    if ((rc = me.init(ctx, M, kmesh, nk))) return rc;
    const int slices = dos_slices(E_n, me.chunk * N);
    double* part = ctx.alloc<double>((int64_t)slices * E_n);
    double* acc = ctx.alloc<double>(2 * E_n);
    if (ctx.rc) return ctx.rc;
    TBG_CUDA(cudaMemsetAsync(acc, 0, sizeof(double) * 2 * E_n, ctx.st));
    for (int64_t c0 = 0; c0 < nk; c0 += me.chunk) {
        const int64_t nkc = std::min(me.chunk, nk - c0);
        if ((rc = me.run(ctx, c0, nkc))) return rc;
        if ((rc = dos_accumulate(ctx.st, nkc * N, me.E, E_n, E_min, step, sigma, part, slices, acc))) return rc;
    }
    std::vector<double> acc_h(2 * E_n);
    TBG_CUDA(cudaMemcpyAsync(acc_h.data(), acc, sizeof(double) * 2 * E_n, cudaMemcpyDeviceToHost, ctx.st));
    if (ctx.sync("tbg_dos")) return ctx.rc;
    if ((rc = check_status(me.status_d, ctx.st))) return rc;
    for (int64_t i = 0; i < E_n; ++i) dos_out[i] = (acc_h[2 * i] - acc_h[2 * i + 1]) / (double)nk;
    return TBG_OK;
}

int tbg_bands_mesh(const tbg_model* m, const int64_t* kmesh, double* E_out) {
    int rc = check_model(m);
    if (rc) return rc;
    const ModelDev& M = m->d;
    int64_t nk = 0;
    if ((rc = check_kmesh(M, kmesh, &nk))) return rc;
    if (!E_out) return set_error(TBG_E_INVALID_ARGUMENT, "null output");
    const int N = (int)M.nsta;
    Ctx ctx;
    MeshEnergies me;
    if ((rc = me.init(ctx, M, kmesh, nk))) return rc;
    for (int64_t c0 = 0; c0 < nk; c0 += me.chunk) {
        const int64_t nkc = std::min(me.chunk, nk - c0);
        if ((rc = me.run(ctx, c0, nkc))) return rc;
        TBG_CUDA(cudaMemcpyAsync(E_out + c0 * N, me.E, sizeof(double) * nkc * N, cudaMemcpyDeviceToHost, ctx.st));
        if (ctx.sync("tbg_bands_mesh")) return ctx.rc;
    }
    if ((rc = check_status(me.status_d, ctx.st))) return rc;
    return ctx.sync("tbg_bands_mesh");
}

int tbg_wilson_loops(const tbg_model* m, int64_t n_loops, int64_t n_k, const double* kvec, int64_t n_occ,
                     const int64_t* occ, int mode, int precision, double* out) {
    int rc = check_model(m);
    if (rc) return rc;
    const ModelDev& M = m->d;
    if (mode != 0 && mode != 1) return set_error(TBG_E_INVALID_ARGUMENT, "mode must be 0 (berry_loop) or 1 (det)");
    if (precision != TBG_PREC_FP64 && precision != TBG_PREC_MIXED)
        return set_error(TBG_E_INVALID_ARGUMENT, "precision must be 0 (FP64) or 1 (mixed)");
    if (n_loops < 0 || n_k < 1 || n_occ < 0) return set_error(TBG_E_INVALID_ARGUMENT, "negative size or empty loop");
    if (n_loops == 0) return TBG_OK;
    if (!kvec || !out || (n_occ > 0 && !occ)) return set_error(TBG_E_INVALID_ARGUMENT, "null argument");
    const int N = (int)M.nsta, dim = M.dim;
    // geometry.rs:160-170: the loop must close modulo an integer vector (else the reference panics)
    for (int64_t l = 0; l < n_loops; ++l)
        for (int d = 0; d < dim; ++d) {
            const double diff = kvec[(l * n_k + n_k - 1) * dim + d] - kvec[(l * n_k) * dim + d];
            if (!(std::fabs(diff - std::round(diff)) <= 1e-9))
                return set_error(TBG_E_INVALID_ARGUMENT,
                                 "wrong, the end of this loop must differ from the beginning by an integer grid vector");
        }
    for (int64_t i = 0; i < n_occ; ++i)
        if (occ[i] < 0 || occ[i] >= N) return set_error(TBG_E_INVALID_ARGUMENT, "occupied band index out of bounds");
    if (n_occ > kWilsonMaxOcc) return set_error(TBG_E_UNSUPPORTED, "Wilson loops support at most 64 occupied bands");
    const int svd = mode == 0;
    // mixed: FP32 eigenpairs refined on the tensor cores (9 .. 2048 bands), else FP64
    const bool mixed = effective_precision(M, precision) == TBG_PREC_MIXED && N > kSmallMaxN;
    if (n_occ == 0) {  // empty product: det 1 (phase 0); no eigenphases
        if (!svd)
            for (int64_t l = 0; l < n_loops; ++l) out[l] = 0.0;
        return TBG_OK;
    }
    const int T = (int)(n_k - 1);
    const int64_t NN = (int64_t)N * N;
    // loops per chunk: eigenpairs at T points per loop plus the loop workspace
    const int64_t per_loop =
        (int64_t)std::max(T, 1) * (sizeof(zc) * NN * 2 + 8 * N + 8 * dim +
                                   (mixed ? (int64_t)(sizeof(float4) * NN + mixed_berry_workspace_bytes(N, 1)) : 0)) +
        (int64_t)wilson_workspace_bytes(N, 1, (int)n_k, (int)n_occ) + 8 * n_k * dim;
    int64_t chunk = std::max<int64_t>(1, std::min<int64_t>(n_loops, chunk_budget_bytes() / per_loop));
    chunk = std::min<int64_t>(chunk, std::max<int64_t>(1, 65535 / std::max(T, 1)));
    Ctx ctx;
    double* kv_d = ctx.alloc<double>(chunk * n_k * dim);
    double* kp_d = ctx.alloc<double>(chunk * std::max(T, 1) * dim);
    zc* H = ctx.alloc<zc>(chunk * std::max(T, 1) * NN);
    zc* U = ctx.alloc<zc>(chunk * std::max(T, 1) * NN);
    double* E = ctx.alloc<double>(chunk * std::max(T, 1) * N);
    int* occ_d = ctx.alloc<int>(n_occ);
    const size_t wb = wilson_workspace_bytes(N, chunk, (int)n_k, (int)n_occ);
    void* work = ctx.alloc<unsigned char>(wb);
    double* out_d = ctx.alloc<double>(chunk * (svd ? n_occ : 1));
    int* status_d = ctx.alloc<int>(1);
    const int64_t npmax = chunk * std::max(T, 1);
    float4* Hp = mixed ? ctx.alloc<float4>(npmax * NN) : nullptr;
    const size_t mwb = mixed ? mixed_berry_workspace_bytes(N, npmax) : 0;
    void* mwork = mixed ? ctx.alloc<unsigned char>(mwb) : nullptr;
    if (ctx.rc) return ctx.rc;
    std::vector<int> occ32(occ, occ + n_occ);
    TBG_CUDA(cudaMemcpyAsync(occ_d, occ32.data(), sizeof(int) * n_occ, cudaMemcpyHostToDevice, ctx.st));
    TBG_CUDA(cudaMemsetAsync(status_d, 0, sizeof(int), ctx.st));
    for (int64_t l0 = 0; l0 < n_loops; l0 += chunk) {
        const int64_t nl = std::min(chunk, n_loops - l0);
        TBG_CUDA(cudaMemcpyAsync(kv_d, kvec + l0 * n_k * dim, sizeof(double) * nl * n_k * dim,
                                 cudaMemcpyHostToDevice, ctx.st));
        if (T > 0) {
            // the loop points k_0 .. k_{T-1} (k_T is k_0 up to the gauge phase)
            TBG_CUDA(cudaMemcpy2DAsync(kp_d, sizeof(double) * T * dim, kv_d, sizeof(double) * n_k * dim,
                                       sizeof(double) * T * dim, nl, cudaMemcpyDeviceToDevice, ctx.st));
            const int64_t np = nl * T;
            if ((rc = fourier_direct(M, ctx.st, np, kp_d, TBG_GAUGE_ATOM, 0, nullptr, H, nullptr, NN, 0))) return rc;
            if (mixed) {
                if ((rc = z_to_pairs(ctx.st, np, NN, H, NN, Hp))) return rc;
                if ((rc = mixed_berry(ctx.st, N, np, Hp, nullptr, nullptr, 0.0, E, nullptr, mwork, mwb, status_d,
                                      nullptr, nullptr, U)))
                    return rc;
            } else if ((rc = eig_batched(ctx.st, N, np, H, E, U, nullptr, 0, status_d))) {
                return rc;
            }
        }
        if ((rc = wilson_from_vectors(ctx.st, M, nl, (int)n_k, kv_d, U, (int)n_occ, occ_d, svd, out_d, work, wb,
                                      status_d)))
            return rc;
        TBG_CUDA(cudaMemcpyAsync(out + l0 * (svd ? n_occ : 1), out_d, sizeof(double) * nl * (svd ? n_occ : 1),
                                 cudaMemcpyDeviceToHost, ctx.st));
        if (ctx.sync("tbg_wilson_loops")) return ctx.rc;
    }
    if ((rc = check_status(status_d, ctx.st))) return rc;
    return ctx.sync("tbg_wilson_loops");
}

int tbg_hall_energy_cut(const tbg_model* m, const int64_t* kmesh, const double* dirs2, int64_t nmu, const double* mu,
                        double T, double eta, int spin, double* sigma_out) {
    int rc = check_model(m);
    if (rc) return rc;
    const ModelDev& M = m->d;
    // validate_rank2 (config.rs:141-147), then the energy-cut checks (linear/mod.rs:177-185)
    int64_t nk = 0;
    if ((rc = check_kmesh(M, kmesh, &nk))) return rc;
    if ((rc = check_dirs(dirs2, 2, M.dim, 2))) return rc;
    if (nmu < 1 || !mu)
        return set_error(TBG_E_INVALID_RESPONSE_PARAMETER, "chemical_potentials: must contain at least one value");
    for (int64_t j = 0; j < nmu; ++j)
        if (!std::isfinite(mu[j]))
            return set_error(TBG_E_INVALID_RESPONSE_PARAMETER, "chemical_potentials: all values must be finite");
    if ((rc = check_eta(eta))) return rc;
    if (!std::isfinite(T) || T < 0.0)
        return set_error(TBG_E_INVALID_RESPONSE_PARAMETER, "T: all values must be finite and non-negative");
    if ((rc = check_spin(m, spin))) return rc;
    for (int64_t j = 0; j + 1 < nmu; ++j)
        if (mu[j] > mu[j + 1]) return set_error(TBG_E_INVALID_RESPONSE_PARAMETER, "mu: must be sorted in ascending order");
    if (M.dim != 2 && M.dim != 3) return set_error(TBG_E_INVALID_DIMENSION, "energy-cut integration supports dim 2 and 3");
    if (!sigma_out) return set_error(TBG_E_INVALID_ARGUMENT, "null output");
    const double det = lattice_det(M.lat, M.dim);
    if (det == 0.0 || !std::isfinite(det)) return set_error(TBG_E_LINALG, "Linear algebra operation failed: singular lattice");
    const int N = (int)M.nsta, dim = M.dim;
    const int64_t NN = (int64_t)N * N;
    Ctx ctx;
    BerryJob J;
    J.m = const_cast<ModelDev*>(&M);
    J.spin = spin;
    J.eta = eta;
    J.precision = TBG_PREC_FP64;
    J.want_metric = false;
    J.chunk = choose_chunk(nk, sizeof(zc) * NN * 5 + 64 * N);
    double* dirs_d = ctx.alloc<double>(2 * dim);
    J.dirs_d = dirs_d;
    double* E_all = ctx.alloc<double>(nk * N);
    double* Om_all = ctx.alloc<double>(nk * N);
    zc* U_all = ctx.alloc<zc>(nk * NN);
    zc* K_all = ctx.alloc<zc>(nk * NN);
    double* Rd = ctx.alloc<double>(J.chunk * NN);
    int* perm_d = ctx.alloc<int>(nk * N);
    if (ctx.rc) return ctx.rc;
    if ((rc = alloc_berry(ctx, J))) return rc;
    TBG_CUDA(cudaMemcpyAsync(dirs_d, dirs2, sizeof(double) * 2 * dim, cudaMemcpyHostToDevice, ctx.st));
    const int64_t n0 = kmesh[0], n1 = dim > 1 ? kmesh[1] : 1, n2 = dim > 2 ? kmesh[2] : 1;
    // 1. vertex data of the whole mesh (compute_velocity_kernel, primitives.rs:33-137)
    for (int64_t c0 = 0; c0 < nk; c0 += J.chunk) {
        const int64_t nkc = std::min(J.chunk, nk - c0);
        kmesh_kernel<<<blocks_for(nkc), 256, 0, ctx.st>>>(c0, nkc, dim, n0, n1, n2, J.k_d);
        TBG_LAUNCHED("kmesh_kernel");
        if ((rc = run_berry_chunk(ctx, J, nkc, nullptr))) return rc;
        TBG_CUDA(cudaMemcpyAsync(E_all + c0 * N, J.E, sizeof(double) * nkc * N, cudaMemcpyDeviceToDevice, ctx.st));
        TBG_CUDA(cudaMemcpyAsync(U_all + c0 * NN, J.U, sizeof(zc) * nkc * NN, cudaMemcpyDeviceToDevice, ctx.st));
        if ((rc = ec_vertex_data(ctx.st, N, nkc, J.V, 2 * NN, J.E, eta, K_all + c0 * NN, Om_all + c0 * N))) return rc;
    }
    // 2. squared overlaps of the forward mesh edges, per dimension
    const int64_t n3[3] = {n0, n1, n2};
    const int64_t stride[3] = {n3[1] * n3[2], n3[2], 1};
    std::vector<double> R_h((size_t)nk * dim * NN, 0.0);
    for (int d = 0; d < dim; ++d) {
        const int64_t sd = stride[d];
        for (int64_t a0 = 0; a0 + sd < nk; a0 += J.chunk) {
            const int64_t na = std::min(J.chunk, nk - sd - a0);
            if ((rc = zgemm_batched(ctx.st, N, na, true, U_all + a0 * NN, NN, U_all + (a0 + sd) * NN, NN, J.scratch,
                                    NN)))
                return rc;
            if ((rc = ec_abs2(ctx.st, na * NN, J.scratch, Rd))) return rc;
            TBG_CUDA(cudaMemcpy2DAsync(R_h.data() + ((size_t)a0 * dim + d) * NN, sizeof(double) * dim * NN, Rd,
                                       sizeof(double) * NN, sizeof(double) * NN, na, cudaMemcpyDeviceToHost, ctx.st));
            if (ctx.sync("tbg_hall_energy_cut overlaps")) return ctx.rc;
        }
    }
    if ((rc = check_status(J.status_d, ctx.st))) return rc;
    // 3. band tracking on the host, permutations to the device
    std::vector<int> perm_h((size_t)nk * N);
    ec_track(dim, kmesh, N, R_h.data(), perm_h.data());
    TBG_CUDA(cudaMemcpyAsync(perm_d, perm_h.data(), sizeof(int) * nk * N, cudaMemcpyHostToDevice, ctx.st));
    // 4. the mu grid: the chemical potentials, or the extended fine grid of the thermal convolution
    const double width = (T <= 0.0) ? 0.0 : T * 8.617333262145e-5;
    std::vector<double> grid;
    double mu_lo = 0.0, dmu = 0.0, beta = 0.0;
    if (width == 0.0) {
        grid.assign(mu, mu + nmu);
    } else {
        beta = 1.0 / width;
        const double x_max = 12.0;
        const double mmin = *std::min_element(mu, mu + nmu), mmax = *std::max_element(mu, mu + nmu);
        mu_lo = mmin - x_max / beta;
        const double mu_hi = mmax + x_max / beta;
        dmu = 0.1 / beta;
        const int64_t n_ext = (int64_t)std::ceil((mu_hi - mu_lo) / dmu) + 1;
        if (n_ext > (int64_t)1 << 26) return set_error(TBG_E_UNSUPPORTED, "thermal grid too fine");
        const double step = n_ext > 1 ? (mu_hi - mu_lo) / (double)(n_ext - 1) : 0.0;
        grid.resize(n_ext);
        for (int64_t i = 0; i < n_ext; ++i) grid[i] = mu_lo + step * (double)i;  // ndarray linspace
    }
    const int ng = (int)grid.size();
    const int window = std::min(ng, kEcWindow);
    const int S = dim == 2 ? 4 : 5;
    const int64_t items = nk * S * N;
    const int nblocks = (int)std::max<int64_t>(1, std::min<int64_t>((items + 127) / 128, 152 * 8));
    double* grid_d = ctx.alloc<double>(ng);
    double* part = ctx.alloc<double>((int64_t)nblocks * window);
    double* fpart = ctx.alloc<double>((int64_t)nblocks * window);
    double* acc_d = ctx.alloc<double>(ng);
    double* full_d = ctx.alloc<double>(ng);
    if (ctx.rc) return ctx.rc;
    TBG_CUDA(cudaMemcpyAsync(grid_d, grid.data(), sizeof(double) * ng, cudaMemcpyHostToDevice, ctx.st));
    // 5. occupancy cut of every simplex
    if ((rc = ec_integrate(ctx.st, dim, kmesh, N, E_all, K_all, Om_all, perm_d, ng, grid_d, eta, part, fpart, nblocks,
                           window, acc_d, full_d)))
        return rc;
    std::vector<double> acc_h(ng), full_h(ng);
    TBG_CUDA(cudaMemcpyAsync(acc_h.data(), acc_d, sizeof(double) * ng, cudaMemcpyDeviceToHost, ctx.st));
    TBG_CUDA(cudaMemcpyAsync(full_h.data(), full_d, sizeof(double) * ng, cudaMemcpyDeviceToHost, ctx.st));
    if (ctx.sync("tbg_hall_energy_cut")) return ctx.rc;
    std::vector<double> s0(ng);
    for (int w0 = 0; w0 < ng; w0 += window) {  // the full-occupancy difference array restarts per window
        double run = 0.0;
        for (int i = w0; i < std::min(ng, w0 + window); ++i) {
            run += full_h[i];
            s0[i] = acc_h[i] + run;
        }
    }
    // 6. thermal convolution (energy_cut.rs:1380-1427), then the Cartesian normalisation
    if (width == 0.0) {
        for (int64_t j = 0; j < nmu; ++j) sigma_out[j] = s0[j] / det;
    } else {
        const double dx = 2.0 * 18.0 / 72.0;
        for (int64_t j = 0; j < nmu; ++j) {
            double sum = 0.0;
            for (int iq = 0; iq < 72; ++iq) {
                const double x = -18.0 + ((double)iq + 0.5) * dx;
                const double w = std::fabs(x) > 50.0 ? 0.0 : std::exp(x) / ((1.0 + std::exp(x)) * (1.0 + std::exp(x)));
                const double i_f = (mu[j] + x / beta - mu_lo) / dmu;
                const int64_t i_lo = std::max<int64_t>((int64_t)std::floor(i_f), 0);
                const int64_t i_hi = std::min<int64_t>(i_lo + 1, ng - 1);
                if (i_hi > i_lo) {
                    const double t = i_f - (double)i_lo;
                    sum += dx * w * (s0[i_lo] + t * (s0[i_hi] - s0[i_lo]));
                }
            }
            sigma_out[j] = sum / det;
        }
    }
    return TBG_OK;
}

int tbg_quantum_geometry(const tbg_model* m, int64_t nk, const double* k, const double* dirs2, double eta,
                         int precision, double* metric_out, double* berry_out, double* E_out) {
    if (nk > 0 && (!metric_out || !berry_out)) return set_error(TBG_E_INVALID_ARGUMENT, "null output");
    // the quantum-geometry kernel always uses the charge current (spin ignored)
    return berry_common(m, nk, k, dirs2, -1, eta, precision, berry_out, E_out, 0, nullptr, 0.0, nullptr,
                        metric_out);
}

int tbg_quantum_geometry_mesh(const tbg_model* m, const int64_t* kmesh, const double* dirs2, int64_t nmu,
                              const double* mu, double T, double eta, int precision, double* metric_out,
                              double* berry_out, tbg_report* report) {
    if (!metric_out) return set_error(TBG_E_INVALID_ARGUMENT, "null output");
    return hall_impl(m, kmesh, 0, 0, true, dirs2, nmu, mu, T, eta, -1, precision, berry_out, report, metric_out);
}

}  // extern "C"
