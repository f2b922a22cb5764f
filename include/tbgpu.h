/*
 * tbgpu.h -- C-ABI of the GB300 k-mesh engine for Rustb tight-binding models.
 *
 * Every entry point replaces one method on Rustb's k-mesh hot path.  The
 * reference interface each one stands in for is cited beside it (paths are
 * relative to the Rustb crate root).  Layout conventions follow Rustb/ndarray:
 *
 *   - all arrays are C (row-major) contiguous;
 *   - a complex number is two doubles {re, im} (binary layout of
 *     num_complex::Complex<f64>);
 *   - k-points are fractional coordinates, shape (nk, dim);
 *   - hamR is int64 (isize on 64-bit targets), shape (nR, dim);
 *   - ham is complex, shape (nR, nsta, nsta), ham[r][i][j] = <i,0|H|j,R_r>;
 *   - orb is (norb, dim) fractional, lat is (dim, dim) with lattice vectors
 *     as rows (src/model.rs:150-158).
 *
 * All pointers are HOST pointers.  Outputs are caller-allocated.  Each call is
 * synchronous: on return the outputs are written.  Calls on different models
 * (or the same model) from different host threads are safe.
 *
 * Every function returns a status (enum tbg_status).  On failure the message
 * of the most recent error of the calling thread is available through
 * tbg_last_error().
 */
#ifndef TBGPU_H
#define TBGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  Codes 1..13 map 1:1 onto TbError variants (src/error.rs). */
enum tbg_status {
    TBG_OK = 0,
    TBG_E_KVECTOR_LENGTH = 1,             /* TbError::KVectorLengthMismatch */
    TBG_E_DIMENSION_MISMATCH = 2,         /* TbError::DimensionMismatch */
    TBG_E_INVALID_RESPONSE_PARAMETER = 3, /* TbError::InvalidResponseParameter */
    TBG_E_SPIN_NOT_ALLOWED = 4,           /* TbError::SpinNotAllowed */
    TBG_E_INVALID_KMESH = 5,              /* TbError::InvalidKmeshDimensions */
    TBG_E_LINALG = 6,                     /* TbError::Linalg (singular lattice) */
    TBG_E_INVALID_DIMENSION = 7,          /* TbError::InvalidDimension */
    TBG_E_INVALID_MODEL = 8,              /* TbError::InvalidModelInvariant */
    TBG_E_INVALID_ARGUMENT = 9,           /* conditions on which Rustb panics */
    TBG_E_INVALID_ENERGY_RANGE = 10,      /* TbError::InvalidEnergyRange */
    TBG_E_INVALID_DOS_PARAMETER = 11,     /* TbError::InvalidDosParameter */
    TBG_E_FILE_PARSE = 12,                /* TbError::FileParse */
    TBG_E_FILE_OPEN = 13,                 /* TbError::FileCreation (a file that cannot be opened) */
    TBG_E_CUDA = 20,                      /* CUDA runtime failure */
    TBG_E_NOCONV = 21,                    /* eigensolver did not converge */
    TBG_E_TIMEOUT = 22,                   /* a bounded device wait ran out */
    TBG_E_OOM = 23,                       /* device allocation failed */
    TBG_E_UNSUPPORTED = 24                /* size or option not supported */
};

/* Gauge (src/model.rs:449-452). */
enum tbg_gauge { TBG_GAUGE_LATTICE = 0, TBG_GAUGE_ATOM = 1 };

/* Spin-current polarisation (src/model.rs:470-474); -1 = None (charge current). */
enum tbg_spin { TBG_SPIN_NONE = -1, TBG_SPIN_X = 0, TBG_SPIN_Y = 1, TBG_SPIN_Z = 2 };

/* Arithmetic of tbg_hall_conductivity / tbg_berry_curvature.  MIXED applies
 * to models with 9 <= nsta <= 2048 (products longer than 256 run in exact
 * chunks); other models run FP64 (tbg_report.precision says which ran). */
enum tbg_precision {
    TBG_PREC_FP64 = 0,  /* plain: FP64 end to end (the drop-in) */
    TBG_PREC_MIXED = 1  /* FP32 eigensolve, refinement and rotation on the
                           tensor cores with FP64-class exact-slice products */
};

typedef struct tbg_model tbg_model;

/* Per-call report filled by tbg_hall_conductivity (may be NULL). */
typedef struct tbg_report {
    int64_t nk;              /* k-points processed */
    int64_t nsta;            /* bands per k-point */
    int32_t precision;       /* tbg_precision used */
    int32_t fourier_mode;    /* 0 = FP64 phase x hop contraction, 1 = exact-slice tensor-core
                                contraction, 2 = fused small-model path (nsta <= 8) */
    int64_t kernel_launches; /* device kernels launched by the call */
    double device_ms;        /* device time of the call (CUDA events) */
    double eig_ms;           /* device time spent in the eigensolver kernels */
    int64_t refine_clusters; /* near-degenerate clusters handled by the refinement */
} tbg_report;

/* ---------------------------------------------------------------- model --- */

/* Upload a model and keep it resident on the device.
 * Replaces: the Model<SPIN,DIM,R> value every hot-path method borrows
 * (src/model.rs:150-158); validation mirrors Model::validate (src/model.rs:564).
 * spin != 0 means nsta = 2*norb (spinful basis [up 0..norb, down norb..2norb]). */
int tbg_model_create(int dim, int spin, int64_t norb, int64_t nR,
                     const int64_t* hamR, const double* ham,
                     const double* orb, const double* lat, tbg_model** out);

/* Attach a position matrix (HasRMatrix models): rmatrix has shape
 * (n_rmat, dim, nsta, nsta) complex, Cartesian; its rows pair with the first
 * n_rmat rows of hamR.  Replaces: RMatrixData / HasRMatrix (src/model.rs:18-76)
 * as read by gen_v (src/velocity.rs:377-401) and gen_v_projected
 * (src/velocity.rs:627-668). */
int tbg_model_set_rmatrix(tbg_model* m, int64_t n_rmat, const double* rmatrix);

int tbg_model_destroy(tbg_model* m);

int tbg_model_info(const tbg_model* m, int* dim, int* spin, int64_t* norb,
                   int64_t* nsta, int64_t* nR);

/* ------------------------------------------------------- per-k primitives --- */

/* H(k) for nk k-points -> H_out (nk, nsta, nsta) complex.
 * Replaces: Model::gen_ham (src/model_physics.rs:43-148). */
int tbg_gen_ham(const tbg_model* m, int64_t nk, const double* k, int gauge,
                double* H_out);

/* Velocity along every Cartesian direction -> V_out (nk, dim, nsta, nsta),
 * H_out (nk, nsta, nsta) (H_out may be NULL).
 * Replaces: Velocity::gen_v (src/velocity.rs:214-441). */
int tbg_gen_v(const tbg_model* m, int64_t nk, const double* k, int gauge,
              double* V_out, double* H_out);

/* Direction-projected velocity: dirs (n_proj, dim) -> V_out (nk, n_proj, nsta,
 * nsta), H_out (nk, nsta, nsta) (may be NULL).
 * Replaces: Model::gen_v_projected (src/velocity.rs:470-731). */
int tbg_gen_v_projected(const tbg_model* m, int64_t nk, const double* k,
                        int gauge, int64_t n_proj, const double* dirs,
                        double* V_out, double* H_out);

/* Band energies (ascending) -> E_out (nk, nsta).
 * Replaces: Solve::solve_band_onek / solve_band_all / solve_band_all_parallel
 * (src/solve_ham.rs:52-107; LAPACK zheev via eigvalsh_v,
 * src/ndarray_lapack.rs:412-448). */
int tbg_solve_band(const tbg_model* m, int64_t nk, const double* k,
                   double* E_out);

/* The same with a precision choice: TBG_PREC_FP64 is tbg_solve_band;
 * TBG_PREC_MIXED runs the FP32 eigensolve with the FP64-class refinement of
 * the eigenvalues (<= 1e-9 ||H||; models of 9..2048 bands, others FP64).  For
 * callers that want band energies faster than the drop-in (the serving loop's
 * bands requests); no counterpart in the reference. */
int tbg_solve_band_prec(const tbg_model* m, int64_t nk, const double* k,
                        int precision, double* E_out);

/* Energies and eigenvectors -> E_out (nk, nsta), U_out (nk, nsta, nsta).
 * evec_rows != 0: U_out[k][n][:] is the n-th eigenvector (the layout of
 * Solve::solve_onek / solve_all_parallel, src/solve_ham.rs:110-184);
 * evec_rows == 0: eigenvectors in columns.  The phase of each eigenvector is
 * arbitrary, as with LAPACK. */
int tbg_solve(const tbg_model* m, int64_t nk, const double* k, double* E_out,
              double* U_out, int evec_rows);

/* ----------------------------------------------------------- response --- */

/* Band-resolved Berry curvature at nk k-points: dirs2 (2, dim) rows = the two
 * tensor indices, spin = tbg_spin, eta >= 0.  Omega_out, E_out (nk, nsta).
 * Replaces: BerryCurvature::berry_curvature_at (src/response/traits.rs:60-78,
 * kernel berry_curvature_at_impl traits.rs:160-200). */
int tbg_berry_curvature(const tbg_model* m, int64_t nk, const double* k,
                        const double* dirs2, int spin, double eta,
                        int precision, double* Omega_out, double* E_out);

/* The same for several models with the same nsta and dim at once: model i
 * takes nk[i] k-points, k is their concatenation (sum nk, dim) and Omega_out,
 * E_out (sum nk, nsta) are concatenated the same way.  The models' H and
 * velocities come from their own hopping tables into one stacked buffer and
 * the eigensolve, rotation and Omega run once over the stacked k-points, so
 * many small models fill the GPU as one large one does; results equal those
 * of tbg_berry_curvature model by model.  Replaces: a loop of
 * berry_curvature_at (src/response/traits.rs:60-78) over models, as Rustb's
 * users batch many models (rayon over models, src/response/linear/mod.rs:198-202). */
int tbg_berry_curvature_multi(int64_t n_models, const tbg_model* const* models,
                              const int64_t* nk, const double* k,
                              const double* dirs2, int spin, double eta,
                              int precision, double* Omega_out, double* E_out);

/* Occupation-weighted Berry curvature sum_n Omega_n f(E_n, mu) per k-point.
 * T in kelvin (0 = step function with f(mu) = 1/2).
 * Replaces: BerryCurvature::occupied_berry_curvature_on
 * (src/response/traits.rs:104-150). */
int tbg_occupied_berry_curvature(const tbg_model* m, int64_t nk,
                                 const double* k, const double* dirs2, int spin,
                                 double eta, double T, double mu, int precision,
                                 double* out);

/* Anomalous / spin Hall conductivity, Direct integration over the uniform
 * mesh kmesh[dim]: sigma_out[j] = sum_k sum_n Omega_n f(E_n, mu_j) / nk / det(lat).
 * Replaces: Model::hall_conductivity with Integration::Direct
 * (src/response/linear/mod.rs:160-225). */
int tbg_hall_conductivity(const tbg_model* m, const int64_t* kmesh,
                          const double* dirs2, int64_t nmu, const double* mu,
                          double T, double eta, int spin, int precision,
                          double* sigma_out, tbg_report* report);

/* Anomalous / spin Hall conductivity with Integration::EnergyCut on the
 * uniform mesh kmesh[dim] (dim 2 or 3; mu sorted ascending): eigenpairs and
 * K_nm = v^a_nm v^b_mn at every mesh point, bands tracked by eigenvector
 * overlap, each triangle (2D, both diagonals) or tetrahedron (3D) cut at every
 * mu -- vertex-averaged Omega where a band is fully occupied, quadrature of
 * the interpolated Kubo term on the occupied part where it is partly occupied
 * -- and, for T > 0, the thermal convolution of the zero-width result.
 * sigma_out[j] / det(lat).  FP64.
 * Replaces: Model::hall_conductivity with Integration::EnergyCut
 * (src/response/linear/mod.rs:226-268, src/response/tracking.rs:123-240,
 * src/response/energy_cut.rs:1120-1849). */
int tbg_hall_energy_cut(const tbg_model* m, const int64_t* kmesh,
                        const double* dirs2, int64_t nmu, const double* mu,
                        double T, double eta, int spin, double* sigma_out);

/* Unnormalised Direct-integration sums over the k-points of the uniform mesh
 * kmesh[dim] with flat indices [k_begin, k_begin + k_count) in gen_kmesh order:
 *   sums_out[j] = sum_k sum_n Omega_n f(E_n, mu_j).
 * The conductivity is the sum over disjoint ranges covering the mesh, divided
 * by nk and det(lat).  This splits one mesh across calls or devices; the
 * reference computes the same sum inside hall_conductivity
 * (src/response/linear/mod.rs:204-223) over the whole mesh at once. */
int tbg_hall_sums_range(const tbg_model* m, const int64_t* kmesh, int64_t k_begin,
                        int64_t k_count, const double* dirs2, int64_t nmu,
                        const double* mu, double T, double eta, int spin,
                        int precision, double* sums_out, tbg_report* report);

/* Band-resolved quantum geometry at nk k-points: the tensor
 *   G_n = sum_{m != n} v^a_nm v^b_mn / ((E_n - E_m)^2 + eta^2)
 * with dirs2 (2, dim) rows = a, b; metric_out = Re G_n, berry_out = -2 Im G_n,
 * E_out (may be NULL) the band energies, all (nk, nsta).  Charge current
 * (no spin dressing).
 * Replaces: QuantumGeometry::quantum_geometry_at / quantum_geometry_on
 * (src/quantum_geometry.rs:88-138, kernel quantum_geometry_at_impl
 * quantum_geometry.rs:149-193). */
int tbg_quantum_geometry(const tbg_model* m, int64_t nk, const double* k,
                         const double* dirs2, double eta, int precision,
                         double* metric_out, double* berry_out, double* E_out);

/* Occupation-weighted quantum geometry, Direct integration over the uniform
 * mesh kmesh[dim]: per mu_j,
 *   metric_out[j] = sum_k sum_n g_n f(E_n, mu_j) / nk / det(lat),
 *   berry_out[j]  = sum_k sum_n Omega_n f(E_n, mu_j) / nk / det(lat).
 * Replaces: Model::quantum_geometry with Integration::Direct
 * (src/quantum_geometry.rs:196-240). */
int tbg_quantum_geometry_mesh(const tbg_model* m, const int64_t* kmesh,
                              const double* dirs2, int64_t nmu, const double* mu,
                              double T, double eta, int precision,
                              double* metric_out, double* berry_out,
                              tbg_report* report);

/* FP64 band energies (ascending) at every point of the uniform mesh
 * kmesh[dim], gen_kmesh order (first dimension outermost) -> E_out (nk, nsta).
 * Replaces: solve_band_all_parallel(&gen_kmesh(k_mesh)) as the mesh consumers
 * call it -- Model::dos (src/model_physics.rs:206-207), write_bxsf and
 * show_fermi_surface (src/fermi_surface.rs:454-463, 848-900), write_spin_frmsf
 * (fermi_surface.rs:637-666). */
int tbg_bands_mesh(const tbg_model* m, const int64_t* kmesh, double* E_out);

/* Density of states with Gaussian smearing on the uniform mesh kmesh[dim]:
 * E_out[i] = E_min + i (E_max - E_min) / (E_n - 1) (E_out may be NULL) and
 *   dos_out[i] = 1/nk sum_{k,n} exp(-((E_i - E_nk) / sigma)^2 / 2) / sigma / sqrt(2 pi),
 * band energies in FP64.  Errors: E_min >= E_max -> INVALID_ENERGY_RANGE;
 * E_n == 0 or sigma not finite and positive -> INVALID_DOS_PARAMETER.
 * Replaces: Model::dos (src/model_physics.rs:179-230). */
int tbg_dos(const tbg_model* m, const int64_t* kmesh, double E_min, double E_max,
            int64_t E_n, double sigma, double* E_out, double* dos_out);

/* Wilson loops over n_loops closed k-paths kvec (n_loops, n_k, dim); each
 * path's last point must equal its first up to an integer vector G (the
 * eigenvectors there are the first point's times exp(-2 pi i G . tau)).
 * occ (n_occ) are the occupied band indices (n_occ <= 64).
 * mode 0: out (n_loops, n_occ) = -arg of the eigenvalues of the product of the
 *         unitary (U V^dagger) parts of the overlap matrices, ascending per loop;
 *         replaces Berry::berry_loop (src/geometry.rs:156-215) and, through the
 *         loops the caller builds, berry_flux / berry_phase / wannier_centre
 *         (geometry.rs:272-420).
 * mode 1: out (n_loops) = -arg det of the product of the raw overlaps;
 *         replaces Berry::berry_loop_det (geometry.rs:217-270).
 * precision: FP64 eigenpairs at the loop points, or MIXED (FP32 eigenpairs
 * refined with FP64-class tensor-core products, <= 2048 bands). */
int tbg_wilson_loops(const tbg_model* m, int64_t n_loops, int64_t n_k, const double* kvec,
                     int64_t n_occ, const int64_t* occ, int mode, int precision, double* out);

/* ------------------------------------------------------ Wannier90 input --- */

/* Native reader of Wannier90 tight-binding tables (host side; the result is
 * uploaded with tbg_model_create / tbg_model_set_rmatrix).  Together with the
 * seedname.win / _centres.xyz parsing of the host mirror it replaces
 * Wannier90::from_hr and Model::from_hr_with_rmatrix
 * (src/wannier90.rs:49-1219).  Call order as the reference reads the files:
 * tbg_w90_read_hr, (win / xyz on the host), tbg_w90_read_r when the model
 * carries a position matrix, tbg_w90_apply_wsvec (no-op when the file is
 * absent), tbg_w90_hermitize_rmatrix; then tbg_w90_info / tbg_w90_copy. */
typedef struct tbg_w90 tbg_w90;

/* seedname_hr.dat -> ham (nR, nsta, nsta) complex with R = 0 first, hamR (nR, 3);
 * zero_energy is subtracted from the R = 0 diagonal (wannier90.rs:85-245). */
int tbg_w90_read_hr(const char* hr_path, double zero_energy, tbg_w90** out);
/* seedname_r.dat -> rmatrix (nR, 3, nsta, nsta) aligned with hamR
 * (wannier90.rs:771-880); TBG_E_FILE_OPEN when the file is missing. */
int tbg_w90_read_r(tbg_w90* h, const char* r_path);
/* seedname_wsvec.dat Wigner-Seitz refolding (wannier90.rs:882-1142);
 * *applied = 0 and TBG_OK when the file does not exist. */
int tbg_w90_apply_wsvec(tbg_w90* h, const char* ws_path, int* applied);
/* rmatrix(R) <- (rmatrix(R) + rmatrix(-R)^dagger) / 2 (wannier90.rs:1146-1167). */
int tbg_w90_hermitize_rmatrix(tbg_w90* h);
int tbg_w90_info(const tbg_w90* h, int64_t* nsta, int64_t* nR, int* has_r);
/* Copies into caller arrays sized from tbg_w90_info (any may be NULL). */
int tbg_w90_copy(const tbg_w90* h, double* ham, int64_t* hamR, double* rmatrix);
int tbg_w90_free(tbg_w90* h);

/* ------------------------------------------- asynchronous batch queue --- */

/* Jobs run on library-owned worker threads, each call on its own CUDA stream,
 * so jobs of different models and sizes overlap on the GPU.  The reference
 * runs the same methods concurrently from rayon workers
 * (src/response/linear/mod.rs:198-202, src/solve_ham.rs:327-332); a Rust
 * caller uses these entry points to keep many batch calls in flight. */
typedef enum {
  TBG_JOB_HALL = 0,      /* tbg_hall_conductivity: out0 = sigma (nmu)         */
  TBG_JOB_BANDS = 1,     /* tbg_solve_band: out0 = E (nk, nsta)               */
  TBG_JOB_BERRY = 2,     /* tbg_berry_curvature: out0 = Omega, out1 = E       */
  TBG_JOB_OCCUPIED = 3   /* tbg_occupied_berry_curvature: out0 (nk), mu[0]    */
} tbg_job_kind;

typedef struct tbg_job {
  int kind;                 /* tbg_job_kind */
  const tbg_model* model;
  const int64_t* kmesh;     /* HALL: (dim) */
  int64_t nk;               /* BANDS, BERRY, OCCUPIED */
  const double* k;          /* (nk, dim) */
  const double* dirs2;      /* (2, dim) */
  int64_t nmu;
  const double* mu;         /* (nmu); OCCUPIED uses mu[0] */
  double T, eta;
  int spin, precision;
  double* out0;
  double* out1;
} tbg_job;

/* Queue a job.  The descriptor, kmesh, dirs2 and mu are copied; k and the
 * outputs must stay valid until the job is reported done.  The job runs on
 * the device current in the calling thread.  *ticket identifies it. */
int tbg_batch_submit(const tbg_job* job, int64_t* ticket);

/* Non-blocking: *done = 1 once the job finished, *status = its tbg_status
 * (and tbg_last_error in this thread holds its message).  A ticket is
 * released by the call that reports it done; an unknown ticket is
 * TBG_E_INVALID_ARGUMENT. */
int tbg_batch_poll(int64_t ticket, int* done, int* status);

/* Block until the job finished; *status as for tbg_batch_poll.  Releases the
 * ticket. */
int tbg_batch_wait(int64_t ticket, int* status);

/* Number of worker threads (default 4; applies to workers not yet started). */
int tbg_batch_set_workers(int n);

/* ------------------------------------------------ no-allocation variant --- */

/* Size of the fixed device scratch array used by tbg_eigvalsh_noalloc, and
 * the largest matrix order it admits (one 1448 x 1448 complex FP64 matrix). */
#define TBG_NOALLOC_SCRATCH_BYTES (32u * 1024u * 1024u)
#define TBG_NOALLOC_MAX_N 1448

/* Band energies (ascending, FP64) of nk device-resident Hermitian matrices,
 * without allocating any device memory.  No counterpart in the reference: it
 * serves callers that cannot call cudaMalloc -- code that hands all device
 * memory to its own allocator or pool, or a latency-critical loop in which
 * cudaMalloc/cudaFree would synchronise the device.
 *
 * H_d (nk, n, n) complex FP64 and E_d (nk, n) FP64 are DEVICE pointers owned
 * by the caller; H_d is not modified.  The solver works on a copy of H_d in a
 * fixed static device array of TBG_NOALLOC_SCRATCH_BYTES that every GPU that
 * loads this library holds until the process exits; a call needs
 * nk * n * n * 16 bytes of it and is rejected with TBG_E_UNSUPPORTED beyond
 * that (so n <= TBG_NOALLOC_MAX_N).  The first call on a device looks up the
 * array's device address (cudaGetSymbolAddress) and keeps it; make that first
 * call before any stream capture, and do not use the entry point on a device
 * after cudaDeviceReset.  Non-finite input is not reported: there is no status
 * word to read back without synchronising, and such a matrix yields NaN
 * energies (check E_d, or use tbg_solve_band, which returns TBG_E_NOCONV).
 * The work is enqueued on `stream` (a cudaStream_t, NULL = default stream) and
 * the call returns without waiting.  All calls share the one array: calls
 * whose work overlaps on the GPU (different streams, no ordering between them)
 * race on it; calls on one stream are ordered and safe.  Each call overwrites
 * the part of the array it uses, so nothing in it has to start at zero. */
int tbg_eigvalsh_noalloc(int64_t n, int64_t nk, const double* H_d, double* E_d,
                         void* stream);

/* ------------------------------------------------------------- utility --- */

/* Measured FMA throughput of this GPU's FP64 and FP32 pipes (TFLOP/s), from a
 * short register-resident FMA loop.  A measurement aid for roofline
 * denominators; no reference counterpart. */
int tbg_measure_fma_peaks(double* fp64_tflops, double* fp32_tflops);

/* Copy the calling thread's last error message into buf (always NUL-terminated).
 * Returns the status of that error. */
int tbg_last_error(char* buf, size_t len);

/* Select the CUDA device used by subsequent calls from the calling thread
 * (models remember the device they were created on). */
int tbg_set_device(int device);

/* Per-kernel device timing (measurement aid; no reference counterpart).
 * While enabled, every kernel family the library launches is bracketed by
 * CUDA events on the stream it is launched on; durations accumulate per
 * family together with the algorithmic flops of those launches.
 * tbg_kernel_timing_read copies up to max_entries records (names:
 * max_entries x 64 chars, NUL-terminated) and returns how many. */
int tbg_kernel_timing_enable(int enable);
int tbg_kernel_timing_read(char* names, int64_t* launches, double* total_ms,
                           double* total_flops, int max_entries, int reset);

/* Bytes of device scratch one call sizes its k-point chunks to at this
 * moment: TBG_CHUNK_BYTES when set, else a sixth of the free device memory
 * between 6 and 40 GB (no reference counterpart; for callers that admit
 * concurrent calls by device footprint). */
int64_t tbg_chunk_budget_bytes(void);

/* Crossover of the FP64 eigensolvers: matrices of 9 .. n bands go to the
 * warp-per-matrix cyclic Jacobi solver, larger ones to the Householder
 * solver (n is clamped to [8, 32]; 8 = Householder from 9 bands on, the
 * default).  Process-wide; returns the previous value.  A tuning knob for the
 * batch autotuner (no reference counterpart). */
int tbg_set_jacobi_max_n(int n);

/* Library version string, e.g. "tbgpu 0.1.0 sm_103a". */
const char* tbg_version(void);

/* Number of tbgpu kernels launched by the calling thread since the last reset
 * (reset != 0 zeroes the counter after reading). */
int64_t tbg_kernel_launch_count(int reset);

#ifdef __cplusplus
}
#endif

#endif /* TBGPU_H */
