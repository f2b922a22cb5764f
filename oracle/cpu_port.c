/*
 * CPU port of Rustb's Direct Hall-conductivity path -- TEST INFRASTRUCTURE /
 * CPU BASELINE ONLY (never part of the product library).
 *
 * Restates, per k-point and in the same order of operations as the reference:
 *   gen_v_projected     src/velocity.rs:470-622   (zaxpy sweeps over R, tau term, Atom gauge)
 *   eigh                src/response/traits.rs:168 (LAPACK zheev, JOBZ='V', UPLO='L',
 *                                                   on the row-major buffer)
 *   U^T V U*            src/response/traits.rs:177-180 (two zgemm per direction)
 *   Omega_n             src/response/traits.rs:181-195
 *   occupation sums     src/response/linear/mod.rs:204-223, src/thermodynamics.rs:100-118
 * and the density of states of Model::dos (src/model_physics.rs:179-230).
 * The BLAS/LAPACK routines are taken at run time from the OpenBLAS that scipy
 * bundles (the routines Rustb's openblas backend links).  k-points run in
 * parallel under OpenMP with single-threaded BLAS, as Rustb's rayon
 * par_iter does.
 */
#include <dlfcn.h>
#include <math.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef void (*zaxpy_t)(const int*, const double*, const double*, const int*, double*, const int*);
typedef void (*zheev_t)(const char*, const char*, const int*, double*, const int*, double*, double*,
                        const int*, double*, int*, size_t, size_t);
typedef void (*cblas_zgemm_t)(int, int, int, int, int, int, const void*, const void*, int, const void*, int,
                              const void*, void*, int);
typedef void (*set_threads_t)(int);

static zaxpy_t p_zaxpy = 0;
static zheev_t p_zheev = 0;
static cblas_zgemm_t p_zgemm = 0;

enum { RowMajor = 101, NoTrans = 111, ConjTrans = 113 };

int port_init(const char* blas_path) {
    void* h = dlopen(blas_path, RTLD_NOW | RTLD_LOCAL);
    if (!h) return -1;
    p_zaxpy = (zaxpy_t)dlsym(h, "scipy_zaxpy_");
    p_zheev = (zheev_t)dlsym(h, "scipy_zheev_");
    p_zgemm = (cblas_zgemm_t)dlsym(h, "scipy_cblas_zgemm");
    set_threads_t st = (set_threads_t)dlsym(h, "scipy_openblas_set_num_threads");
    if (!p_zaxpy || !p_zheev || !p_zgemm) return -2;
    if (st) st(1);
    return 0;
}

static double fermi(double e, double mu, double width) {
    if (width == 0.0) return e < mu ? 1.0 : (e > mu ? 0.0 : 0.5);
    double x = (e - mu) / width;
    if (x > 50.0) return 0.0;
    if (x < -50.0) return 1.0;
    return 1.0 / (1.0 + exp(x));
}

/* Per-k Berry curvature (Omega, E) following berry_curvature_at_impl.
 * ham: (nR, N, N) interleaved complex; hamR (nR, dim); Rcart (nR, 3);
 * tau (N, 3) fractional per state; taucart (N, 3). */
static int berry_one(int dim, int N, int norb, int nR, const double* ham, const int64_t* hamR,
                     const double* Rcart, const double* tau, const double* taucart, const double* k,
                     const double* dirs, int spin, double eta, double* Om, double* E, double* ws) {
    const size_t NN = (size_t)N * N;
    double* H = ws;               /* 2NN */
    double* V = H + 2 * NN;       /* 2 x 2NN */
    double* T = V + 4 * NN;       /* 2NN */
    double* Jb = T + 2 * NN;      /* 2NN */
    double* Vb = Jb + 2 * NN;     /* 2NN */
    double* u = Vb + 2 * NN;      /* 2 nR */
    double* phi = u + 2 * nR;     /* 2 N */
    double* work = phi + 2 * N;   /* 2 * lwork */
    const int lwork = 66 * N;
    double* rwork = work + 2 * lwork; /* 3N */
    const int one = 1, nn = (int)NN;
    memset(H, 0, sizeof(double) * 6 * NN);
    for (int r = 0; r < nR; ++r) {
        double s = (double)hamR[r * dim] * k[0];
        if (dim > 1) s += (double)hamR[r * dim + 1] * k[1];
        if (dim > 2) s += (double)hamR[r * dim + 2] * k[2];
        u[2 * r] = cos(2.0 * M_PI * s);
        u[2 * r + 1] = sin(2.0 * M_PI * s);
        p_zaxpy(&nn, u + 2 * r, ham + 2 * NN * r, &one, H, &one);
    }
    for (int p = 0; p < 2; ++p) {
        const double* w = dirs + p * dim;
        for (int r = 0; r < nR; ++r) {
            double rw = w[0] * Rcart[3 * r];
            if (dim > 1) rw += w[1] * Rcart[3 * r + 1];
            if (dim > 2) rw += w[2] * Rcart[3 * r + 2];
            if (rw != 0.0) {
                double a[2] = {-u[2 * r + 1] * rw, u[2 * r] * rw}; /* i (w.R) u */
                p_zaxpy(&nn, a, ham + 2 * NN * r, &one, V + 2 * NN * p, &one);
            }
        }
    }
    for (int s = 0; s < N; ++s) {
        double t = tau[3 * s] * k[0];
        if (dim > 1) t += tau[3 * s + 1] * k[1];
        if (dim > 2) t += tau[3 * s + 2] * k[2];
        phi[2 * s] = cos(2.0 * M_PI * t);
        phi[2 * s + 1] = sin(2.0 * M_PI * t);
    }
    for (int p = 0; p < 2; ++p) {
        const double* w = dirs + p * dim;
        double* vv = V + 2 * NN * p;
        for (int m = 0; m < N; ++m) {
            double tm = w[0] * taucart[3 * m] + (dim > 1 ? w[1] * taucart[3 * m + 1] : 0) +
                        (dim > 2 ? w[2] * taucart[3 * m + 2] : 0);
            for (int n = 0; n < N; ++n) {
                double tn = w[0] * taucart[3 * n] + (dim > 1 ? w[1] * taucart[3 * n + 1] : 0) +
                            (dim > 2 ? w[2] * taucart[3 * n + 2] : 0);
                double diff = tn - tm;
                const size_t e = (size_t)m * N + n;
                double hr = H[2 * e], hi = H[2 * e + 1];
                double vr = vv[2 * e] - diff * hi, vi = vv[2 * e + 1] + diff * hr;
                /* * conj(phi_m) * phi_n */
                double gr = phi[2 * m] * phi[2 * n] + phi[2 * m + 1] * phi[2 * n + 1];
                double gi = phi[2 * m] * phi[2 * n + 1] - phi[2 * m + 1] * phi[2 * n];
                vv[2 * e] = vr * gr - vi * gi;
                vv[2 * e + 1] = vr * gi + vi * gr;
            }
        }
    }
    for (int m = 0; m < N; ++m)
        for (int n = 0; n < N; ++n) {
            const size_t e = (size_t)m * N + n;
            double gr = phi[2 * m] * phi[2 * n] + phi[2 * m + 1] * phi[2 * n + 1];
            double gi = phi[2 * m] * phi[2 * n + 1] - phi[2 * m + 1] * phi[2 * n];
            double hr = H[2 * e], hi = H[2 * e + 1];
            H[2 * e] = hr * gr - hi * gi;
            H[2 * e + 1] = hr * gi + hi * gr;
        }
    if (spin >= 0) { /* J = 1/2 {S, V_0}, S = sigma (x) I / 2 */
        double* V0 = V;
        memcpy(T, V0, sizeof(double) * 2 * NN);
        for (int i = 0; i < N; ++i)
            for (int j = 0; j < N; ++j) {
                int pi, pj;
                double sir, sii, sjr, sji;
#define SPIN_ENTRY(idx, pidx, sr, si)                                   \
    {                                                                   \
        int up = (idx) < norb;                                          \
        if (spin == 0) { pidx = up ? (idx) + norb : (idx) - norb; sr = 0.5; si = 0.0; } \
        else if (spin == 1) { pidx = up ? (idx) + norb : (idx) - norb; sr = 0.0; si = up ? -0.5 : 0.5; } \
        else { pidx = (idx); sr = up ? 0.5 : -0.5; si = 0.0; }         \
    }
                int ppj;
                SPIN_ENTRY(i, pi, sir, sii);
                SPIN_ENTRY(j, pj, sjr, sji);
                /* (V S)[i][j] = V[i][pi(j)] S[pi(j)][j]: the weight of row pi(j) */
                SPIN_ENTRY(pj, ppj, sjr, sji);
                (void)ppj;
                const double* a = T + 2 * ((size_t)pi * N + j);
                const double* b = T + 2 * ((size_t)i * N + pj);
                double ar = sir * a[0] - sii * a[1], ai = sir * a[1] + sii * a[0];
                double br = b[0] * sjr - b[1] * sji, bi = b[0] * sji + b[1] * sjr;
                V0[2 * ((size_t)i * N + j)] = 0.5 * (ar + br);
                V0[2 * ((size_t)i * N + j) + 1] = 0.5 * (ai + bi);
            }
    }
    int info = 0, n = N;
    p_zheev("V", "L", &n, H, &n, E, work, &lwork, rwork, &info, 1, 1);
    if (info != 0) return info;
    /* H now holds, row n (row-major view), the conjugated eigenvector n. */
    const double alpha[2] = {1.0, 0.0}, beta[2] = {0.0, 0.0};
    for (int p = 0; p < 2; ++p) {
        double* out = p == 0 ? Jb : Vb;
        p_zgemm(RowMajor, NoTrans, ConjTrans, N, N, N, alpha, V + 2 * NN * p, N, H, N, beta, T, N);
        p_zgemm(RowMajor, NoTrans, NoTrans, N, N, N, alpha, H, N, T, N, beta, out, N);
    }
    const double eta2 = eta * eta;
    for (int b = 0; b < N; ++b) {
        double v = 0.0;
        for (int o = 0; o < N; ++o) {
            if (o == b) continue;
            const double* x = Jb + 2 * ((size_t)b * N + o);
            const double* y = Vb + 2 * ((size_t)o * N + b);
            double im = x[0] * y[1] + x[1] * y[0];
            double d = E[b] - E[o];
            v += -2.0 * im / (d * d + eta2);
        }
        Om[b] = v;
    }
    return 0;
}

size_t port_workspace_doubles(int N, int nR) {
    const size_t NN = (size_t)N * N;
    return 14 * NN + 2 * (size_t)nR + 2 * (size_t)N + 2 * 66 * (size_t)N + 3 * (size_t)N + 64;
}

/* Occupation-weighted sums S[k][j] = sum_n Omega_n f(E_n, mu_j) over the k-points
 * of the uniform mesh with flat indices [k0, k0 + nk) (gen_kmesh order), or over
 * the explicit list klist (nk, dim) when klist != NULL.  Returns 0 or the first
 * non-zero LAPACK info. */
int port_hall_sums(int dim, int spin_model, int norb, int nR, const double* ham, const int64_t* hamR,
                   const double* orb, const double* lat, const int64_t* kmesh, int64_t k0, int64_t nk,
                   const double* klist, const double* dirs, int spin, double eta, int nmu, const double* mu,
                   double width, int nthreads, double* S, double* Om_out, double* E_out) {
    const int N = spin_model ? 2 * norb : norb;
    double* Rcart = (double*)calloc((size_t)nR * 3, sizeof(double));
    double* tau = (double*)calloc((size_t)N * 3, sizeof(double));
    double* taucart = (double*)calloc((size_t)N * 3, sizeof(double));
    for (int r = 0; r < nR; ++r)
        for (int c = 0; c < dim; ++c) {
            double s = 0;
            for (int d = 0; d < dim; ++d) s += (double)hamR[r * dim + d] * lat[d * dim + c];
            Rcart[3 * r + c] = s;
        }
    for (int s = 0; s < N; ++s) {
        int o = s % norb;
        for (int d = 0; d < dim; ++d) tau[3 * s + d] = orb[o * dim + d];
        for (int c = 0; c < dim; ++c) {
            double v = 0;
            for (int d = 0; d < dim; ++d) v += orb[o * dim + d] * lat[d * dim + c];
            taucart[3 * s + c] = v;
        }
    }
    const size_t wsz = port_workspace_doubles(N, nR);
    int err = 0;
#pragma omp parallel num_threads(nthreads)
    {
        double* ws = (double*)malloc(sizeof(double) * wsz);
        double* Om = (double*)malloc(sizeof(double) * N);
        double* E = (double*)malloc(sizeof(double) * N);
#pragma omp for schedule(dynamic, 1)
        for (int64_t t = 0; t < nk; ++t) {
            double k[3] = {0, 0, 0};
            if (klist) {
                for (int d = 0; d < dim; ++d) k[d] = klist[t * dim + d];
            } else {
                const int64_t idx = k0 + t;
                const int64_t n0 = kmesh[0], n1 = dim > 1 ? kmesh[1] : 1, n2 = dim > 2 ? kmesh[2] : 1;
                if (dim == 1) k[0] = (double)idx / (double)n0;
                if (dim == 2) { k[0] = (double)(idx / n1) / (double)n0; k[1] = (double)(idx % n1) / (double)n1; }
                if (dim == 3) {
                    k[0] = (double)(idx / (n1 * n2)) / (double)n0;
                    k[1] = (double)((idx / n2) % n1) / (double)n1;
                    k[2] = (double)(idx % n2) / (double)n2;
                }
            }
            int info = berry_one(dim, N, norb, nR, ham, hamR, Rcart, tau, taucart, k, dirs, spin, eta, Om, E, ws);
            if (info) {
#pragma omp critical
                err = info;
            }
            for (int j = 0; j < nmu; ++j) {
                double s = 0.0;
                for (int b = 0; b < N; ++b) s += Om[b] * fermi(E[b], mu[j], width);
                S[t * nmu + j] = s;
            }
            if (Om_out) memcpy(Om_out + t * N, Om, sizeof(double) * N);
            if (E_out) memcpy(E_out + t * N, E, sizeof(double) * N);
        }
        free(ws);
        free(Om);
        free(E);
    }
    free(Rcart);
    free(tau);
    free(taucart);
    return err;
}

/* H(k) in the Atom gauge (src/velocity.rs Fourier sum, then conj(phi_m) phi_n),
 * as berry_one builds it.  u: 2 nR, phi: 2 N scratch. */
static void ham_one(int dim, int N, int nR, const double* ham, const int64_t* hamR, const double* tau,
                    const double* k, double* H, double* u, double* phi) {
    const size_t NN = (size_t)N * N;
    const int one = 1, nn = (int)NN;
    memset(H, 0, sizeof(double) * 2 * NN);
    for (int r = 0; r < nR; ++r) {
        double s = (double)hamR[r * dim] * k[0];
        if (dim > 1) s += (double)hamR[r * dim + 1] * k[1];
        if (dim > 2) s += (double)hamR[r * dim + 2] * k[2];
        u[2 * r] = cos(2.0 * M_PI * s);
        u[2 * r + 1] = sin(2.0 * M_PI * s);
        p_zaxpy(&nn, u + 2 * r, ham + 2 * NN * r, &one, H, &one);
    }
    for (int s = 0; s < N; ++s) {
        double t = tau[3 * s] * k[0];
        if (dim > 1) t += tau[3 * s + 1] * k[1];
        if (dim > 2) t += tau[3 * s + 2] * k[2];
        phi[2 * s] = cos(2.0 * M_PI * t);
        phi[2 * s + 1] = sin(2.0 * M_PI * t);
    }
    for (int m = 0; m < N; ++m)
        for (int n = 0; n < N; ++n) {
            const size_t e = (size_t)m * N + n;
            double gr = phi[2 * m] * phi[2 * n] + phi[2 * m + 1] * phi[2 * n + 1];
            double gi = phi[2 * m] * phi[2 * n + 1] - phi[2 * m + 1] * phi[2 * n];
            double hr = H[2 * e], hi = H[2 * e + 1];
            H[2 * e] = hr * gr - hi * gi;
            H[2 * e + 1] = hr * gi + hi * gr;
        }
}

/* Model::dos (src/model_physics.rs:179-230) on the mesh points [k0, k0 + nk)
 * (gen_kmesh order): band energies by zheev JOBZ='N' (solve_band_onek,
 * src/solve_ham.rs:52-62), then, as the reference's fold does, every energy
 * against every one of the E_n grid points:
 *   A = (E_i - x) / sigma;  acc[i] += exp(-A^2 / 2) / sigma / sqrt(2 pi).
 * acc (E_n) receives the sum over the range (not divided by nk); threads keep
 * private accumulators that are added in thread order at the end.  Returns 0
 * or the first non-zero LAPACK info. */
int port_dos(int dim, int spin_model, int norb, int nR, const double* ham, const int64_t* hamR, const double* orb,
             const int64_t* kmesh, int64_t k0, int64_t nk, int64_t E_n, double E_min, double E_max, double sigma,
             int nthreads, double* acc) {
    const int N = spin_model ? 2 * norb : norb;
    const size_t NN = (size_t)N * N;
    double* tau = (double*)calloc((size_t)N * 3, sizeof(double));
    for (int s = 0; s < N; ++s)
        for (int d = 0; d < dim; ++d) tau[3 * s + d] = orb[(s % norb) * dim + d];
    const double step = E_n > 1 ? (E_max - E_min) / (double)(E_n - 1) : 0.0;
    const double sigma0 = 1.0 / sigma, pi0 = 1.0 / sqrt(2.0 * M_PI);
    double* Eg = (double*)malloc(sizeof(double) * E_n);
    for (int64_t i = 0; i < E_n; ++i) Eg[i] = E_min + step * (double)i;
    double* parts = (double*)calloc((size_t)nthreads * E_n, sizeof(double));
    int err = 0;
#pragma omp parallel num_threads(nthreads)
    {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        double* mine = parts + (size_t)tid * E_n;
        const int lwork = 66 * N;
        double* H = (double*)malloc(sizeof(double) * (2 * NN + 2 * (size_t)nR + 2 * (size_t)N + 2 * (size_t)lwork +
                                                      3 * (size_t)N + (size_t)N));
        double* u = H + 2 * NN;
        double* phi = u + 2 * nR;
        double* work = phi + 2 * N;
        double* rwork = work + 2 * lwork;
        double* E = rwork + 3 * N;
#pragma omp for schedule(dynamic, 16)
        for (int64_t t = 0; t < nk; ++t) {
            double k[3] = {0, 0, 0};
            const int64_t idx = k0 + t;
            const int64_t n0 = kmesh[0], n1 = dim > 1 ? kmesh[1] : 1, n2 = dim > 2 ? kmesh[2] : 1;
            if (dim == 1) k[0] = (double)idx / (double)n0;
            if (dim == 2) { k[0] = (double)(idx / n1) / (double)n0; k[1] = (double)(idx % n1) / (double)n1; }
            if (dim == 3) {
                k[0] = (double)(idx / (n1 * n2)) / (double)n0;
                k[1] = (double)((idx / n2) % n1) / (double)n1;
                k[2] = (double)(idx % n2) / (double)n2;
            }
            ham_one(dim, N, nR, ham, hamR, tau, k, H, u, phi);
            int info = 0, n = N;
            p_zheev("N", "L", &n, H, &n, E, work, &lwork, rwork, &info, 1, 1);
            if (info) {
#pragma omp critical
                err = info;
            }
            for (int b = 0; b < N; ++b) {
                const double x = E[b];
                for (int64_t i = 0; i < E_n; ++i) {
                    const double A = (Eg[i] - x) * sigma0;
                    mine[i] += exp(-A * A / 2.0) * sigma0 * pi0;
                }
            }
        }
        free(H);
    }
    for (int t = 0; t < nthreads; ++t)
        for (int64_t i = 0; i < E_n; ++i) acc[i] += parts[(size_t)t * E_n + i];
    free(parts);
    free(Eg);
    free(tau);
    return err;
}

/* Wannier90 _hr.dat as from_hr reads it (src/wannier90.rs:85-245), on one
 * thread: every line kept, then the values taken by position (tokens 5 and 6
 * of each data line) and divided by the block's weight.  ham_out receives the
 * n_R blocks in file order (n_R, nsta, nsta) complex, transposed as the
 * reference stores them.  Returns n_R * nsta^2, or -1 on a malformed file. */
int64_t port_read_hr(const char* path, double zero_energy, double* ham_out, int64_t cap_values) {
    FILE* f = fopen(path, "r");
    if (!f) return -1;
    size_t nl = 0, capl = 1024;
    char** lines = (char**)malloc(sizeof(char*) * capl);
    char* buf = NULL;
    size_t bl = 0;
    ssize_t got;
    while ((got = getline(&buf, &bl, f)) >= 0) {
        if (nl == capl) {
            capl *= 2;
            lines = (char**)realloc(lines, sizeof(char*) * capl);
        }
        lines[nl++] = strdup(buf);
    }
    free(buf);
    fclose(f);
    int64_t result = -1;
    if (nl >= 3) {
        const long nsta = strtol(lines[1], NULL, 10), n_R = strtol(lines[2], NULL, 10);
        long* w = (long*)malloc(sizeof(long) * (n_R > 0 ? n_R : 1));
        long nw = 0;
        size_t n_line = 0;
        for (size_t i = 3; i < nl; ++i) {
            if (strchr(lines[i], '.')) {
                n_line = i;
                break;
            }
            char* p = lines[i];
            char* e;
            for (long v = strtol(p, &e, 10); e != p; v = strtol(p, &e, 10)) {
                if (nw < n_R) w[nw++] = v;
                p = e;
            }
        }
        const int64_t NN = (int64_t)nsta * nsta;
        if (nsta > 0 && nw >= n_R && n_line + (size_t)(n_R * NN) <= nl && n_R * NN * 2 <= cap_values) {
            for (long r = 0; r < n_R; ++r)
                for (long a = 0; a < nsta; ++a)
                    for (long b = 0; b < nsta; ++b) {
                        char* p = lines[n_line + r * NN + a * nsta + b];
                        char* e;
                        for (int t = 0; t < 5; ++t) {
                            strtod(p, &e);
                            p = e;
                        }
                        const double re = strtod(p, &e);
                        p = e;
                        const double im = strtod(p, &e);
                        double* o = ham_out + 2 * (r * NN + b * nsta + a);
                        o[0] = re / (double)w[r];
                        o[1] = im / (double)w[r];
                    }
            (void)zero_energy;
            result = n_R * NN;
        }
        free(w);
    }
    for (size_t i = 0; i < nl; ++i) free(lines[i]);
    free(lines);
    return result;
}
