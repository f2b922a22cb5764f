// Wilson loops over closed k-paths (src/geometry.rs:156-270): for loop l with
// points k_0 .. k_{T} (k_T = k_0 + G, G integer), occupied bands occ,
//   O_t[i][j] = <u_occ_i(k_t) | u_occ_j(k_t+1)>,   t = 0 .. T-1,
//   u(k_T) = diag(exp(-2 pi i G . tau)) u(k_0)        (the loop's periodic gauge),
// SVD mode (berry_loop): W_t = U V^dagger of O_t = U S V^dagger, P = W_0 ... W_{T-1},
//   phases = -arg(eigenvalues of P);
// det mode (berry_loop_det): P = O_0 ... O_{T-1}, phase = -arg det P.
// Eigenvectors are the columns of the batched FP64 eigensolver's U at the
// Atom-gauge H(k_t) (solve_all, src/solve_ham.rs:110-184).
//
// GB300 form: one block per segment forms O_t from the eigenvector columns
// (L2-resident) and, in another launch, takes it to its unitary factor by the
// Newton-Schulz iteration X <- X (3 - X^dagger X) / 2 (the singular values of
// an overlap of orthonormal sets lie in (0, 1], where it converges
// quadratically; a bounded number of steps, a singular overlap -- the gap
// closing on the path -- is reported); one block per loop multiplies the
// chain in shared memory.  P is unitary, so its eigenvectors are those of the Hermitian
// Re(e^{-i phi} P) = (e^{-i phi} P + e^{i phi} P^dagger) / 2 (eigenvalues
// cos(theta - phi), distinct unless theta_i + theta_j = 2 phi): that matrix
// goes through the batched Hermitian eigensolver for two angles phi, and
// lambda_j = v_j^dagger P v_j is taken from the angle whose |lambda| are
// closest to 1.  The phases of a loop are returned in ascending order (the
// reference returns LAPACK zgeev's order, which carries no meaning).

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "tbgpu_internal.cuh"

namespace tbg {
namespace {

constexpr double kTwoPiW = 6.283185307179586476925286766559;
constexpr int kMaxNS = 80;  // Newton-Schulz steps (quadratic from sigma_min >= 1e-6 needs ~45)

// endphase[l][a] = exp(-2 pi i (k_T - k_0) . tau_a)
__global__ void wl_endphase_kernel(int64_t n_loops, int n_k, int dim, const double* __restrict__ kv, int N,
                                   const double* __restrict__ tau, zc* __restrict__ endphase) {
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < n_loops * N;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t l = idx / N;
        const int a = (int)(idx % N);
        const double* k0 = kv + (l * n_k) * dim;
        const double* kT = kv + (l * n_k + n_k - 1) * dim;
        double x = 0.0;
        for (int d = 0; d < dim; ++d) x += (kT[d] - k0[d]) * tau[3 * a + d];
        double s, c;
        sincos(-kTwoPiW * x, &s, &c);
        endphase[idx] = mk(c, s);
    }
}

// O[l][t] (n_occ x n_occ) from the eigenvector matrices U[l][t] (N x N, columns),
// t = 0 .. T-1, T = n_k - 1 points solved per loop.
__global__ void __launch_bounds__(256) wl_overlap_kernel(int N, int n_occ, int T, const zc* __restrict__ U,
                                                         const int* __restrict__ occ,
                                                         const zc* __restrict__ endphase, zc* __restrict__ O) {
    const int64_t seg = blockIdx.x;  // l * T + t
    const int64_t l = seg / T;
    const int t = (int)(seg % T);
    const int64_t NN = (int64_t)N * N;
    const zc* A = U + (l * T + t) * NN;
    const bool last = (t == T - 1);
    const zc* B = U + (l * T + (last ? 0 : t + 1)) * NN;
    const zc* ph = endphase + l * N;
    zc* Ob = O + seg * (int64_t)n_occ * n_occ;
    for (int e = threadIdx.x; e < n_occ * n_occ; e += blockDim.x) {
        const int i = e / n_occ, j = e % n_occ;
        const int ci = occ[i], cj = occ[j];
        zc s = mk(0.0, 0.0);
        for (int a = 0; a < N; ++a) {
            zc b = B[(int64_t)a * N + cj];
            if (last) b = ph[a] * b;
            fma_cjx(s, A[(int64_t)a * N + ci], b);
        }
        Ob[e] = s;
    }
}

// C = A B (n x n, shared memory), all threads of the block.
__device__ void smem_mm(int n, const zc* A, const zc* B, zc* C) {
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
        const int i = e / n, j = e % n;
        zc s = mk(0.0, 0.0);
        for (int k = 0; k < n; ++k) fma_cx(s, A[i * n + k], B[k * n + j]);
        C[e] = s;
    }
}

// O[seg] <- its unitary factor U V^dagger, one block per segment, by the
// Newton-Schulz iteration: stop when X is unitary to rounding, or one step
// after the error fell below 1e-8 (that step squares it).
__global__ void __launch_bounds__(256) wl_polar_kernel(int n, zc* __restrict__ O, int* __restrict__ status) {
    extern __shared__ zc wsm[];
    zc* X = wsm;
    zc* Y = X + n * n;
    zc* Z = Y + n * n;
    __shared__ double s_err;
    const int nn = n * n;
    zc* Ot = O + (int64_t)blockIdx.x * nn;
    for (int e = threadIdx.x; e < nn; e += blockDim.x) X[e] = Ot[e];
    __syncthreads();
    double err = 1.0;
    for (int it = 0; it < kMaxNS; ++it) {
        // Y = X^dagger X
        for (int e = threadIdx.x; e < nn; e += blockDim.x) {
            const int i = e / n, j = e % n;
            zc s = mk(0.0, 0.0);
            for (int k = 0; k < n; ++k) fma_cjx(s, X[k * n + i], X[k * n + j]);
            Y[e] = s;
        }
        if (threadIdx.x == 0) s_err = 0.0;
        __syncthreads();
        double m = 0.0;
        for (int e = threadIdx.x; e < nn; e += blockDim.x) {
            const double dr = Y[e].re - ((e / n == e % n) ? 1.0 : 0.0);
            m = fmax(m, fabs(dr) + fabs(Y[e].im));
        }
        // block max (non-negative doubles order like their bit patterns)
        atomicMax(reinterpret_cast<unsigned long long*>(&s_err), (unsigned long long)__double_as_longlong(m));
        __syncthreads();
        err = s_err;
        if (err <= 4e-16 * n) break;  // uniform: every thread read the same s_err
        // Y <- (3 I - Y) / 2, X <- X Y
        for (int e = threadIdx.x; e < nn; e += blockDim.x)
            Y[e] = mk(((e / n == e % n) ? 1.5 : 0.0) - 0.5 * Y[e].re, -0.5 * Y[e].im);
        __syncthreads();
        smem_mm(n, X, Y, Z);
        __syncthreads();
        for (int e = threadIdx.x; e < nn; e += blockDim.x) X[e] = Z[e];
        __syncthreads();
        if (err <= 1e-8) {
            err = 0.0;
            break;
        }
    }
    for (int e = threadIdx.x; e < nn; e += blockDim.x) Ot[e] = X[e];
    if (threadIdx.x == 0 && err > 1e-8) atomicOr(status, 4);
}

// P[l] = O[l][0] ... O[l][T-1] (unitary factors in SVD mode, raw overlaps in det mode).
__global__ void __launch_bounds__(256) wl_chain_kernel(int n, int T, const zc* __restrict__ O, zc* __restrict__ P) {
    extern __shared__ zc wsm[];
    zc* X = wsm;
    zc* Z = X + n * n;
    zc* Pc = Z + n * n;
    const int64_t l = blockIdx.x;
    const int nn = n * n;
    for (int e = threadIdx.x; e < nn; e += blockDim.x) Pc[e] = mk((e / n == e % n) ? 1.0 : 0.0, 0.0);
    __syncthreads();
    for (int t = 0; t < T; ++t) {
        const zc* Ot = O + (l * T + t) * (int64_t)nn;
        for (int e = threadIdx.x; e < nn; e += blockDim.x) X[e] = Ot[e];
        __syncthreads();
        smem_mm(n, Pc, X, Z);  // Pc <- Pc X
        __syncthreads();
        for (int e = threadIdx.x; e < nn; e += blockDim.x) Pc[e] = Z[e];
        __syncthreads();
    }
    for (int e = threadIdx.x; e < nn; e += blockDim.x) P[l * nn + e] = Pc[e];
}

// Hz[l] = (e^{-i phi} P + e^{i phi} P^dagger) / 2
__global__ void wl_hermitian_kernel(int64_t n_loops, int n, double phi, const zc* __restrict__ P,
                                    zc* __restrict__ Hz) {
    const int64_t nn = (int64_t)n * n;
    double s, c;
    sincos(phi, &s, &c);
    const zc w = mk(c, -s), wc = mk(c, s);
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < n_loops * nn;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t l = idx / nn;
        const int e = (int)(idx % nn), i = e / n, j = e % n;
        const zc a = w * P[l * nn + i * n + j];
        const zc b = wc * conj(P[l * nn + j * n + i]);
        Hz[idx] = mk(0.5 * (a.re + b.re), 0.5 * (a.im + b.im));
    }
}

// For each loop: lambda_j = v_j^dagger P v_j from the eigenvectors V (columns) of
// the two Hermitian combinations; keep the angle whose min |lambda| is larger;
// phases -arg(lambda), ascending.
__global__ void wl_phases_kernel(int64_t n_loops, int n, const zc* __restrict__ P, const zc* __restrict__ V1,
                                 const zc* __restrict__ V2, double* __restrict__ out) {
    extern __shared__ double ph_sm[];  // 2n phases + 2 mins
    double* ph = ph_sm;
    __shared__ double s_min[2];
    const int64_t nn = (int64_t)n * n;
    for (int64_t l = blockIdx.x; l < n_loops; l += gridDim.x) {
        const zc* Pl = P + l * nn;
        if (threadIdx.x < 2) s_min[threadIdx.x] = 2.0;
        __syncthreads();
        for (int q = threadIdx.x; q < 2 * n; q += blockDim.x) {
            const int pass = q / n, j = q % n;
            const zc* V = (pass == 0 ? V1 : V2) + l * nn;
            zc lam = mk(0.0, 0.0);
            for (int a = 0; a < n; ++a) {
                zc pv = mk(0.0, 0.0);
                for (int b = 0; b < n; ++b) fma_cx(pv, Pl[a * n + b], V[(int64_t)b * n + j]);
                fma_cjx(lam, V[(int64_t)a * n + j], pv);
            }
            ph[q] = -atan2(lam.im, lam.re);
            const double mag = sqrt(abs2(lam));
            atomicMin(reinterpret_cast<unsigned long long*>(&s_min[pass]),
                      (unsigned long long)__double_as_longlong(mag));
        }
        __syncthreads();
        const int pass = (s_min[0] >= s_min[1]) ? 0 : 1;
        // rank sort of the chosen pass (n is small)
        for (int j = threadIdx.x; j < n; j += blockDim.x) {
            const double v = ph[pass * n + j];
            int r = 0;
            for (int q = 0; q < n; ++q) {
                const double u = ph[pass * n + q];
                r += (u < v) || (u == v && q < j);
            }
            out[l * n + r] = v;
        }
        __syncthreads();
    }
}

// det mode: -arg det P[l] by LU with partial pivoting (one thread per loop; n small).
__global__ void wl_det_kernel(int64_t n_loops, int n, zc* __restrict__ P, double* __restrict__ out) {
    const int64_t nn = (int64_t)n * n;
    for (int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; l < n_loops;
         l += (int64_t)gridDim.x * blockDim.x) {
        zc* A = P + l * nn;
        zc det = mk(1.0, 0.0);
        for (int k = 0; k < n; ++k) {
            int p = k;
            double best = abs2(A[k * n + k]);
            for (int i = k + 1; i < n; ++i) {
                const double v = abs2(A[i * n + k]);
                if (v > best) {
                    best = v;
                    p = i;
                }
            }
            if (p != k) {
                for (int j = 0; j < n; ++j) {
                    const zc tmp = A[k * n + j];
                    A[k * n + j] = A[p * n + j];
                    A[p * n + j] = tmp;
                }
                det = mk(-det.re, -det.im);
            }
            const zc piv = A[k * n + k];
            det = det * piv;
            if (best == 0.0) break;
            const double inv = 1.0 / best;
            const zc rp = mk(piv.re * inv, -piv.im * inv);  // 1 / piv
            for (int i = k + 1; i < n; ++i) {
                const zc f = A[i * n + k] * rp;
                for (int j = k + 1; j < n; ++j) A[i * n + j] = A[i * n + j] - f * A[k * n + j];
            }
        }
        out[l] = -atan2(det.im, det.re);
    }
}

template <typename K>
int wl_allow_smem(K kern, size_t need) {
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaFuncAttributes fa;
    cudaError_t e = cudaFuncGetAttributes(&fa, kern);
    if (e != cudaSuccess) return cuda_error(e, "cudaFuncGetAttributes(wilson kernel)");
    // static and dynamic shared memory together stay within the opt-in limit
    const int dyn_max = optin - (int)fa.sharedSizeBytes;
    if (need > (size_t)dyn_max) return set_error(TBG_E_UNSUPPORTED, "Wilson loop: too many occupied bands");
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn_max);
    if (e != cudaSuccess) return cuda_error(e, "cudaFuncSetAttribute(wilson kernel)");
    return TBG_OK;
}

inline unsigned nblk(int64_t total) {
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>((total + 255) / 256, 152LL * 64));
}

}  // namespace

size_t wilson_chain_smem(int n_occ) { return sizeof(zc) * 3 * (size_t)n_occ * n_occ; }

// kv_d: (n_loops, n_k, dim) k-points; U: eigenvectors at points t < n_k - 1 of
// every loop, (n_loops * (n_k - 1), N, N).  out: (n_loops, n_occ) or (n_loops).
int wilson_from_vectors(cudaStream_t st, const ModelDev& m, int64_t n_loops, int n_k, const double* kv_d, const zc* U,
                        int n_occ, const int* occ_d, int svd, double* out, void* work, size_t work_bytes,
                        int* status_d) {
    if (n_loops <= 0) return TBG_OK;
    const int N = (int)m.nsta, T = n_k - 1;
    const int64_t nn = (int64_t)n_occ * n_occ;
    unsigned char* p = static_cast<unsigned char*>(work);
    auto take = [&](size_t b) {
        void* q = p;
        p += (b + 255) & ~size_t(255);
        return q;
    };
    zc* endph = static_cast<zc*>(take(sizeof(zc) * n_loops * N));
    zc* O = static_cast<zc*>(take(sizeof(zc) * n_loops * std::max(T, 1) * nn));
    zc* P = static_cast<zc*>(take(sizeof(zc) * n_loops * nn));
    zc* Hz = static_cast<zc*>(take(sizeof(zc) * n_loops * nn));
    zc* V1 = static_cast<zc*>(take(sizeof(zc) * n_loops * nn));
    zc* V2 = static_cast<zc*>(take(sizeof(zc) * n_loops * nn));
    double* Ez = static_cast<double*>(take(sizeof(double) * n_loops * n_occ));
    if ((size_t)(p - static_cast<unsigned char*>(work)) > work_bytes)
        return set_error(TBG_E_OOM, "wilson workspace too small");
    if (T > 0) {
        wl_endphase_kernel<<<nblk(n_loops * N), 256, 0, st>>>(n_loops, n_k, m.dim, kv_d, N, m.tau_d, endph);
        TBG_LAUNCHED("wl_endphase_kernel");
        KTimer kt(st, "wl_overlap_kernel");
        wl_overlap_kernel<<<(unsigned)(n_loops * T), 256, 0, st>>>(N, n_occ, T, U, occ_d, endph, O);
        TBG_LAUNCHED("wl_overlap_kernel");
    }
    const size_t smem = wilson_chain_smem(n_occ);
    if (svd && T > 0) {
        KTimer kt(st, "wl_polar_kernel");
        if (int rc = wl_allow_smem(wl_polar_kernel, smem)) return rc;
        wl_polar_kernel<<<(unsigned)(n_loops * T), 256, smem, st>>>(n_occ, O, status_d);
        TBG_LAUNCHED("wl_polar_kernel");
    }
    {
        KTimer kt(st, "wl_chain_kernel");
        if (int rc = wl_allow_smem(wl_chain_kernel, smem)) return rc;
        wl_chain_kernel<<<(unsigned)n_loops, 256, smem, st>>>(n_occ, T, O, P);
        TBG_LAUNCHED("wl_chain_kernel");
    }
    if (!svd) {
        wl_det_kernel<<<nblk(n_loops), 256, 0, st>>>(n_loops, n_occ, P, out);
        TBG_LAUNCHED("wl_det_kernel");
        return TBG_OK;
    }
    const double phis[2] = {0.7390851332151607, 2.3999632297286535};  // two generic angles
    zc* Vs[2] = {V1, V2};
    for (int q = 0; q < 2; ++q) {
        wl_hermitian_kernel<<<nblk(n_loops * nn), 256, 0, st>>>(n_loops, n_occ, phis[q], P, Hz);
        TBG_LAUNCHED("wl_hermitian_kernel");
        if (int rc = eig_batched(st, n_occ, n_loops, Hz, Ez, Vs[q], nullptr, 0, status_d)) return rc;
    }
    wl_phases_kernel<<<(unsigned)std::min<int64_t>(n_loops, 152 * 16), 128, sizeof(double) * 2 * n_occ, st>>>(
        n_loops, n_occ, P, V1, V2, out);
    TBG_LAUNCHED("wl_phases_kernel");
    return TBG_OK;
}

size_t wilson_workspace_bytes(int N, int64_t n_loops, int n_k, int n_occ) {
    const size_t nn = (size_t)n_occ * n_occ;
    const size_t T = (size_t)std::max(n_k - 1, 1);
    return sizeof(zc) * n_loops * ((size_t)N + T * nn + 4 * nn) + sizeof(double) * n_loops * n_occ + 8 * 256;
}

}  // namespace tbg
