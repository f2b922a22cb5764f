// Fused path for small models (nsta <= 8): one thread per k-point runs the
// whole of berry_curvature_at_impl (src/response/traits.rs:160-200) in
// registers / local memory, FP64:
//   H, V_0, V_1 by the Fourier sum over R with the Atom gauge and tau term
//   (src/velocity.rs:538-622), optional spin dressing (traits.rs:170-175),
//   eigenpairs by cyclic complex Jacobi, U^H V U, Omega_n (and optionally
//   the quantum metric, src/quantum_geometry.rs:160-187), and the
//   occupation sums per chemical potential (linear/mod.rs:204-223).
// For nsta <= 8 the per-k work is a few thousand flops, so one launch covers
// tens of thousands of k-points and the batched per-matrix kernels would be
// dominated by launch and synchronisation overhead.

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "tbgpu_internal.cuh"

namespace tbg {
namespace {

constexpr double kTwoPiS = 6.283185307179586476925286766559;

__device__ __forceinline__ double fermi_s(double e, double mu, double width) {
    if (width == 0.0) return (e < mu) ? 1.0 : ((e > mu) ? 0.0 : 0.5);
    const double x = (e - mu) / width;
    if (x > 50.0) return 0.0;
    if (x < -50.0) return 1.0;
    return 1.0 / (1.0 + exp(x));
}

// Cyclic complex Jacobi on the Hermitian NM x NM (active N) matrix A; W gets
// the eigenvectors in columns.  Rotation: G = diag(1, e^{-i phi}) [[c,-s],[s,c]]
// with e^{i phi} = a_pq / |a_pq|, tan 2 theta = 2 |a_pq| / (a_pp - a_qq).
template <int NM, bool WANT_W>
__device__ void jacobi(int N, zc (&A)[NM][NM], zc (&W)[NM][NM]) {
    if (WANT_W)
        for (int i = 0; i < NM; ++i)
            for (int j = 0; j < NM; ++j) W[i][j] = mk(i == j ? 1.0 : 0.0, 0.0);
    for (int sweep = 0; sweep < 40; ++sweep) {
        double off = 0.0, dia = 0.0;
        for (int i = 0; i < N; ++i)
            for (int j = 0; j < N; ++j) {
                if (i != j)
                    off += abs2(A[i][j]);
                else
                    dia += abs2(A[i][j]);
            }
        if (off <= 1e-32 * dia || off == 0.0) break;
        for (int p = 0; p < N - 1; ++p)
            for (int q = p + 1; q < N; ++q) {
                const zc apq = A[p][q];
                const double mag = sqrt(abs2(apq));
                if (mag == 0.0) continue;
                const double app = A[p][p].re, aqq = A[q][q].re;
                const zc ph = mk(apq.re / mag, apq.im / mag);
                const zc emi = conj(ph);
                const double theta = 0.5 * atan2(2.0 * mag, app - aqq);
                double sn, cs;
                sincos(theta, &sn, &cs);
                for (int k = 0; k < N; ++k) {
                    const zc akp = A[k][p], akq = emi * A[k][q];
                    A[k][p] = cs * akp + sn * akq;
                    A[k][q] = cs * akq - sn * akp;
                }
                for (int k = 0; k < N; ++k) {
                    const zc apk = A[p][k], aqk = ph * A[q][k];
                    A[p][k] = cs * apk + sn * aqk;
                    A[q][k] = cs * aqk - sn * apk;
                }
                A[p][q] = mk(0.0, 0.0);
                A[q][p] = mk(0.0, 0.0);
                A[p][p].im = 0.0;
                A[q][q].im = 0.0;
                if (WANT_W)
                    for (int k = 0; k < N; ++k) {
                        const zc wkp = W[k][p], wkq = emi * W[k][q];
                        W[k][p] = cs * wkp + sn * wkq;
                        W[k][q] = cs * wkq - sn * wkp;
                    }
            }
    }
}

// VALS: band energies only (E_out); no velocities, eigenvectors or curvature.
template <int NM, bool VALS>
__global__ void __launch_bounds__(128) small_fused_kernel(
    int N, int norb, int dim, int nR, int64_t nk, const double* __restrict__ klist, int64_t k0, int64_t n0,
    int64_t n1, int64_t n2, const zc* __restrict__ ham, const int* __restrict__ hamR, const double* __restrict__ Rcart,
    const double* __restrict__ tau, const double* __restrict__ taucart, const double* __restrict__ dirs, int spin,
    double eta, int nmu, const double* __restrict__ mu, double width, double* __restrict__ Om_out,
    double* __restrict__ E_out, double* __restrict__ S_out, double* __restrict__ Met_out, double* __restrict__ SM_out) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= nk) return;
    double kv[3] = {0.0, 0.0, 0.0};
    if (klist) {
        for (int d = 0; d < dim; ++d) kv[d] = klist[t * dim + d];
    } else {
        const int64_t idx = k0 + t;  // gen_kmesh order (src/kpoints.rs:49-87)
        if (dim == 1) {
            kv[0] = (double)idx / (double)n0;
        } else if (dim == 2) {
            kv[0] = (double)(idx / n1) / (double)n0;
            kv[1] = (double)(idx % n1) / (double)n1;
        } else {
            kv[0] = (double)(idx / (n1 * n2)) / (double)n0;
            kv[1] = (double)((idx / n2) % n1) / (double)n1;
            kv[2] = (double)(idx % n2) / (double)n2;
        }
    }
    zc H[NM][NM], V0[NM][NM], V1[NM][NM];
    for (int i = 0; i < NM; ++i)
        for (int j = 0; j < NM; ++j) H[i][j] = V0[i][j] = V1[i][j] = mk(0.0, 0.0);
    const double* w0 = dirs;
    const double* w1 = dirs + dim;
    for (int r = 0; r < nR; ++r) {
        const int* R = hamR + 3 * r;
        double s = (double)R[0] * kv[0];
        if (dim > 1) s += (double)R[1] * kv[1];
        if (dim > 2) s += (double)R[2] * kv[2];
        double sn, cs;
        sincos(kTwoPiS * s, &sn, &cs);
        const zc u = mk(cs, sn);
        const zc* hr = ham + (int64_t)r * N * N;
        if (VALS) {
            for (int i = 0; i < N; ++i)
                for (int j = 0; j < N; ++j) H[i][j] = H[i][j] + u * hr[i * N + j];
            continue;
        }
        const double* rc = Rcart + 3 * r;
        double c0 = w0[0] * rc[0], c1 = w1[0] * rc[0];
        if (dim > 1) {
            c0 += w0[1] * rc[1];
            c1 += w1[1] * rc[1];
        }
        if (dim > 2) {
            c0 += w0[2] * rc[2];
            c1 += w1[2] * rc[2];
        }
        for (int i = 0; i < N; ++i)
            for (int j = 0; j < N; ++j) {
                const zc tt = u * hr[i * N + j];
                H[i][j] = H[i][j] + tt;
                V0[i][j] = V0[i][j] + mk(-c0 * tt.im, c0 * tt.re);  // i c0 t
                V1[i][j] = V1[i][j] + mk(-c1 * tt.im, c1 * tt.re);
            }
    }
    // Atom gauge + tau term
    zc ph[NM];
    double tp0[NM], tp1[NM];
    // energies only: the Atom-gauge phase is a unitary similarity and leaves them unchanged
    for (int s = 0; s < (VALS ? 0 : N); ++s) {
        const double* ts = tau + 3 * s;
        double a = ts[0] * kv[0];
        if (dim > 1) a += ts[1] * kv[1];
        if (dim > 2) a += ts[2] * kv[2];
        double sn, cs;
        sincos(kTwoPiS * a, &sn, &cs);
        ph[s] = mk(cs, sn);
        const double* tc = taucart + 3 * s;
        double p0 = w0[0] * tc[0], p1 = w1[0] * tc[0];
        if (dim > 1) {
            p0 += w0[1] * tc[1];
            p1 += w1[1] * tc[1];
        }
        if (dim > 2) {
            p0 += w0[2] * tc[2];
            p1 += w1[2] * tc[2];
        }
        tp0[s] = p0;
        tp1[s] = p1;
    }
    for (int m = 0; m < (VALS ? 0 : N); ++m)
        for (int n = 0; n < N; ++n) {
            const zc g = cmul(ph[m], ph[n]);
            const zc hl = H[m][n];
            const double d0 = tp0[n] - tp0[m], d1 = tp1[n] - tp1[m];
            V0[m][n] = (V0[m][n] + mk(-d0 * hl.im, d0 * hl.re)) * g;
            V1[m][n] = (V1[m][n] + mk(-d1 * hl.im, d1 * hl.re)) * g;
            H[m][n] = hl * g;
        }
    if (!VALS && spin >= 0) {  // J = 1/2 (S V0 + V0 S), S = sigma (x) I / 2
        zc J[NM][NM];
        for (int i = 0; i < N; ++i)
            for (int j = 0; j < N; ++j) {
                auto ent = [&](int x, int& px, zc& sx) {
                    const bool up = x < norb;
                    if (spin == TBG_SPIN_X) {
                        px = up ? x + norb : x - norb;
                        sx = mk(0.5, 0.0);
                    } else if (spin == TBG_SPIN_Y) {
                        px = up ? x + norb : x - norb;
                        sx = up ? mk(0.0, -0.5) : mk(0.0, 0.5);
                    } else {
                        px = x;
                        sx = up ? mk(0.5, 0.0) : mk(-0.5, 0.0);
                    }
                };
                int pi, pj, ppj;
                zc si, sj;
                ent(i, pi, si);
                ent(j, pj, sj);
                ent(pj, ppj, sj);  // (V S)[i][j] = V[i][pi(j)] S[pi(j)][j]
                const zc a = si * V0[pi][j];
                const zc c = V0[i][pj] * sj;
                J[i][j] = mk(0.5 * (a.re + c.re), 0.5 * (a.im + c.im));
            }
        for (int i = 0; i < N; ++i)
            for (int j = 0; j < N; ++j) V0[i][j] = J[i][j];
    }
    zc W[NM][NM];
    jacobi<NM, !VALS>(N, H, W);
    double E[NM];
    int ord[NM];
    for (int i = 0; i < N; ++i) {
        E[i] = H[i][i].re;
        ord[i] = i;
    }
    for (int i = 1; i < N; ++i) {  // ascending order (insertion sort of the index)
        const int oi = ord[i];
        int j = i - 1;
        while (j >= 0 && E[ord[j]] > E[oi]) {
            ord[j + 1] = ord[j];
            --j;
        }
        ord[j + 1] = oi;
    }
    if (VALS) {
        for (int i = 0; i < N; ++i) E_out[t * N + i] = E[ord[i]];
        return;
    }
    // band-basis velocities B = W^H V W (H reused as scratch)
    zc Bx[NM][NM], By[NM][NM];
    for (int a = 0; a < N; ++a)
        for (int b = 0; b < N; ++b) {
            zc sx = mk(0.0, 0.0), sy = mk(0.0, 0.0);
            for (int i = 0; i < N; ++i) {
                zc tx = mk(0.0, 0.0), ty = mk(0.0, 0.0);
                for (int j = 0; j < N; ++j) {
                    fma_cx(tx, V0[i][j], W[j][b]);
                    fma_cx(ty, V1[i][j], W[j][b]);
                }
                fma_cjx(sx, W[i][a], tx);
                fma_cjx(sy, W[i][a], ty);
            }
            Bx[a][b] = sx;
            By[a][b] = sy;
        }
    const double eta2 = eta * eta;
    const bool met = Met_out || SM_out;
    double Om[NM], G[NM];
    for (int a = 0; a < N; ++a) {
        double v = 0.0, g = 0.0;
        for (int b = 0; b < N; ++b) {
            if (a == b) continue;
            const double im = Bx[a][b].re * By[b][a].im + Bx[a][b].im * By[b][a].re;
            const double de = E[a] - E[b];
            const double den = de * de + eta2;
            v += -2.0 * im / den;
            if (met) g += (Bx[a][b].re * By[b][a].re - Bx[a][b].im * By[b][a].im) / den;
        }
        Om[a] = v;
        G[a] = g;
    }
    for (int i = 0; i < N; ++i) {
        if (Om_out) Om_out[t * N + i] = Om[ord[i]];
        if (E_out) E_out[t * N + i] = E[ord[i]];
        if (Met_out) Met_out[t * N + i] = G[ord[i]];
    }
    if (S_out) {
        for (int j = 0; j < nmu; ++j) {
            double s = 0.0, sg = 0.0;
            for (int i = 0; i < N; ++i) {
                const double f = fermi_s(E[ord[i]], mu[j], width);
                s += Om[ord[i]] * f;
                sg += G[ord[i]] * f;
            }
            S_out[t * nmu + j] = s;
            if (SM_out) SM_out[t * nmu + j] = sg;
        }
    }
}

// Eigenpairs of batched N x N (N <= 8) Hermitian matrices, one thread per
// matrix: cyclic Jacobi in registers, E ascending, U with the eigenvectors in
// columns (row-major, the layout of the batched solver); U may be null.
// Non-finite input sets bit 0 of *status, as the batched solver does.
template <int NM>
__global__ void __launch_bounds__(128) small_eig_kernel(int N, int64_t batch, const zc* __restrict__ H,
                                                       double* __restrict__ E_out, zc* __restrict__ U_out,
                                                       int* __restrict__ status) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= batch) return;
    const int64_t NN = (int64_t)N * N;
    zc A[NM][NM], W[NM][NM];
    for (int i = 0; i < NM; ++i)
        for (int j = 0; j < NM; ++j) A[i][j] = (i < N && j < N) ? H[t * NN + i * N + j] : mk(0.0, 0.0);
    jacobi<NM, true>(N, A, W);
    double E[NM];
    int ord[NM];
    for (int i = 0; i < N; ++i) {
        E[i] = A[i][i].re;
        ord[i] = i;
    }
    for (int i = 1; i < N; ++i) {  // ascending (insertion sort of the index)
        const int oi = ord[i];
        int j = i - 1;
        while (j >= 0 && E[ord[j]] > E[oi]) {
            ord[j + 1] = ord[j];
            --j;
        }
        ord[j + 1] = oi;
    }
    bool bad = false;
    for (int i = 0; i < N; ++i) {
        E_out[t * N + i] = E[ord[i]];
        bad = bad || !isfinite(E[i]);
    }
    if (bad && status) atomicOr(status, 1);
    if (U_out)
        for (int r = 0; r < N; ++r)
            for (int c = 0; c < N; ++c) U_out[t * NN + r * N + c] = W[r][ord[c]];
}

}  // namespace

int small_fused(const ModelDev& m, cudaStream_t st, int64_t nk, const double* klist_d, int64_t k0,
                const int64_t* kmesh, const double* dirs_d, int spin, double eta, int nmu, const double* mu_d,
                double width, double* Om, double* E, double* S, double* Met, double* SM) {
    if (nk <= 0) return TBG_OK;
    const int N = (int)m.nsta;
    const int64_t n0 = kmesh ? kmesh[0] : 1, n1 = (kmesh && m.dim > 1) ? kmesh[1] : 1,
                  n2 = (kmesh && m.dim > 2) ? kmesh[2] : 1;
    const unsigned blocks = (unsigned)((nk + 127) / 128);
    KTimer kt(st, "small_fused_kernel");
    // energies only when nothing else is asked for
    const bool vals = !Om && !S && !Met && !SM;
    if (vals && !E) return TBG_OK;
#define SMALL_LAUNCH(NM)                                                                                             \
    do {                                                                                                             \
        if (vals)                                                                                                    \
            small_fused_kernel<NM, true><<<blocks, 128, 0, st>>>(                                                    \
                N, (int)m.norb, m.dim, (int)m.nR, nk, klist_d, k0, n0, n1, n2, m.ham, m.hamR_d, m.Rcart_d, m.tau_d, \
                m.taucart_d, dirs_d, spin, eta, nmu, mu_d, width, Om, E, S, Met, SM);                               \
        else                                                                                                         \
            small_fused_kernel<NM, false><<<blocks, 128, 0, st>>>(                                                   \
                N, (int)m.norb, m.dim, (int)m.nR, nk, klist_d, k0, n0, n1, n2, m.ham, m.hamR_d, m.Rcart_d, m.tau_d, \
                m.taucart_d, dirs_d, spin, eta, nmu, mu_d, width, Om, E, S, Met, SM);                               \
    } while (0)
    if (N <= 2)
        SMALL_LAUNCH(2);
    else if (N <= 4)
        SMALL_LAUNCH(4);
    else if (N <= 8)
        SMALL_LAUNCH(8);
    else
        return set_error(TBG_E_UNSUPPORTED, "small_fused: nsta > 8");
#undef SMALL_LAUNCH
    TBG_LAUNCHED("small_fused_kernel");
    return TBG_OK;
}

}  // namespace tbg

namespace tbg {
int eig_small(cudaStream_t st, int N, int64_t batch, const zc* H, double* E, zc* U, int* status) {
    if (batch <= 0) return TBG_OK;
    const unsigned blocks = (unsigned)((batch + 127) / 128);
    if (N <= 2)
        small_eig_kernel<2><<<blocks, 128, 0, st>>>(N, batch, H, E, U, status);
    else if (N <= 4)
        small_eig_kernel<4><<<blocks, 128, 0, st>>>(N, batch, H, E, U, status);
    else
        small_eig_kernel<8><<<blocks, 128, 0, st>>>(N, batch, H, E, U, status);
    TBG_LAUNCHED("small_eig_kernel");
    return TBG_OK;
}
}  // namespace tbg

namespace tbg {
namespace {

// Warp-per-matrix cyclic complex Jacobi (FP64) for kSmallMaxN < N <= 32.  The
// matrix (upper triangle read, as by the Householder solver) and the
// eigenvector accumulator sit in shared memory; the N(N-1)/2 rotations of a
// sweep run as N-1 rounds of N/2 disjoint pairs (circle-method round robin:
// the last index fixed, the others turning), and in each round every 2x2 block
// (rows of pair I, columns of pair J) becomes G_I^H B G_J, one block per lane,
// with the rotation of the one-thread solver above:
//   G = [[c, -s], [s e^{-i phi}, c e^{-i phi}]],  e^{i phi} = a_pq / |a_pq|,
//   tan 2 theta = 2 |a_pq| / (a_pp - a_qq), |theta| <= pi/4
// (the small angle: with every pair of a round rotated at once, the near-swaps
// that the angle up to pi/2 allows make the rounds cycle without converging).
// Sweeps stop when the off-diagonal norm is 1e-15 of the diagonal's: blocks
// off the diagonal only reach rounding level, never exact zeros (at most 40).
template <int NP>
struct JacobiWarp {
    zc A[NP * NP];
    zc V[NP * NP];
    zc em[NP / 2];
    double c[NP / 2], s[NP / 2];
    int p[NP / 2], q[NP / 2], rank[NP];
};

template <int NP>
__global__ void __launch_bounds__(64) jacobi_warp_kernel(int N, int64_t batch, const zc* __restrict__ H,
                                                         double* __restrict__ E_out, zc* __restrict__ U_out,
                                                         int* __restrict__ status) {
    extern __shared__ __align__(16) unsigned char jacobi_smem[];
    const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    JacobiWarp<NP>& w = reinterpret_cast<JacobiWarp<NP>*>(jacobi_smem)[threadIdx.x >> 5];
    const int n2 = (N + 1) & ~1, nh = n2 / 2, NN = N * N;
    for (int64_t m = blockIdx.x * (int64_t)nw + (threadIdx.x >> 5); m < batch; m += (int64_t)gridDim.x * nw) {
        const zc* h = H + m * NN;
        for (int e = lane; e < n2 * n2; e += 32) {
            const int i = e / n2, j = e - i * n2;
            zc a = mk(0.0, 0.0);
            if (i < N && j < N) a = j >= i ? h[i * N + j] : conj(h[j * N + i]);
            if (i == j) a.im = 0.0;
            w.A[i * NP + j] = a;
            w.V[i * NP + j] = mk(i == j ? 1.0 : 0.0, 0.0);
        }
        __syncwarp();
        for (int sweep = 0; sweep < 40; ++sweep) {
            double off = 0.0, dia = 0.0;
            for (int e = lane; e < n2 * n2; e += 32) {
                const int i = e / n2, j = e - i * n2;
                const double v = abs2(w.A[i * NP + j]);
                if (i == j)
                    dia += v;
                else
                    off += v;
            }
            for (int o = 16; o; o >>= 1) {
                off += __shfl_xor_sync(0xffffffffu, off, o);
                dia += __shfl_xor_sync(0xffffffffu, dia, o);
            }
            if (off <= 1e-30 * dia || off == 0.0) break;  // warp-uniform
            for (int r = 0; r < n2 - 1; ++r) {
                if (lane < nh) {
                    const int p = lane == 0 ? r : (r + lane) % (n2 - 1);
                    const int q = lane == 0 ? n2 - 1 : (r - lane + n2 - 1) % (n2 - 1);
                    const zc apq = w.A[p * NP + q];
                    const double mag = sqrt(abs2(apq));
                    double sn = 0.0, cs = 1.0;
                    zc em = mk(1.0, 0.0);
                    if (mag > 0.0) {
                        em = mk(apq.re / mag, -apq.im / mag);
                        const double dl = w.A[p * NP + p].re - w.A[q * NP + q].re;
                        sincos(0.5 * atan2(copysign(2.0 * mag, dl), fabs(dl)), &sn, &cs);
                    }
                    w.p[lane] = p;
                    w.q[lane] = q;
                    w.c[lane] = cs;
                    w.s[lane] = sn;
                    w.em[lane] = em;
                }
                __syncwarp();
                for (int b = lane; b < nh * nh; b += 32) {
                    const int I = b / nh, J = b - I * nh;
                    const int pi = w.p[I], qi = w.q[I], pj = w.p[J], qj = w.q[J];
                    const double ci = w.c[I], si = w.s[I], cj = w.c[J], sj = w.s[J];
                    const zc ei = conj(w.em[I]), ej = w.em[J];
                    const zc b00 = w.A[pi * NP + pj], b01 = w.A[pi * NP + qj];
                    const zc b10 = w.A[qi * NP + pj], b11 = w.A[qi * NP + qj];
                    // columns: B G_J
                    const zc t01 = ej * b01, t11 = ej * b11;
                    const zc r00 = cj * b00 + sj * t01, r01 = cj * t01 - sj * b00;
                    const zc r10 = cj * b10 + sj * t11, r11 = cj * t11 - sj * b10;
                    // rows: G_I^H (B G_J)
                    const zc u10 = ei * r10, u11 = ei * r11;
                    zc a00 = ci * r00 + si * u10, a01 = ci * r01 + si * u11;
                    zc a10 = ci * u10 - si * r00, a11 = ci * u11 - si * r01;
                    if (I == J) {
                        a00.im = 0.0;
                        a11.im = 0.0;
                        a01 = mk(0.0, 0.0);
                        a10 = mk(0.0, 0.0);
                    }
                    w.A[pi * NP + pj] = a00;
                    w.A[pi * NP + qj] = a01;
                    w.A[qi * NP + pj] = a10;
                    w.A[qi * NP + qj] = a11;
                }
                for (int e = lane; e < n2 * nh; e += 32) {
                    const int row = e / nh, J = e - row * nh;
                    const int pj = w.p[J], qj = w.q[J];
                    const double cj = w.c[J], sj = w.s[J];
                    const zc v0 = w.V[row * NP + pj], v1 = w.em[J] * w.V[row * NP + qj];
                    w.V[row * NP + pj] = cj * v0 + sj * v1;
                    w.V[row * NP + qj] = cj * v1 - sj * v0;
                }
                __syncwarp();
            }
        }
        // ascending order: rank of each diagonal entry, ties by index
        for (int i = lane; i < N; i += 32) {
            const double di = w.A[i * NP + i].re;
            int rk = 0;
            for (int j = 0; j < N; ++j) {
                const double dj = w.A[j * NP + j].re;
                rk += (dj < di) || (dj == di && j < i);
            }
            w.rank[i] = rk;
            E_out[m * N + rk] = di;
            if (!isfinite(di) && status) atomicOr(status, 1);
        }
        __syncwarp();
        if (U_out)
            for (int e = lane; e < NN; e += 32) {
                const int r = e / N, c = e - r * N;
                U_out[m * NN + r * N + w.rank[c]] = w.V[r * NP + c];
            }
        __syncwarp();
    }
}

template <int NP>
int launch_jacobi(cudaStream_t st, int N, int64_t batch, const zc* H, double* E, zc* U, int* status) {
    constexpr int kWarps = 2;
    const size_t smem = kWarps * sizeof(JacobiWarp<NP>);
    auto kern = jacobi_warp_kernel<NP>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_error(e, "jacobi_warp_kernel smem");
    int dev = 0, nsm = 0, perSM = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, kern, 32 * kWarps, smem);
    if (e != cudaSuccess || perSM < 1) perSM = 1;
    const int64_t grid = std::min<int64_t>((int64_t)nsm * perSM, (batch + kWarps - 1) / kWarps);
    KTimer kt(st, "jacobi_warp_kernel");
    kern<<<(unsigned)grid, 32 * kWarps, smem, st>>>(N, batch, H, E, U, status);
    TBG_LAUNCHED("jacobi_warp_kernel");
    return TBG_OK;
}

}  // namespace

int eig_jacobi(cudaStream_t st, int N, int64_t batch, const zc* H, double* E, zc* U, int* status) {
    if (batch <= 0) return TBG_OK;
    if (N < 2 || N > kJacobiMaxN) return set_error(TBG_E_UNSUPPORTED, "eig_jacobi: N outside [2, 32]");
    return N <= 16 ? launch_jacobi<16>(st, N, batch, H, E, U, status)
                   : launch_jacobi<32>(st, N, batch, H, E, U, status);
}

}  // namespace tbg
