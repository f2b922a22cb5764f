// Energy-cut Hall integration (Integration::EnergyCut of hall_conductivity,
// src/response/linear/mod.rs:226-268): vertex kernels on the whole mesh
// (primitives.rs:33-137), band tracking by eigenvector overlap
// (tracking.rs:123-240), occupancy cut of every simplex with vertex-averaged
// Omega where a band is fully occupied and K-quadrature on the clipped region
// where it is partly occupied (energy_cut.rs:1120-1352 for 2D triangles,
// 1449-1795 for 3D tetrahedra), thermal convolution of the zero-width result
// (energy_cut.rs:1355-1428, 1797-1849).
//
// GB300 form: the vertex data (E, eigenvectors, K_nm = va_nm vb_mn, vertex
// Omega) come from the FP64 per-chunk pipeline and stay resident; the squared
// overlaps |<u_n(a)|u_m(b)>|^2 of every mesh edge are batched complex GEMMs
// over strided vertex pairs; the breadth-first tracking -- a sequential walk
// whose every step depends on the previous ones -- runs on the host over those
// overlaps, composing permutations instead of moving data; one GPU thread
// then integrates one (simplex, band) pair over the whole sorted mu grid,
// reading the vertex data through the permutations, and adds into
// shared-memory accumulators per mu (a difference array for the fully
// occupied mu range); block partials are summed in block order.

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <deque>
#include <numeric>
#include <vector>

#include "tbgpu_internal.cuh"

namespace tbg {
namespace {

constexpr double kEcEps = 1e-12;                                  // energy_cut.rs:47
__constant__ int c_cube_tets[5][4] = {{0, 1, 2, 4}, {3, 1, 2, 7}, {5, 1, 4, 7}, {6, 2, 4, 7}, {1, 2, 4, 7}};
__constant__ double c_tet_vol_factor[5] = {1.0 / 6.0, 1.0 / 6.0, 1.0 / 6.0, 1.0 / 6.0, 1.0 / 3.0};
__constant__ double c_tri_q[3][3] = {{2.0 / 3.0, 1.0 / 6.0, 1.0 / 6.0},
                                     {1.0 / 6.0, 2.0 / 3.0, 1.0 / 6.0},
                                     {1.0 / 6.0, 1.0 / 6.0, 2.0 / 3.0}};
__constant__ double c_tet_q[4][4] = {
    {0.5854101966249685, 0.1381966011250105, 0.1381966011250105, 0.1381966011250105},
    {0.1381966011250105, 0.5854101966249685, 0.1381966011250105, 0.1381966011250105},
    {0.1381966011250105, 0.1381966011250105, 0.5854101966249685, 0.1381966011250105},
    {0.1381966011250105, 0.1381966011250105, 0.1381966011250105, 0.5854101966249685}};

// K[b][n][m] = Bx[n][m] By[m][n];  Om[b][n] = -2 Im sum_{m != n} K_nm / ((E_n - E_m)^2 + eta^2),
// terms with a denominator below 1e-30 skipped (kernel.rs:54-80).  One warp per row.
__global__ void ec_vertex_kernel(int N, int64_t batch, const zc* __restrict__ V, int64_t ldV,
                                 const double* __restrict__ E, double eta2, zc* __restrict__ K,
                                 double* __restrict__ Om) {
    const int lane = threadIdx.x & 31;
    const int64_t NN = (int64_t)N * N;
    const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t w = gw; w < batch * N; w += nw) {
        const int64_t b = w / N;
        const int n = (int)(w % N);
        const zc* bx = V + b * ldV + (int64_t)n * N;
        const zc* by = V + b * ldV + NN;
        const double* Eb = E + b * N;
        zc* Kr = K + b * NN + (int64_t)n * N;
        double gi = 0.0;
        for (int m = lane; m < N; m += 32) {
            const zc x = bx[m];
            const zc y = by[(int64_t)m * N + n];
            const zc k = x * y;
            Kr[m] = k;
            if (m == n) continue;
            const double de = Eb[n] - Eb[m];
            const double den = de * de + eta2;
            if (den < 1e-30) continue;
            gi += k.im / den;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) gi += __shfl_xor_sync(0xffffffffu, gi, o);
        if (lane == 0) Om[b * N + n] = -2.0 * gi;
    }
}

// R[i] = |C[i]|^2
__global__ void ec_abs2_kernel(int64_t n, const zc* __restrict__ C, double* __restrict__ R) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        R[i] = abs2(C[i]);
}

// Omega of band n at barycentric lam (eval_berry_band_at_lam_buf, kernel.rs:138-182),
// vertex data read through the vertex permutations.
template <int NV>
__device__ double ec_eval(int n, int N, const int64_t (&vs)[NV], const double* __restrict__ E,
                          const zc* __restrict__ K, const int* __restrict__ perm, const double (&lam)[NV],
                          double eta2) {
    const int64_t NN = (int64_t)N * N;
    auto e_of = [&](int m) {
        double e = 0.0;
#pragma unroll
        for (int j = 0; j < NV; ++j)
            if (lam[j] != 0.0) e += E[vs[j] * N + perm[vs[j] * N + m]] * lam[j];
        return e;
    };
    const double en = e_of(n);
    double gi = 0.0;
    for (int m = 0; m < N; ++m) {
        if (m == n) continue;
        const double de = en - e_of(m);
        const double den = de * de + eta2;
        if (den < 1e-30) continue;
        double ki = 0.0;
#pragma unroll
        for (int j = 0; j < NV; ++j)
            if (lam[j] != 0.0) {
                const int* p = perm + vs[j] * N;
                ki += K[vs[j] * NN + (int64_t)p[n] * N + p[m]].im * lam[j];
            }
        gi += ki / den;
    }
    return -2.0 * gi;
}

__device__ __forceinline__ int upper_bound_d(const double* a, int n, double x) {  // first a[i] > x
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (a[mid] <= x)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

__device__ __forceinline__ int lower_bound_d(const double* a, int n, double x) {  // first a[i] >= x
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (a[mid] < x)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

// ---------------------------------------------------------------- 2D ------
__device__ double tri_partial(int n, int N, const int64_t (&vs)[3], const double (&cx)[3], const double (&cy)[3],
                              const double (&ev)[3], double mu, const double* E, const zc* K, const int* perm,
                              double eta2) {
    // clip_triangle (energy_cut.rs:1120-1170): barycentric sub-triangles of E <= mu
    int a = 0, b = 1, c = 2;  // sort the three vertices by energy (stable)
    if (ev[b] < ev[a]) { const int t = a; a = b; b = t; }
    if (ev[c] < ev[b]) { const int t = b; b = c; c = t; }
    if (ev[b] < ev[a]) { const int t = a; a = b; b = t; }
    auto cut = [&](int i, int j, double (&l)[3]) {
        const double de = ev[j] - ev[i];
        const double t = fabs(de) < kEcEps ? 0.5 : fmin(fmax((mu - ev[i]) / de, 0.0), 1.0);
        l[0] = l[1] = l[2] = 0.0;
        l[i] = 1.0 - t;
        l[j] = t;
    };
    double sub[2][3][3];
    int nsub;
    auto unit = [](int i, double (&l)[3]) {
        l[0] = l[1] = l[2] = 0.0;
        l[i] = 1.0;
    };
    if (mu <= ev[b] + kEcEps) {
        unit(a, sub[0][0]);
        cut(a, b, sub[0][1]);
        cut(a, c, sub[0][2]);
        nsub = 1;
    } else {
        unit(a, sub[0][0]);
        unit(b, sub[0][1]);
        cut(a, c, sub[0][2]);
        unit(b, sub[1][0]);
        cut(a, c, sub[1][1]);
        cut(b, c, sub[1][2]);
        nsub = 2;
    }
    double total = 0.0;
    for (int s = 0; s < nsub; ++s) {
        double px[3], py[3];
        for (int q = 0; q < 3; ++q) {
            px[q] = sub[s][q][0] * cx[0] + sub[s][q][1] * cx[1] + sub[s][q][2] * cx[2];
            py[q] = sub[s][q][0] * cy[0] + sub[s][q][1] * cy[1] + sub[s][q][2] * cy[2];
        }
        const double sub_area = 0.5 * fabs((px[1] - px[0]) * (py[2] - py[0]) - (px[2] - px[0]) * (py[1] - py[0]));
        if (sub_area < 1e-30) continue;
        for (int q = 0; q < 3; ++q) {
            double lam[3];
            for (int i = 0; i < 3; ++i)
                lam[i] = c_tri_q[q][0] * sub[s][0][i] + c_tri_q[q][1] * sub[s][1][i] + c_tri_q[q][2] * sub[s][2][i];
            total += sub_area * (1.0 / 3.0) * ec_eval<3>(n, N, vs, E, K, perm, lam, eta2);
        }
    }
    return total;
}

// ---------------------------------------------------------------- 3D ------
__device__ __forceinline__ double tet_vol(const double (&p)[4][3]) {
    const double x0 = p[0][0], y0 = p[0][1], z0 = p[0][2];
    const double x1 = p[1][0], y1 = p[1][1], z1 = p[1][2];
    const double x2 = p[2][0], y2 = p[2][1], z2 = p[2][2];
    const double x3 = p[3][0], y3 = p[3][1], z3 = p[3][2];
    const double det = (x1 - x0) * ((y2 - y0) * (z3 - z0) - (z2 - z0) * (y3 - y0)) -
                       (y1 - y0) * ((x2 - x0) * (z3 - z0) - (z2 - z0) * (x3 - x0)) +
                       (z1 - z0) * ((x2 - x0) * (y3 - y0) - (y2 - y0) * (x3 - x0));
    return fabs(det) / 6.0;
}

__device__ double sub_tet(const double (&sub)[4][4], const double (&co)[4][3], int n, int N, const int64_t (&vs)[4],
                          const double* E, const zc* K, const int* perm, double eta2) {
    double p[4][3];
    for (int k = 0; k < 4; ++k)
        for (int d = 0; d < 3; ++d)
            p[k][d] = sub[k][0] * co[0][d] + sub[k][1] * co[1][d] + sub[k][2] * co[2][d] + sub[k][3] * co[3][d];
    const double vol = tet_vol(p);
    if (vol < 1e-30) return 0.0;
    double total = 0.0;
    for (int q = 0; q < 4; ++q) {
        double lam[4] = {0.0, 0.0, 0.0, 0.0};
        for (int k = 0; k < 4; ++k)
            for (int i = 0; i < 4; ++i) lam[i] += c_tet_q[q][k] * sub[k][i];
        total += vol * 0.25 * ec_eval<4>(n, N, vs, E, K, perm, lam, eta2);
    }
    return total;
}

__device__ double tet_partial(int n, int N, const int64_t (&vs)[4], const double (&co)[4][3], const double (&ev)[4],
                              const double (&ov)[4], double full_vol, double mu, const double* E, const zc* K,
                              const int* perm, double eta2) {
    int idx[4] = {0, 1, 2, 3};  // stable insertion sort by energy
    for (int i = 1; i < 4; ++i) {
        const int v = idx[i];
        int j = i - 1;
        while (j >= 0 && ev[idx[j]] > ev[v]) {
            idx[j + 1] = idx[j];
            --j;
        }
        idx[j + 1] = v;
    }
    const int a = idx[0], b = idx[1], c = idx[2], d = idx[3];
    auto unit = [](int i, double (&l)[4]) {
        l[0] = l[1] = l[2] = l[3] = 0.0;
        l[i] = 1.0;
    };
    auto cut = [&](int i, int j, double (&l)[4]) {
        const double de = ev[j] - ev[i];
        const double t = fabs(de) < kEcEps ? 0.5 : fmin(fmax((mu - ev[i]) / de, 0.0), 1.0);
        l[0] = l[1] = l[2] = l[3] = 0.0;
        l[i] = 1.0 - t;
        l[j] = t;
    };
    double s[4][4];
    if (mu <= ev[b] + kEcEps) {
        unit(a, s[0]); cut(a, b, s[1]); cut(a, c, s[2]); cut(a, d, s[3]);
        return sub_tet(s, co, n, N, vs, E, K, perm, eta2);
    }
    if (mu <= ev[c] + kEcEps) {
        double r = 0.0;
        unit(a, s[0]); unit(b, s[1]); cut(a, c, s[2]); cut(b, d, s[3]);
        r += sub_tet(s, co, n, N, vs, E, K, perm, eta2);
        unit(a, s[0]); cut(a, c, s[1]); cut(a, d, s[2]); cut(b, d, s[3]);
        r += sub_tet(s, co, n, N, vs, E, K, perm, eta2);
        unit(b, s[0]); cut(b, c, s[1]); cut(b, d, s[2]); cut(a, c, s[3]);
        r += sub_tet(s, co, n, N, vs, E, K, perm, eta2);
        return r;
    }
    const double full_val = full_vol * (ov[0] + ov[1] + ov[2] + ov[3]) / 4.0;
    unit(d, s[0]); cut(a, d, s[1]); cut(b, d, s[2]); cut(c, d, s[3]);
    return full_val - sub_tet(s, co, n, N, vs, E, K, perm, eta2);
}

// One thread per (cell, simplex, band); acc[im] gets the partial-occupation
// values, fdiff[im] the fully occupied value at the first mu of its range
// (prefix-summed later).  mu window [mu0, mu0 + nmu) of the sorted grid.
template <int DIM>
__global__ void __launch_bounds__(128) ec_integrate_kernel(int N, int nx, int ny, int nz, const double* __restrict__ E,
                                                           const zc* __restrict__ K, const double* __restrict__ Om,
                                                           const int* __restrict__ perm, int nmu_all,
                                                           const double* __restrict__ mu_all, int mu0, int nmu,
                                                           double eta, double* __restrict__ part,
                                                           double* __restrict__ fpart) {
    extern __shared__ double ec_sm[];
    double* acc = ec_sm;        // nmu
    double* fd = ec_sm + nmu;   // nmu + 1
    for (int i = threadIdx.x; i < 2 * nmu + 1; i += blockDim.x) ec_sm[i] = 0.0;
    __syncthreads();
    const double eta2 = eta * eta;
    constexpr int S = DIM == 2 ? 4 : 5;
    const int64_t ncells = (int64_t)nx * ny * (DIM == 3 ? nz : 1);
    const int64_t items = ncells * S * N;
    const double* mu = mu_all;
    for (int64_t it = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; it < items;
         it += (int64_t)gridDim.x * blockDim.x) {
        const int n = (int)(it % N);
        const int s = (int)((it / N) % S);
        const int64_t cell = it / ((int64_t)N * S);
        double scale, full;
        double e_min = INFINITY, e_max = -INFINITY;
        if (DIM == 2) {
            const int ix = (int)(cell / ny), iy = (int)(cell % ny);
            const int ixp = (ix + 1) % nx, iyp = (iy + 1) % ny;
            const int64_t i00 = (int64_t)ix * ny + iy, i10 = (int64_t)ixp * ny + iy, i11 = (int64_t)ixp * ny + iyp,
                          i01 = (int64_t)ix * ny + iyp;
            const double inx = 1.0 / nx, iny = 1.0 / ny;
            int64_t vs[3];
            // build_triangles_2d_diagavg (tracking.rs:278-341)
            if (s == 0) { vs[0] = i00; vs[1] = i10; vs[2] = i01; }
            else if (s == 1) { vs[0] = i11; vs[1] = i10; vs[2] = i01; }
            else if (s == 2) { vs[0] = i00; vs[1] = i10; vs[2] = i11; }
            else { vs[0] = i00; vs[1] = i11; vs[2] = i01; }
            double cx[3], cy[3];
            for (int j = 0; j < 3; ++j) {  // coord_of: the first corner whose index matches
                const int64_t v = vs[j];
                if (v == i00) { cx[j] = ix * inx; cy[j] = iy * iny; }
                else if (v == i10) { cx[j] = (ix + 1) * inx; cy[j] = iy * iny; }
                else if (v == i11) { cx[j] = (ix + 1) * inx; cy[j] = (iy + 1) * iny; }
                else { cx[j] = ix * inx; cy[j] = (iy + 1) * iny; }
            }
            const double area = 0.5 * fabs((cx[1] - cx[0]) * (cy[2] - cy[0]) - (cx[2] - cx[0]) * (cy[1] - cy[0]));
            if (area < kEcEps) continue;
            scale = (inx * iny / 4.0) / area;
            double ev[3], ov[3];
            for (int j = 0; j < 3; ++j) {
                const int pn = perm[vs[j] * N + n];
                ev[j] = E[vs[j] * N + pn];
                ov[j] = Om[vs[j] * N + pn];
                e_min = fmin(e_min, ev[j]);
                e_max = fmax(e_max, ev[j]);
            }
            full = area * (ov[0] + ov[1] + ov[2]) / 3.0;
            const int ip = upper_bound_d(mu, nmu_all, e_min + kEcEps);
            const int iff = lower_bound_d(mu, nmu_all, e_max - kEcEps);
            const int lo = max(ip, mu0), hi = min(iff, mu0 + nmu);
            for (int im = lo; im < hi; ++im)
                atomicAdd(&acc[im - mu0], scale * tri_partial(n, N, vs, cx, cy, ev, mu[im], E, K, perm, eta2));
            if (iff < mu0 + nmu) atomicAdd(&fd[max(iff, mu0) - mu0], scale * full);
        } else {
            const int iz = (int)(cell % nz), iy = (int)((cell / nz) % ny), ix = (int)(cell / ((int64_t)ny * nz));
            const int ixp = (ix + 1) % nx, iyp = (iy + 1) % ny, izp = (iz + 1) % nz;
            auto i3 = [&](int x, int y, int z) { return ((int64_t)x * ny + y) * nz + z; };
            const int64_t c[8] = {i3(ix, iy, iz),  i3(ixp, iy, iz),  i3(ix, iyp, iz),  i3(ixp, iyp, iz),
                                  i3(ix, iy, izp), i3(ixp, iy, izp), i3(ix, iyp, izp), i3(ixp, iyp, izp)};
            const double inx = 1.0 / nx, iny = 1.0 / ny, inz = 1.0 / nz;
            int64_t vs[4];
            double co[4][3];
            for (int j = 0; j < 4; ++j) {
                const int l = c_cube_tets[s][j];
                vs[j] = c[l];
                co[j][0] = (ix + (l & 1)) * inx;
                co[j][1] = (iy + ((l >> 1) & 1)) * iny;
                co[j][2] = (iz + ((l >> 2) & 1)) * inz;
            }
            const double vol = tet_vol(co);
            if (vol < kEcEps) continue;
            scale = (inx * iny * inz * c_tet_vol_factor[s]) / vol;
            double ev[4], ov[4];
            for (int j = 0; j < 4; ++j) {
                const int pn = perm[vs[j] * N + n];
                ev[j] = E[vs[j] * N + pn];
                ov[j] = Om[vs[j] * N + pn];
                e_min = fmin(e_min, ev[j]);
                e_max = fmax(e_max, ev[j]);
            }
            full = vol * (ov[0] + ov[1] + ov[2] + ov[3]) / 4.0;
            const int ip = upper_bound_d(mu, nmu_all, e_min + kEcEps);
            const int iff = lower_bound_d(mu, nmu_all, e_max - kEcEps);
            const int lo = max(ip, mu0), hi = min(iff, mu0 + nmu);
            for (int im = lo; im < hi; ++im)
                atomicAdd(&acc[im - mu0],
                          scale * tet_partial(n, N, vs, co, ev, ov, vol, mu[im], E, K, perm, eta2));
            if (iff < mu0 + nmu) atomicAdd(&fd[max(iff, mu0) - mu0], scale * full);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nmu; i += blockDim.x) {
        part[(int64_t)blockIdx.x * nmu + i] = acc[i];
        fpart[(int64_t)blockIdx.x * nmu + i] = fd[i];
    }
}

// out[i] = sum over blocks of p[b][i]: one warp per column, lane-strided
// partial sums combined by a fixed shuffle tree (the same order every run).
__global__ void ec_colsum_kernel(int nblocks, int nmu, const double* __restrict__ p, double* __restrict__ out) {
    const int lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < nmu; i += nw) {
        double s = 0.0;
        for (int b = lane; b < nblocks; b += 32) s += p[(int64_t)b * nmu + i];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) out[i] = s;
    }
}

// greedy_assign (tracking.rs:43-68)
void greedy_assign(int N, const double* ov, int* perm, std::vector<int>& rows, std::vector<double>& best,
                   std::vector<char>& taken) {
    for (int i = 0; i < N; ++i) {
        double b = -1.0;
        for (int j = 0; j < N; ++j) b = std::max(b, ov[(size_t)i * N + j]);
        best[i] = b;
        rows[i] = i;
    }
    std::stable_sort(rows.begin(), rows.end(), [&](int x, int y) { return best[x] > best[y]; });
    std::fill(taken.begin(), taken.end(), 0);
    for (int i : rows) {
        int bj = 0;
        double bv = -1.0;
        for (int j = 0; j < N; ++j)
            if (!taken[j] && ov[(size_t)i * N + j] > bv) {
                bv = ov[(size_t)i * N + j];
                bj = j;
            }
        taken[bj] = 1;
        perm[i] = bj;
    }
}

}  // namespace

// global_band_track (tracking.rs:123-175) over the squared overlaps of the
// forward mesh edges: R[(a * dim + d) * N^2 + n * N + m] = |<u_n(a)|u_m(a + e_d)>|^2.
// perm (nk, N): tracked band n of vertex v is raw band perm[v][n].
void ec_track(int dim, const int64_t* kmesh, int N, const double* R, int* perm) {
    int64_t n3[3] = {kmesh[0], dim > 1 ? kmesh[1] : 1, dim > 2 ? kmesh[2] : 1};
    const int64_t nk = n3[0] * n3[1] * n3[2];
    const int64_t stride[3] = {n3[1] * n3[2], n3[2], 1};
    for (int64_t v = 0; v < nk; ++v)
        for (int n = 0; n < N; ++n) perm[v * N + n] = n;
    if (nk <= 1) return;
    const size_t NN = (size_t)N * N;
    std::vector<char> visited(nk, 0);
    std::deque<int64_t> q;
    visited[0] = 1;
    q.push_back(0);
    std::vector<double> ov(NN), acc(NN), best(N);
    std::vector<int> rows(N);
    std::vector<char> taken(N);
    // neighbour_indices (tracking.rs:177-240): non-periodic, +x, -x, +y, -y, +z, -z
    auto neighbours = [&](int64_t i, int64_t* out, int* dims, int* signs) {
        int cnt = 0;
        for (int d = 0; d < dim; ++d) {
            const int64_t cd = (i / stride[d]) % n3[d];
            for (int sgn : {1, -1}) {
                const int64_t j = cd + sgn;
                if (j >= 0 && j < n3[d]) {
                    out[cnt] = i + sgn * stride[d];
                    dims[cnt] = d;
                    signs[cnt] = sgn;
                    ++cnt;
                }
            }
        }
        return cnt;
    };
    int64_t nb_list[6], vn_list[6];
    int nb_d[6], nb_s[6], vn_d[6], vn_s[6];
    while (!q.empty()) {
        const int64_t cur = q.front();
        q.pop_front();
        const int cn = neighbours(cur, nb_list, nb_d, nb_s);
        for (int a = 0; a < cn; ++a) {
            const int64_t nb = nb_list[a];
            if (visited[nb]) continue;
            int cnt = 0;
            std::fill(acc.begin(), acc.end(), 0.0);
            const int vc = neighbours(nb, vn_list, vn_d, vn_s);
            for (int b = 0; b < vc; ++b) {
                const int64_t vn = vn_list[b];
                if (!visited[vn]) continue;
                const int d = vn_d[b];
                const int* pv = perm + vn * N;
                // raw[n][m] = |<u_n(vn)|u_m(nb)>|^2, rows taken through vn's permutation
                if (vn_s[b] < 0) {  // vn = nb - e_d: the forward edge (vn, nb)
                    const double* Rf = R + ((size_t)vn * dim + d) * NN;
                    for (int n = 0; n < N; ++n)
                        for (int m = 0; m < N; ++m) ov[(size_t)n * N + m] = Rf[(size_t)pv[n] * N + m];
                } else {  // vn = nb + e_d: the forward edge (nb, vn), transposed
                    const double* Rf = R + ((size_t)nb * dim + d) * NN;
                    for (int n = 0; n < N; ++n)
                        for (int m = 0; m < N; ++m) ov[(size_t)n * N + m] = Rf[(size_t)m * N + pv[n]];
                }
                if (cnt == 0)
                    std::copy(ov.begin(), ov.end(), acc.begin());
                else
                    for (size_t e = 0; e < NN; ++e) acc[e] += ov[e];
                ++cnt;
            }
            if (cnt > 0) {
                for (size_t e = 0; e < NN; ++e) acc[e] /= (double)cnt;
                greedy_assign(N, acc.data(), perm + nb * N, rows, best, taken);
            }
            visited[nb] = 1;
            q.push_back(nb);
        }
    }
}

// one value for every call (a per-call value would race between host threads)
size_t ec_smem_max() { return sizeof(double) * (2 * (size_t)kEcWindow + 1); }

int ec_vertex_data(cudaStream_t st, int N, int64_t batch, const zc* V, int64_t ldV, const double* E, double eta,
                   zc* K, double* Om) {
    const unsigned g = (unsigned)std::max<int64_t>(1, std::min<int64_t>((batch * N * 32 + 255) / 256, 152LL * 64));
    KTimer kt(st, "ec_vertex_kernel");
    ec_vertex_kernel<<<g, 256, 0, st>>>(N, batch, V, ldV, E, eta * eta, K, Om);
    TBG_LAUNCHED("ec_vertex_kernel");
    return TBG_OK;
}

int ec_abs2(cudaStream_t st, int64_t n, const zc* C, double* R) {
    ec_abs2_kernel<<<(unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152LL * 64)), 256, 0, st>>>(
        n, C, R);
    TBG_LAUNCHED("ec_abs2_kernel");
    return TBG_OK;
}

// sigma0 (nmu) on the sorted mu grid (device); part/fpart scratch of
// nblocks * window doubles each.
int ec_integrate(cudaStream_t st, int dim, const int64_t* kmesh, int N, const double* E, const zc* K, const double* Om,
                 const int* perm, int nmu, const double* mu_d, double eta, double* part, double* fpart, int nblocks,
                 int window, double* acc_out, double* full_out) {
    const int nx = (int)kmesh[0], ny = (int)kmesh[1], nz = dim == 3 ? (int)kmesh[2] : 1;
    for (int mu0 = 0; mu0 < nmu; mu0 += window) {
        const int w = std::min(window, nmu - mu0);
        const size_t smem = sizeof(double) * (2 * (size_t)w + 1);
        {
            KTimer kt(st, "ec_integrate_kernel");
            if (dim == 2) {
                cudaFuncSetAttribute(ec_integrate_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)ec_smem_max());
                ec_integrate_kernel<2><<<nblocks, 128, smem, st>>>(N, nx, ny, nz, E, K, Om, perm, nmu, mu_d, mu0, w,
                                                                   eta, part, fpart);
            } else {
                cudaFuncSetAttribute(ec_integrate_kernel<3>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)ec_smem_max());
                ec_integrate_kernel<3><<<nblocks, 128, smem, st>>>(N, nx, ny, nz, E, K, Om, perm, nmu, mu_d, mu0, w,
                                                                   eta, part, fpart);
            }
            TBG_LAUNCHED("ec_integrate_kernel");
        }
        const unsigned cg = (unsigned)std::min(152 * 16, (w * 32 + 255) / 256);
        ec_colsum_kernel<<<cg, 256, 0, st>>>(nblocks, w, part, acc_out + mu0);
        TBG_LAUNCHED("ec_colsum_kernel");
        ec_colsum_kernel<<<cg, 256, 0, st>>>(nblocks, w, fpart, full_out + mu0);
        TBG_LAUNCHED("ec_colsum_kernel");
    }
    return TBG_OK;
}

}  // namespace tbg
