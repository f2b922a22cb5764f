// Gaussian-smeared density of states (src/model_physics.rs:179-230):
//   dos(E_i) = 1/nk sum_{k,n} exp(-A^2 / 2) / sigma / sqrt(2 pi),  A = (E_i - E_nk) / sigma,
//   E_i = E_min + i (E_max - E_min) / (E_n - 1)   (ndarray linspace).
//
// The band energies of one mesh chunk are already on the device.  One block
// owns a tile of 256 consecutive energy bins (one per thread, accumulated in a
// register) and one slice of the chunk's energies.  The term of energy x is
// non-zero only where exp(-A^2/2) does not underflow in FP64, |A| < 38.6, so
// each staged energy carries the bin range of |E_i - x| <= 38.7 sigma (one bin
// of slack either side) within the tile, and only those terms are formed (see
// dos_kernel for the recurrence that replaces most exponentials).  Per-slice
// partials are then added in slice order into a compensated running total
// per bin, so the result does not depend on scheduling.

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "tbgpu_internal.cuh"

namespace tbg {
namespace {

constexpr int kBins = 256;     // bins per block (one per thread)
constexpr int kRun = 64;       // table entries per exponential start
constexpr int kMaxE = 128;     // energies staged per pass (upper bound)
constexpr int kChunks = 8;     // runs per energy: <= 4 walking up, <= 4 down (kBins / kRun each)
constexpr int kTableBytes = 36 * 1024;
constexpr double kCut = 38.7;  // exp(-kCut^2 / 2) underflows to 0 in FP64

// One pass stages up to `epp` band energies.  For energy x the bins of the
// tile inside its window form one contiguous range [s, s + L); the table row
// of x holds its Gaussian on that range.  From the bin c nearest x the row is
// walked outward in both directions, in runs of at most kRun bins, each run
// started by two exponentials at its end nearest x and extended by
//   g(j + k) = g(j) rho(j),  rho(j + k) = rho(j) exp(-d^2),  d = step / sigma, k = +-1,
// (A(j + k) = A(j) + k d).  Values only shrink along a run, so nothing
// underflows early, and a run of 64 multiplies loses ~1e-12 relative at most.
// Each thread then adds, for its own bin, the table entries of every staged
// energy in staging order.
__global__ void __launch_bounds__(kBins) dos_kernel(int64_t count, int64_t per_slice, const double* __restrict__ ev,
                                                    int64_t E_n, double E_min, double step, double sigma,
                                                    double sigma0, double pi0, double rho_step, double inv_step,
                                                    int lmax, int epp, double* __restrict__ part) {
    extern __shared__ double table[];  // epp * lmax
    __shared__ double xs[kMaxE];
    __shared__ int s_lo[kMaxE], s_len[kMaxE], s_c[kMaxE], s_pre[kMaxE + 1];
    __shared__ unsigned short runmap[kMaxE * kChunks];
    const int lane = threadIdx.x & 31;
    const int64_t b0 = (int64_t)blockIdx.x * kBins;
    const int64_t bin = b0 + threadIdx.x;
    const int tile = (int)std::min<int64_t>(kBins, E_n - b0);
    const int64_t s0 = (int64_t)blockIdx.y * per_slice;
    const int64_t s1 = std::min<int64_t>(count, s0 + per_slice);
    const double w = kCut * sigma;
    const double d = step * sigma0;
    double acc = 0.0;
    for (int64_t c0 = s0; c0 < s1; c0 += epp) {
        const int nc = (int)std::min<int64_t>(epp, s1 - c0);
        __syncthreads();
        // 1. window of each staged energy within this tile, and its centre bin
        if (threadIdx.x < kMaxE) {
            int lo = 0, len = 0, c = 0;
            double x = 0.0;
            if (threadIdx.x < nc) {
                x = ev[c0 + threadIdx.x];
                if (step > 0.0) {
                    // bounds by the reciprocal step: a rounding shift of one bin stays inside the slack
                    const double u = (x - E_min) * inv_step, hw = w * inv_step;
                    double a = ceil(u - hw) - 1.0;
                    double b = floor(u + hw) + 1.0;
                    a = fmax(a, (double)b0);
                    b = fmin(b, (double)(b0 + tile - 1));
                    if (a <= b) {
                        lo = (int)(a - (double)b0);
                        len = min((int)(b - a) + 1, lmax);  // lmax holds the widest window; guard rounding
                        double cr = rint(u) - (double)(b0 + lo);
                        c = (int)fmin(fmax(cr, -1.0), (double)len);
                    }
                } else if (fabs(x - E_min) <= w && b0 == 0) {
                    len = 1;
                }
            }
            const int up = len - max(c, 0) > 0 ? len - max(c, 0) : 0;
            const int down = min(len, c) > 0 ? min(len, c) : 0;
            const int n = (up + kRun - 1) / kRun + (down + kRun - 1) / kRun;
            xs[threadIdx.x] = x;
            s_lo[threadIdx.x] = lo;
            s_len[threadIdx.x] = len;
            s_c[threadIdx.x] = c;
            s_pre[threadIdx.x] = n;
        }
        __syncthreads();
        if (threadIdx.x < 32) {  // exclusive scan of the run counts (4 per lane)
            int v[kMaxE / 32], t = 0;
#pragma unroll
            for (int q = 0; q < kMaxE / 32; ++q) {
                v[q] = s_pre[lane * (kMaxE / 32) + q];
                t += v[q];
            }
            int incl = t;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += y;
            }
            int ex = incl - t;
#pragma unroll
            for (int q = 0; q < kMaxE / 32; ++q) {
                s_pre[lane * (kMaxE / 32) + q] = ex;
                ex += v[q];
            }
            if (lane == 31) s_pre[kMaxE] = incl;
        }
        __syncthreads();
        if (threadIdx.x < nc) {
            const int e = threadIdx.x, len = s_len[e], c = s_c[e];
            const int up = len - max(c, 0) > 0 ? len - max(c, 0) : 0;
            const int down = min(len, c) > 0 ? min(len, c) : 0;
            const int nu = (up + kRun - 1) / kRun, nd = (down + kRun - 1) / kRun;
            int p = s_pre[e];
            for (int i = 0; i < nu; ++i) runmap[p++] = (unsigned short)(e * kChunks + i);
            for (int i = 0; i < nd; ++i) runmap[p++] = (unsigned short)(e * kChunks + kChunks / 2 + i);
        }
        __syncthreads();
        // 2. table rows, one run per thread
        const int runs = s_pre[nc];
        for (int t = threadIdx.x; t < runs; t += kBins) {
            const int e = runmap[t] / kChunks, q = runmap[t] % kChunks;
            const int len = s_len[e], c = s_c[e];
            const bool upward = q < kChunks / 2;
            const int i = upward ? q : q - kChunks / 2;
            const int k = upward ? 1 : -1;
            const int from = upward ? max(c, 0) + i * kRun : min(len - 1, c - 1) - i * kRun;
            const int to = upward ? min(from + kRun - 1, len - 1) : max(from - (kRun - 1), 0);
            const double x = xs[e];
            double* row = table + e * lmax;
            const double Ej = __dadd_rn(E_min, __dmul_rn(step, (double)(b0 + s_lo[e] + from)));
            const double A = (Ej - x) * sigma0;
            double g = exp(-A * A / 2.0) * sigma0 * pi0;
            double rho = exp(-(double)k * d * A - d * d / 2.0);
            for (int j = from;; j += k) {
                row[j] = g;
                if (j == to) break;
                g *= rho;
                rho *= rho_step;
            }
        }
        __syncthreads();
        // 3. each bin adds the staged energies' entries in order
        if (threadIdx.x < tile) {
            const int ib = threadIdx.x;
            for (int e = 0; e < nc; ++e) {
                const int j = ib - s_lo[e];
                if (j >= 0 && j < s_len[e]) acc += table[e * lmax + j];
            }
        }
    }
    if (bin < E_n) part[(int64_t)blockIdx.y * E_n + bin] = acc;
}

// One warp per bin: the slices' partials in a fixed order (lane-strided
// compensated sums, then a fixed shuffle tree of two-sums), added to the
// running compensated total.
__device__ __forceinline__ void two_sum(double a, double b, double& s, double& e) {
    s = a + b;
    const double bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

__global__ void dos_reduce_kernel(int64_t E_n, int slices, const double* __restrict__ part, double* __restrict__ acc) {
    const int lane = threadIdx.x & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t i = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; i < E_n; i += nw) {
        double s = 0.0, c = 0.0;
        for (int y = lane; y < slices; y += 32) {
            double t, e;
            two_sum(s, part[(int64_t)y * E_n + i], t, e);
            s = t;
            c += e;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const double so = __shfl_xor_sync(0xffffffffu, s, o), co = __shfl_xor_sync(0xffffffffu, c, o);
            double t, e;
            // lanes l and l^o combine in the same order on both sides
            if (lane & o) two_sum(so, s, t, e); else two_sum(s, so, t, e);
            s = t;
            c = c + co + e;
        }
        if (lane == 0) {
            double t, e;
            two_sum(acc[2 * i], s, t, e);
            acc[2 * i] = t;
            acc[2 * i + 1] += e + c;
        }
    }
}

int dos_lmax(int64_t E_n, double step, double sigma) {
    if (step <= 0.0) return 1;
    // |window| <= floor(2 w / step) + 3 bins; two more absorb rounding of the bounds
    const double wb = std::floor(2.0 * kCut * sigma / step) + 5.0;
    return (int)std::max(1.0, std::min((double)std::min<int64_t>(kBins, E_n), wb));
}

}  // namespace

int dos_slices(int64_t E_n, int64_t count) {
    const int64_t tiles = (E_n + kBins - 1) / kBins;
    const int64_t want = std::max<int64_t>(1, (152 * 8 + tiles - 1) / tiles);
    const int64_t most = std::max<int64_t>(1, count / kBins);
    return (int)std::min<int64_t>({want, most, 4096});
}

int dos_accumulate(cudaStream_t st, int64_t count, const double* ev, int64_t E_n, double E_min, double step,
                   double sigma, double* part, int slices, double* acc) {
    if (count <= 0) return TBG_OK;
    const int64_t per_slice = (count + slices - 1) / slices;
    const double pi0 = 1.0 / std::sqrt(2.0 * M_PI);
    const double sigma0 = 1.0 / sigma;
    const double d = step * sigma0;
    const int lmax = dos_lmax(E_n, step, sigma);
    // about two runs per energy: a multiple of 16 energies keeps the run-building warps full
    int epp = std::max(1, std::min(kMaxE, kTableBytes / (8 * lmax)));
    if (epp >= 16) epp &= ~15;
    {
        KTimer kt(st, "dos_kernel");
        dim3 grid((unsigned)((E_n + kBins - 1) / kBins), (unsigned)slices);
        dos_kernel<<<grid, kBins, sizeof(double) * epp * lmax, st>>>(count, per_slice, ev, E_n, E_min, step, sigma,
                                                                      sigma0, pi0, std::exp(-d * d),
                                                                      step > 0.0 ? 1.0 / step : 0.0, lmax, epp, part);
        TBG_LAUNCHED("dos_kernel");
    }
    KTimer kt(st, "dos_reduce_kernel");
    dos_reduce_kernel<<<(unsigned)std::min<int64_t>((E_n * 32 + 255) / 256, 152 * 16), 256, 0, st>>>(E_n, slices,
                                                                                                      part, acc);
    TBG_LAUNCHED("dos_reduce_kernel");
    return TBG_OK;
}

}  // namespace tbg
