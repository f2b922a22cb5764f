// Gaussian-smeared density of states (src/model_physics.rs:179-230):
//   dos(E_i) = 1/nk sum_{k,n} exp(-A^2 / 2) / sigma / sqrt(2 pi),  A = (E_i - E_nk) / sigma,
//   E_i = E_min + i (E_max - E_min) / (E_n - 1)   (ndarray linspace).
//
// The band energies of one mesh chunk are already on the device.  One block
// owns a tile of 256 consecutive energy bins (one per thread, accumulated in a
// register) and one slice of the chunk's energies, staged through shared
// memory.  The term of energy x is non-zero only where exp(-A^2/2) does not
// underflow in FP64, |A| < 38.6; each staged energy carries the integer bin
// range [lo, hi] of |E_i - x| <= 38.7 sigma (one bin of slack either side),
// so the per-pair test is two integer compares and only terms the reference
// sums as non-zero reach the FP64 exponential.  Per-slice partials are then
// added in slice order into a compensated running total per bin, so the
// result does not depend on scheduling.

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "tbgpu_internal.cuh"

namespace tbg {
namespace {

constexpr int kBins = 256;     // bins per block (one per thread)
constexpr int kStage = 1024;   // energies staged per pass
constexpr double kCut = 38.7;  // exp(-kCut^2 / 2) underflows to 0 in FP64

__global__ void __launch_bounds__(kBins) dos_kernel(int64_t count, int64_t per_slice, const double* __restrict__ ev,
                                                    int64_t E_n, double E_min, double step, double sigma,
                                                    double sigma0, double pi0, double* __restrict__ part) {
    __shared__ double xs[kStage];
    __shared__ int2 win[kStage];
    const int64_t bin = (int64_t)blockIdx.x * kBins + threadIdx.x;
    // the grid point exactly as the host returns it (no FMA contraction)
    const double Ei = __dadd_rn(E_min, __dmul_rn(step, (double)bin));
    const int64_t s0 = (int64_t)blockIdx.y * per_slice;
    const int64_t s1 = std::min<int64_t>(count, s0 + per_slice);
    const double w = kCut * sigma;
    double acc = 0.0;
    for (int64_t c0 = s0; c0 < s1; c0 += kStage) {
        const int nc = (int)std::min<int64_t>(kStage, s1 - c0);
        __syncthreads();
        for (int j = threadIdx.x; j < nc; j += kBins) {
            const double x = ev[c0 + j];
            int lo = 1, hi = 0;  // empty
            if (step > 0.0) {
                double a = ceil((x - w - E_min) / step) - 1.0;
                double b = floor((x + w - E_min) / step) + 1.0;
                a = fmax(a, 0.0);
                b = fmin(b, (double)(E_n - 1));
                if (a <= b) {
                    lo = (int)a;
                    hi = (int)b;
                }
            } else if (fabs(x - E_min) <= w) {  // a single bin at E_min
                lo = 0;
                hi = 0;
            }
            xs[j] = x;
            win[j] = make_int2(lo, hi);
        }
        __syncthreads();
        if (bin < E_n) {
            const int ib = (int)bin;
            for (int j = 0; j < nc; ++j) {
                const int2 r = win[j];
                if (ib < r.x || ib > r.y) continue;
                const double A = (Ei - xs[j]) * sigma0;
                acc += exp(-A * A / 2.0) * sigma0 * pi0;
            }
        }
    }
    if (bin < E_n) part[(int64_t)blockIdx.y * E_n + bin] = acc;
}

__global__ void dos_reduce_kernel(int64_t E_n, int slices, const double* __restrict__ part, double* __restrict__ acc) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < E_n; i += (int64_t)gridDim.x * blockDim.x) {
        double s = acc[2 * i], c = acc[2 * i + 1];
        for (int y = 0; y < slices; ++y) {
            const double v = part[(int64_t)y * E_n + i] - c;
            const double t = s + v;
            c = (t - s) - v;
            s = t;
        }
        acc[2 * i] = s;
        acc[2 * i + 1] = c;
    }
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
    {
        KTimer kt(st, "dos_kernel");
        dim3 grid((unsigned)((E_n + kBins - 1) / kBins), (unsigned)slices);
        dos_kernel<<<grid, kBins, 0, st>>>(count, per_slice, ev, E_n, E_min, step, sigma, 1.0 / sigma, pi0, part);
        TBG_LAUNCHED("dos_kernel");
    }
    KTimer kt(st, "dos_reduce_kernel");
    dos_reduce_kernel<<<(unsigned)std::min<int64_t>((E_n + 255) / 256, 152 * 8), 256, 0, st>>>(E_n, slices, part, acc);
    TBG_LAUNCHED("dos_reduce_kernel");
    return TBG_OK;
}

}  // namespace tbg
