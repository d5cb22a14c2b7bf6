// Per-combo weight rows of the weighted-window moving averages, generated on
// the device and right-aligned into a [n_combos][kmax] f32 matrix
// (zero-padded on the left), normalised so each row sums to one.
//
// Weight definitions follow the crate:
//   ALMA   w_i = exp(-(i - m)^2 / (2 s^2)), m = offset (p-1), s = p / sigma
//          (alma.rs:1426-1437; the exponent is formed in f64 and exponentiated
//          as expf(a_hi) * (1 + a_lo) so the weights keep ~1e-7 accuracy)
//   WMA    w_i = (i + 1) / (p (p + 1) / 2)                       (wma.rs:295-336)
//   SWMA   symmetric triangle = box(a) * box(b)        (swma.rs:320-400, 406-482)
//   PWMA   binomial row C(p-1, r) / sum                  (pwma.rs:1367-1408)
//   SINWMA w_k = sin((k+1) pi / (p+1)) / sum             (sinwma.rs:271-289)
//   TRIMA  box(m1) * box(m2), m1 = (p+1)/2, m2 = p - m1 + 1 (trima.rs:277-364)
#include "vta_internal.h"

namespace vta {

namespace {

__device__ double raw_weight(int kind, int i, int p, double a, double b) {
    switch (kind) {
        case WT_ALMA: {
            const double m = a * (double)(p - 1);
            const double s = (double)p / b;
            const double s2 = 2.0 * s * s;
            const double d = (double)i - m;
            const double e = -(d * d) / s2;
            const float hi = (float)e;
            const float lo = (float)(e - (double)hi);
            return (double)expf(hi) * (1.0 + (double)lo);
        }
        case WT_WMA: return (double)(i + 1);
        case WT_SWMA: {
            int aa, bb;
            if (p & 1) { aa = bb = (p + 1) >> 1; }
            else { aa = p >> 1; bb = aa + 1; }
            return (double)min(min(i + 1, p - i), min(aa, bb));
        }
        case WT_PWMA: {
            const int n = p - 1;
            const int r = min(i, n - i);
            double res = 1.0;
            for (int k = 0; k < r; ++k) {
                res *= (double)(n - k);
                res /= (double)(k + 1);
            }
            return res;
        }
        case WT_SINWMA: return (double)sinpif((float)(i + 1) / (float)(p + 1));
        case WT_TRIMA: {
            const int m1 = (p + 1) / 2, m2 = p - m1 + 1;
            return (double)min(min(i + 1, p - i), min(m1, m2));
        }
    }
    return 0.0;
}

// One block per combo: raw weights, f64 block sum, normalise, store.
__global__ void k_weights(int kind, const int* periods, const double* pa, const double* pb, int kmax,
                          float* w) {
    __shared__ double red[256];
    const int c = blockIdx.x;
    const int p = periods[c];
    const double a = pa ? pa[c] : 0.0, b = pb ? pb[c] : 0.0;
    double s = 0.0;
    for (int i = threadIdx.x; i < p; i += blockDim.x) s += raw_weight(kind, i, p, a, b);
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    const double inv = 1.0 / red[0];
    float* row = w + (size_t)c * kmax;
    for (int k = threadIdx.x; k < kmax; k += blockDim.x) {
        const int i = k - (kmax - p);
        row[k] = i >= 0 ? (float)(raw_weight(kind, i, p, a, b) * inv) : 0.f;
    }
}

}  // namespace

vta_status launch_weights(int kind, const int* periods, const double* pa, const double* pb, int n_combos,
                          int kmax, float* w, cudaStream_t st) {
    k_weights<<<n_combos, 256, 0, st>>>(kind, periods, pa, pb, kmax, w);
    return check_launch("k_weights");
}

}  // namespace vta
