// Nearest-rank percentile over a sliding window kept sorted in registers
// (shared by the batch kernel in k_window.cu and the many-series plan in
// k_tm_plan.cu).
//
// percentile_nearest_rank over a window of `len` values (NaN excluded):
// out = sorted[k], k = round(p * wl) - 1 clamped to [0, wl - 1], wl the number
// of non-NaN values in the window (percentile_nearest_rank.rs:190-266).  The
// sorted window lives in W >= len registers padded with +inf; each step
// removes the value leaving the window and inserts the one entering it with
// constant-index mask / min / max passes (about 5 W operations), and the k-th
// value is read by a select tree on the bits of k.
//
// Why not a sort per window (the reference's bitonic path): a bitonic sort of
// a 64-slot window is 21 compare-exchange stages of 32 pairs, about 670
// min/max pairs per output, against about 5 W operations here (280 for
// W = 56) for the incremental update.
#pragma once

#include <cuda_runtime.h>

namespace vta {
namespace pnr {

__device__ __forceinline__ int rank(double pf, int wl) {
    const long long raw = (long long)round(fma(pf, (double)wl, 0.0)) - 1;
    const int k = raw <= 0 ? 0 : (int)raw;
    return k >= wl ? wl - 1 : k;
}

// Insert v (not NaN) into the ascending window, dropping the last (+inf)
// slot: w'[i] = min(w[i], max(w[i-1], v)) -- two min/max per slot, no
// predicates, every slot independent.
template <int W>
__device__ __forceinline__ void insert(float (&w)[W], float v) {
#pragma unroll
    for (int i = W - 1; i > 0; --i) w[i] = fminf(w[i], fmaxf(w[i - 1], v));
    w[0] = fminf(w[0], v);
}
// Remove one element equal to v (v is in the window): slots below v keep their
// value, the others take their right neighbour.  "w[i] < v" is the sign of
// w[i] - v (exact: a difference of distinct floats is never zero with
// denormals kept, and equal values give +0), turned into a bit mask, so the
// select is one logic operation and no predicate register is used (a
// compare-and-select form measured 14% slower in the many-series plan).
template <int W>
__device__ __forceinline__ void remove(float (&w)[W], float v) {
    constexpr unsigned kInf = 0x7f800000u;
#pragma unroll
    for (int i = 0; i < W; ++i) {
        const unsigned m = (unsigned)((int)__float_as_uint(__fsub_rn(w[i], v)) >> 31);
        const unsigned nxt = i + 1 < W ? __float_as_uint(w[i + 1]) : kInf;
        w[i] = __uint_as_float((__float_as_uint(w[i]) & m) | (nxt & ~m));
    }
}
// One step of the sliding window: remove vo and insert vi, each when not NaN
// (NaN values never enter the window).
template <int W>
__device__ __forceinline__ void replace(float (&w)[W], float vo, float vi) {
    if (!isnan(vo)) remove(w, vo);
    if (!isnan(vi)) insert(w, vi);
}

// w[k] for a runtime k by a select tree on the bits of k (depth log2 W
// instead of a W-long chain of dependent selects)
template <int W>
__device__ __forceinline__ float pick_tree(const float (&w)[W], int k) {
    constexpr int P = W <= 16 ? 16 : (W <= 32 ? 32 : 64);
    float v[P];
#pragma unroll
    for (int i = 0; i < P; ++i) v[i] = i < W ? w[i] : 0.f;
#pragma unroll
    for (int step = 1; step < P; step <<= 1) {
        const bool hi = (k & step) != 0;
#pragma unroll
        for (int i = 0; i + step < P; i += 2 * step) v[i] = hi ? v[i + step] : v[i];
    }
    return v[0];
}

// The output for a window of wl non-NaN values (kfull: the rank of a full
// window of len values); NaN for an empty window.
template <int W>
__device__ __forceinline__ float pick(const float (&w)[W], int wl, int len, int kfull, double pf) {
    const int k = wl == len ? kfull : (wl > 0 ? rank(pf, wl) : 0);
    const float r = pick_tree(w, k);
    return wl > 0 ? r : __int_as_float(0x7fc00000);
}

}  // namespace pnr
}  // namespace vta
