// Weighted-window moving averages as a split-precision tcgen05 contraction.
//
//   out[c][t] = sum_k W[c][k] * x[t - K + 1 + k]        (rows of W right-aligned)
//
// is a GEMM D[M = combos][N = times] = A[M][K] * B[K][N] whose B operand is the
// Hankel matrix B[k][n] = x[base + k + n].  Work items are (tile of 128
// combos, 256-wide time tile) pairs, combo-tile major, cut into short chunks
// that a persistent grid of one CTA per SM takes round-robin (ItemIter).  A
// (K-major, packed in core-matrix order) is bulk-copied to shared memory with
// cp.async.bulk whenever a CTA enters a new combo tile.  B is never
// materialised as a K x 256 tile: the producer writes an "8-shift expanded
// strip" E[q] = x16[base + q .. base + q + 7] (16 bytes per q), so the 8x8 core
// matrix (kc, nc) of the MN-major canonical layout is the contiguous 128-byte
// block at q = 8*(kc + nc) and both descriptor strides are 128 bytes.  A K x 256
// tile therefore costs (K/8 + 31) * 128 bytes of shared memory, and stepping K
// by 16 just advances the descriptor start by 256 bytes.
//
// Precision: operands are split into FP16 hi + lo parts after exact power-of-
// two scaling (per weight row; per time tile after centring x on a tile
// reference value r, using sum_k w_k = S_c):
//   y = 2^-(e_c + e_x) * (Ah Bh + Ah Bl + Al Bh) + r * S_c,
// three tcgen05.mma.kind::f16 per K step with FP32 accumulation in TMEM.  The
// split keeps ~22 significant bits per operand (FP16 has 11), so the result is
// within ~1e-7 relative of the FP64 sum.  A BF16 hi/lo variant (8-bit
// significands, ~16 bits per operand) is selectable for comparison.
//
// Two kernels.  k_hankel_strips builds, once per 256-wide time tile, the hi/lo
// strips for the largest period in the sweep (plus the tile's centring value
// and x scale) in global memory; a combo tile of smaller period K reads the
// same strip starting 16 * (Kmax - K) bytes in, so every combo tile shares it.
// k_wwma_tc (288 threads): thread 0 bulk-copies the weights of the current
// combo tile, then per item waits for its strip (double-buffered, cp.async.bulk + mbarrier
// complete_tx), issues the MMAs into one of two 256-column TMEM accumulators,
// and starts the copy of the next strip as soon as the MMAs that read that
// buffer have completed.  Warps 1-8 drain the other accumulator (tcgen05.ld),
// apply scale and centring, stage 32x32 blocks in 128-byte-swizzled shared
// memory, patch warm-up / NaN positions there, and write them with TMA tensor
// stores.  Every mbarrier wait is bounded by a time limit after which the
// kernel records an error code, stops issuing work, drains its own MMAs and
// bulk copies and frees TMEM.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "tc_ops.cuh"
#include "vta_internal.h"

namespace vta {
namespace {

using namespace tc;

constexpr int kM = 128;          // combos per tile (MMA M)
constexpr int kN = 256;          // times per tile (MMA N)
constexpr int kThreads = 288;     // warp 0: TMA + MMA issue; warps 1-8: epilogue
constexpr int kEpiThreads = 256;
constexpr int kMaxK = 272;       // largest tile K whose whole A tile the shared memory holds
constexpr int kSliceK = 256;     // K slice of a larger tile: its A slice and strip part are
                                 // copied per (item, slice) and its MMAs accumulate in TMEM
constexpr int kStripBufs = 3;    // strip buffers: copies for items i+1 and i+2 in flight during item i
constexpr int kStageLd = 36;     // epilogue staging row stride (floats) of the st.global path
constexpr int kStageTma = 32 * 32 * 4;  // epilogue staging per warp for a TMA store (bytes)
constexpr uint32_t kTmemCols = 512;
constexpr unsigned long long kWaitNs = 2000000000ull;  // 2 s per wait

__device__ __forceinline__ float qnan() { return __int_as_float(0x7fc00000); }
// Instruction descriptor of kind::f16: D f32, A/B f16 (0) or bf16 (1),
// A K-major, B MN-major, N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t instr_desc(uint32_t ab_type) { return tc::instr_desc_f16(ab_type, kM, kN, 1u); }

// ------------------------------------------------------------ A packing ---
// Per combo tile m (rows c = 128 m + r): K_m = roundup16(max period), the last
// K_m columns of the right-aligned weight matrix, scaled by 2^e_r so the row
// maximum lies in [2^13, 2^14), split hi/lo and laid out as core matrices
// [K_m/8][16 row groups][8 rows][8 elements].
struct PackArgs {
    const float* w;
    int kmax, n_combos;
    const int* tile_k;          // [tiles] K_m
    const long long* tile_off;  // [tiles] offset (elements) of the hi block; lo follows
    uint16_t* packed;
    float* row_scale;           // [tiles*128] 2^-e_r
    float* row_sum;             // [tiles*128] sum of the f32 weights
};

constexpr int kPackThreads = 512;

template <int VARIANT>
__global__ void __launch_bounds__(kPackThreads) k_pack_a(PackArgs a) {
    __shared__ float sc_sh[kM];
    const int m = blockIdx.x;
    const int K = a.tile_k[m];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int col0 = a.kmax - K;  // weight column of k = 0 (negative: zero padding)
    // row statistics, one warp per row (coalesced along the row): maximum
    // magnitude and the row sum as a compensated float pair (Neumaier; an f64
    // running sum is a chain of slow FP64 adds on GB300)
    constexpr int kSlots = (kMaxK + 31) / 32;  // row elements per lane per pass
    for (int r = warp; r < kM; r += kPackThreads / 32) {
        const int c = m * kM + r;
        float mx = 0.f, sum = 0.f, comp = 0.f;
        if (c < a.n_combos) {
            const float* row = a.w + (size_t)c * a.kmax;
            for (int k0 = 0; k0 < K; k0 += 32 * kSlots) {
                // all of the lane's loads first (independent), then the sums
                float v[kSlots];
#pragma unroll
                for (int j = 0; j < kSlots; ++j) {
                    const int k = k0 + lane + 32 * j;
                    v[j] = (k < K && col0 + k >= 0) ? row[col0 + k] : 0.f;
                }
#pragma unroll
                for (int j = 0; j < kSlots; ++j) {
                    mx = fmaxf(mx, fabsf(v[j]));
                    const float t = sum + v[j];
                    comp += fabsf(sum) >= fabsf(v[j]) ? (sum - t) + v[j] : (v[j] - t) + sum;
                    sum = t;
                }
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
            const float so = __shfl_xor_sync(0xffffffffu, sum, o);
            const float co = __shfl_xor_sync(0xffffffffu, comp, o);
            const float t = sum + so;
            comp += co + (fabsf(sum) >= fabsf(so) ? (sum - t) + so : (so - t) + sum);
            sum = t;
        }
        if (lane == 0) {
            int e = 0;
            if (mx > 0.f) {
                int ex;
                frexpf(mx, &ex);  // mx = f * 2^ex, f in [0.5, 1)
                e = 14 - ex;
            }
            sc_sh[r] = ldexpf(1.f, e);
            a.row_scale[(size_t)m * kM + r] = mx > 0.f ? ldexpf(1.f, -e) : 0.f;
            a.row_sum[(size_t)m * kM + r] = sum + comp;
        }
    }
    __syncthreads();
    // packed element o = ((k / 8) * 16 + g) * 64 + rr * 8 + (k % 8) of row
    // r = 8 g + rr: consecutive threads write consecutive elements and read 8
    // consecutive weights of one row
    uint16_t* hi = a.packed + a.tile_off[m];
    uint16_t* lo = hi + (size_t)kM * K;
    const int total = kM * K;
#pragma unroll 4
    for (int o = threadIdx.x; o < total; o += kPackThreads) {
        const int kb = o >> 10, rem = o & 1023;
        const int r = ((rem >> 6) << 3) | ((rem >> 3) & 7);
        const int k = (kb << 3) | (rem & 7);
        const int c = m * kM + r;
        float v = 0.f;
        if (c < a.n_combos && col0 + k >= 0) v = a.w[(size_t)c * a.kmax + col0 + k] * sc_sh[r];
        uint16_t h, l;
        Split<VARIANT>::run(v, h, l);
        hi[o] = h;
        lo[o] = l;
    }
}

// Warm-up / NaN masks of one staged row of 32 consecutive outputs (tiles that
// need them are few; kept out of line so the hot epilogue loop stays small).
// `swz` selects the 128-byte-swizzled staging layout of the TMA store path.
__device__ __noinline__ void mask_staged(float* row, bool swz, int lane, int tb, int warm, int p, bool has_nan,
                                         int n, int nan_mode, const double* nanp) {
    for (int j = 0; j < 32; ++j) {
        const int t = tb + j;
        bool bad = t < warm;
        if (!bad && has_nan && t < n) {
            const double hi = nanp[t];
            const double lo = (nan_mode == 0 && t - p >= 0) ? nanp[t - p] : 0.0;
            bad = hi - lo > 0.5;
        }
        if (bad) {
            const int pos = swz ? ((((j >> 2) ^ (lane & 7)) << 2) | (j & 3)) : j;
            row[pos] = qnan();
        }
    }
}

// ------------------------------------------------------------ B strips ----
// One expanded Hankel strip per 256-wide time tile, built once for the largest
// tile K (Kmax) and shared by every combo tile: E[q] = lin[q .. q+7] (16 bytes)
// with lin[i] = split((x[base + i] - r) * 2^e_x), base = t0 - Kmax + 1.  A
// combo tile with K < Kmax uses the same strip from block (Kmax - K) on.
struct StripArgs {
    const float* x;
    int n, first;
    int kmax;
    int jmax;                 // strip blocks of 8 shifts: Kmax/8 + 31
    uint8_t* strips_hi;       // [n_time_tiles][jmax * 8 * 16]
    uint8_t* strips_lo;
    float* ref;               // [n_time_tiles] centring value r
    float* xscale;            // [n_time_tiles] 2^-e_x
};

template <int VARIANT>
__global__ void __launch_bounds__(128) k_hankel_strips(StripArgs a) {
    extern __shared__ uint8_t sm[];
    const int g = blockIdx.x;
    const int t0 = g * kN;
    const int base = t0 - a.kmax + 1;
    const int L = a.jmax * 8 + 8;  // linear values needed
    float* xf = reinterpret_cast<float*>(sm);
    uint16_t* lh = reinterpret_cast<uint16_t*>(xf + L);
    uint16_t* ll = lh + ((L + 7) & ~7);
    __shared__ float red[4];
    const int gref = min(t0 + kN - 1, a.n - 1);
    const float vref = (gref >= a.first && gref >= 0) ? a.x[gref] : 0.f;
    const float ref = isfinite(vref) ? vref : 0.f;
    float mx = 0.f;
    for (int q = threadIdx.x; q < L; q += 128) {
        const int gi = base + q;
        float v = __int_as_float(0x7fc00000);  // outside the series / not finite: zero after centring
        if (gi >= a.first && gi < a.n) {
            const float u = a.x[gi];
            if (isfinite(u)) v = u;
        }
        xf[q] = v;
        if (!isnan(v)) mx = fmaxf(mx, fabsf(v - ref));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
    __syncthreads();
    mx = fmaxf(fmaxf(red[0], red[1]), fmaxf(red[2], red[3]));
    int ex = 0;
    if (mx > 0.f) {
        int e2;
        frexpf(mx, &e2);
        ex = 13 - e2;
    }
    const float sc = ldexpf(1.f, ex);
    for (int q = threadIdx.x; q < L; q += 128) {
        const float v = isnan(xf[q]) ? 0.f : (xf[q] - ref) * sc;
        uint16_t h, l;
        Split<VARIANT>::run(v, h, l);
        lh[q] = h;
        ll[q] = l;
    }
    if (threadIdx.x == 0) {
        a.ref[g] = ref;
        a.xscale[g] = ldexpf(1.f, -ex);
    }
    __syncthreads();
    const uint32_t* wh = reinterpret_cast<const uint32_t*>(lh);
    const uint32_t* wl = reinterpret_cast<const uint32_t*>(ll);
    uint4* oh = reinterpret_cast<uint4*>(a.strips_hi + (size_t)g * a.jmax * 128);
    uint4* ol = reinterpret_cast<uint4*>(a.strips_lo + (size_t)g * a.jmax * 128);
    for (int q = threadIdx.x; q < a.jmax * 8; q += 128) {
        const int w0 = q >> 1;
        uint4 h4, l4;
        if (q & 1) {
            h4 = make_uint4(__byte_perm(wh[w0], wh[w0 + 1], 0x5432), __byte_perm(wh[w0 + 1], wh[w0 + 2], 0x5432),
                            __byte_perm(wh[w0 + 2], wh[w0 + 3], 0x5432), __byte_perm(wh[w0 + 3], wh[w0 + 4], 0x5432));
            l4 = make_uint4(__byte_perm(wl[w0], wl[w0 + 1], 0x5432), __byte_perm(wl[w0 + 1], wl[w0 + 2], 0x5432),
                            __byte_perm(wl[w0 + 2], wl[w0 + 3], 0x5432), __byte_perm(wl[w0 + 3], wl[w0 + 4], 0x5432));
        } else {
            h4 = make_uint4(wh[w0], wh[w0 + 1], wh[w0 + 2], wh[w0 + 3]);
            l4 = make_uint4(wl[w0], wl[w0 + 1], wl[w0 + 2], wl[w0 + 3]);
        }
        oh[q] = h4;
        ol[q] = l4;
    }
}

// ------------------------------------------------------------ main kernel -
struct TcArgs {
    int n, first;
    const int* periods;
    int n_combos;
    const int* tile_k;
    const long long* tile_off;
    const uint16_t* packed;
    const float* row_scale;
    const float* row_sum;
    int kmax, jmax;       // the sweep's largest tile K and its strip blocks (global strips)
    int ka, jcap;         // shared-memory capacities: A tile K and strip blocks per buffer
    const uint8_t* strips_hi;
    const uint8_t* strips_lo;
    const float* ref;
    const float* xscale;
    int nan_mode;
    const double* nanp;
    const int* warm_extra;  // [n_combos] extra warm-up steps (null: 0)
    float* out;
    int n_time_tiles;     // time tiles per combo tile
    int items;            // combo tiles x time tiles, combo-tile major
    int nchunks;          // items are cut into nchunks near-equal runs; CTA b takes b, b+G, ...
    int* err;             // error word (0 = ok)
    unsigned long long* trace;  // optional pipeline trace of CTA (0, 0): [tile][event]
};
// trace events per tile (globaltimer ns)
enum { TR_P_STRIP = 0, TR_P_ACC = 1, TR_P_ISSUED = 2, TR_E_START = 3, TR_E_END = 4, TR_N = 8 };
constexpr int kTraceTiles = 64;

struct __align__(16) SmemCtl {
    uint64_t a_full;
    uint64_t strip_full[kStripBufs];
    uint64_t unit_done[kStripBufs];  // MMAs of the (item, slice) unit using strip buffer u % kStripBufs
    uint64_t mma_done[2];
    uint64_t acc_empty[2];
    uint32_t tmem_base;
    int abort_flag;
    int issued;  // tiles whose MMAs were committed
};


// Walks a CTA's items: chunk c holds items [c*items/nchunks, (c+1)*items/nchunks),
// and a CTA takes chunks blockIdx.x, blockIdx.x + gridDim.x, ...  At any moment
// the grid works on a window of about gridDim.x consecutive chunks, i.e. a few
// combo tiles, which keeps the output rows being written (and their pages)
// few, while every CTA gets the same number of items to within one.
struct ItemIter {
    int q, end, chunk;
    // combo tile of the current item.  Combos are period-major, so tile K
    // grows with the tile index; the item order visits tiles 0, n-1, 1, n-2, ...
    // so the grid's window mixes tensor-heavy (large K) and write-heavy (small
    // K) tiles instead of running all SMs through one kind at a time.
    __device__ int tile(const TcArgs& a) const {
        const int j = q / a.n_time_tiles;
        const int n = a.items / a.n_time_tiles;
        return (j & 1) ? n - 1 - (j >> 1) : (j >> 1);
    }
    __device__ int time_tile(const TcArgs& a) const { return q % a.n_time_tiles; }
    __device__ void start(const TcArgs& a, int c) {
        chunk = c;
        q = (int)((long long)c * a.items / a.nchunks);
        end = (int)((long long)(c + 1) * a.items / a.nchunks);
    }
    __device__ void advance(const TcArgs& a) {
        if (++q >= end) start(a, chunk + (int)gridDim.x);
    }
};

template <int VARIANT, bool TMA_STORE>
__global__ void __launch_bounds__(kThreads, 1) k_wwma_tc(TcArgs a, const __grid_constant__ CUtensorMap tmap_out) {
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    // layout (capacities for the largest tile K): A hi | A lo | strip[kStripBufs] hi |
    // strip[kStripBufs] lo | staging (1024-aligned) | ctl
    const uint32_t strip_cap = (uint32_t)a.jcap * 128;
    uint8_t* p = smem_raw;
    uint16_t* a_hi = reinterpret_cast<uint16_t*>(p);
    p += (size_t)kM * a.ka * 2;
    uint16_t* a_lo = reinterpret_cast<uint16_t*>(p);
    p += (size_t)kM * a.ka * 2;
    uint8_t* strip_hi[kStripBufs];
    uint8_t* strip_lo[kStripBufs];
    for (int j = 0; j < kStripBufs; ++j) strip_hi[j] = p + (size_t)j * strip_cap;
    p += kStripBufs * (size_t)strip_cap;
    for (int j = 0; j < kStripBufs; ++j) strip_lo[j] = p + (size_t)j * strip_cap;
    p += kStripBufs * (size_t)strip_cap;
    p = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(p) + 1023) & ~uintptr_t(1023));
    float* stage = reinterpret_cast<float*>(p);  // [8 epilogue warps][32][kStageLd] or [8][4 KB swizzled]
    p += (size_t)8 * 32 * kStageLd * sizeof(float);
    SmemCtl* ctl = reinterpret_cast<SmemCtl*>(p);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // persistent schedule (ItemIter): this CTA's item count
    int ntiles = 0;
    for (int c = blockIdx.x; c < a.nchunks; c += gridDim.x)
        ntiles += (int)((long long)(c + 1) * a.items / a.nchunks - (long long)c * a.items / a.nchunks);
    volatile int* abort_flag = &ctl->abort_flag;
    const bool tracing = a.trace != nullptr && blockIdx.x == 0;

    if (tid == 0) {
        mbar_init(&ctl->a_full, 1);
        for (int b = 0; b < kStripBufs; ++b) {
            mbar_init(&ctl->strip_full[b], 1);
            mbar_init(&ctl->unit_done[b], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&ctl->mma_done[b], 1);
            mbar_init(&ctl->acc_empty[b], kEpiThreads);
        }
        ctl->abort_flag = 0;
        ctl->issued = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(&ctl->tmem_base)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = ctl->tmem_base;

    if (tid == 0) {
        // ================= producer: TMA copies + MMA issue (one thread) ======
        // The work of an item is one or more units (item, slice): a tile whose
        // K fits the shared memory (K <= ka) is one unit and keeps its A tile
        // resident across items; a larger tile is cut into K slices of
        // kSliceK whose A slice and strip part are copied per unit and whose
        // MMAs accumulate into the item's TMEM accumulator.  Strip buffers
        // cycle per unit (copies for units u+1 and u+2 in flight during u).
        const uint32_t idesc = instr_desc(VARIANT);
        auto nslices = [&](int K) { return K <= a.ka ? 1 : (K + kSliceK - 1) / kSliceK; };
        auto slice_k0 = [&](int K, int sl) { return K <= a.ka ? 0 : sl * kSliceK; };
        auto slice_len = [&](int K, int sl) { return K <= a.ka ? K : min(kSliceK, K - sl * kSliceK); };
        // a unit with its item's tile K and slice count read once per item
        // (the producer is one thread: every global load sits on its path)
        struct Unit {
            ItemIter it;
            int sl, mt, K, S;
        };
        auto unit_load = [&](Unit& un) {
            if (un.it.q >= a.items) {  // past this CTA's last item: nothing to read
                un.mt = -1;
                un.K = 0;
                un.S = 1;
                return;
            }
            un.mt = un.it.tile(a);
            un.K = a.tile_k[un.mt];
            un.S = nslices(un.K);
        };
        auto unit_advance = [&](Unit& un) {
            if (++un.sl >= un.S) {
                un.sl = 0;
                un.it.advance(a);
                unit_load(un);
            }
        };
        // strip part of unit u: the Kmax strip of its time tile, entered
        // 16 (Kmax - K + k0) bytes in
        auto copy_strip = [&](int u, const Unit& un) {
            const int bb = u % kStripBufs;
            const int Ki = un.K;
            const int k0 = slice_k0(Ki, un.sl), ks = slice_len(Ki, un.sl);
            const uint32_t sb = (uint32_t)(ks / 8 + kN / 8 - 1) * 128;
            const size_t g = (size_t)un.it.time_tile(a) * a.jmax * 128 + (size_t)(a.kmax - Ki + k0) * 16;
            mbar_arrive_tx(&ctl->strip_full[bb], 2 * sb);
            bulk_g2s(strip_hi[bb], a.strips_hi + g, sb, &ctl->strip_full[bb]);
            bulk_g2s(strip_lo[bb], a.strips_lo + g, sb, &ctl->strip_full[bb]);
        };
        int a_mt = -1, a_loads = 0;
        bool a_pending = false;
        // A of unit (tile mt, slice sl): the whole tile, or the slice's K range
        auto load_a = [&](int mt, int sl) {
            const int Km = a.tile_k[mt];
            const int k0 = slice_k0(Km, sl), ks = slice_len(Km, sl);
            const uint32_t abytes = (uint32_t)kM * ks * 2;
            const uint16_t* src = a.packed + a.tile_off[mt];
            const size_t koff = (size_t)k0 * kM;  // core-matrix rows of k < k0 come first
            mbar_arrive_tx(&ctl->a_full, 2 * abytes);
            bulk_g2s(a_hi, src + koff, abytes, &ctl->a_full);
            bulk_g2s(a_lo, src + (size_t)kM * Km + koff, abytes, &ctl->a_full);
            a_mt = nslices(Km) == 1 ? mt : -1;
            a_pending = true;
        };
        // (units are walked until the CTA's items run out: counting them up
        // front cost the producer a serial pass over every item)
        bool ok = true;
        Unit cur, nxt;  // nxt: the unit whose strip is copied next
        cur.it.start(a, blockIdx.x);
        cur.sl = 0;
        unit_load(cur);
        nxt = cur;
        int copies = 0;  // strips requested (units 0 .. copies-1)
        for (; copies < 2 && nxt.mt >= 0; ++copies, unit_advance(nxt)) copy_strip(copies, nxt);
        int consumed = 0;
        int i = 0;  // item of the current unit
        for (int u = 0; ok && cur.mt >= 0; ++u) {
            const int b = i & 1;
            const int sbuf = u % kStripBufs;
            const int mt = cur.mt, K = cur.K, S = cur.S, sl = cur.sl;
            ok = mbar_wait(&ctl->strip_full[sbuf], (u / kStripBufs) & 1, abort_flag);
            if (ok) consumed = u + 1;
            if (tracing && sl == 0 && i < kTraceTiles) a.trace[i * TR_N + TR_P_STRIP] = now_ns();
            if (ok && sl == 0 && i >= 2) ok = mbar_wait(&ctl->acc_empty[b], ((i >> 1) - 1) & 1, abort_flag);
            if (ok && (S > 1 || mt != a_mt)) {
                // every MMA that reads the current A (unit u-1 and earlier)
                // must have completed before A is overwritten
                if (u >= 1)
                    ok = mbar_wait(&ctl->unit_done[(u - 1) % kStripBufs], ((u - 1) / kStripBufs) & 1, abort_flag);
                if (ok) {
                    load_a(mt, sl);
                    ok = mbar_wait(&ctl->a_full, a_loads & 1, abort_flag);
                    ++a_loads;
                    if (ok) a_pending = false;
                }
            }
            if (!ok) break;
            if (tracing && sl == 0 && i < kTraceTiles) a.trace[i * TR_N + TR_P_ACC] = now_ns();
            const int ks = slice_len(K, sl);
            tc_fence_after();
            const uint32_t d = tmem + (uint32_t)(b * kN);
            const uint32_t ah = smem_u32(a_hi), al = smem_u32(a_lo);
            const uint32_t bh = smem_u32(strip_hi[sbuf]), bl = smem_u32(strip_lo[sbuf]);
            for (int kk = 0; kk < (ks >> 4); ++kk) {
                // A: next 2 K-chunks (16 row groups * 128 B each); B: next 2 strip blocks
                const uint32_t ao = (uint32_t)kk * 2 * 16 * 128, bo = (uint32_t)kk * 256;
                const uint64_t dah = smem_desc(ah + ao, 16 * 128, 128);
                const uint64_t dal = smem_desc(al + ao, 16 * 128, 128);
                const uint64_t dbh = smem_desc(bh + bo, 128, 128);
                const uint64_t dbl = smem_desc(bl + bo, 128, 128);
                tc_mma(d, dah, dbh, idesc, (sl > 0 || kk > 0) ? 1u : 0u);
                tc_mma(d, dah, dbl, idesc, 1u);
                tc_mma(d, dal, dbh, idesc, 1u);
            }
            tc_commit(&ctl->unit_done[sbuf]);
            if (sl == S - 1) {
                tc_commit(&ctl->mma_done[b]);
                ctl->issued = i + 1;
                if (tracing && i < kTraceTiles) a.trace[i * TR_N + TR_P_ISSUED] = now_ns();
                ++i;
            }
            unit_advance(cur);
            // strip of unit u + 2 into the buffer of unit u - 1, once the MMAs
            // of unit u - 1 (its last reader) are done
            if (nxt.mt >= 0) {
                if (u >= 1)
                    ok = mbar_wait(&ctl->unit_done[(u - 1) % kStripBufs], ((u - 1) / kStripBufs) & 1, abort_flag);
                if (ok) {
                    copy_strip(copies, nxt);
                    ++copies;
                    unit_advance(nxt);
                }
            }
        }
        if (!ok) {
            ctl->abort_flag = 1;
            // copies still in flight land in this CTA's shared memory: wait
            // for them (bounded) before the CTA may exit
            volatile int no_abort = 0;
            for (int j = consumed; j < copies; ++j)
                mbar_wait(&ctl->strip_full[j % kStripBufs], (j / kStripBufs) & 1, &no_abort);
            if (a_pending) mbar_wait(&ctl->a_full, a_loads & 1, &no_abort);
        }
    } else if (warp >= 1) {
        // ================= epilogue: warps 1-8 ================================
        // warp w reads TMEM lane quarter w % 4 (its 32 combo rows) and column
        // half (w - 1) / 4 of the 256 times of a tile.
        const int q4 = warp & 3;
        const int half = (warp - 1) >> 2;
        const int r = q4 * 32 + lane;  // accumulator row = combo within tile
        int cur_mt = -1, p = 1, warm = 0, rbase = 0;
        float rscale = 0.f, rsum = 0.f;
        const bool vec_ok = (a.n & 3) == 0;
        const bool has_nan = a.nanp != nullptr && a.nanp[a.n - 1] > 0.5;
        float* st = TMA_STORE ? reinterpret_cast<float*>(reinterpret_cast<uint8_t*>(stage) + (size_t)(warp - 1) * kStageTma)
                              : stage + (size_t)(warp - 1) * 32 * kStageLd;
        ItemIter it;
        it.start(a, blockIdx.x);
        for (int i = 0; i < ntiles; ++i, it.advance(a)) {
            const int b = i & 1;
            const int mt = it.tile(a);
            const int g = it.time_tile(a);
            const int t0 = g * kN;
            if (mt != cur_mt) {
                cur_mt = mt;
                const int c = mt * kM + r;
                p = c < a.n_combos ? a.periods[c] : 1;
                warm = a.first + p - 1 + (a.warm_extra && c < a.n_combos ? a.warm_extra[c] : 0);
                rscale = a.row_scale[(size_t)mt * kM + r];
                rsum = a.row_sum[(size_t)mt * kM + r];
                rbase = mt * kM + q4 * 32;  // first combo of this warp's rows
            }
            const float ref = __ldg(a.ref + g), xs = __ldg(a.xscale + g);
            // one lane waits, the warp follows (tcgen05.ld is warp-collective)
            int ok = 1;
            if (lane == 0) {
                ok = mbar_wait(&ctl->mma_done[b], (i >> 1) & 1, abort_flag);
                if (!ok) ctl->abort_flag = 1;
            }
            ok = __shfl_sync(0xffffffffu, ok, 0);
            if (!ok) break;
            __syncwarp();
            tc_fence_after();
            const bool tr = tracing && warp == 1 && lane == 0 && i < kTraceTiles;
            if (tr) a.trace[i * TR_N + TR_E_START] = now_ns();
            const float scale = rscale * xs;
            const float off = ref * rsum;
            // tiles past every row's warm-up with a NaN-free series need no masks
            const bool plain = !has_nan && __all_sync(0xffffffffu, t0 >= warm);
            const uint32_t tbase = tmem + ((uint32_t)(q4 * 32) << 16) + (uint32_t)(b * kN + half * 128);
            // the TMEM load of block k + 1 is issued before block k is staged, so
            // it overlaps the wait for the previous block's TMA store
            uint32_t v[32];
            TC_LD32(tbase, v);
#pragma unroll 1
            for (int k = 0; k < 4; ++k) {
                TC_WAIT_LD32(v);
                const int cb = half * 128 + k * 32;
                float y[32];
#pragma unroll
                for (int j = 0; j < 32; ++j) y[j] = fmaf(__uint_as_float(v[j]), scale, off);
                if (k < 3) TC_LD32(tbase + (uint32_t)((k + 1) * 32), v);
                if constexpr (TMA_STORE) {
                    // the staging block is rewritten: wait until the previous
                    // block's store has read it
                    if (lane == 0) asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
                    __syncwarp();
                    // 128-byte swizzle: 16-byte chunk j4 of row `lane` goes to chunk j4 ^ (lane & 7)
                    uint8_t* row8 = reinterpret_cast<uint8_t*>(st) + lane * 128;
#pragma unroll
                    for (int j4 = 0; j4 < 8; ++j4)
                        *reinterpret_cast<float4*>(row8 + ((j4 ^ (lane & 7)) << 4)) =
                            make_float4(y[4 * j4], y[4 * j4 + 1], y[4 * j4 + 2], y[4 * j4 + 3]);
                    if (!plain)
                        mask_staged(reinterpret_cast<float*>(row8), true, lane, t0 + cb, warm, p, has_nan, a.n,
                                    a.nan_mode, a.nanp);
                    // the TMA engine writes the 32 x 32 block (clipping rows / times past the ends)
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                    __syncwarp();
                    if (lane == 0) {
                        asm volatile(
                            "cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%1, %2}], [%3];" ::"l"(
                                reinterpret_cast<uint64_t>(&tmap_out)),
                            "r"(t0 + cb), "r"(rbase), "r"(smem_u32(st))
                            : "memory");
                        asm volatile("cp.async.bulk.commit_group;" ::: "memory");
                    }
                    __syncwarp();
                } else {
#pragma unroll
                    for (int j4 = 0; j4 < 8; ++j4)
                        *reinterpret_cast<float4*>(st + lane * kStageLd + 4 * j4) =
                            make_float4(y[4 * j4], y[4 * j4 + 1], y[4 * j4 + 2], y[4 * j4 + 3]);
                    if (!plain)
                        mask_staged(st + lane * kStageLd, false, lane, t0 + cb, warm, p, has_nan, a.n, a.nan_mode,
                                    a.nanp);
                    __syncwarp();
                    // 8 lanes per row: each store instruction writes 4 rows x 128 B
                    const int c4 = lane & 7;
                    const int tcol = t0 + cb + 4 * c4;
#pragma unroll
                    for (int kk = 0; kk < 8; ++kk) {
                        const int rr = 4 * kk + (lane >> 3);
                        const int cr = rbase + rr;
                        if (cr < a.n_combos) {
                            const float4 yv = *reinterpret_cast<const float4*>(st + rr * kStageLd + 4 * c4);
                            float* o = a.out + (size_t)cr * a.n + tcol;
                            if (vec_ok && tcol + 4 <= a.n) {
                                *reinterpret_cast<float4*>(o) = yv;
                            } else {
                                if (tcol < a.n) o[0] = yv.x;
                                if (tcol + 1 < a.n) o[1] = yv.y;
                                if (tcol + 2 < a.n) o[2] = yv.z;
                                if (tcol + 3 < a.n) o[3] = yv.w;
                            }
                        }
                    }
                    __syncwarp();
                }
            }
            tc_fence_before();
            mbar_arrive(&ctl->acc_empty[b]);
            if (tr) a.trace[i * TR_N + TR_E_END] = now_ns();
        }
        if (TMA_STORE && lane == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
    }

    // drain: the last committed MMAs must have completed before TMEM is freed
    __syncthreads();
    if (tid == 0) {
        const int last = ctl->issued - 1;
        if (last >= 0) {
            const unsigned long long t0 = now_ns();
            while (!mbar_try(&ctl->mma_done[last & 1], (last >> 1) & 1) && now_ns() - t0 < kWaitNs) {
            }
        }
        if (ctl->abort_flag) atomicExch(a.err, 1);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols)
                     : "memory");
    }
}

// Dynamic shared memory for an A capacity of K (whole tiles up to K; larger
// tiles run in kSliceK slices).
size_t smem_bytes_for(int K) {
    const int J = K / 8 + kN / 8 - 1;
    return (size_t)kM * K * 2 * 2 + 2 * kStripBufs * (size_t)J * 128 + 1024 + (size_t)8 * 32 * kStageLd * sizeof(float) +
           sizeof(SmemCtl) + 128;
}

}  // namespace

vta_status launch_wwma_batch_tc(const WwmaBatchArgs& a, int variant, vta_ctx* ctx, cudaStream_t st) {
    const int n_tiles_m = (a.n_combos + kM - 1) / kM;
    const int* per = a.periods_host;
    std::vector<int> tk(n_tiles_m);
    std::vector<long long> toff(n_tiles_m);
    long long off = 0;
    int kbig = 16;
    for (int mt = 0; mt < n_tiles_m; ++mt) {
        int mx = 1;
        for (int r = 0; r < kM && mt * kM + r < a.n_combos; ++r) mx = std::max(mx, per[mt * kM + r]);
        const int K = (mx + 15) & ~15;
        tk[mt] = K;
        toff[mt] = off;
        off += 2LL * kM * K;
        kbig = std::max(kbig, K);
    }
    // A capacity: whole tiles up to kMaxK; larger tiles run in kSliceK slices
    const int ka = std::min(kbig, kMaxK);
    const size_t smem = std::max<size_t>(smem_bytes_for(ka), 160 * 1024);
    if (smem > ctx->smem_optin) return fail(VTA_ERR_NOT_IMPLEMENTED, "tcgen05 path: shared memory");
    const int n_time_tiles = (a.n + kN - 1) / kN;
    const int jmax = kbig / 8 + kN / 8 - 1;
    const size_t strip_tile = (size_t)jmax * 128;
    // operands in the context's second workspace (the first holds the
    // caller's weights and periods during this call)
    auto al256 = [](size_t b) { return (b + 255) & ~size_t(255); };
    const size_t total = al256(n_tiles_m * sizeof(int)) + al256(n_tiles_m * sizeof(long long)) +
                         al256((size_t)off * sizeof(uint16_t)) + 2 * al256((size_t)n_tiles_m * kM * sizeof(float)) +
                         2 * al256(strip_tile * n_time_tiles) + 2 * al256(n_time_tiles * sizeof(float)) +
                         al256(sizeof(int));
    void* buf = nullptr;
    VTA_TRY(ctx_aux(ctx, total, &buf));
    char* bp = static_cast<char*>(buf);
    auto take = [&](size_t bytes) {
        char* r = bp;
        bp += al256(bytes);
        return r;
    };
    int* d_tk = reinterpret_cast<int*>(take(n_tiles_m * sizeof(int)));
    long long* d_toff = reinterpret_cast<long long*>(take(n_tiles_m * sizeof(long long)));
    uint16_t* d_packed = reinterpret_cast<uint16_t*>(take((size_t)off * sizeof(uint16_t)));
    float* d_rs = reinterpret_cast<float*>(take((size_t)n_tiles_m * kM * sizeof(float)));
    float* d_rsum = reinterpret_cast<float*>(take((size_t)n_tiles_m * kM * sizeof(float)));
    uint8_t* d_sh = reinterpret_cast<uint8_t*>(take(strip_tile * n_time_tiles));
    uint8_t* d_sl = reinterpret_cast<uint8_t*>(take(strip_tile * n_time_tiles));
    float* d_ref = reinterpret_cast<float*>(take(n_time_tiles * sizeof(float)));
    float* d_xs = reinterpret_cast<float*>(take(n_time_tiles * sizeof(float)));
    int* d_err = reinterpret_cast<int*>(take(sizeof(int)));
    VTA_TRY(upload_async(ctx, d_tk, tk.data(), n_tiles_m * sizeof(int), st));
    VTA_TRY(upload_async(ctx, d_toff, toff.data(), n_tiles_m * sizeof(long long), st));
    VTA_CUDA_TRY(cudaMemsetAsync(d_err, 0, sizeof(int), st));
    PackArgs pa{a.w, a.kmax, a.n_combos, d_tk, d_toff, d_packed, d_rs, d_rsum};
    if (variant == 1) k_pack_a<1><<<n_tiles_m, kPackThreads, 0, st>>>(pa);
    else k_pack_a<0><<<n_tiles_m, kPackThreads, 0, st>>>(pa);
    VTA_TRY(check_launch("k_pack_a"));
    StripArgs sa{a.x, a.n, a.first, kbig, jmax, d_sh, d_sl, d_ref, d_xs};
    const int L = jmax * 8 + 8;
    const size_t ssmem = (size_t)L * 4 + 2 * (size_t)((L + 7) & ~7) * 2 + 64;
    if (ssmem > ctx->smem_optin) return fail(VTA_ERR_NOT_IMPLEMENTED, "tcgen05 path: period above the strip limit");
    if (variant == 1) {
        VTA_CUDA_TRY(cudaFuncSetAttribute(k_hankel_strips<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ssmem));
        k_hankel_strips<1><<<n_time_tiles, 128, ssmem, st>>>(sa);
    } else {
        VTA_CUDA_TRY(cudaFuncSetAttribute(k_hankel_strips<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ssmem));
        k_hankel_strips<0><<<n_time_tiles, 128, ssmem, st>>>(sa);
    }
    VTA_TRY(check_launch("k_hankel_strips"));

    TcArgs t{};
    t.n = a.n;
    t.first = a.first;
    t.periods = a.periods;
    t.n_combos = a.n_combos;
    t.tile_k = d_tk;
    t.tile_off = d_toff;
    t.packed = d_packed;
    t.row_scale = d_rs;
    t.row_sum = d_rsum;
    t.kmax = kbig;
    t.jmax = jmax;
    t.ka = ka;
    t.jcap = ka / 8 + kN / 8 - 1;
    t.strips_hi = d_sh;
    t.strips_lo = d_sl;
    t.ref = d_ref;
    t.xscale = d_xs;
    t.nan_mode = a.nan_mode;
    t.nanp = a.nanp;
    t.warm_extra = a.warm_extra;
    t.out = a.out;
    t.err = d_err;
    unsigned long long* d_trace = nullptr;
    const char* tr_env = std::getenv("VTA_TC_TRACE");
    if (tr_env && tr_env[0] == '1') {
        VTA_CUDA_TRY(cudaMallocAsync((void**)&d_trace, kTraceTiles * TR_N * 8, st));
        VTA_CUDA_TRY(cudaMemsetAsync(d_trace, 0, kTraceTiles * TR_N * 8, st));
    }
    t.trace = d_trace;
    // persistent: one CTA per SM (the shared memory allows one); the items are
    // cut into grid * k chunks of ~kItemsPerChunk items that the CTAs take
    // round-robin (measured on the 17,920-combo ALMA grid: 1 item 3.69 ms,
    // 8 -> 2.98, 24 -> 2.98, 64 -> 2.93, 128 -> 3.02; a CTA reloads its A tile
    // at every combo-tile change, which drains its MMA pipeline)
    constexpr double kItemsPerChunk = 64.0;
    const long long items = (long long)n_tiles_m * n_time_tiles;
    if (items > INT32_MAX / 2) return fail(VTA_ERR_LAUNCH_CONFIG_TOO_LARGE, "tcgen05 path: too many tiles");
    const int G = (int)std::min<long long>(items, ctx->num_sms);
    int k = std::max(1, (int)std::llround((double)items / ((double)G * kItemsPerChunk)));
    // with few combo tiles every CTA should see each of them (large and small
    // K tiles cost very different MMA time): at least two chunks per tile
    if (n_tiles_m <= 4) k = std::max(k, 2 * n_tiles_m);
    // every chunk must hold at least one item (the CTAs' item walk assumes it)
    k = std::min<long long>(k, std::max<long long>(1, items / G));
    t.n_time_tiles = n_time_tiles;
    t.items = (int)items;
    t.nchunks = G * k;
    dim3 grid((unsigned)G);
    // TMA store path when rows are 16-byte aligned (len % 4 == 0); st.global otherwise
    CUtensorMap tmap;
    std::memset(&tmap, 0, sizeof tmap);
    bool use_tma = (a.n % 4) == 0 && (reinterpret_cast<uintptr_t>(a.out) & 15) == 0;
    if (use_tma) {
        static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
        if (!encode) {
            cudaDriverEntryPointQueryResult q;
            void* fn = nullptr;
            if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
                    cudaSuccess && q == cudaDriverEntryPointSuccess)
                encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
            cudaGetLastError();
        }
        const cuuint64_t dims[2] = {(cuuint64_t)a.n, (cuuint64_t)a.n_combos};
        const cuuint64_t strides[1] = {(cuuint64_t)a.n * sizeof(float)};
        const cuuint32_t box[2] = {32, 32};
        const cuuint32_t estr[2] = {1, 1};
        use_tma = encode && encode(&tmap, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, a.out, dims, strides, box, estr,
                                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                                   CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
    }
    auto kern = variant == 1 ? (use_tma ? k_wwma_tc<1, true> : k_wwma_tc<1, false>)
                             : (use_tma ? k_wwma_tc<0, true> : k_wwma_tc<0, false>);
    VTA_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    ktimer_begin(st);
    kern<<<grid, kThreads, smem, st>>>(t, tmap);
    ktimer_end(st);
    VTA_TRY(check_launch("k_wwma_tc"));
    if (ctx->async_alloc && !d_trace) {
        // server slot: the error word is read when the request completes
        VTA_CUDA_TRY(cudaMemcpyAsync(ctx->err_host, d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
        return VTA_OK;
    }
    int err = 0;
    VTA_CUDA_TRY(cudaMemcpyAsync(&err, d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
    VTA_CUDA_TRY(cudaStreamSynchronize(st));
    if (d_trace) {
        std::vector<unsigned long long> h(kTraceTiles * TR_N);
        cudaMemcpy(h.data(), d_trace, h.size() * 8, cudaMemcpyDeviceToHost);
        cudaFree(d_trace);
        const unsigned long long t0 = h[0];
        std::fprintf(stderr, "tc trace (ns): tile strip_in acc_free issued e_start e_end\n");
        for (int i = 0; i < std::min<long long>(kTraceTiles, items / grid.x); ++i) {
            std::fprintf(stderr, "%3d", i);
            for (int e = 0; e < 5; ++e)
                std::fprintf(stderr, " %8lld", h[i * TR_N + e] ? (long long)(h[i * TR_N + e] - t0) : -1LL);
            std::fprintf(stderr, "\n");
        }
    }
    if (err) return fail(VTA_ERR_CUDA, "tcgen05 contraction: pipeline wait timed out");
    return VTA_OK;
}

}  // namespace vta
