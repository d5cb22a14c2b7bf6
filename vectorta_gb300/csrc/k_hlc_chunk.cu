// Time-chunked single-series sweeps of ADX and SuperTrend (batch layout:
// one series, lane = parameter combo).
//
// The sequential kernels (k_hlc.cu) run one lane per combo over the whole
// series, so a sweep of a few hundred combos keeps a few warps busy for the
// series' full length.  Here the combos of a 32-combo group are also cut into
// time chunks with the verified warm restart of the many-series plans: a
// chunk that starts past the seeding phase first runs `warm` steps from a
// guessed state (the state decays by (1 - 1/p) per step), records the state
// it reaches at its start and at its end, and k_hlc_chunk_fixup recomputes,
// per combo and in chunk order, every chunk whose recorded start state differs
// (bit for bit) from its predecessor's end state.  Results are therefore
// bit-identical to the sequential kernels.
//
// A warp owns one (group, chunk) item.  The shared inputs of each 32-step tile
// are loaded once per warp (lane j loads step tb + j, one coalesced 128-byte
// row per array) and broadcast step by step with shuffles; outputs are staged
// per warp in shared memory and written as 32 rows x 128 bytes.
#include <algorithm>
#include <type_traits>

#include "hlc_ops.cuh"
#include "vta_internal.h"

namespace vta {
namespace {

constexpr int kCW = 4;  // warps per block

// ops with a wide-tile step form (hlc_ops.cuh)
template <class Op, class = void> struct HasWide : std::false_type {};
template <class Op> struct HasWide<Op, std::void_t<decltype(Op::kWide)>> : std::true_type {};

struct In1 {
    const float *h, *l, *c;
    __device__ float H(int t) const { return __ldg(h + t); }
    __device__ float L(int t) const { return __ldg(l + t); }
    __device__ float C(int t) const { return __ldg(c + t); }
};

__device__ __forceinline__ void store_state(float* dst, const float (&w)[8]) {
    float4* d = reinterpret_cast<float4*>(dst);
    d[0] = make_float4(w[0], w[1], w[2], w[3]);
    d[1] = make_float4(w[4], w[5], w[6], w[7]);
}

template <class Op>
__global__ void __launch_bounds__(kCW * 32) k_hlc_chunk(HlcChunkArgs a) {
    __shared__ float stage0[kCW][32][33];
    __shared__ float stage1[kCW][Op::kTwo ? 32 : 1][33];
    __shared__ float4 xin[kCW][3][8];  // a running tile's high, low and close
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int item = blockIdx.x * kCW + warp;
    if (item >= a.n_items) return;
    const int2 it = a.items[item];
    const int g = it.x, k = it.y;
    const int chunk = a.group_chunk[g];
    const int c0 = k * chunk;
    const int c1 = min(c0 + chunk, a.n);
    const int li = g * 32 + lane;
    const bool valid = li < a.n_combos;
    const int lc = valid ? li : g * 32;  // idle lanes shadow the group's first combo (nothing written)
    Op op;
    op.init(a.periods[lc], a.factors ? a.factors[lc] : 0.f, a.first);
    const In1 in{a.h, a.l, a.c};
    const int W = a.group_warm[g];  // multiple of 32
    const bool warm = k > 0 && __all_sync(0xffffffffu, c0 - W >= op.run_from());
    int t0;
    if (warm) {
        t0 = c0 - W;
        op.start_warm(in, t0);
    } else {
        t0 = min(a.first, c0) & ~31;
        op.start_exact();
    }
    // from rf on every lane of the warp is in its running phase
    const int rf = __reduce_max_sync(0xffffffffu, op.run_from());
    // tiles of 32 steps over [tb0, tend); with `emit` the outputs go to the rows
    auto tiles = [&](int tb0, int tend, bool emit) {
        for (int tb = tb0; tb < tend; tb += 32) {
            const int nt = min(32, tend - tb);
            const int tj = tb + lane;
            float xh = 0.f, xl = 0.f, xc = 0.f;
            if (lane < nt) {
                xh = __ldg(a.h + tj);
                xl = __ldg(a.l + tj);
                xc = __ldg(a.c + tj);
            }
            if (tb >= rf && nt == 32) {
                // the tile's bars from shared memory, four steps per 16-byte
                // broadcast load
                float* xs = reinterpret_cast<float*>(&xin[warp][0][0]);
                __syncwarp();  // the previous tile's reads are done
                xs[lane] = xh;
                xs[32 + lane] = xl;
                xs[64 + lane] = xc;
                __syncwarp();
                auto run32 = [&](auto wide_tag) {
#pragma unroll 2
                    for (int q = 0; q < 8; ++q) {
                        const float4 h4 = xin[warp][0][q], l4 = xin[warp][1][q], c4 = xin[warp][2][q];
                        const float hv[4] = {h4.x, h4.y, h4.z, h4.w}, lv[4] = {l4.x, l4.y, l4.z, l4.w},
                                    cv[4] = {c4.x, c4.y, c4.z, c4.w};
#pragma unroll
                        for (int u = 0; u < 4; ++u) {
                            float o1;
                            const float o0 =
                                op.template step_run<decltype(wide_tag)::value>(hv[u], lv[u], cv[u], o1);
                            if (emit) {
                                stage0[warp][lane][4 * q + u] = o0;
                                if (Op::kTwo) stage1[warp][lane][4 * q + u] = o1;
                            }
                        }
                    }
                };
                bool wide = false;
                if constexpr (HasWide<Op>::value) wide = __all_sync(0xffffffffu, op.wide_ok(xh, xl, xc));
                if (wide)
                    run32(std::true_type{});
                else
                    run32(std::false_type{});
            } else {
                for (int j = 0; j < nt; ++j) {
                    const float hv = __shfl_sync(0xffffffffu, xh, j);
                    const float lv = __shfl_sync(0xffffffffu, xl, j);
                    const float cv = __shfl_sync(0xffffffffu, xc, j);
                    float o1;
                    const float o0 = op.stepv(tb + j, hv, lv, cv, o1);
                    if (emit) {
                        stage0[warp][lane][j] = o0;
                        if (Op::kTwo) stage1[warp][lane][j] = o1;
                    }
                }
            }
            if (emit) {
                __syncwarp();
                if (lane < nt) {
                    for (int r = 0; r < 32; ++r) {
                        const int row = g * 32 + r;
                        if (row >= a.n_combos) break;
                        a.out0[(size_t)row * a.n + tj] = stage0[warp][r][lane];
                        if (Op::kTwo) a.out1[(size_t)row * a.n + tj] = stage1[warp][r][lane];
                    }
                }
                __syncwarp();
            }
        }
    };
    tiles(t0, c0, false);
    float w[8];
    const size_t sidx = (size_t)k * a.n_combos + li;
    if (k > 0 && valid) {
        op.save(w);
        store_state(a.st_start + sidx * 8, w);
        a.exact[sidx] = warm ? 0 : 1;
    }
    tiles(c0, c1, true);
    if (valid) {
        op.save(w);
        store_state(a.st_end + sidx * 8, w);
    }
}

__device__ __forceinline__ bool same_state(const float* x, const float* y) {
    const uint4* p = reinterpret_cast<const uint4*>(x);
    const uint4* q = reinterpret_cast<const uint4*>(y);
    const uint4 a0 = p[0], a1 = p[1], b0 = q[0], b1 = q[1];
    return a0.x == b0.x && a0.y == b0.y && a0.z == b0.z && a0.w == b0.w && a1.x == b1.x && a1.y == b1.y &&
           a1.z == b1.z && a1.w == b1.w;
}

// All (chunk, combo) pairs in parallel: count, per combo, the warm-restarted
// chunks whose start state differs from the end state the kernel left before
// them.  Combos with none need no sequential pass.
__global__ void k_hlc_mismatch(HlcChunkArgs a) {
    const int li = blockIdx.x * blockDim.x + threadIdx.x;
    const int k = blockIdx.y + 1;
    if (li >= a.n_combos) return;
    if ((long long)k * a.group_chunk[li >> 5] >= a.n) return;
    const size_t sidx = (size_t)k * a.n_combos + li;
    if (a.exact[sidx]) return;
    if (!same_state(a.st_start + sidx * 8, a.st_end + (sidx - a.n_combos) * 8)) atomicAdd(&a.need[li], 1);
}

// Per combo with a mismatch, chunks in order: a warm-restarted chunk whose
// start state is not its predecessor's end state is recomputed from that end
// state (which may itself have been recomputed just before).
template <class Op>
__global__ void k_hlc_chunk_fixup(HlcChunkArgs a) {
    const int li = blockIdx.x * blockDim.x + threadIdx.x;
    if (li >= a.n_combos || a.need[li] == 0) return;
    const int chunk = a.group_chunk[li >> 5];
    const In1 in{a.h, a.l, a.c};
    for (int k = 1; (long long)k * chunk < a.n; ++k) {
        const size_t sidx = (size_t)k * a.n_combos + li, pidx = sidx - a.n_combos;
        if (a.exact[sidx]) continue;
        if (same_state(a.st_start + sidx * 8, a.st_end + pidx * 8)) continue;
        const int c0 = k * chunk, c1 = min(c0 + chunk, a.n);
        Op op;
        op.init(a.periods[li], a.factors ? a.factors[li] : 0.f, a.first);
        float w[8];
        for (int i = 0; i < 8; ++i) w[i] = a.st_end[pidx * 8 + i];
        op.load(w, in, c0);
        for (int t = c0; t < c1; ++t) {
            float o1;
            const float o0 = op.step(in, t, o1);
            a.out0[(size_t)li * a.n + t] = o0;
            if (Op::kTwo) a.out1[(size_t)li * a.n + t] = o1;
        }
        op.save(w);
        store_state(a.st_end + sidx * 8, w);
        atomicAdd(a.fixups, 1);
    }
}

}  // namespace

vta_status launch_hlc_chunk(const HlcChunkArgs& a, cudaStream_t st) {
    const unsigned blocks = ceil_div(a.n_items, kCW);
    const unsigned fix_blocks = ceil_div(a.n_combos, 128);
    const dim3 mm_grid(fix_blocks, (unsigned)std::max(1, a.max_chunks - 1));
    ktimer_begin(st);
    if (a.kind == 0) k_hlc_chunk<hlc::PAdx><<<blocks, kCW * 32, 0, st>>>(a);
    else k_hlc_chunk<hlc::PSuperTrend><<<blocks, kCW * 32, 0, st>>>(a);
    VTA_TRY(check_launch("k_hlc_chunk"));
    if (a.max_chunks > 1) {
        k_hlc_mismatch<<<mm_grid, 128, 0, st>>>(a);
        VTA_TRY(check_launch("k_hlc_mismatch"));
    }
    if (a.kind == 0) k_hlc_chunk_fixup<hlc::PAdx><<<fix_blocks, 128, 0, st>>>(a);
    else k_hlc_chunk_fixup<hlc::PSuperTrend><<<fix_blocks, 128, 0, st>>>(a);
    ktimer_end(st);
    return check_launch("k_hlc_chunk_fixup");
}

}  // namespace vta
