// Many-series work-list kernels: several indicators over one set of ragged
// time-major OHLC series in one persistent launch.
//
// Work items are (job, tile of 32 consecutive series, time chunk).  A warp
// takes items from a global counter; lane l of the warp owns series
// 32 * tile + l, so every load and store of a time step is one coalesced
// 128-byte row segment.  Series of uneven length stop at their own length:
// cells past it are neither read nor written.
//
// Recurrent jobs (ATR, ADX, SuperTrend) are cut into time chunks with a
// verified warm restart.  Chunk k (c0 = k * chunk) that starts past the
// indicator's seeding phase runs `warm` steps before c0 from a state guessed
// from the inputs; since every state component decays by (1 - 1/p) per step
// the guess is forgotten, and the state it reaches at c0 is recorded.  Every
// chunk also records its state at its end.  k_tm_fixup then walks each
// series' chunks in order and compares (bit for bit) the recorded start state
// of chunk k with the end state of chunk k - 1; where they differ it recomputes
// chunk k from that exact end state.  The outputs are therefore bit-identical
// to one sequential pass over the series, whatever the chunk and warm lengths.
// The percentile job is exact per chunk by construction (its window is
// rebuilt from the `length` inputs before c0).
#include <cfloat>

#include "vta_internal.h"
#include "vta_plan.h"
#include "hlc_ops.cuh"
#include "pnr_ops.cuh"

namespace vta {
namespace {

constexpr int kPlanWarps = 4;
__device__ __forceinline__ float qnan() { return __int_as_float(0x7fc00000); }

struct TmIn {
    const float *h, *l, *c;
    size_t cols, s;
    __device__ float H(int t) const { return __ldg(h + (size_t)t * cols + s); }
    __device__ float L(int t) const { return __ldg(l + (size_t)t * cols + s); }
    __device__ float C(int t) const { return __ldg(c + (size_t)t * cols + s); }
};

using hlc::PAtr;
using hlc::PAdx;
using hlc::PSuperTrend;

// ------------------------------------------------ nearest-rank percentile ---
// (the sorted register window of pnr_ops.cuh)
using pnr::pick;
using pnr::rank;

// ------------------------------------------------ chunk runners -------------
// Inputs are staged per warp in shared memory: a double buffer of kPB steps
// x {high, low, close} x 32 lanes, filled with cp.async (4 bytes per lane and
// value, so each step of a warp is one 128-byte row segment).  Each lane
// copies and reads only its own column, so no cross-lane synchronisation is
// needed; while a block is computed the next one is in flight, so a warp
// waits for memory about once per kPB steps instead of once per step.
constexpr int kPB = 16;
constexpr int kStageFloats = 2 * 3 * kPB * 32;  // per warp
constexpr size_t kPlanSmem = (size_t)kPlanWarps * kStageFloats * sizeof(float);

__device__ __forceinline__ void cp_async4(float* dst, const float* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)),
                 "l"(src)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }

struct Stage {
    float* base;  // this warp's [2][3][kPB][32]
    int lane;
    __device__ float* at(int buf, int arr, int j) const { return base + ((buf * 3 + arr) * kPB + j) * 32 + lane; }
    // copies of steps [tb, min(tb + kPB, tend)) of the given arrays into `buf`
    __device__ void load(int buf, const float* a0, const float* a1, const float* a2, size_t cols, size_t s,
                         int tb, int tend) const {
        for (int j = 0; j < kPB && tb + j < tend; ++j) {
            const size_t g = (size_t)(tb + j) * cols + s;
            if (a0) cp_async4(at(buf, 0, j), a0 + g);
            if (a1) cp_async4(at(buf, 1, j), a1 + g);
            if (a2) cp_async4(at(buf, 2, j), a2 + g);
        }
        cp_async_commit();
    }
};

// Steps t in [t, tend); with `emit` writes the outputs of each step.
template <class Op>
__device__ void run_span(Op& op, const TmIn& in, const Stage& sg, int t, int tend, bool emit, float* out0,
                         float* out1) {
    if (t >= tend) return;
    const int rf = op.run_from();  // from here on the running update alone
    sg.load(0, in.h, in.l, in.c, in.cols, in.s, t, tend);
    int buf = 0;
    for (int tb = t; tb < tend; tb += kPB, buf ^= 1) {
        // next block in flight (an empty group at the end keeps the count)
        sg.load(buf ^ 1, in.h, in.l, in.c, in.cols, in.s, tb + kPB, tend);
        cp_async_wait1();
        const int te = min(tb + kPB, tend);
        for (int tt = tb; tt < te; ++tt) {
            const int j = tt - tb;
            float o1;
            const float hv = *sg.at(buf, 0, j), lv = *sg.at(buf, 1, j), cv = *sg.at(buf, 2, j);
            const float o0 = tt >= rf ? op.step_run(hv, lv, cv, o1) : op.stepv(tt, hv, lv, cv, o1);
            if (emit) {
                out0[(size_t)tt * in.cols + in.s] = o0;
                if (Op::kTwo) out1[(size_t)tt * in.cols + in.s] = o1;
            }
        }
    }
}

// Percentile chunk [c0, c1) of each lane.  All lanes of the warp run one
// time loop over [c0 - len + 1, max c1) in step: each step removes the value
// leaving the window and inserts the one entering (NaN values are never in
// the window, which also covers the NaN lead), and writes its output when
// the step is inside the lane's own chunk.  A lane whose series has ended
// follows along without inserting or writing.  Keeping the lanes on one
// loop (instead of each running its own window build and loop) keeps the
// warp converged.
template <int W>
__device__ void pnr_chunk(const TmIn& in, const Stage& sg, unsigned mask, int f, int L, int len, double pf, int c0,
                          int c1, float* out) {
    const int tend = __reduce_max_sync(mask, c1);
    if (tend <= c0) return;  // warp-uniform
    const int tbeg = max(0, c0 - len + 1);
    const int start = f + len - 1;
    const int kfull = rank(pf, len);
    float w[W];
#pragma unroll
    for (int i = 0; i < W; ++i) w[i] = __int_as_float(0x7f800000);
    int wl = 0;
    // staged arrays: 0 = entering x[u], 1 = leaving x[u - len]
    auto load = [&](int buf, int ub) {
        for (int j = 0; j < kPB && ub + j < tend; ++j) {
            const int u = ub + j, uo = u - len;
            if (u < L) cp_async4(sg.at(buf, 0, j), in.c + (size_t)u * in.cols + in.s);
            if (uo >= tbeg && uo < L) cp_async4(sg.at(buf, 1, j), in.c + (size_t)uo * in.cols + in.s);
        }
        cp_async_commit();
    };
    load(0, tbeg);
    int buf = 0;
    for (int ub = tbeg; ub < tend; ub += kPB, buf ^= 1) {
        load(buf ^ 1, ub + kPB);
        cp_async_wait1();
        const int ue = min(ub + kPB, tend);
        for (int u = ub; u < ue; ++u) {
            const int j = u - ub, uo = u - len;
            const float vo = (uo >= tbeg && uo < L) ? *sg.at(buf, 1, j) : qnan();
            const float vi = u < L ? *sg.at(buf, 0, j) : qnan();
            pnr::replace(w, vo, vi);
            wl += (isnan(vi) ? 0 : 1) - (isnan(vo) ? 0 : 1);
            if (u >= c0 && u < c1)
                out[(size_t)u * in.cols + in.s] = u < start ? qnan() : pick(w, wl, len, kfull, pf);
        }
    }
}

template <class Op>
__device__ void run_chunk(const PlanArgs& a, const PlanJob& J, int s, int k, const Stage& sg) {
    const int L = a.len[s];
    const int c0 = k * J.chunk;
    if (c0 >= L) return;
    const int c1 = min(c0 + J.chunk, L);
    const int f = a.first_hlc[s];
    Op op;
    op.init(J.period, J.param, f);
    const TmIn in{a.h, a.l, a.c, (size_t)a.cols, (size_t)s};
    const size_t sidx = (size_t)k * a.cols + s;
    int t;
    bool exact = true;
    if (k > 0 && f < L && c0 - J.warm >= op.run_from()) {
        t = c0 - J.warm;
        op.start_warm(in, t);
        exact = false;
    } else {
        t = min(f, c0);
        op.start_exact();
    }
    run_span(op, in, sg, t, c0, false, J.out0, J.out1);
    float w[8];
    if (k > 0) {
        op.save(w);
        float4* d = reinterpret_cast<float4*>(J.st_start + sidx * 8);
        d[0] = make_float4(w[0], w[1], w[2], w[3]);
        d[1] = make_float4(w[4], w[5], w[6], w[7]);
        J.exact[sidx] = exact ? 1 : 0;
    }
    run_span(op, in, sg, c0, c1, true, J.out0, J.out1);
    op.save(w);
    float4* d = reinterpret_cast<float4*>(J.st_end + sidx * 8);
    d[0] = make_float4(w[0], w[1], w[2], w[3]);
    d[1] = make_float4(w[4], w[5], w[6], w[7]);
}

// `mask`: the lanes of the warp working on this item (all of them call).
__device__ void run_pnr(const PlanArgs& a, const PlanJob& J, int s, int k, const Stage& sg, unsigned mask) {
    const int L = a.len[s];
    const int c0 = k * J.chunk;
    const int c1 = max(c0, min(c0 + J.chunk, L));
    const TmIn in{a.h, a.l, a.c, (size_t)a.cols, (size_t)s};
    const int f = a.first_c[s];
    // window registers: the length rounded up to a multiple of 8
    switch ((J.period + 7) >> 3) {
        case 1: case 2: pnr_chunk<16>(in, sg, mask, f, L, J.period, J.pfrac, c0, c1, J.out0); break;
        case 3: pnr_chunk<24>(in, sg, mask, f, L, J.period, J.pfrac, c0, c1, J.out0); break;
        case 4: pnr_chunk<32>(in, sg, mask, f, L, J.period, J.pfrac, c0, c1, J.out0); break;
        case 5: pnr_chunk<40>(in, sg, mask, f, L, J.period, J.pfrac, c0, c1, J.out0); break;
        case 6: pnr_chunk<48>(in, sg, mask, f, L, J.period, J.pfrac, c0, c1, J.out0); break;
        case 7: pnr_chunk<56>(in, sg, mask, f, L, J.period, J.pfrac, c0, c1, J.out0); break;
        default: pnr_chunk<64>(in, sg, mask, f, L, J.period, J.pfrac, c0, c1, J.out0); break;
    }
}

// Persistent work-list kernel: each warp takes items until the list is done.
__global__ void __launch_bounds__(kPlanWarps * 32) k_tm_plan(PlanArgs a) {
    extern __shared__ float plan_smem[];
    const int lane = threadIdx.x & 31;
    const Stage sg{plan_smem + (threadIdx.x >> 5) * kStageFloats, lane};
    for (;;) {
        int it = 0;
        if (lane == 0) it = atomicAdd(a.counter, 1);
        it = __shfl_sync(0xffffffffu, it, 0);
        if (it >= a.n_items) break;
        const int4 w = a.items[it];
        const int s = w.y * 32 + lane;
        const unsigned mask = __ballot_sync(0xffffffffu, s < a.cols);
        if (s >= a.cols) continue;
        const PlanJob& J = a.jobs[w.x];
        switch (J.kind) {
            case PJ_ATR: run_chunk<PAtr>(a, J, s, w.z, sg); break;
            case PJ_ADX: run_chunk<PAdx>(a, J, s, w.z, sg); break;
            case PJ_SUPERTREND: run_chunk<PSuperTrend>(a, J, s, w.z, sg); break;
            default: run_pnr(a, J, s, w.z, sg, mask); break;
        }
    }
}

// Fix-up: per (recurrent job, series), chunks in order; a warm-restarted
// chunk whose recorded start state differs from the previous chunk's end
// state is recomputed from that end state.
template <class Op>
__device__ void fixup_series(const PlanArgs& a, const PlanJob& J, int s) {
    const int L = a.len[s];
    const TmIn in{a.h, a.l, a.c, (size_t)a.cols, (size_t)s};
    for (int k = 1; k * J.chunk < L; ++k) {
        const size_t sidx = (size_t)k * a.cols + s;
        if (J.exact[sidx]) continue;
        const size_t pidx = sidx - a.cols;
        const uint4* ps = reinterpret_cast<const uint4*>(J.st_start + sidx * 8);
        const uint4* pe = reinterpret_cast<const uint4*>(J.st_end + pidx * 8);
        const uint4 s0 = ps[0], s1 = ps[1], e0 = pe[0], e1 = pe[1];
        if (s0.x == e0.x && s0.y == e0.y && s0.z == e0.z && s0.w == e0.w && s1.x == e1.x && s1.y == e1.y &&
            s1.z == e1.z && s1.w == e1.w)
            continue;
        const int c0 = k * J.chunk;
        const int c1 = min(c0 + J.chunk, L);
        Op op;
        op.init(J.period, J.param, a.first_hlc[s]);
        const float* we = J.st_end + pidx * 8;
        float w[8];
        for (int i = 0; i < 8; ++i) w[i] = we[i];
        op.load(w, in, c0);
        float o1;
        for (int t = c0; t < c1; ++t) {
            const float o0 = op.step(in, t, o1);
            J.out0[(size_t)t * a.cols + s] = o0;
            if (Op::kTwo) J.out1[(size_t)t * a.cols + s] = o1;
        }
        op.save(w);
        float4* d = reinterpret_cast<float4*>(J.st_end + sidx * 8);
        d[0] = make_float4(w[0], w[1], w[2], w[3]);
        d[1] = make_float4(w[4], w[5], w[6], w[7]);
        atomicAdd(&a.stats[0], 1);
    }
}

__global__ void k_tm_fixup(PlanArgs a) {
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int j = (int)(g / a.cols), s = (int)(g % a.cols);
    if (j >= a.n_jobs) return;
    const PlanJob& J = a.jobs[j];
    switch (J.kind) {
        case PJ_ATR: fixup_series<PAtr>(a, J, s); break;
        case PJ_ADX: fixup_series<PAdx>(a, J, s); break;
        case PJ_SUPERTREND: fixup_series<PSuperTrend>(a, J, s); break;
        default: break;
    }
}

// First valid index per series within its own length: close alone and
// high, low and close together (len[s] when there is none).
// First valid row of each series: close alone (percentile) and high, low and
// close together (the high/low/close jobs).  Rows are examined kFirstRows at a
// time; the block's loads are all issued before any is tested (rows clamped
// into the series, no short-circuit), so the NaN lead costs few memory round
// trips.
constexpr int kFirstRows = 16;

__global__ void k_plan_first(PlanArgs a, int* first_hlc, int* first_c) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= a.cols) return;
    const int L = a.len[s];
    const TmIn in{a.h, a.l, a.c, (size_t)a.cols, (size_t)s};
    int fc = L, fh = L;
    for (int t0 = 0; t0 < L && fh == L; t0 += kFirstRows) {
        float hv[kFirstRows], lv[kFirstRows], cv[kFirstRows];
#pragma unroll
        for (int j = 0; j < kFirstRows; ++j) {
            const int t = min(t0 + j, L - 1);
            cv[j] = in.C(t);
            hv[j] = in.H(t);
            lv[j] = in.L(t);
        }
        int bc = L, bh = L;  // first hit of this block
#pragma unroll
        for (int j = kFirstRows - 1; j >= 0; --j) {
            const bool okc = (t0 + j < L) & !isnan(cv[j]);
            if (okc) bc = t0 + j;
            if (okc & !isnan(hv[j]) & !isnan(lv[j])) bh = t0 + j;
        }
        if (fc == L) fc = bc;
        fh = bh;
    }
    first_c[s] = fc;
    first_hlc[s] = fh;
}

}  // namespace

vta_status launch_plan_first(const PlanArgs& a, int* first_hlc, int* first_c, cudaStream_t st) {
    k_plan_first<<<(a.cols + 127) / 128, 128, 0, st>>>(a, first_hlc, first_c);
    return check_launch("k_plan_first");
}

int tm_plan_blocks(int num_sms) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_tm_plan, kPlanWarps * 32, kPlanSmem) != cudaSuccess ||
        per_sm < 1) {
        cudaGetLastError();
        per_sm = 1;
    }
    return num_sms * per_sm;
}

vta_status launch_tm_plan(const PlanArgs& a, int blocks, cudaStream_t st) {
    k_tm_plan<<<blocks, kPlanWarps * 32, kPlanSmem, st>>>(a);
    return check_launch("k_tm_plan");
}

vta_status launch_tm_fixup(const PlanArgs& a, cudaStream_t st) {
    const long long n = (long long)a.n_jobs * a.cols;
    k_tm_fixup<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(a);
    return check_launch("k_tm_fixup");
}

}  // namespace vta
