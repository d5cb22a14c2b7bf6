// Exact chunked scan of batch ADX sweeps with long periods.
//
// Past its seeding phase (t >= f + 2p) ADX is two linear Wilder levels with a
// pointwise function between them:
//   s <- s * omr + u        s = (atr, +DM, -DM) sums, u = (TR, +DM, -DM) of bar t
//   dx = DX(s)              adx_dx (hlc_ops.cuh)
//   adx <- (adx * pm1 + dx) * rp
// (omr = 1 - 1/p, pm1 = p - 1, rp = 1/p, all f32 as in PAdx).  The
// warm-restart chunking of k_hlc_chunk.cu runs 32 p + 64 steps before every
// chunk, which for periods in the thousands is many times the chunk itself.
// Here a 32-combo group's time axis after its seeding is cut into chunks of L
// steps and processed exactly, like the chunked linear recurrences:
//   AGG1   per (group, chunk): the first level from a zero state over the chunk;
//   CARRY1 per lane: chunk-entry first-level states, s_{k+1} = omr^L s_k + a_k
//          (double-single; s_1 is the seeding run's end state);
//   AGG2   per (group, chunk): the first level from its exact entry state, DX,
//          and the second level from a zero state;
//   CARRY2 per lane: chunk-entry ADX, adx_{k+1} = (pm1 rp)^L adx_k + b_k;
//   EMIT   per (group, chunk): both levels from their entry states, outputs.
// The seeding run (chunk 0, up to the group's s0) is k_hlc_chunk's exact
// chunk-0 item.  Outputs differ from one sequential f32 pass by the rounding
// of the composed carries (a few 1e-7 relative); a NaN bar enters the sums
// through the same NaN-skipping max and comparisons as in the sequential
// pass.
#include <algorithm>
#include <type_traits>

#include "hlc_ops.cuh"
#include "vta_internal.h"

namespace vta {
namespace {

constexpr int kSW = 4;  // warps per block

struct D2s {
    float hi, lo;
};
__device__ __forceinline__ D2s ds_norm(float s, float e) {
    const float hi = s + e;
    return {hi, e - (hi - s)};
}
__device__ __forceinline__ D2s ds_mul(D2s a, D2s b) {
    const float p = a.hi * b.hi;
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e));
    return ds_norm(p, e);
}
__device__ __forceinline__ D2s ds_add(D2s a, D2s b) {
    const float s = a.hi + b.hi;
    const float bb = s - a.hi;
    const float e = ((a.hi - (s - bb)) + (b.hi - bb)) + (a.lo + b.lo);
    return ds_norm(s, e);
}
__device__ __forceinline__ D2s ds_pow(D2s b, long long n) {
    D2s r = {1.f, 0.f};
    while (n > 0) {
        if (n & 1) r = ds_mul(r, b);
        b = ds_mul(b, b);
        n >>= 1;
    }
    return r;
}

struct Lane {
    float omr, pm1, rp;
    __device__ void init(int p) {
        rp = (float)(1.0 / (double)p);
        omr = (float)(1.0 - 1.0 / (double)p);
        pm1 = (float)p - 1.f;
    }
};

enum { PASS_AGG1 = 0, PASS_AGG2 = 1, PASS_EMIT = 2 };


// One (group, chunk >= 1) item per warp; lane = combo of the group.
template <int PASS>
__global__ void __launch_bounds__(kSW * 32) k_adx_scan(AdxScanArgs a) {
    __shared__ float stage[kSW][32][33];
    __shared__ float4 xin[kSW][3][8];  // a full tile's high, low and close
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int item = blockIdx.x * kSW + warp;
    if (item >= a.n_items) return;
    const int2 it = a.items[item];
    const int gi = it.x, k = it.y;
    const int g = a.groups[gi];
    const int c0 = a.group_s0[gi] + (k - 1) * a.L;
    const int c1 = min(c0 + a.L, a.n);
    const int ci = g * 32 + lane;  // combo
    const bool valid = ci < a.n_combos;
    const size_t si = (size_t)k * a.n_slots + gi * 32 + lane;  // state slot
    Lane ln;
    ln.init(__ldg(a.periods + (valid ? ci : g * 32)));
    float atr = 0.f, pdm = 0.f, mdm = 0.f, adx = 0.f;
    if (PASS != PASS_AGG1) {
        const float4 s = a.carry1[si];
        atr = s.x;
        pdm = s.y;
        mdm = s.z;
    }
    if (PASS == PASS_EMIT) adx = a.carry2[si];
    // inputs of the bar before the chunk (c0 >= 1)
    float ph = __ldg(a.h + c0 - 1), pl = __ldg(a.l + c0 - 1), pc = __ldg(a.c + c0 - 1);
    for (int tb = c0; tb < c1; tb += 32) {
        const int nt = min(32, c1 - tb);
        float xh = 0.f, xl = 0.f, xc = 0.f;
        if (lane < nt) {
            xh = __ldg(a.h + tb + lane);
            xl = __ldg(a.l + tb + lane);
            xc = __ldg(a.c + tb + lane);
        }
        // one step on the bar (ch, cl, cc): PAdx::step_run's arithmetic
        auto step = [&](int j, float ch, float cl, float cc, auto wide_tag) {
            constexpr bool WIDE = decltype(wide_tag)::value;
            const float tr = fmaxf(fmaxf(ch - cl, fabsf(ch - pc)), fabsf(cl - pc));
            const float up = ch - ph, down = pl - cl;
            const float dp = (up > down && up > 0.f) ? up : 0.f;
            const float dm = (down > up && down > 0.f) ? down : 0.f;
            atr = atr * ln.omr + tr;
            pdm = pdm * ln.omr + dp;
            mdm = mdm * ln.omr + dm;
            if (PASS != PASS_AGG1) {
                const float dx = WIDE ? hlc::adx_dx_wide(pdm, mdm) : hlc::adx_dx(pdm, mdm, atr);
                adx = (adx * ln.pm1 + dx) * ln.rp;
            }
            if (PASS == PASS_EMIT) stage[warp][lane][j] = adx;
            ph = ch;
            pl = cl;
            pc = cc;
        };
        // A full tile reads its bars from shared memory, four steps per
        // 16-byte broadcast load, in a fully unrolled loop; a partial tile
        // broadcasts them by shuffles.
        auto steps = [&](auto wide_tag) {
            if (nt == 32) {
                float* xs = reinterpret_cast<float*>(&xin[warp][0][0]);
                __syncwarp();  // the previous tile's reads are done
                xs[lane] = xh;
                xs[32 + lane] = xl;
                xs[64 + lane] = xc;
                __syncwarp();
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    const float4 h4 = xin[warp][0][q], l4 = xin[warp][1][q], c4 = xin[warp][2][q];
                    step(4 * q, h4.x, l4.x, c4.x, wide_tag);
                    step(4 * q + 1, h4.y, l4.y, c4.y, wide_tag);
                    step(4 * q + 2, h4.z, l4.z, c4.z, wide_tag);
                    step(4 * q + 3, h4.w, l4.w, c4.w, wide_tag);
                }
            } else {
                for (int j = 0; j < nt; ++j)
                    step(j, __shfl_sync(0xffffffffu, xh, j), __shfl_sync(0xffffffffu, xl, j),
                         __shfl_sync(0xffffffffu, xc, j), wide_tag);
            }
        };
        // DX by the hardware reciprocal where the sums stay normal over
        // these steps (hlc::adx_wide_ok)
        const bool wide = PASS != PASS_AGG1 &&
                          __all_sync(0xffffffffu, hlc::adx_wide_ok(atr, pdm, mdm, xh, xl, xc, ph, pl, pc));
        if (wide)
            steps(std::true_type{});
        else
            steps(std::false_type{});
        if (PASS == PASS_EMIT) {
            __syncwarp();
            if (lane < nt)
                for (int r = 0; r < 32; ++r) {
                    const int row = g * 32 + r;
                    if (row >= a.n_combos) break;
                    a.out[(size_t)row * a.n + tb + lane] = stage[warp][r][lane];
                }
            __syncwarp();
        }
    }
    if (PASS == PASS_AGG1) a.agg1[si] = make_float4(atr, pdm, mdm, 0.f);
    if (PASS == PASS_AGG2) a.agg2[si] = adx;
}

// Chunk-entry states per lane slot, in double-single: one warp per slot.
// LEVEL 1: s_1 = the seeding run's end state, s_{k+1} = m s_k + agg1_k with
// m = omr^L; LEVEL 2: adx_1 likewise with m = (pm1 rp)^L and agg2.  Every
// transition k = 1 .. nch - 2 is over a full chunk, so all share m: the warp
// splits them into 32 consecutive blocks, each thread composes its block into
// one affine map x -> A x + B, the maps are scanned across the warp (five
// shuffle levels), and each thread then walks its block again from its
// entry state, writing the entries.
struct Aff {
    D2s A, B[3];
};
__device__ __forceinline__ D2s ds_shfl_up(D2s v, int o) {
    return {__shfl_up_sync(0xffffffffu, v.hi, o), __shfl_up_sync(0xffffffffu, v.lo, o)};
}
template <int LEVEL>
__global__ void __launch_bounds__(128) k_adx_carry(AdxScanArgs a) {
    constexpr int NC = LEVEL == 1 ? 3 : 1;
    const int slot = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (slot >= a.n_slots) return;  // warp-uniform
    const int gi = slot >> 5;
    const int ci = a.groups[gi] * 32 + (slot & 31);
    if (ci >= a.n_combos) return;  // warp-uniform
    Lane ln;
    ln.init(__ldg(a.periods + ci));
    const int s0 = a.group_s0[gi];
    const int nch = 1 + (a.n - s0 + a.L - 1) / a.L;  // chunks of the group, chunk 0 included
    const float* seed = a.seed_state + (size_t)ci * 8;  // k_hlc_chunk's chunk-0 end state
    const D2s m = LEVEL == 1 ? D2s{ln.omr, 0.f} : ds_mul({ln.pm1, 0.f}, {ln.rp, 0.f});
    const D2s mL = ds_pow(m, a.L);
    auto agg = [&](int k) {
        const size_t si = (size_t)k * a.n_slots + slot;
        return LEVEL == 1 ? __ldg(a.agg1 + si) : make_float4(__ldg(a.agg2 + si), 0.f, 0.f, 0.f);
    };
    auto put = [&](int k, const D2s (&x)[NC]) {
        const size_t si = (size_t)k * a.n_slots + slot;
        if (LEVEL == 1)
            a.carry1[si] = make_float4(x[0].hi + x[0].lo, x[1].hi + x[1].lo, x[2].hi + x[2].lo, 0.f);
        else
            a.carry2[si] = x[0].hi + x[0].lo;
    };
    // transitions 1 .. T, T = nch - 2; this thread's block [k0, k1)
    const int T = nch - 2;
    const int per = T > 0 ? (T + 31) / 32 : 0;
    const int k0 = 1 + min(T, lane * per), k1 = 1 + min(T, (lane + 1) * per);
    Aff f;
    f.A = {1.f, 0.f};
#pragma unroll
    for (int c = 0; c < NC; ++c) f.B[c] = {0.f, 0.f};
#pragma unroll 1
    for (int k = k0; k < k1; ++k) {
        const float4 g4 = agg(k);
        const float g[3] = {g4.x, g4.y, g4.z};
        f.A = ds_mul(mL, f.A);
#pragma unroll
        for (int c = 0; c < NC; ++c) f.B[c] = ds_add(ds_mul(mL, f.B[c]), {g[c], 0.f});
    }
    // inclusive scan of the maps in lane order: (later) o (earlier)
#pragma unroll 1
    for (int o = 1; o < 32; o <<= 1) {
        Aff e;
        e.A = ds_shfl_up(f.A, o);
#pragma unroll
        for (int c = 0; c < NC; ++c) e.B[c] = ds_shfl_up(f.B[c], o);
        if (lane >= o) {
#pragma unroll
            for (int c = 0; c < NC; ++c) f.B[c] = ds_add(ds_mul(f.A, e.B[c]), f.B[c]);
            f.A = ds_mul(f.A, e.A);
        }
    }
    // exclusive map of this thread: the previous lane's inclusive one
    Aff x;
    x.A = ds_shfl_up(f.A, 1);
#pragma unroll
    for (int c = 0; c < NC; ++c) x.B[c] = ds_shfl_up(f.B[c], 1);
    D2s st[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) {
        const D2s sd = {seed[LEVEL == 1 ? c : 3], 0.f};
        st[c] = lane == 0 ? sd : ds_add(ds_mul(x.A, sd), x.B[c]);
    }
#pragma unroll 1
    for (int k = k0; k < k1; ++k) {
        put(k, st);
        const float4 g4 = agg(k);
        const float g[3] = {g4.x, g4.y, g4.z};
#pragma unroll
        for (int c = 0; c < NC; ++c) st[c] = ds_add(ds_mul(mL, st[c]), {g[c], 0.f});
    }
    // the last chunk's entry (k = nch - 1) from the thread whose block ends there
    if (nch >= 2 && k1 == nch - 1 && (k0 < k1 || lane == 0)) put(nch - 1, st);
}

}  // namespace

vta_status launch_adx_scan(const AdxScanArgs& a, cudaStream_t st) {
    if (a.n_items <= 0) return VTA_OK;
    const unsigned blocks = ceil_div(a.n_items, kSW);
    const unsigned cblocks = ceil_div((size_t)a.n_slots * 32, 128);  // a warp per lane slot
    k_adx_scan<PASS_AGG1><<<blocks, kSW * 32, 0, st>>>(a);
    VTA_TRY(check_launch("k_adx_scan<agg1>"));
    k_adx_carry<1><<<cblocks, 128, 0, st>>>(a);
    VTA_TRY(check_launch("k_adx_carry<1>"));
    k_adx_scan<PASS_AGG2><<<blocks, kSW * 32, 0, st>>>(a);
    VTA_TRY(check_launch("k_adx_scan<agg2>"));
    k_adx_carry<2><<<cblocks, 128, 0, st>>>(a);
    VTA_TRY(check_launch("k_adx_carry<2>"));
    k_adx_scan<PASS_EMIT><<<blocks, kSW * 32, 0, st>>>(a);
    return check_launch("k_adx_scan<emit>");
}

}  // namespace vta
