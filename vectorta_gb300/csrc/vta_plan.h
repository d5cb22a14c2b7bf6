// Shared by the many-series work-list kernels (k_tm_plan.cu) and the plan
// host code (vta_plan.cu).  Not part of the C ABI.
#pragma once

#include "vta_internal.h"

namespace vta {

enum PlanKind { PJ_ATR = 0, PJ_ADX = 1, PJ_SUPERTREND = 2, PJ_PERCENTILE = 3 };

// One indicator over all series of a plan (device copy).
struct PlanJob {
    int kind;
    int period;           // ATR length, ADX / SuperTrend period, percentile length
    float param;          // SuperTrend factor
    double pfrac;         // percentile percentage * 0.01
    int chunk;            // time-chunk length of the work items
    int warm;             // warm-restart steps before a chunk (recurrent jobs)
    float* out0;          // [rows][cols]: atr / adx / trend / percentile
    float* out1;          // SuperTrend changed
    float* st_start;      // [n_chunks][cols][8] state entering each chunk (warm runs)
    float* st_end;        // [n_chunks][cols][8] state at each chunk's end
    unsigned char* exact; // [n_chunks][cols] chunk computed from the series start
};

struct PlanArgs {
    const float* h;
    const float* l;
    const float* c;
    int cols, rows;
    const int* len;        // [cols] series lengths (<= rows)
    const int* first_hlc;  // [cols] first index with high, low and close valid
    const int* first_c;    // [cols] first valid close
    const PlanJob* jobs;
    int n_jobs;
    const int4* items;     // {job, tile, chunk, 0}
    int n_items;
    int* counter;          // work-list head (zeroed before each launch)
    int* stats;            // [0] chunks recomputed by the fix-up pass
};

inline bool plan_job_recurrent(int kind) { return kind != PJ_PERCENTILE; }
constexpr int kPlanMaxPnrWindow = 64;  // percentile windows kept in registers

// First valid index per series within its length (close; high+low+close).
vta_status launch_plan_first(const PlanArgs& a, int* first_hlc, int* first_c, cudaStream_t st);
// Persistent work-list launch (`blocks` CTAs) and the fix-up pass.
vta_status launch_tm_plan(const PlanArgs& a, int blocks, cudaStream_t st);
vta_status launch_tm_fixup(const PlanArgs& a, cudaStream_t st);
// CTAs of the persistent launch that fit on the device at once.
int tm_plan_blocks(int num_sms);

}  // namespace vta
