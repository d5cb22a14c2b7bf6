// vta_sma_batch_device_noalloc: the SMA parameter sweep over a device-resident
// series (same result as vta_sma_batch_device, sma_wrapper.rs:830) without any
// device memory allocation.  The crate's sma_batch_dev_from_device allocates
// its period list, f64 prefix and output per call (sma_wrapper.rs:838-841) and
// vta_sma_batch_device grows the context workspace with cudaMalloc; this entry
// point instead carves its working buffers out of one file-scope scratch array
// in static device memory, whose address is looked up once per device.
//
// Scratch layout (256-byte aligned pieces):
//   [0, kPeriodBytes)                  int periods[kMaxCombos]
//   [kBadOff, + 256)                   int bad[2]: first NaN / infinite input
// No piece has to start at zero: the period list is copied in before use and
// the window launcher sets bad[] before its scan.
#include <cstdio>
#include <mutex>

#include "vta_internal.h"

namespace vta {
namespace {

constexpr size_t kMaxLen = VTA_NOALLOC_MAX_LEN;
constexpr size_t kMaxCombos = VTA_NOALLOC_MAX_COMBOS;
constexpr size_t align256(size_t b) { return (b + 255) & ~size_t(255); }
constexpr size_t kPeriodBytes = align256(kMaxCombos * sizeof(int));
constexpr size_t kBadOff = kPeriodBytes;
constexpr size_t kScratchBytes = kBadOff + 256;
static_assert(kScratchBytes == VTA_NOALLOC_SCRATCH_BYTES, "header and layout disagree");

// One copy per device (per CUDA context of the process).  Uninitialised, so it
// takes no space in the shared library; the driver reserves it on a device
// when this translation unit's module is first loaded there.
static __device__ __align__(256) unsigned char g_sma_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
void* g_scratch_ptr[kMaxDevices] = {};

// Address of the scratch on `device`, which the caller has made current.
// First use per device: cudaGetSymbolAddress (loads the module there).
vta_status scratch_on(int device, unsigned char** out) {
    if (device < 0 || device >= kMaxDevices)
        return fail(VTA_ERR_INVALID_INPUT, "sma_batch_device_noalloc: device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if (!g_scratch_ptr[device]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_sma_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(sma no-alloc scratch)");
        if (!p) return fail(VTA_ERR_CUDA, "sma_batch_device_noalloc: null scratch address");
        g_scratch_ptr[device] = p;
    }
    *out = static_cast<unsigned char*>(g_scratch_ptr[device]);
    return VTA_OK;
}

}  // namespace
}  // namespace vta

using namespace vta;

extern "C" vta_status vta_sma_batch_device_noalloc(vta_ctx* ctx, const float* d_data, size_t len,
                                                   size_t first_valid, const vta_period_batch_range* sweep,
                                                   float* d_out) {
    VTA_TRY(enter_call(ctx));
    if (!sweep) return fail(VTA_ERR_INVALID_INPUT, "null sweep");
    if (!d_data) return fail(VTA_ERR_INVALID_INPUT, "null input pointer");
    if (!d_out) return fail(VTA_ERR_INVALID_INPUT, "null output pointer");
    if (len == 0) return fail(VTA_ERR_INVALID_INPUT, "sma: empty data");
    char buf[240];
    if (len > kMaxLen) {
        std::snprintf(buf, sizeof buf,
                      "sma_batch_device_noalloc: len %zu exceeds this entry point's limit of %zu bars "
                      "(VTA_NOALLOC_MAX_LEN); use vta_sma_batch_device",
                      len, kMaxLen);
        return fail(VTA_ERR_INVALID_INPUT, buf);
    }
    // The period count comes from the range arithmetic, so an oversized sweep
    // is rejected before anything is built; the periods are then written
    // straight into a fixed array (no host or device allocation).
    const size_t nc = sma_period_count(sweep->period);
    if (nc > kMaxCombos) {
        std::snprintf(buf, sizeof buf,
                      "sma_batch_device_noalloc: %zu periods exceed the fixed scratch limit of %zu "
                      "(VTA_NOALLOC_MAX_COMBOS); use vta_sma_batch_device",
                      nc, kMaxCombos);
        return fail(VTA_ERR_INVALID_INPUT, buf);
    }
    VTA_TRY(validate_sma_range(sweep->period, nc, len, first_valid));
    const int n = (int)len;

    int periods[kMaxCombos];  // 16 KiB of the caller's stack
    int pmax = 0;
    for (size_t i = 0; i < nc; ++i) {
        periods[i] = (int)sma_period_at(sweep->period, i);
        pmax = periods[i] > pmax ? periods[i] : pmax;
    }

    unsigned char* base = nullptr;
    VTA_TRY(scratch_on(ctx->device, &base));
    int* d_per = reinterpret_cast<int*>(base);
    int* d_bad = reinterpret_cast<int*>(base + kBadOff);

    cudaStream_t st = ctx->stream;
    VTA_CUDA_TRY(cudaMemcpyAsync(d_per, periods, nc * sizeof(int), cudaMemcpyHostToDevice, st));
    PrefixWinArgs a{};
    a.kind = WK_SMA;
    a.x = d_data;
    a.bad = d_bad;
    a.n = n;
    a.first = (int)first_valid;
    a.periods = d_per;
    a.n_combos = (int)nc;
    a.out0 = d_out;
    ctx->last_kernel = "sma_noalloc";
    VTA_TRY(launch_prefix_window_batch(a, pmax, ctx->smem_optin, st));
    // Synchronous like every entry point: the scratch is free again on return.
    VTA_CUDA_TRY(cudaStreamSynchronize(st));
    return check_async("stream");
}
