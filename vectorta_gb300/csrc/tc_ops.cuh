// tcgen05 / bulk-copy / mbarrier primitives shared by the tensor-core
// contraction kernels (inline PTX for sm_103a).  Every wait on an mbarrier is
// bounded: past its time limit it returns false so the caller can raise an
// error flag, drain its own copies and MMAs, free TMEM and return.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdint.h>

namespace vta {
namespace tc {

constexpr unsigned long long kTcWaitNs = 2000000000ull;  // 2 s per wait

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ unsigned long long now_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// ------------------------------------------------------------ mbarrier ----
__device__ __forceinline__ void mbar_init(uint64_t* b, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* b) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(b)) : "memory");
}
__device__ __forceinline__ void mbar_arrive_tx(uint64_t* b, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try(uint64_t* b, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_u32(b)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait: false on timeout or when another thread raised the abort flag.
__device__ inline bool mbar_wait(uint64_t* b, uint32_t parity, volatile int* abort_flag,
                                 unsigned long long limit_ns = kTcWaitNs) {
    const unsigned long long t0 = now_ns();
    for (;;) {
        if (mbar_try(b, parity)) return true;
        if (*abort_flag) return false;
        if (now_ns() - t0 > limit_ns) return false;
    }
}

// ------------------------------------------------------------ tcgen05 -----
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Shared-memory matrix descriptor, no swizzle: start, leading / stride byte
// offsets (>> 4), descriptor version 1 at bits 46-47.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46);
}

__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}
__device__ __forceinline__ void tc_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_u32(bar))
                 : "memory");
}

#define TC_LD32(taddr, r)                                                                                   \
    asm volatile(                                                                                           \
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16," \
        "%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"                              \
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),   \
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),          \
          "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),        \
          "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),        \
          "=r"(r[29]), "=r"(r[30]), "=r"(r[31])                                                              \
        : "r"(taddr))

// Waits for this thread's tcgen05.ld to complete; the 32 destination registers
// are operands, so no use of them can be scheduled before the wait.
#define TC_WAIT_LD32(r)                                                                                   \
    asm volatile("tcgen05.wait::ld.sync.aligned;"                                                         \
                 : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]),     \
                   "+r"(r[7]), "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), \
                   "+r"(r[14]), "+r"(r[15]), "+r"(r[16]), "+r"(r[17]), "+r"(r[18]), "+r"(r[19]),          \
                   "+r"(r[20]), "+r"(r[21]), "+r"(r[22]), "+r"(r[23]), "+r"(r[24]), "+r"(r[25]),          \
                   "+r"(r[26]), "+r"(r[27]), "+r"(r[28]), "+r"(r[29]), "+r"(r[30]), "+r"(r[31])           \
                 :                                                                                        \
                 : "memory")

// ------------------------------------------------------------ splitting ---
template <int VARIANT>
struct Split;
template <>
struct Split<0> {  // FP16 hi/lo
    static __device__ __forceinline__ void run(float v, uint16_t& hi, uint16_t& lo) {
        const __half h = __float2half_rn(v);
        const __half l = __float2half_rn(v - __half2float(h));
        hi = __half_as_ushort(h);
        lo = __half_as_ushort(l);
    }
};
template <>
struct Split<1> {  // BF16 hi/lo
    static __device__ __forceinline__ void run(float v, uint16_t& hi, uint16_t& lo) {
        const __nv_bfloat16 h = __float2bfloat16_rn(v);
        const __nv_bfloat16 l = __float2bfloat16_rn(v - __bfloat162float(h));
        hi = __bfloat16_as_ushort(h);
        lo = __bfloat16_as_ushort(l);
    }
};

__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

// Instruction descriptor of kind::f16: D f32, A/B f16 (0) or bf16 (1), A
// K-major, B MN-major (b_mn = 1) or K-major (0), N >> 3 at bit 17, M >> 4 at
// bit 24.
__host__ __device__ constexpr uint32_t instr_desc_f16(uint32_t ab_type, int m, int n, uint32_t b_mn) {
    return (1u << 4) | (ab_type << 7) | (ab_type << 10) | (0u << 15) | (b_mn << 16) | ((uint32_t)(n >> 3) << 17) |
           ((uint32_t)(m >> 4) << 24);
}

}  // namespace tc
}  // namespace vta
