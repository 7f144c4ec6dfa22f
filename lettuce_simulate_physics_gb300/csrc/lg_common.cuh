// Shared host and device helpers of the GB300 engine: errors, device buffers, and the inline PTX
// used by the kernels (bulk async copies with mbarrier completion, MUFU reciprocal square root).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>

namespace lg {

// ---- errors ---------------------------------------------------------------------------------
// Status-carrying exception; the C ABI turns it into an lg_status and a thread-local message.
struct Error : std::runtime_error {
    int status;
    Error(int s, const std::string& m) : std::runtime_error(m), status(s) {}
};
constexpr int kRuntime = 1, kLogic = 2, kArg = 3, kUnavailable = 4;

[[noreturn]] inline void fail(int status, const std::string& msg) { throw Error(status, msg); }

inline void check_cuda(cudaError_t e, const char* what, const char* file, int line) {
    if (e != cudaSuccess) {
        cudaGetLastError();
        fail(kRuntime, std::string(what) + " failed: " + cudaGetErrorString(e) + " (" + file + ":" +
                           std::to_string(line) + ")");
    }
}
#define LG_CK(x) ::lg::check_cuda((x), #x, __FILE__, __LINE__)
#define LG_LAUNCHED() ::lg::check_cuda(cudaGetLastError(), "kernel launch", __FILE__, __LINE__)

// ---- device buffers -------------------------------------------------------------------------
// Grow-only device allocation; contents are not preserved when it grows.
class DevBuf {
public:
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { release(); }
    void reserve(size_t bytes) {
        if (bytes <= cap_) return;
        release();
        size_t want = bytes < 256 ? 256 : bytes;
        void* p = nullptr;
        cudaError_t e = cudaMalloc(&p, want);
        if (e != cudaSuccess) {
            cudaGetLastError();
            fail(kRuntime, "cudaMalloc(" + std::to_string(want) + " bytes) failed: " + cudaGetErrorString(e));
        }
        p_ = p;
        cap_ = want;
    }
    void release() {
        if (p_) cudaFree(p_);
        p_ = nullptr;
        cap_ = 0;
    }
    template <class T>
    T* as() const { return static_cast<T*>(p_); }
    size_t capacity() const { return cap_; }

private:
    void* p_ = nullptr;
    size_t cap_ = 0;
};

// Device-side error word bits (read back by the host after a synchronising call).
enum : unsigned {
    kErrWaitTimeout = 1u,    // an mbarrier or flag wait hit its iteration cap
    kErrStackOverflow = 2u,  // walk traversal stack full
    kErrNodeOverflow = 4u,   // tree node capacity exceeded
    kErrDeepKeys = 8u,       // key restarts deeper than the engine supports (kept as one leaf)
    kErrListOverflow = 16u,  // interaction-list capacity exceeded
};

// Iteration cap of every device-side wait; a wait that reaches it records kErrWaitTimeout and
// returns instead of spinning on.
constexpr unsigned kSpinCap = 1u << 22;

#ifdef __CUDACC__
// ---- PTX: MUFU reciprocal square root ------------------------------------------------------
__device__ __forceinline__ float rsqrt_mufu(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// ---- PTX: mbarrier and bulk async copy (TMA engine, non-tensor form) -----------------------
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_fence_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Arms the barrier for one arrival plus `bytes` of transaction count.
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait for the barrier phase `parity` to complete; false after `cap` polls.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned parity, unsigned cap = kSpinCap) {
    for (unsigned it = 0; it < cap; ++it)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// Global -> shared bulk copy of `bytes` (multiple of 16, both addresses 16-byte aligned),
// completing as transaction bytes on `bar`.
__device__ __forceinline__ void bulk_g2s(void* dst_smem, const void* src_gmem, unsigned bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst_smem)),
        "l"(src_gmem), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

// ---- PTX: packed FP32 pairs (sm_100+ f32x2 arithmetic) ----------------------------------------
// One instruction operates on two floats held in a 64-bit register pair: the same FP32 pipe
// throughput as scalar FFMA, at half the issue slots.
typedef unsigned long long f2x;

__device__ __forceinline__ f2x f2_pack(float lo, float hi) {
    f2x d;
    asm("mov.b64 %0, {%1, %2};" : "=l"(d) : "f"(lo), "f"(hi));
    return d;
}
__device__ __forceinline__ void f2_unpack(f2x v, float& lo, float& hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ f2x f2_add(f2x a, f2x b) {
    f2x d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2x f2_sub(f2x a, f2x b) {
    f2x d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2x f2_mul(f2x a, f2x b) {
    f2x d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2x f2_fma(f2x a, f2x b, f2x c) {
    f2x d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ f2x f2_rsqrt(f2x a) {
    float lo, hi;
    f2_unpack(a, lo, hi);
    return f2_pack(rsqrt_mufu(lo), rsqrt_mufu(hi));
}
__device__ __forceinline__ f2x f2_bcast(float v) { return f2_pack(v, v); }
__device__ __forceinline__ float f2_sum(f2x v) {
    float lo, hi;
    f2_unpack(v, lo, hi);
    return lo + hi;
}

// ---- compensated summation ---------------------------------------------------------------
// Kahan step: adds x to (s, c), c carrying the low-order bits lost by s.
__device__ __forceinline__ void kahan_add(float& s, float& c, float x) {
    float y = x - c;
    float t = s + y;
    c = (t - s) - y;
    s = t;
}
#endif

}  // namespace lg
