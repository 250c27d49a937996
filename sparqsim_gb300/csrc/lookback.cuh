// lookback.cuh — decoupled look-back (single-pass chained scan) helpers.
//
// Tiles take their index from an atomic counter in the order they start, so a
// tile only ever waits on tiles that are already resident and running; that is
// what guarantees progress. Every wait is still bounded: after a limit of
// polls (word 1 of the device error block, sq_set_wait_limit; kSpinLimit when
// 0) the waiting tile raises bit 0 of the device error word, treats the
// missing predecessor as zero and finishes, and the host reports
// SQ_ERR_DEVICE_TIMEOUT for the operation instead of hanging.
#pragma once
#include <cuda/atomic>
#include <cstdint>

namespace sq {

constexpr unsigned kSpinLimit = 1u << 22;

// The poll limit of bounded waits: word 1 of the error block `err` points
// into (written by the host between launches), kSpinLimit when it is 0.
__device__ __forceinline__ unsigned spin_limit(const unsigned* err) {
    const unsigned v = *(const volatile unsigned*)(err + 1);
    return v ? v : kSpinLimit;
}

// 64-bit status word: bits 63..62 = flag (0 none, 1 aggregate, 2 inclusive
// prefix), bits 61..0 = value.
constexpr unsigned long long kFlagAgg = 1ull << 62;
constexpr unsigned long long kFlagPre = 2ull << 62;
constexpr unsigned long long kValMask = (1ull << 62) - 1;

__device__ __forceinline__ void lb_store(unsigned long long* p, unsigned long long v) {
    cuda::atomic_ref<unsigned long long, cuda::thread_scope_device> a(*p);
    a.store(v, cuda::memory_order_release);
}
__device__ __forceinline__ unsigned long long lb_load(unsigned long long* p) {
    cuda::atomic_ref<unsigned long long, cuda::thread_scope_device> a(*p);
    return a.load(cuda::memory_order_acquire);
}

// Called by all 32 lanes of one warp. Publishes `aggregate` for `tile`, walks
// back over predecessors 32 at a time, publishes the inclusive prefix and
// returns the exclusive prefix (same value in every lane).
__device__ __forceinline__ unsigned long long lb_warp_exclusive(unsigned long long* status, long long tile,
                                                                unsigned long long aggregate, unsigned* err) {
    const unsigned lane = threadIdx.x & 31u;
    if (tile == 0) {
        if (lane == 0) lb_store(&status[0], kFlagPre | aggregate);
        return 0;
    }
    if (lane == 0) lb_store(&status[tile], kFlagAgg | aggregate);
    unsigned long long exclusive = 0;
    long long base = tile - 1;
    unsigned spins = 0;
    const unsigned limit = spin_limit(err);
    while (true) {
        const long long idx = base - (long long)lane;
        unsigned long long s = idx >= 0 ? lb_load(&status[idx]) : kFlagPre;
        unsigned flag = (unsigned)(s >> 62);
        const unsigned pre_mask = __ballot_sync(0xffffffffu, flag == 2u);
        const unsigned bad_mask = __ballot_sync(0xffffffffu, flag == 0u);
        const int first_pre = pre_mask ? __ffs(pre_mask) - 1 : 32;
        const unsigned needed = first_pre >= 31 ? 0xffffffffu : ((2u << first_pre) - 1u);
        if (bad_mask & needed) {
            if (++spins > limit) {
                if (lane == 0) atomicOr(err, 1u);
                // give up: count missing predecessors as zero
                unsigned long long v = (lane <= (unsigned)first_pre && flag != 0u) ? (s & kValMask) : 0ull;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
                exclusive += __shfl_sync(0xffffffffu, v, 0);
                break;
            }
            __nanosleep(32);
            continue;
        }
        unsigned long long v = ((int)lane <= first_pre) ? (s & kValMask) : 0ull;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        exclusive += __shfl_sync(0xffffffffu, v, 0);
        if (first_pre < 32) break;
        base -= 32;
        spins = 0;
    }
    if (lane == 0) lb_store(&status[tile], kFlagPre | (exclusive + aggregate));
    return exclusive;
}

// 32-bit status for per-digit look-back in the radix sort: bits 31..30 flag,
// bits 29..0 count (sorts are limited to < 2^30 keys).
constexpr unsigned kFlag32Agg = 1u << 30;
constexpr unsigned kFlag32Pre = 2u << 30;
constexpr unsigned kVal32Mask = (1u << 30) - 1;

__device__ __forceinline__ void lb32_store(unsigned* p, unsigned v) {
    cuda::atomic_ref<unsigned, cuda::thread_scope_device> a(*p);
    a.store(v, cuda::memory_order_release);
}
__device__ __forceinline__ unsigned lb32_load(unsigned* p) {
    cuda::atomic_ref<unsigned, cuda::thread_scope_device> a(*p);
    return a.load(cuda::memory_order_acquire);
}

// Relaxed forms for status words that carry their own payload (flag and
// count in one word): nothing else is published through them.
__device__ __forceinline__ void lb32_store_relaxed(unsigned* p, unsigned v) {
    cuda::atomic_ref<unsigned, cuda::thread_scope_device> a(*p);
    a.store(v, cuda::memory_order_relaxed);
}
__device__ __forceinline__ unsigned lb32_load_relaxed(unsigned* p) {
    cuda::atomic_ref<unsigned, cuda::thread_scope_device> a(*p);
    return a.load(cuda::memory_order_relaxed);
}

}  // namespace sq
