// Device helpers shared by the chunked scan kernels (segment index, segment
// masks): asynchronous chunk copies, the compiled PAM test and warp-aggregated
// hit emission.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace bgo {

// Asynchronous 16-byte global -> shared copy (completes at cp.async.wait_group).
__device__ __forceinline__ void cp_async16(void *smem_dst, const void *gmem_src) {
    const uint32_t d = (uint32_t)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(gmem_src));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N));
}

__device__ __forceinline__ uint32_t sfshr(uint32_t lo, uint32_t hi, uint32_t s) {
    return __funnelshift_r(lo, hi, s);
}

// Positions (bits) whose base passes one compiled PAM test.
__device__ __forceinline__ uint32_t pam_test(uint32_t h, uint32_t l, uint32_t code) {
    if (code & 0x100u) {  // generic allowed set
        const uint32_t m0 = 0u - (code & 1u), m1 = 0u - ((code >> 1) & 1u);
        const uint32_t m2 = 0u - ((code >> 2) & 1u), m3 = 0u - ((code >> 3) & 1u);
        return (~h & ~l & m0) | (~h & l & m1) | (h & ~l & m2) | (h & l & m3);
    }
    const uint32_t hv = 0u - (code & 1u), hc = 0u - ((code >> 1) & 1u);
    const uint32_t lv = 0u - ((code >> 2) & 1u), lc = 0u - ((code >> 3) & 1u);
    return ~(((h ^ hv) & hc) | ((l ^ lv) & lc));
}

// Marks the granule (4,096 positions of one strand) of a key that did not fit
// the hit buffer.
__device__ __forceinline__ void mark_dropped(uint64_t pos, uint64_t slot, uint32_t *drop_bits,
                                             int64_t base1) {
    if (!drop_bits) return;
    const int64_t g = (slot ? base1 : 0) + (int64_t)(pos / 4096);
    atomicOr(drop_bits + (g >> 5), 1u << (g & 31));
}

// Appends `key`; the lanes executing this call together share one atomicAdd.
// Returns true when the key did not fit (it is counted; the caller marks its
// granule, so that this path stays small).
__device__ __forceinline__ bool semit(uint64_t key, uint64_t *keys, int64_t cap,
                                      unsigned long long *counter) {
    unsigned act = __activemask();
    int lane = threadIdx.x & 31;
    int leader = __ffs(act) - 1;
    unsigned long long base = 0;
    if (lane == leader) base = atomicAdd(counter, (unsigned long long)__popc(act));
    base = __shfl_sync(act, base, leader);
    unsigned long long slot = base + (unsigned long long)__popc(act & ((1u << lane) - 1u));
    if (slot < (unsigned long long)cap) {
        keys[slot] = key;
        return false;
    }
    return true;
}

}  // namespace bgo
