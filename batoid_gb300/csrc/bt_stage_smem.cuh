// Staging of a program blob from global into shared memory with one TMA bulk
// copy (cp.async.bulk) completed on an mbarrier.  The wait is bounded: if the
// copy does not complete within the iteration limit the kernel records
// BT_ERR_TIMEOUT in the device status word, waits once more (bounded) for the
// copy in flight and returns without touching any ray.
#pragma once
#include <stdint.h>

#define BT_WAIT_LIMIT (1u << 24)

// One status word per translation unit that stages blobs (no relocatable
// device code is needed); the TU exports a host reader for it.
static __device__ int bt_dev_status = 0;

__device__ __forceinline__ uint32_t bt_smem_addr(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ bool bt_mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bt_smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Returns false (after recording the timeout) if the blob did not arrive.
// Must be called by every thread of the block, before any other use of smem.
__device__ __forceinline__ bool bt_stage_blob(unsigned char* smem, const unsigned char* gblob, int bytes,
                                              uint64_t* bar) {
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bt_smem_addr(bar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                     ::"r"(bt_smem_addr(bar)), "r"((uint32_t)bytes) : "memory");
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
            ::"r"(bt_smem_addr(smem)), "l"(gblob), "r"((uint32_t)bytes), "r"(bt_smem_addr(bar))
            : "memory");
    }
    for (uint32_t i = 0; i < BT_WAIT_LIMIT; i++) {
        if (bt_mbar_try_wait(bar, 0)) return true;
    }
    atomicExch(&bt_dev_status, 5 /* BT_ERR_TIMEOUT */);
    for (uint32_t i = 0; i < BT_WAIT_LIMIT; i++) {
        if (bt_mbar_try_wait(bar, 0)) break;
    }
    return false;
}
