// Tensor memory accelerator (TMA) loads as inline PTX: a tiled box of a 4-D
// tensor map copied from global into shared memory, completing on an mbarrier
// with its byte count (complete_tx).  The mbarrier helpers (init, bounded
// parity wait) are those of tcgen05.cuh.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "tcgen05.cuh"

namespace ocfd {
namespace tma {

// the calling thread arrives on `bar` and adds `bytes` to the transaction count
// the current phase waits for
__device__ __forceinline__ void expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(tc::smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// box of `map` at element coordinates (x, y, z, c) into dst (128-byte aligned
// shared memory, the box stored densely with x fastest); x times the element
// size must be a multiple of 16 bytes.  Elements outside the tensor read as 0.
__device__ __forceinline__ void load_4d(void* dst, const CUtensorMap* map, int x, int y, int z, int c,
                                        uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
        "%5}], [%6];" ::"r"(tc::smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(c), "r"(tc::smem_u32(bar))
        : "memory");
}

// a tensor map in global memory written by the generic proxy (the host's copy
// of a box table) made visible to the tensormap proxy before a TMA uses it
__device__ __forceinline__ void fence_tensormap_acquire(const CUtensorMap* map) {
    asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(reinterpret_cast<uint64_t>(map))
                 : "memory");
}

// generic-proxy accesses of shared memory ordered before later async-proxy
// (TMA) writes to it
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

}  // namespace tma
}  // namespace ocfd
