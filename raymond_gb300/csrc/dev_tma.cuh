// Tensor-memory-accelerator copies (cp.async.bulk.tensor) into shared
// memory, completing on an mbarrier by transaction bytes, and the host's
// tensor-map encoder (cuTensorMapEncodeTiled through the runtime's
// driver-entry-point query, so nothing links libcuda directly).
#pragma once
#include <cuda.h>
#include <cudaTypedefs.h>

#include <cstdint>

#include "dev_tcgen05.cuh"

namespace rmd {

// Arrives on *bar and adds `bytes` to the transaction count it waits for.
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(tc::smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// The box of `map` at coordinates (c0, c1) into dst; dst 128-byte aligned,
// c0 × element size a multiple of 16 bytes.
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int c0, int c1, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            tc::smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(tc::smem_u32(bar))
        : "memory");
}

// As tma_load_2d for a rank-4 map.
__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* map, int c0, int c1, int c2, int c3,
                                            uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
        "[%6];" ::"r"(tc::smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(tc::smem_u32(bar))
        : "memory");
}

// As tma_load_2d for a rank-5 map.
__device__ __forceinline__ void tma_load_5d(void* dst, const CUtensorMap* map, int c0, int c1, int c2, int c3, int c4,
                                            uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.5d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, %6}], "
        "[%7];" ::"r"(tc::smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(tc::smem_u32(bar))
        : "memory");
}

// cuTensorMapEncodeTiled, or null when the driver does not offer it.
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder();

}  // namespace rmd
