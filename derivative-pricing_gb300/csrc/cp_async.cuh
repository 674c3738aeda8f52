// cp_async.cuh -- 16-byte asynchronous copies from global to shared memory
// (cp.async.cg), completed per thread by commit / wait groups: no barrier and
// no spin-wait involved.  Both addresses must be 16-byte aligned.  A thread
// waits for its groups before it reads the copied data and before it exits.
#pragma once

#include <cstdint>

namespace mcdg {

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    const uint32_t s = static_cast<uint32_t>(__cvta_generic_to_shared(smem));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s), "l"(gmem) : "memory");
}

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }

__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

}  // namespace mcdg
