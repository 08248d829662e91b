// TMA tile copies and mbarrier waits (inline PTX, sm_90+ / sm_103a).
#pragma once

#include <cuda.h>

#include <cstdint>

namespace fdtd {

// Tensor maps of one copy of the state: the six hi arrays and, for the
// compensated form, the six lo arrays (passed to the fused kernel by value).
struct TmaMaps {
  CUtensorMap hi[6];
  CUtensorMap lo[6];
};

// Maps of one fused step launch: tile loads from the current copy and tile
// stores into the second copy (maps of the grid rows and their x margins, so
// stores past the grid's last row are clipped by the copy engine).
struct StepMaps {
  TmaMaps ld;
  TmaMaps st;
};

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

// Makes barrier initialisation visible to the async (TMA) proxy.
__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return done != 0;
}

// Bounded waits.  A wait polls the barrier at most `polls` times; on giving
// up it records bit 0 in *err and returns false.  The fused kernels then stop
// their tile loops uniformly (the CTA's barrier reduces every thread's
// outcome), wait (again bounded) for the copies they still have in flight,
// record bit 1 if one of those waits gives up too, and return: no thread is
// left at a barrier and no copy lands in a CTA that has exited.
constexpr uint32_t kMaxBarrierPolls = 1u << 24;

struct WaitCtl {
  int* err;        // device status word, read and cleared by fdtd_synchronize
  uint32_t polls;  // polls before a wait gives up (kMaxBarrierPolls)
  int withhold;    // test hook of the timeout path: issue no tile loads, so
                   // every wait gives up with no copy in flight (0: off)
};

__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, const WaitCtl& wc, int code = 1) {
  for (uint32_t n = 0; n < wc.polls; ++n)
    if (mbar_try_wait(bar, parity)) return true;
  atomicOr(wc.err, code);
  return false;
}

// 3-D tiled TMA load of the box at element coordinates (x, y, z) of `map`
// into shared memory, completing on `bar` (transaction bytes).
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_addr(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
      : "memory");
}

// 3-D tiled TMA store of a box from shared memory to element coordinates
// (x, y, z) of `map`; completes as part of the thread's bulk async-group.
// Elements outside the map's extent are not written.
__device__ __forceinline__ void tma_store_3d(const CUtensorMap* map, const void* src, int x, int y, int z) {
  asm volatile(
      "cp.async.bulk.tensor.3d.global.shared::cta.tile.bulk_group [%0, {%2, %3, %4}], [%1];" ::"l"(
          reinterpret_cast<uint64_t>(map)),
      "r"(smem_addr(src)), "r"(x), "r"(y), "r"(z)
      : "memory");
}

// Brings a tensor map (in global, constant or parameter memory) into the
// copy engine's descriptor cache ahead of its first use.
__device__ __forceinline__ void prefetch_tensormap(const CUtensorMap* map) {
  asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(map)) : "memory");
}

__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }

// Waits until every committed bulk store of this thread has read its shared
// memory source (the buffer may then be rewritten).
__device__ __forceinline__ void bulk_wait_read_all() {
  asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}

// Waits until every committed bulk store of this thread has completed.
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

// Orders this thread's shared-memory writes before later async-proxy (TMA)
// reads of them.
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

}  // namespace fdtd
