// Tensor-copy (TMA) and mbarrier helpers shared by the stage kernels that
// fill shared-memory tiles with bulk asynchronous copies.
#pragma once

#include <cuda.h>

namespace mamr {

// cuTensorMapEncodeTiled, from the driver through the runtime (no link
// against the driver library); null if unavailable.
using EncodeTiledFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType,
                                   cuuint32_t, void *, const cuuint64_t *,
                                   const cuuint64_t *, const cuuint32_t *,
                                   const cuuint32_t *, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion,
                                   CUtensorMapFloatOOBfill);
EncodeTiledFn encode_tiled();

__device__ __forceinline__ unsigned smem_addr(const void *p)
{
   return (unsigned) __cvta_generic_to_shared(p);
}

// An mbarrier expecting one arrival per phase.
__device__ __forceinline__ void mbar_init(unsigned bar)
{
   asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar)
                : "memory");
}

__device__ __forceinline__ void mbar_init_fence()
{
   asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// The single arrival of the current phase, which also announces the bytes
// the phase's copies deliver.
__device__ __forceinline__ void mbar_expect_tx(unsigned bar, unsigned bytes)
{
   asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::
                   "r"(bar), "r"(bytes)
                : "memory");
}

// Waits for phase `parity` of the mbarrier at shared address bar; false if
// it has not completed after 64 tries.  Each try suspends the thread until
// the phase completes or a time hint of 10 ms runs out, so a waiting warp
// takes no issue slots from the warps that compute.
__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity)
{
   for (int it = 0; it < 64; it++) {
      unsigned ok;
      asm volatile("{\n\t.reg .pred p;\n\t"
                   "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, "
                   "%3;\n\t"
                   "selp.u32 %0, 1, 0, p;\n\t}"
                   : "=r"(ok)
                   : "r"(bar), "r"(parity), "r"(10000000u)
                   : "memory");
      if (ok)
         return true;
   }
   return false;
}

// Orders this thread's earlier generic-proxy accesses of shared memory
// before later tensor copies into it.
__device__ __forceinline__ void fence_proxy_async_smem()
{
   asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// A box of the 4-d tensor tm at coordinates (c0 .. c3) into shared memory
// at dst (128-byte aligned), completing on the mbarrier bar.  c0 (the
// innermost) times the element size must be a multiple of 16 bytes.
__device__ __forceinline__ void tma_load_4d(void *dst, const CUtensorMap *tm,
                                            int c0, int c1, int c2, int c3,
                                            unsigned bar)
{
   asm volatile("cp.async.bulk.tensor.4d.shared::cluster.global.tile"
                ".mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
                "[%6];"
                ::"r"(smem_addr(dst)),
                "l"(reinterpret_cast<unsigned long long>(tm)), "r"(c0),
                "r"(c1), "r"(c2), "r"(c3), "r"(bar)
                : "memory");
}

// bytes (a multiple of 16) from global src to shared dst, both 16-byte
// aligned, completing on the mbarrier bar.
__device__ __forceinline__ void bulk_load(void *dst, const void *src,
                                          unsigned bytes, unsigned bar)
{
   asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx"
                "::bytes [%0], [%1], %2, [%3];"
                ::"r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(bar)
                : "memory");
}

}  // namespace mamr
