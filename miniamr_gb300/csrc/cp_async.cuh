// cp.async helpers shared by the stage kernels.
#pragma once

namespace mamr {

// 16 bytes global -> shared, bypassing L1; both addresses 16-byte aligned.
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem)
{
   unsigned s = (unsigned) __cvta_generic_to_shared(smem);
   asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s),
                "l"(gmem));
}
// One element (4 or 8 bytes) global -> shared, through L1; both addresses
// aligned to the element size.
template <typename T>
__device__ __forceinline__ void cp_async_elem(T *smem, const T *gmem)
{
   static_assert(sizeof(T) == 4 || sizeof(T) == 8, "4- or 8-byte elements");
   unsigned s = (unsigned) __cvta_generic_to_shared(smem);
   if (sizeof(T) == 4)
      asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s),
                   "l"(gmem));
   else
      asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s),
                   "l"(gmem));
}
// Waits until at most N of this thread's committed groups are pending.
template <int N> __device__ __forceinline__ void cp_async_wait_group()
{
   asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}
__device__ __forceinline__ void cp_async_commit()
{
   asm volatile("cp.async.commit_group;\n" ::);
}
__device__ __forceinline__ void cp_async_wait_all()
{
   asm volatile("cp.async.wait_all;\n" ::: "memory");
}

}  // namespace mamr
