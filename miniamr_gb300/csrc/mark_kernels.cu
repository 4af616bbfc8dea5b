// Refinement marking on the device (mamr_mark_refine): reset_all,
// check_objects / the uniform assignment and refine_level of one rank
// (ref/refine.c:500-527, ref/move.c:65-623, ref/refine.c:68-74, 325-496).
//
// The flags only rise (-1 < 0 < 1) under every rule of those routines, so
// the reference's result is the least fixed point of the rules above the
// initial state, whatever order they run in.  The initial flags come from
// the FP64 object tests of mark_geometry.h (one thread per block); every
// rule is then applied to every block and parent with atomicMax in passes
// until a pass changes nothing -- across the whole GPU in one cooperative
// launch with grid-wide barriers between passes.  Each change raises one
// of at most 2 (blocks + parents) flag steps, so that many passes bound
// the loop; running out sets ERR_MARK instead of spinning.
#include <cmath>

#include <cooperative_groups.h>

#include "mamr_internal.h"

#define MAMR_MFN static __device__ __forceinline__
#include "mark_geometry.h"
#undef MAMR_MFN

namespace mamr {

namespace {

// Slots not listed hold this value; rules never raise them.
constexpr int32_t UNLISTED = (int32_t) 0x80808080;

__global__ void mark_init_kernel(const mamr_mark_block *__restrict__ mb,
                                 int nb, mamr_mark_params p, int3 bs,
                                 const mamr_object *__restrict__ objs,
                                 int n_objs,
                                 const mamr_mark_parent *__restrict__ pa,
                                 int np, int32_t *__restrict__ ref,
                                 int32_t *__restrict__ pref)
{
   const int bsize[3] = {bs.x, bs.y, bs.z};
   for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nb + np;
        i += gridDim.x * blockDim.x) {
      if (i < nb) {
         const mamr_mark_block &b = mb[i];
         int r;
         if (p.uniform_refine) {
            r = b.level < p.num_refine ? 1 : 0;
         } else {
            r = mamr_mg_block_state(b.cen, b.level, &p, bsize, objs, n_objs);
            if (r == 1 && b.level == p.num_refine)
               r = 0;
            if (r == -1 && b.level == 0)
               r = 0;
         }
         ref[b.slot] = r;
      } else {
         const int q = i - nb;
         int r = -1;
         for (int k = 0; k < 8; k++)
            if (pa[q].child[k] < 0)
               r = 0;
         pref[q] = r;
      }
   }
}

__device__ __forceinline__ int32_t load_flag(const int32_t *x)
{
   return *(const volatile int32_t *) x;
}

// Raises a listed flag to v; returns whether it changed.
__device__ __forceinline__ bool raise_flag(int32_t *x, int32_t v)
{
   const int32_t cur = load_flag(x);
   if (cur == UNLISTED || cur >= v)
      return false;
   return atomicMax(x, v) < v;
}

__global__ void __launch_bounds__(1024)
mark_fixpoint_kernel(const mamr_mark_block *__restrict__ mb, int nb,
                     const mamr_mark_parent *__restrict__ pa, int np,
                     int uniform, int max_passes, int32_t *ref,
                     int32_t *pref, unsigned *err)
{
   __shared__ int changed;
   for (int pass = 0;; pass++) {
      if (threadIdx.x == 0)
         changed = 0;
      __syncthreads();
      bool mine = false;
      for (int i = threadIdx.x; i < nb; i += blockDim.x) {
         const mamr_mark_block &b = mb[i];
         const int32_t v = load_flag(&ref[b.slot]);
         // family: a block at 1 (or at 0, but not an initial zero of the
         // uniform assignment) keeps its parent from coarsening
         if ((v == 1 || (v == 0 && !uniform)) && b.parent >= 0)
            mine |= raise_flag(&pref[b.parent], 0);
         for (int l = 0; l < 6; l++) {
            const int nl = b.nei_level[l];
            if (nl == b.level + 1)
               mine |= raise_flag(&ref[b.slot], 0);      // finer neighbour
            else if (v == 1 && nl == b.level)
               mine |= raise_flag(&ref[b.nei[l]], 0);
            else if (v >= 0 && nl == b.level - 1)
               mine |= raise_flag(&ref[b.nei[l]], v);    // 1: must refine
         }
      }
      for (int q = threadIdx.x; q < np; q += blockDim.x)
         if (pa[q].active && load_flag(&pref[q]) >= 0)
            for (int k = 0; k < 8; k++) {
               const int32_t ch = pa[q].child[k];
               if (ch >= 0)
                  mine |= raise_flag(&ref[ch], 0);
            }
      if (mine)
         changed = 1;
      __syncthreads();
      const bool again = changed != 0;
      __syncthreads();
      if (!again)
         break;
      if (pass + 1 >= max_passes) {
         if (threadIdx.x == 0)
            atomicOr(err, ERR_MARK);
         break;
      }
   }
}

// The whole marking in one cooperative launch: initial flags, then rule
// passes separated by grid-wide barriers until one pass changes nothing,
// then the gather.  Pass p reports changes in flags[p % 3]; after the
// barrier every thread reads it, and CTA 0 clears flags[(p + 2) % 3], which
// nobody writes before the barrier that ends pass p + 1.
__global__ void __launch_bounds__(256)
mark_grid_kernel(const mamr_mark_block *__restrict__ mb, int nb,
                 const mamr_mark_parent *__restrict__ pa, int np,
                 mamr_mark_params p, int3 bs,
                 const mamr_object *__restrict__ objs, int n_objs,
                 int max_passes, int32_t *ref, int32_t *pref,
                 int32_t *__restrict__ out, int *flags, unsigned *err)
{
   namespace cg = cooperative_groups;
   cg::grid_group grid = cg::this_grid();
   const int bsize[3] = {bs.x, bs.y, bs.z};
   const int uniform = p.uniform_refine != 0;
   const int t0 = blockIdx.x * blockDim.x + threadIdx.x;
   const int nt = gridDim.x * blockDim.x;
   for (int i = t0; i < nb + np; i += nt) {
      if (i < nb) {
         const mamr_mark_block &b = mb[i];
         int r;
         if (uniform) {
            r = b.level < p.num_refine ? 1 : 0;
         } else {
            r = mamr_mg_block_state(b.cen, b.level, &p, bsize, objs, n_objs);
            if (r == 1 && b.level == p.num_refine)
               r = 0;
            if (r == -1 && b.level == 0)
               r = 0;
         }
         ref[b.slot] = r;
      } else {
         const int q = i - nb;
         int r = -1;
         for (int k = 0; k < 8; k++)
            if (pa[q].child[k] < 0)
               r = 0;
         pref[q] = r;
      }
   }
   grid.sync();
   for (int pass = 0;; pass++) {
      bool mine = false;
      for (int i = t0; i < nb + np; i += nt) {
         if (i < nb) {
            const mamr_mark_block &b = mb[i];
            const int32_t v = load_flag(&ref[b.slot]);
            if ((v == 1 || (v == 0 && !uniform)) && b.parent >= 0)
               mine |= raise_flag(&pref[b.parent], 0);
            for (int l = 0; l < 6; l++) {
               const int nl = b.nei_level[l];
               if (nl == b.level + 1)
                  mine |= raise_flag(&ref[b.slot], 0);
               else if (v == 1 && nl == b.level)
                  mine |= raise_flag(&ref[b.nei[l]], 0);
               else if (v >= 0 && nl == b.level - 1)
                  mine |= raise_flag(&ref[b.nei[l]], v);
            }
         } else {
            const int q = i - nb;
            if (pa[q].active && load_flag(&pref[q]) >= 0)
               for (int k = 0; k < 8; k++) {
                  const int32_t ch = pa[q].child[k];
                  if (ch >= 0)
                     mine |= raise_flag(&ref[ch], 0);
               }
         }
      }
      if (__any_sync(0xffffffffu, mine) && (threadIdx.x & 31) == 0)
         atomicExch(&flags[pass % 3], 1);
      grid.sync();
      const bool again = *(volatile int *) &flags[pass % 3] != 0;
      if (t0 == 0)
         flags[(pass + 2) % 3] = 0;
      if (!again)
         break;
      if (pass + 1 >= max_passes) {
         if (t0 == 0)
            atomicOr(err, ERR_MARK);
         break;
      }
   }
   for (int i = t0; i < nb; i += nt)
      out[i] = load_flag(&ref[mb[i].slot]);
}

__global__ void mark_gather_kernel(const mamr_mark_block *__restrict__ mb,
                                   int nb, const int32_t *__restrict__ ref,
                                   int32_t *__restrict__ out)
{
   for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nb;
        i += gridDim.x * blockDim.x)
      out[i] = ref[mb[i].slot];
}

int grid_for(int n)
{
   const int g = (n + 255) / 256;
   return g < 1 ? 1 : (g > 152 * 16 ? 152 * 16 : g);
}

}  // namespace

// Device buffers (d_ref: max_blocks flags, then the block and parent
// lists) are the caller's; returns the number of kernels launched or -1.
// Device buffers (d_ref: max_blocks flags, d_flags: 3 ints) are the
// caller's.  With cooperative launch support the marking is one grid-wide
// kernel; otherwise the initial flags, one CTA for the passes and the
// gather.  Returns the number of kernels launched or -1.
int launch_mark_refine(const mamr_mark_params &p, int3 bsize,
                       const mamr_object *d_objs, int n_objs,
                       const mamr_mark_block *d_mb, int nb,
                       const mamr_mark_parent *d_pa, int np, int max_blocks,
                       int32_t *d_ref, int32_t *d_pref, int32_t *d_out,
                       int *d_flags, unsigned *err, cudaStream_t s)
{
   if (cudaMemsetAsync(d_ref, 0x80, sizeof(int32_t) * (size_t) max_blocks,
                       s) != cudaSuccess ||
       cudaMemsetAsync(d_flags, 0, 3 * sizeof(int), s) != cudaSuccess)
      return -1;
   const long long bound = 2LL * ((long long) nb + np) + 2;
   int max_passes = (int) (bound < (1 << 30) ? bound : (1 << 30));
   // a caller's cap (a test knob): running out sets ERR_MARK as above
   if (p.max_passes > 0 && p.max_passes < max_passes)
      max_passes = p.max_passes;
   int dev = 0, coop = 0, sms = 0, per_sm = 0;
   cudaGetDevice(&dev);
   cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
   cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
   cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mark_grid_kernel,
                                                 256, 0);
   if (coop && per_sm > 0) {
      // enough CTAs for one item per thread, at most what stays resident
      const int want = (nb + np + 255) / 256;
      const int grid = want < 1 ? 1 : (want < per_sm * sms ? want
                                                           : per_sm * sms);
      mamr_mark_params pc = p;
      void *args[] = {(void *) &d_mb, (void *) &nb, (void *) &d_pa,
                      (void *) &np, (void *) &pc, (void *) &bsize,
                      (void *) &d_objs, (void *) &n_objs,
                      (void *) &max_passes, (void *) &d_ref,
                      (void *) &d_pref, (void *) &d_out, (void *) &d_flags,
                      (void *) &err};
      if (cudaLaunchCooperativeKernel((const void *) mark_grid_kernel,
                                      dim3(grid), dim3(256), args, 0, s) !=
          cudaSuccess)
         return -1;
      return 1;
   }
   mark_init_kernel<<<grid_for(nb + np), 256, 0, s>>>(
      d_mb, nb, p, bsize, d_objs, n_objs, d_pa, np, d_ref, d_pref);
   mark_fixpoint_kernel<<<1, 1024, 0, s>>>(
      d_mb, nb, d_pa, np, p.uniform_refine != 0, max_passes, d_ref, d_pref,
      err);
   mark_gather_kernel<<<grid_for(nb), 256, 0, s>>>(d_mb, nb, d_ref, d_out);
   return cudaPeekAtLastError() == cudaSuccess ? 3 : -1;
}

}  // namespace mamr
