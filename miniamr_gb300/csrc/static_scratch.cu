// An allocation-free variant of the FP64 checksum for callers that cannot
// call cudaMalloc -- for instance code running where another allocator has
// reserved all device memory up front (a framework's caching allocator or a
// serving process with a fixed arena), or code on a latency-critical path
// that must not take the device-wide synchronisation an allocation can
// imply.  The checksum's only scratch, one partial sum per block, lives in
// the file-scope device array below instead of a context buffer.
//
// The array is a module global: every GPU that loads this library holds its
// 512 KiB until the process exits, and every call on a device shares it.
#include <mutex>

#include "mamr_internal.h"

namespace {

constexpr int kMaxDevices = 64;

// One FP64 partial per block, written by the first pass before the second
// pass reads it; nothing in it needs to start at zero.
static __device__ __align__(256) double g_block_partials[MAMR_STATIC_MAX_BLOCKS];

std::mutex g_setup_mutex;
double *g_partials_ptr[kMaxDevices];

// Once per device, with that device current: the device address of
// g_block_partials.  In host code the array's name is only a host-side
// stand-in, so kernels must be given this address.  Failures are reported
// here, with their own message.
int partials_address(double **out)
{
   int dev = 0;
   cudaError_t e = cudaGetDevice(&dev);
   if (e != cudaSuccess)
      return mamr::report_error(MAMR_ECUDA, "noalloc checksum: no current "
                                "device: %s", cudaGetErrorString(e));
   if (dev < 0 || dev >= kMaxDevices)
      return mamr::report_error(MAMR_EUNSUP, "noalloc checksum: device "
                                "ordinal %d is beyond the %d devices it "
                                "serves", dev, kMaxDevices);
   std::lock_guard<std::mutex> lock(g_setup_mutex);
   if (!g_partials_ptr[dev]) {
      void *p = nullptr;
      e = cudaGetSymbolAddress(&p, g_block_partials);
      if (e != cudaSuccess)
         return mamr::report_error(MAMR_ECUDA, "noalloc checksum: device "
                                   "address of the static scratch: %s",
                                   cudaGetErrorString(e));
      g_partials_ptr[dev] = static_cast<double *>(p);
   }
   *out = g_partials_ptr[dev];
   return MAMR_OK;
}

}  // namespace

extern "C" int mamr_check_sum_fp64_noalloc(const double *blocks,
                                           const mamr_config *cfg,
                                           const int32_t *slots,
                                           int32_t n_blocks, int32_t var,
                                           double *sum, void *stream)
{
   if (!blocks || !cfg || !sum || n_blocks < 0 || (n_blocks && !slots))
      return mamr::report_error(MAMR_EINVAL, "noalloc checksum: null "
                                "pointer or negative block count");
   if (n_blocks > MAMR_STATIC_MAX_BLOCKS)
      return mamr::report_error(MAMR_EINVAL, "noalloc checksum: %d blocks "
                                "exceed the static scratch of %d blocks",
                                n_blocks, MAMR_STATIC_MAX_BLOCKS);
   if (cfg->nx < 1 || cfg->ny < 1 || cfg->nz < 1 || cfg->num_vars < 1 ||
       var < 0 || var >= cfg->num_vars)
      return mamr::report_error(MAMR_EINVAL, "noalloc checksum: bad shape "
                                "or variable %d", var);
   double *partials = nullptr;
   int r = partials_address(&partials);
   if (r != MAMR_OK)
      return r;
   // the dense layout of the ABI's host buffers: no row padding
   mamr::Geom g;
   g.nx = cfg->nx; g.ny = cfg->ny; g.nz = cfg->nz; g.V = cfg->num_vars;
   g.X = g.nx + 2; g.Y = g.ny + 2; g.Z = g.nz + 2;
   g.Zp = g.Z;
   g.koff = 0;
   g.kplane = -1;
   g.bv = (long long) g.X * g.Y * g.Z;
   int n = mamr::launch_checksum_fp64(blocks, g, slots, n_blocks, var,
                                      partials, sum,
                                      static_cast<cudaStream_t>(stream));
   if (n < 0)
      return mamr::report_error(MAMR_ECUDA, "noalloc checksum launch: %s",
                                cudaGetErrorString(cudaGetLastError()));
   return MAMR_OK;
}
