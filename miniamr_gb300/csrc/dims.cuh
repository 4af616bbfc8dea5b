// Compile-time block dimensions for the device kernels (CUDA only).
#pragma once

#include "mamr_internal.h"

namespace mamr {

// Block dimensions: compile-time constants for the common block sizes (so
// that every index folds), taken from g when zero.
template <int BX, int BY, int BZ> struct Dims {
   const int nx, ny, nz, X, Y;
   __device__ explicit Dims(const Geom &g)
      : nx(BX ? BX : g.nx), ny(BY ? BY : g.ny), nz(BZ ? BZ : g.nz),
        X((BX ? BX : g.nx) + 2), Y((BY ? BY : g.ny) + 2)
   {
   }
   // cell (i, j, k) of a block-variable in the split layout (contexts
   // always use it): interior rows of nz values, then the k = 0 and
   // k = nz+1 planes
   __device__ __forceinline__ int cell(int i, int j, int k) const
   {
      const int row = i * Y + j;
      if (k >= 1 && k <= nz)
         return row * nz + (k - 1);
      return X * Y * nz + (k == 0 ? 0 : X * Y) + row;
   }
   __device__ __forceinline__ int fcell(int dir, int nc, int a, int b) const
   {
      if (dir == 0) return cell(nc, a, b);
      if (dir == 1) return cell(a, nc, b);
      return cell(a, b, nc);
   }
};

// Compile-time block size of a geometry: 8^3 and 16^3 get their own
// instantiations, anything else the run-time one.
inline int dims_kind(const Geom &g)
{
   if (g.nx == 8 && g.ny == 8 && g.nz == 8)
      return 1;
   if (g.nx == 16 && g.ny == 16 && g.nz == 16)
      return 2;
   return 0;
}

}  // namespace mamr
