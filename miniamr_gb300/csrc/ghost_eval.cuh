// Evaluation of the 27-point edge and corner ghost recipes (batched.h) in
// the stage kernels (CUDA only).
#pragma once

#include "batched.h"
#include "arith.cuh"

namespace mamr {

// The value of an edge or corner ghost cell from its recipe (batched.h):
// t is the cell's index along the edge (unused for corners).  Transforms
// across a level jump are the face gathers' own (coarse/4, the 4-cell sum
// in the reference's order); stale cells come from the pool the run
// started from, which no stage before the last writes ghosts into.
template <typename T, class DM>
__device__ __forceinline__ T eval_recipe(const GhostRecipe &r, int t,
                                         const T *__restrict__ src,
                                         const T *__restrict__ stale,
                                         const Geom &g, const DM &D, int var)
{
   // the cell, with the edge index in place (selects, not an indexed
   // array, so that nothing goes to local memory)
   const int c0 = r.vax == 0 ? t : r.c[0];
   const int c1 = r.vax == 1 ? t : r.c[1];
   const int c2 = r.vax == 2 ? t : r.c[2];
   // an interior cell now, or a ghost cell as the previous stage left it
   // (the stage that wrote the source pool wrote it there)
   if (r.kind == GR_INTERIOR || r.kind == GR_PREV)
      return src[bv_offset(g, r.nb[0], var) + D.cell(c0, c1, c2)];
   if (r.kind == GR_STALE)
      return stale[bv_offset(g, r.nb[0], var) + D.cell(c0, c1, c2)];
   const int dir = r.l >> 1;
   const bool low = !(r.l & 1);
   const int n = dir == 0 ? D.nx : (dir == 1 ? D.ny : D.nz);
   const int na = dir == 0 ? D.ny : D.nx;
   const int nbb = dir == 2 ? D.ny : D.nz;
   const int ha = na / 2, hb = nbb / 2;
   const int a = dir == 0 ? c1 : c0;
   const int b = dir == 2 ? c1 : c2;
   if (r.kind == GR_COARSE) {
      const int iq = r.iqjq & 1, jq = r.iqjq >> 1;
      return quarter(src[bv_offset(g, r.nb[0], var) +
                         D.fcell(dir, low ? n : 1, (a + 1) / 2 + jq * ha,
                                 (b + 1) / 2 + iq * hb)]);
   }
   const int jq = a > ha, iq = b > hb;
   const int a2 = a - jq * ha, b2 = b - iq * hb;
   const int p = low ? n : 1;
   const T *f = src + bv_offset(g, r.nb[iq * 2 + jq], var);
   T s = f[D.fcell(dir, p, 2 * a2 - 1, 2 * b2 - 1)] +
         f[D.fcell(dir, p, 2 * a2 - 1, 2 * b2)];
   s = s + f[D.fcell(dir, p, 2 * a2, 2 * b2 - 1)];
   s = s + f[D.fcell(dir, p, 2 * a2, 2 * b2)];
   return s;
}

}  // namespace mamr
