// Variable-work stencils of --stencil 0 (ref/stencil.c:43-74 dispatch,
// :147-983 kernels) on the device, FP64, over every active block.  The
// per-cell formulas are work_formulas.h; the launch structure follows what
// the reference's loops allow:
//   stencil_0, stencil_check  one thread per cell (each cell reads only
//                             its own variables)
//   stencil_x / _y / _z       one thread per line along the axis, walking
//                             it in increasing order (the reference updates
//                             in place, so each cell sees its predecessor's
//                             new value)
//   stencil_7 / _27           one thread per cell into a scratch buffer of
//                             work values, then a copy back (the
//                             reference's per-block work array: every read
//                             sees the values before the call)
#include <cmath>

#include "mamr_internal.h"
#include "dims.cuh"

namespace mamr {

namespace {

// One block's variables: variable v at cell (i, j, k) is
// base[v * bv + D.cell(i, j, k)].
template <int BX, int BY, int BZ> struct WView {
   const double *base;
   long long bv;
   Dims<BX, BY, BZ> D;
};

}  // namespace

// The formulas become templates over the view type.
#define MAMR_WFN template <typename WV> static __device__ __forceinline__
#define MAMR_WFN0 static __device__ __forceinline__
#define MAMR_WVIEW WV
#define MAMR_AT(w, v, i, j, k)                                                \
   ((w)->base[(long long) (v) * (w)->bv + (w)->D.cell((i), (j), (k))])
#include "work_formulas.h"
#undef MAMR_AT
#undef MAMR_WVIEW
#undef MAMR_WFN0
#undef MAMR_WFN

namespace {

// kind: 0 stencil_0, 6 stencil_check.  (No __restrict__ on the pool in
// the two in-place kernels: their reads must see their own stores.)
template <int BX, int BY, int BZ>
__global__ void work_cell_kernel(double *pool, Geom g,
                                 const int32_t *__restrict__ slots, int nb,
                                 int var, int kind, mamr_work_par P)
{
   const Dims<BX, BY, BZ> D(g);
   const int cells = D.nx * D.ny * D.nz;
   const long long total = (long long) cells * nb;
   for (long long e = blockIdx.x * (long long) blockDim.x + threadIdx.x;
        e < total; e += (long long) gridDim.x * blockDim.x) {
      const int b = (int) (e / cells);
      const int c = (int) (e - (long long) b * cells);
      const int i = c / (D.ny * D.nz) + 1, r = c % (D.ny * D.nz);
      const int j = r / D.nz + 1, k = r % D.nz + 1;
      const WView<BX, BY, BZ> w{pool + bv_offset(g, slots[b], 0), g.bv, D};
      double *p = pool + bv_offset(g, slots[b], var) + D.cell(i, j, k);
      *p = kind == 0 ? mamr_w_stencil0(&w, var, i, j, k, &P)
                     : mamr_w_check(*p, &P);
   }
}

// One thread per (block, line along axis).
template <int BX, int BY, int BZ>
__global__ void work_line_kernel(double *pool, Geom g,
                                 const int32_t *__restrict__ slots, int nb,
                                 int var, int axis, mamr_work_par P)
{
   const Dims<BX, BY, BZ> D(g);
   const int n = axis == 0 ? D.nx : (axis == 1 ? D.ny : D.nz);
   const int lines = D.nx * D.ny * D.nz / n;
   const long long total = (long long) lines * nb;
   for (long long e = blockIdx.x * (long long) blockDim.x + threadIdx.x;
        e < total; e += (long long) gridDim.x * blockDim.x) {
      const int b = (int) (e / lines);
      const int l = (int) (e - (long long) b * lines);
      // the two coordinates across the axis, in i, j, k order
      int a0, a1;
      if (axis == 0) { a0 = l / D.nz; a1 = l % D.nz; }
      else if (axis == 1) { a0 = l / D.nz; a1 = l % D.nz; }
      else { a0 = l / D.ny; a1 = l % D.ny; }
      const WView<BX, BY, BZ> w{pool + bv_offset(g, slots[b], 0), g.bv, D};
      double *base = pool + bv_offset(g, slots[b], var);
      for (int t = 1; t <= n; t++) {
         int i, j, k;
         if (axis == 0) { i = t; j = a0 + 1; k = a1 + 1; }
         else if (axis == 1) { i = a0 + 1; j = t; k = a1 + 1; }
         else { i = a0 + 1; j = a1 + 1; k = t; }
         base[D.cell(i, j, k)] = mamr_w_line(&w, var, axis, i, j, k, &P);
      }
   }
}

// Work values into scratch[b][cell] (seven: 1 for stencil_7, 0 for _27).
template <int BX, int BY, int BZ>
__global__ void work_jacobi_kernel(const double *__restrict__ pool, Geom g,
                                   const int32_t *__restrict__ slots, int nb,
                                   int var, int seven, mamr_work_par P,
                                   double *__restrict__ scratch)
{
   const Dims<BX, BY, BZ> D(g);
   const int cells = D.nx * D.ny * D.nz;
   const long long total = (long long) cells * nb;
   for (long long e = blockIdx.x * (long long) blockDim.x + threadIdx.x;
        e < total; e += (long long) gridDim.x * blockDim.x) {
      const int b = (int) (e / cells);
      const int c = (int) (e - (long long) b * cells);
      const int i = c / (D.ny * D.nz) + 1, r = c % (D.ny * D.nz);
      const int j = r / D.nz + 1, k = r % D.nz + 1;
      const WView<BX, BY, BZ> w{pool + bv_offset(g, slots[b], 0), g.bv, D};
      scratch[e] = seven ? mamr_w_seven(&w, var, i, j, k, &P)
                         : mamr_w_twentyseven(&w, var, i, j, k, &P);
   }
}

template <int BX, int BY, int BZ>
__global__ void work_copy_kernel(double *__restrict__ pool, Geom g,
                                 const int32_t *__restrict__ slots, int nb,
                                 int var, const double *__restrict__ scratch)
{
   const Dims<BX, BY, BZ> D(g);
   const int cells = D.nx * D.ny * D.nz;
   const long long total = (long long) cells * nb;
   for (long long e = blockIdx.x * (long long) blockDim.x + threadIdx.x;
        e < total; e += (long long) gridDim.x * blockDim.x) {
      const int b = (int) (e / cells);
      const int c = (int) (e - (long long) b * cells);
      const int i = c / (D.ny * D.nz) + 1, r = c % (D.ny * D.nz);
      const int j = r / D.nz + 1, k = r % D.nz + 1;
      pool[bv_offset(g, slots[b], var) + D.cell(i, j, k)] = scratch[e];
   }
}

int grid_for(long long items)
{
   const long long blocks = (items + 255) / 256;
   return (int) (blocks < 152 * 32 ? (blocks > 0 ? blocks : 1) : 152 * 32);
}

}  // namespace

template <int BX, int BY, int BZ>
static int launch_work(double *pool, const Geom &g, const int32_t *slots,
                       int nb, int var, int calc_stage,
                       const mamr_work_par &P, double *scratch,
                       cudaStream_t s)
{
   const long long cells = (long long) g.nx * g.ny * g.nz * nb;
   int launches = 0;
   switch (calc_stage % 6) {
   case 0:
      work_cell_kernel<BX, BY, BZ><<<grid_for(cells), 256, 0, s>>>(
         pool, g, slots, nb, var, 0, P);
      launches = 1;
      break;
   case 1:
   case 2:
   case 3: {
      const int axis = calc_stage % 6 - 1;
      const int n = axis == 0 ? g.nx : (axis == 1 ? g.ny : g.nz);
      work_line_kernel<BX, BY, BZ><<<grid_for(cells / n), 256, 0, s>>>(
         pool, g, slots, nb, var, axis, P);
      launches = 1;
      break;
   }
   default:
      work_jacobi_kernel<BX, BY, BZ><<<grid_for(cells), 256, 0, s>>>(
         pool, g, slots, nb, var, calc_stage % 6 == 4, P, scratch);
      work_copy_kernel<BX, BY, BZ><<<grid_for(cells), 256, 0, s>>>(
         pool, g, slots, nb, var, scratch);
      launches = 2;
      break;
   }
   work_cell_kernel<BX, BY, BZ><<<grid_for(cells), 256, 0, s>>>(
      pool, g, slots, nb, var, 6, P);
   launches++;
   return cudaPeekAtLastError() == cudaSuccess ? launches : -1;
}

// stencil_driver's variable-work branch for one variable (1 <= var <
// 4*mat): the kernel of calc_stage % 6, then stencil_check.
int launch_work_stencil(double *pool, const Geom &g, const int32_t *slots,
                        int nb, int var, int calc_stage,
                        const mamr_work_par &P, double *scratch,
                        cudaStream_t s)
{
   if (nb == 0)
      return 0;
   switch (dims_kind(g)) {
   case 1:
      return launch_work<8, 8, 8>(pool, g, slots, nb, var, calc_stage, P,
                                  scratch, s);
   case 2:
      return launch_work<16, 16, 16>(pool, g, slots, nb, var, calc_stage, P,
                                     scratch, s);
   default:
      return launch_work<0, 0, 0>(pool, g, slots, nb, var, calc_stage, P,
                                  scratch, s);
   }
}

}  // namespace mamr
