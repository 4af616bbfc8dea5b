// Internal declarations shared by the host side (api.cu) and the kernels
// (plain_kernels.cu, batched_kernels.cu) of the GB300 library.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstddef>

#include "miniamr_gb300.h"
#include "work_formulas.h"

namespace mamr {

// Pool geometry.  Two layouts of one block-variable:
//  - split (kplane >= 0; the device pool): the X*Y rows hold only the
//    interior k = 1..nz, back to back (row i*Y + j at (i*Y + j)*nz), so the
//    128-byte lines DRAM delivers carry nothing but interior cells; the
//    ghost values k = 0 and k = nz+1 of row (i, j) sit in two planes after
//    the rows, at kplane + i*Y + j and kplane + X*Y + i*Y + j.  bv is
//    rounded up to whole 128-byte lines, and the device pools start where
//    interior row (1, 1) of every block-variable begins a line.
//  - inline (kplane < 0; host buffers): rows of Zp elements holding
//    k = 0..nz+1 at columns koff .. koff+nz+1.
struct Geom {
   int nx, ny, nz, V;
   int X, Y, Z;       // nx+2, ny+2, nz+2
   int Zp, koff;      // inline layout: row length, column of k = 0
   long long kplane;  // split layout: offset of the k = 0 plane, else -1
   long long bv;      // elements per block-variable
};

__host__ __device__ inline long long bv_offset(const Geom &g, int slot,
                                               int var)
{
   return ((long long) slot * g.V + var) * g.bv;
}

__host__ __device__ inline long long cell_offset(const Geom &g, int i, int j,
                                                 int k)
{
   const long long row = (long long) i * g.Y + j;
   if (g.kplane < 0)
      return row * g.Zp + g.koff + k;
   if (k >= 1 && k <= g.nz)
      return row * g.nz + (k - 1);
   return g.kplane + (k == 0 ? 0 : (long long) g.X * g.Y) + row;
}

// z-face arrays of the warp-per-block and tile kernels: each stage of a
// batched run also stores every block-variable's k = 1 and k = nz planes
// (side 0 and 1, nx * ny values each at (i-1)*ny + (j-1)) contiguously,
// and the next stage reads its z ghosts from there instead of one value
// per row of the neighbour; splits and consolidations store the planes of
// the blocks they write while the arrays are live.  Elements of one
// array, and the offset of a plane.
inline size_t zface_elems(const Geom &g, int max_blocks)
{
   return (size_t) max_blocks * g.V * 2 * g.nx * g.ny;
}
__host__ __device__ inline long long zface_at(const Geom &g, int slot,
                                              int var, int side)
{
   return (((long long) slot * g.V + var) * 2 + side) * g.nx * g.ny;
}

// Offset of interior row (i, j), k = 1, in the split layout.
__host__ __device__ inline long long row_offset(const Geom &g, int i, int j)
{
   return ((long long) i * g.Y + j) * g.nz;
}

// Same-level exchange across one face: lo is the block on the low side
// (west / south / down), hi the one on the high side.
struct SameTask { int32_t lo, hi; };
// Coarse/fine exchange: face l of the coarse block, quarter (iq, jq) of it.
struct DiffTask { int32_t coarse, fine, l, iq, jq; };
// Reflective boundary on face l of a block.
struct BcTask { int32_t slot, l; };

struct DirTasks {
   const SameTask *same; int n_same;
   const DiffTask *diff; int n_diff;
   const BcTask *bc; int n_bc;
};

// Marks an FP32 checksum slot (lo, hi) whose lo word holds the bits of a
// double (the compensated FP64 fallback's result) instead of a fixed-point
// sum: a genuine sum has |hi| < 2^40, so hi never takes this value.
constexpr unsigned long long kChecksumFallbackMark = 0x8000000000000000ull;

// Error word bits written by kernels (context error word).
enum : unsigned {
   ERR_FIXED_RANGE = 1u,   // a cell outside the fixed-point checksum range
   ERR_TASK = 2u,          // a task that does not fit the geometry
   ERR_MARK = 4u,          // refinement marking did not settle
   ERR_WAIT = 8u           // a bounded wait for a bulk copy ran out
};

// --stencil 0: the variable-work kernel of calc_stage % 6 and
// stencil_check for one variable (1 <= var < 4*mat), FP64 pools; scratch
// holds nb * nx*ny*nz doubles.
int launch_work_stencil(double *pool, const Geom &g, const int32_t *slots,
                        int nb, int var, int calc_stage,
                        const mamr_work_par &P, double *scratch,
                        cudaStream_t s);

// Records a failure for mamr_last_error() and returns code.
int report_error(int code, const char *fmt, ...);

// Kernel launchers (plain path).  All return the launch count they issued
// (>= 0) or -1 after a launch error (cudaGetLastError is left set).
template <typename T>
int launch_comm_dir(T *pool, const Geom &g, int dir, int stencil, int code,
                    const DirTasks &t, int var0, int nvar, const T *zc,
                    cudaStream_t s);
template <typename T>
int launch_stencil(T *pool, const Geom &g, int stencil, const int32_t *slots,
                   int n, int var, T *zc, cudaStream_t s);
// The plain path's z-face cache: for every block-variable its interior
// planes k = 1 (side 0) and k = nz (side 1), nx*ny values each at
// (i-1)*ny + (j-1), as the last stencil left them.  The stencil writes it
// (zc non-null) beside the pool; the z-direction face exchange reads the
// interior rows' k = 1 / k = nz values from it (zc non-null) instead of
// one value per 32-byte sector of the pool.
__host__ __device__ inline long long zcache_at(const Geom &g, int slot,
                                               int var, int side, int i,
                                               int j)
{
   return (((long long) slot * g.V + var) * 2 + side) * (g.nx * g.ny) +
          (long long) (i - 1) * g.ny + (j - 1);
}
inline size_t zcache_elems(const Geom &g, int max_blocks)
{
   return (size_t) max_blocks * g.V * 2 * g.nx * g.ny;
}
// The plain stencil stages a whole block-variable in shared memory up to
// kPlainTileBytes and streams larger ones along i through a ring of three
// planes, which must fit kPlainRingBytes (plain_stencil_fits).
constexpr size_t kPlainTileBytes = 200 * 1024;
constexpr size_t kPlainRingBytes = 200 * 1024;
bool plain_stencil_fits(const Geom &g, size_t elem);
// FP64: serial per-block sums in exact reference order, then a serial sum
// over blocks; result in *d_out.
int launch_checksum_fp64(const double *pool, const Geom &g,
                         const int32_t *slots, int n, int var,
                         double *d_partials, double *d_out, cudaStream_t s);
// FP64 checksums of every variable at once into d_sums[V] (d_partials:
// n * V doubles); the same bits as launch_checksum_fp64 per variable.
int launch_checksum_fp64_all(const double *pool, const Geom &g,
                             const int32_t *slots, int n, double *d_partials,
                             double *d_sums, cudaStream_t s);
// FP32, every variable at once into acc[2 * V] (zeroed first).
int launch_checksum_fp32_all(const float *pool, const Geom &g,
                             const int32_t *slots, int n,
                             unsigned long long *acc, unsigned *err,
                             cudaStream_t s);
// FP32 checksum fallback for the variables var0 .. var0+nvar-1 whose cells
// leave the fixed-point window: flags[0] is the miss word the checksum set
// (nothing runs while it is clear), flags[1 .. nvar] per-variable miss
// words and flags[1 + nvar] a counter (all zeroed first), partials
// n * nvar doubles, acc the checksum slots of var0 .. (two words each),
// overwritten for the variables that missed with the compensated FP64 sum
// under kChecksumFallbackMark.  Returns 1 (kernels launched) or -1.
int launch_fp32_checksum_fallback(const float *pool, const Geom &g,
                                  const int32_t *slots, int n, int var0,
                                  int nvar, unsigned *flags,
                                  double *partials, unsigned long long *acc,
                                  cudaStream_t s);
// FP32: exact 128-bit fixed-point accumulation into acc[2] (lo, hi),
// which must be zeroed first.
int launch_checksum_fp32(const float *pool, const Geom &g,
                         const int32_t *slots, int n, int var,
                         unsigned long long *acc, unsigned *err,
                         cudaStream_t s);
template <typename T>
int launch_stage_blocks(T *stage, const T *pool, const Geom &g,
                        const int32_t *slots, int n, cudaStream_t s);
// Data-movement reads with a negative slot s come from staging entry -s-1;
// zf (may be null): the live z-face array, into which the kernels also
// store the k = 1 and k = nz planes of the blocks they write.
template <typename T>
int launch_split(T *pool, const T *stage, const Geom &g,
                 const mamr_split_job *jobs, int n, T *zf, cudaStream_t s);
template <typename T>
int launch_consolidate(T *pool, const T *stage, const Geom &g,
                       const mamr_consolidate_job *jobs, int n, T *zf,
                       cudaStream_t s);
template <typename T>
int launch_upload(T *pool, const Geom &g, const int32_t *slots, int n,
                  const double *dense, cudaStream_t s);
template <typename T>
int launch_download(const T *pool, const Geom &g, const int32_t *slots,
                    int n, double *dense, cudaStream_t s);

// Refinement marking (mark_kernels.cu): flags of the listed blocks into
// d_out (list order) and of the parents into d_pref; d_ref holds
// max_blocks flags by slot, d_flags 3 pass flags.  Returns kernels
// launched or -1.
int launch_mark_refine(const mamr_mark_params &p, int3 bsize,
                       const mamr_object *d_objs, int n_objs,
                       const mamr_mark_block *d_mb, int nb,
                       const mamr_mark_parent *d_pa, int np, int max_blocks,
                       int32_t *d_ref, int32_t *d_pref, int32_t *d_out,
                       int *d_flags, unsigned *err, cudaStream_t s);

}  // namespace mamr
