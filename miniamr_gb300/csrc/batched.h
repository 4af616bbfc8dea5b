// Batched path: one fused launch per stage over every (block, variable) --
// ghost gather from the neighbours' interiors, stencil, checksum -- reading
// one pool and writing the other (ping-pong), so that no grid-wide barrier
// separates the exchange from the update.
#pragma once

#include <vector>

#include "mamr_internal.h"

namespace mamr {

// How one face of a block gets its ghost layer in the batched path.
enum : int32_t {
   FACE_SAME = 0,    // same-level neighbour nb[0]
   FACE_BC = 1,      // domain boundary: reflect the block's own plane
   FACE_COARSE = 2,  // coarser neighbour nb[0]; this block is quarter
                     // (iq, jq) of the neighbour's face
   FACE_FINE = 3     // four finer neighbours nb[iq*2 + jq]
};

struct BFace {
   int32_t type;
   int32_t nb[4];
   int32_t iq, jq;
};

// Per active block, in sorted_list order.
struct BItem {
   int32_t slot;
   int32_t bmask;      // bit l: face l is a domain boundary
   BFace f[6];
   int32_t nb27[27];   // neighbour at offset (dx,dy,dz), index
                       // (dx+1) + 3(dy+1) + 9(dz+1); single-level meshes
};

// One tile of a pencil: the block and its in-plane neighbours at offset
// (dx, dy), index (dx+1) + 3(dy+1), with bmask as in BItem.
struct TileDesc {
   int32_t slot;
   int32_t bmask;
   int32_t nb9[9];
};
// Longest pencil (blocks along z) the pencil kernel takes.
constexpr int PENCIL_MAX = 64;

struct BatchedState;

void batched_destroy(BatchedState *b);
void batched_mesh_changed(BatchedState *b);

// Launch shape of a stage kernel, one of the autotuner's candidates.
//   generic kernel: `threads` per variable (whole warps), `vpc` variables
//                   of one block per CTA (blockDim = vpc * threads)
//   pencil kernel:  `rows` j-rows and `planes` i-planes per thread
//                   (threads = 1024 / (rows * planes))
//   both:           `grid` CTAs
//   warp-per-item kernel (8^3 blocks, 7-point; kernel = 1): threads = 32,
//                   vpc = warps per CTA, rows = 2, planes = 0
struct StageShape {
   int threads = 0, vpc = 1, rows = 1, planes = 4, grid = 1;
   int kernel = 0;
};

// Launches one fused stage: src -> dst for every block and variable.
// FP64 checksums: per-block serial sums into partials[var][block], then
// finalize into sums[var]; FP32: exact fixed-point into acc[var][2].
template <typename T>
int launch_batched_stage(const T *src, T *dst, const Geom &g, int stencil,
                         const BItem *items, int n_blocks,
                         const StageShape &sh, int write_ghosts, int do_cs,
                         double *partials, double *sums,
                         unsigned long long *acc, unsigned *err,
                         cudaStream_t s);
// The generic kernel's launch shapes for this geometry (first = default).
template <typename T>
void batched_candidates(const Geom &g, int stencil, int n_blocks,
                        std::vector<StageShape> &out);

// Warp-per-item variant for 8^3 blocks and the 7-point stencil (any mesh):
// its launch shapes, and one stage (FP32 checksums fused into acc).
template <typename T>
void brick_candidates(const Geom &g, int stencil, int n_blocks,
                      std::vector<StageShape> &out);
template <typename T>
int launch_brick_stage(const T *src, T *dst, const Geom &g,
                       const BItem *items, int n_blocks, const StageShape &sh,
                       int write_ghosts, int do_cs, unsigned long long *acc,
                       unsigned *err, cudaStream_t s);

// Pencil variant for single-level meshes of 16^3 blocks: CTAs walk chains
// of blocks along z (chain[pencils[p].x .. +pencils[p].y), bottom to
// top).  FP32 checksums are fused (acc); FP64 checksums run as a separate
// all-variable pass into partials and sums.
template <typename T>
int launch_pencil_stage(const T *src, T *dst, const Geom &g, int stencil,
                        const BItem *items, int n_blocks,
                        const TileDesc *chain, const int2 *pencils,
                        int n_pencils, const StageShape &sh, int write_ghosts,
                        int do_cs, double *partials, double *sums,
                        unsigned long long *acc, unsigned *err,
                        cudaStream_t s);
// FP64 checksums of every (block, variable) of a pool in the reference's
// order: per-block serial sums into partials[var][block] (one thread per
// block-variable), then sums[var] serially over blocks.  Returns the
// number of kernels launched.
int launch_fp64_checksums(const double *pool, const Geom &g,
                          const BItem *items, int n_blocks, double *partials,
                          double *sums, cudaStream_t s);

// Per-block descriptors (items[0..n)) built on the device from the mesh
// and its slot -> index map; single: also the edge and corner neighbours
// (nb27).  *bad (set above n first) is lowered to the index of a block
// whose coarser neighbour does not list it.
int launch_build_items(const mamr_block *mesh, int n, const int32_t *slot_pos,
                       int single, BItem *items, int *bad, cudaStream_t s);

// The pencil kernel's launch shapes for n_work = pencils x variables.
template <typename T>
void pencil_candidates(int stencil, int n_work, std::vector<StageShape> &out);

}  // namespace mamr
