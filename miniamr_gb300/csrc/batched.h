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
   int32_t bmask;      // bit l: face l is a domain boundary; bit 8 + l:
                       // f[l] is FACE_COARSE; bit 16 + l: FACE_FINE
   BFace f[6];
   int32_t nb27[27];   // neighbour at offset (dx,dy,dz), index
                       // (dx+1) + 3(dy+1) + 9(dz+1); single-level meshes
};

// Sets the level-jump bits of it.bmask from its faces' types.
__host__ __device__ inline void set_jump_bits(BItem &it)
{
   for (int l = 0; l < 6; l++) {
      if (it.f[l].type == FACE_COARSE)
         it.bmask |= 1 << (8 + l);
      else if (it.f[l].type == FACE_FINE)
         it.bmask |= 1 << (16 + l);
   }
}

// ---- 27-point edge and corner ghosts on multi-level meshes ---------------
// comm() (code 0) runs its phases x, y, z in turn, each writing the ghost
// cells on its axis over fixed ranges (ref/comm.c:1473-1534, 1597-1688,
// 1911-1965): across a same-level face the x phase writes cells whose j, k
// are interior, the y phase those whose k is interior, the z phase all;
// a boundary face (27-point) writes all; a level jump only cells whose
// other two coordinates are interior (coarse/4, or the ordered 4-cell
// sum).  A ghost cell's value after a stage is that of its last writer.
// A writer copies a cell of the neighbour (or of the block itself) as the
// earlier phases of the stage left it -- a cell no earlier phase wrote
// still holds what the previous stage gave it.  Resolving the chain gives
// each edge and corner one recipe, the same for every variable and stage:
// an interior cell (current values), a transform of interior cells, a
// ghost cell as the previous stage left it (PREV: read from the stage's
// source pool, whose marked ghost cells every stage writes), or a cell no
// exchange writes while the mesh stands (STALE: read from the pool the
// run started from).
enum : int8_t {
   GR_INTERIOR = 0,   // an interior cell of block nb[0]
   GR_STALE = 1,      // a ghost cell of block nb[0] no exchange writes
   GR_COARSE = 2,     // coarse/4 across face l of the chain's last block
   GR_FINE = 3,       // the 4-cell sum across face l (fine blocks nb[])
   GR_PREV = 4        // a ghost cell of block nb[0] after the last stage
};
struct GhostRecipe {
   int8_t kind;       // GR_*
   int8_t l;          // GR_COARSE / GR_FINE: the face crossed
   int8_t vax;        // edges: the axis the cells run along; corners: -1
   int8_t iqjq;       // GR_COARSE: quarter iq | jq << 1 of the coarse face
   int16_t c[3];      // the cell in the chain's last block (c[vax] unused)
   int16_t pad;
   int32_t nb[4];
};
// 12 edges -- 0..3 along z (i, j sides from bits 0, 1), 4..7 along y (i, k
// sides), 8..11 along x (j, k sides) -- and 8 corners 12..19 (i, j, k
// sides from bits 0, 1, 2).
constexpr int kGhostRecipes = 20;
// A block's "keep" mask: ghost cells some recipe reads as PREV, which
// every stage writes to its destination pool -- bit l (0..5) the face
// plane l, bit 6 + e the edge e.
// Face l of block bp as the batched kernels gather it; false when a
// coarser neighbour does not list bp on the shared face (the face is then
// left as a boundary).
__host__ __device__ inline bool face_desc(const mamr_block *mesh,
                                          const int32_t *slot_pos,
                                          const mamr_block &bp, int l,
                                          BFace &f)
{
   f.nb[0] = f.nb[1] = f.nb[2] = f.nb[3] = 0;
   f.iq = f.jq = 0;
   const int nl = bp.nei_level[l];
   if (nl == -2) {
      f.type = FACE_BC;
      return true;
   }
   if (nl == bp.level) {
      f.type = FACE_SAME;
      f.nb[0] = bp.nei[l][0][0];
      return true;
   }
   if (nl == bp.level + 1) {
      f.type = FACE_FINE;
      for (int iq = 0; iq < 2; iq++)
         for (int jq = 0; jq < 2; jq++)
            f.nb[iq * 2 + jq] = bp.nei[l][iq][jq];
      return true;
   }
   const int m = bp.nei[l][0][0];
   const int pm = slot_pos[m];
   if (pm >= 0)
      for (int iq = 0; iq < 2; iq++)
         for (int jq = 0; jq < 2; jq++)
            if (mesh[pm].nei[l ^ 1][iq][jq] == bp.slot) {
               f.type = FACE_COARSE;
               f.nb[0] = m;
               f.iq = iq;
               f.jq = jq;
               return true;
            }
   f.type = FACE_BC;
   return false;
}

// Whether the phase of axis a writes ghost cell c (c[a] a ghost index) of
// block bp; f receives the face's descriptor.
__host__ __device__ inline bool phase_writes(const mamr_block *mesh,
                                             const int32_t *slot_pos,
                                             const mamr_block &bp,
                                             const int (&c)[3],
                                             const int (&n)[3], int a,
                                             BFace &f, bool &ok)
{
   const int l = 2 * a + (c[a] == n[a] + 1);
   ok = face_desc(mesh, slot_pos, bp, l, f);
   auto interior = [&](int ax) { return c[ax] >= 1 && c[ax] <= n[ax]; };
   if (f.type == FACE_BC)
      return true;
   if (f.type == FACE_SAME)
      return a == 2 || (a == 1 ? interior(2) : interior(1) && interior(2));
   for (int ax = 0; ax < 3; ax++)
      if (ax != a && !interior(ax))
         return false;
   return true;
}

// The mask bit (above) of ghost cell c, which has one or two ghost axes.
__host__ __device__ inline int keep_bit(const int (&c)[3], const int (&n)[3])
{
   int g[3], ng = 0;
   for (int ax = 0; ax < 3; ax++)
      if (c[ax] == 0 || c[ax] == n[ax] + 1)
         g[ng++] = ax;
   auto hi = [&](int ax) { return c[ax] == n[ax] + 1 ? 1 : 0; };
   if (ng == 1)
      return 2 * g[0] + hi(g[0]);
   // edge along the axis that is not a ghost axis
   const int vax = 3 - g[0] - g[1];
   return 6 + 4 * (2 - vax) + (hi(g[0]) | hi(g[1]) << 1);
}

// The recipe of edge or corner e (numbering above) of mesh block q; false
// for a misconnected mesh.  *keep_q / *keep_bit receive the block (mesh
// index) and mask bit of a PREV cell, else -1.
__host__ __device__ inline bool resolve_ghost(const mamr_block *mesh,
                                              const int32_t *slot_pos, int q,
                                              int nx, int ny, int nz, int e,
                                              GhostRecipe &r, int &keep_q,
                                              int &keep_b)
{
   const int n[3] = {nx, ny, nz};
   int c[3], vax;
   if (e < 12) {
      const int s = e & 3;
      vax = 2 - e / 4;                       // 2 (z), 1 (y), 0 (x)
      const int a0 = vax == 0 ? 1 : 0, a1 = vax == 2 ? 1 : 2;
      c[vax] = 1;                            // any interior index
      c[a0] = (s & 1) ? n[a0] + 1 : 0;
      c[a1] = (s & 2) ? n[a1] + 1 : 0;
   } else {
      const int s = e - 12;
      vax = -1;
      for (int ax = 0; ax < 3; ax++)
         c[ax] = (s >> ax & 1) ? n[ax] + 1 : 0;
   }
   r.kind = -1;
   r.vax = (int8_t) vax;
   r.l = 0;
   r.iqjq = 0;
   r.pad = 0;
   r.nb[0] = r.nb[1] = r.nb[2] = r.nb[3] = 0;
   keep_q = keep_b = -1;
   int cur = q, lim = 3;
   for (int hop = 0; hop < 4 && r.kind < 0; hop++) {
      // the last phase before `lim` that writes the cell
      int a = -1;
      BFace f;
      for (int ax = lim - 1; ax >= 0 && a < 0; ax--) {
         if (c[ax] != 0 && c[ax] != n[ax] + 1)
            continue;
         bool ok = true;
         const bool w = phase_writes(mesh, slot_pos, mesh[cur], c, n, ax, f,
                                     ok);
         if (!ok)
            return false;
         if (w)
            a = ax;
      }
      bool ghost = false;
      for (int ax = 0; ax < 3; ax++)
         ghost |= c[ax] == 0 || c[ax] == n[ax] + 1;
      if (!ghost) {
         r.kind = GR_INTERIOR;
         r.nb[0] = mesh[cur].slot;
         break;
      }
      if (a < 0) {
         // no writer this stage so far: a later phase may write it (its
         // value is then the previous stage's), or none does
         bool later = false;
         for (int ax = 0; ax < 3 && !later; ax++)
            if (c[ax] == 0 || c[ax] == n[ax] + 1) {
               bool ok = true;
               later = phase_writes(mesh, slot_pos, mesh[cur], c, n, ax, f,
                                    ok);
               if (!ok)
                  return false;
            }
         r.kind = later ? GR_PREV : GR_STALE;
         r.nb[0] = mesh[cur].slot;
         if (later) {
            keep_q = cur;
            keep_b = keep_bit(c, n);
         }
         break;
      }
      const bool hi = c[a] == n[a] + 1;
      if (f.type == FACE_SAME) {
         cur = slot_pos[f.nb[0]];
         if (cur < 0)
            return false;
         c[a] = hi ? 1 : n[a];
      } else if (f.type == FACE_BC) {
         c[a] = hi ? n[a] : 1;
      } else {
         r.kind = f.type == FACE_COARSE ? GR_COARSE : GR_FINE;
         r.l = (int8_t) (2 * a + hi);
         r.iqjq = (int8_t) (f.iq | f.jq << 1);
         for (int t = 0; t < 4; t++)
            r.nb[t] = f.nb[t];
      }
      lim = a;
   }
   for (int ax = 0; ax < 3; ax++)
      r.c[ax] = (int16_t) c[ax];
   return r.kind >= 0;
}

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
//   pencil kernel with tensor copies (FP32; kernel = 3): the interior and
//                   x-face planes of each tile arrive by bulk tensor copy
//   warp-per-item kernel (8^3 blocks, 7-point; kernel = 1): threads = 32
//                   or 64 per item, vpc = items per CTA, rows = rows per
//                   thread, planes = variables per item (1 or 2); tma = 1:
//                   its tensor-copy form (FP32)
struct StageShape {
   int threads = 0, vpc = 1, rows = 1, planes = 4, grid = 1;
   int kernel = 0;
   int tma = 0;
};

// Launches one fused stage: src -> dst for every block and variable.
// FP64 checksums: per-block serial sums into partials[var][block], then
// finalize into sums[var]; FP32: exact fixed-point into acc[var][2].
// recipes: the 27-point edge and corner recipes of a multi-level mesh
// (n_blocks * kGhostRecipes, mesh order) and keep, the blocks' keep masks,
// or null on one level; stale: the pool the run started from (recipes'
// stale cells); zf_src / zf_dst: the warp-per-block kernel's z-face arrays
// of the source (null when the previous stage wrote none) and the
// destination (null: none written); ctx_err: the context's error word (a
// bounded wait that ran out); n_bv: block-variables the pools hold.
template <typename T>
int launch_batched_stage(const T *src, T *dst, const Geom &g, int stencil,
                         const BItem *items, const GhostRecipe *recipes,
                         const int *keep, const T *stale, int n_blocks,
                         const StageShape &sh, int write_ghosts, int do_cs,
                         double *partials, double *sums,
                         unsigned long long *acc, unsigned *err,
                         unsigned *ctx_err, long long n_bv,
                         const T *zf_src, T *zf_dst, cudaStream_t s);
// The generic kernel's launch shapes for this geometry (first = default).
template <typename T>
void batched_candidates(const Geom &g, int stencil, int n_blocks,
                        std::vector<StageShape> &out);

// Tile kernel for 8^3 and 16^3 blocks, 7 or 27 points, any mesh
// (tile_kernels.cu): its launch shapes (kernel 2) and one stage.
template <typename T>
void tile_candidates(const Geom &g, int stencil, int n_blocks,
                     std::vector<StageShape> &out);
template <typename T>
int launch_tile_stage(const T *src, T *dst, const Geom &g, int stencil,
                      const BItem *items, const GhostRecipe *recipes,
                      const int *keep, const T *stale, int n_blocks,
                      const StageShape &sh, int write_ghosts, int do_cs,
                      unsigned long long *acc, unsigned *err,
                      const T *zf_src, T *zf_dst, cudaStream_t s);

// Warp-per-item variant for 8^3 blocks and the 7-point stencil (any mesh):
// its launch shapes, and one stage (FP32 checksums fused into acc).
template <typename T>
void brick_candidates(const Geom &g, int stencil, int n_blocks,
                      std::vector<StageShape> &out);
template <typename T>
int launch_brick_stage(const T *src, T *dst, const Geom &g,
                       const BItem *items, int n_blocks, const StageShape &sh,
                       int write_ghosts, int do_cs, unsigned long long *acc,
                       unsigned *err, unsigned *ctx_err, long long n_bv,
                       const T *zf_src, T *zf_dst, cudaStream_t s);
// zface_elems / zface_at: mamr_internal.h.

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
                        unsigned *ctx_err, long long n_bv, cudaStream_t s);
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
// The edge and corner recipes (kGhostRecipes per block, mesh order) of a
// multi-level mesh and the blocks' keep masks (keep[n], zeroed first);
// *bad (set above n first) is lowered to the index of a block whose chain
// meets a misconnected face.
int launch_build_recipes(const mamr_block *mesh, int n,
                         const int32_t *slot_pos, const Geom &g,
                         GhostRecipe *out, int *keep, int *bad,
                         cudaStream_t s);

// The pencil kernel's launch shapes for n_work = pencils x variables.
template <typename T>
void pencil_candidates(int stencil, int n_work, std::vector<StageShape> &out);

}  // namespace mamr
