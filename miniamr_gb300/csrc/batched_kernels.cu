// Batched stage kernel: one persistent launch per stage covering every
// (block, variable) item.  Each item stages its block-variable in shared
// memory with a ghost layer gathered straight from the neighbours'
// interiors in the source pool -- the values comm() would have written
// (same-level copy, coarse/4 prolongation, 4-cell restriction sum,
// reflection; ref/comm.c:1465-1965) -- applies the stencil in the
// reference's operation order (ref/stencil.c:82-144), writes the interior
// to the destination pool and, for FP32 pools, folds the exact fixed-point
// checksum of the result into the same pass (FP64 checksums, serial in the
// reference's order ref/check_sum.c:44-53, run as a separate pass over all
// block-variables).
//
// Exactness: face ghosts are exact for every mesh.  27-point edge and
// corner ghosts are resolved axis by axis (neighbour across each
// out-of-range axis, reflection where that axis is a domain boundary),
// which is what comm()'s x, y, z sweeps compose to when all blocks share
// one level; the host only selects this path for 27-point stencils on such
// meshes.
#include <algorithm>
#include <vector>

#include "batched.h"
#include "arith.cuh"
#include "dims.cuh"
#include "ghost_eval.cuh"

namespace mamr {

template <typename T> struct Vec16;
template <> struct Vec16<float> { using type = float4; };
template <> struct Vec16<double> { using type = double2; };

// Shared-memory row length: column KO holds k = 0 so that k = 1 starts a
// 16-byte vector.
__host__ __device__ inline int tile_zs(int nz, int vw)
{
   return ((vw - 1 + nz + 2 + vw - 1) / vw) * vw;
}

template <typename T>
__host__ __device__ inline size_t tile_bytes(const Geom &g)
{
   const int vw = 16 / (int) sizeof(T);
   return (size_t) g.X * g.Y * tile_zs(g.nz, vw) * sizeof(T);
}


// A CTA takes the variables [vg * vpc, vg * vpc + vpc) of one block per
// work item: blockDim.x / vpc threads (whole warps) and one shared tile
// per variable, the block's neighbour record loaded once.
template <typename T, int ST, int BX, int BY, int BZ>
__global__ void __launch_bounds__(512)
batched_stage_kernel(const T *__restrict__ src, T *__restrict__ dst, Geom g,
                     const BItem *__restrict__ items,
                     const GhostRecipe *__restrict__ recipes,
                     const int *__restrict__ keep,
                     const T *__restrict__ stale, int nb, int vpc,
                     int write_ghosts, int do_cs,
                     unsigned long long *__restrict__ acc,
                     unsigned *__restrict__ err)
{
   extern __shared__ __align__(16) unsigned char smem_raw[];
   __shared__ BItem sI;
   constexpr int VW = 16 / (int) sizeof(T), KO = VW - 1;
   const Dims<BX, BY, BZ> D(g);
   const int nx = D.nx, ny = D.ny, nz = D.nz, Y = D.Y;
   const int Zs = tile_zs(nz, VW);
   const int gthreads = blockDim.x / vpc;
   const int grp = threadIdx.x / gthreads, gtid = threadIdx.x - grp * gthreads;
   T *tile = reinterpret_cast<T *>(smem_raw) + (size_t) grp * D.X * Y * Zs;
#define TS(i, j, k) tile[((i) * Y + (j)) * Zs + KO + (k)]
   const int n_groups = (g.V + vpc - 1) / vpc;
   const int n_items = nb * n_groups;
   const int nvec = nz / VW;
   const bool vec = (nz % VW) == 0;
   // FP32 checksum terms of this thread's variable, flushed per warp when
   // the variable changes and at the end
   unsigned long long lo = 0, hi = 0;
   Fixed52 part;
   bool ok = true;
   int cs_var = -1;

   for (int it = blockIdx.x; it < n_items; it += gridDim.x) {
      const int vg = it / nb, b = it - vg * nb;
      const int var = vg * vpc + grp;
      const bool active = var < g.V;
      if (sizeof(T) == 4 && do_cs && var != cs_var) {
         if (cs_var >= 0) {
            warp_acc128_flush(lo, hi, acc + 2 * cs_var);
            lo = hi = 0;
         }
         cs_var = active ? var : -1;
      }
      {
         const int32_t *from = reinterpret_cast<const int32_t *>(items + b);
         int32_t *to = reinterpret_cast<int32_t *>(&sI);
         for (int q = threadIdx.x; q < (int) (sizeof(BItem) / 4);
              q += blockDim.x)
            to[q] = from[q];
      }
      __syncthreads();
      const T *s = src + bv_offset(g, sI.slot, active ? var : 0);
      T *d = dst + bv_offset(g, sI.slot, active ? var : 0);
      // ghost cells the next stage reads as they stand after this one
      const int kb = keep ? keep[b] : 0;

      if (active) {
         // interior rows, 16-byte vectors (rows start on a sector boundary)
         if (vec) {
            using V = typename Vec16<T>::type;
            for (int e = gtid; e < nx * ny * nvec; e += gthreads) {
               int r = e / nvec, q = e - r * nvec;
               int i = r / ny + 1, j = r - (i - 1) * ny + 1;
               V v = __ldg(reinterpret_cast<const V *>(
                              s + D.cell(i, j, 1)) + q);
               *reinterpret_cast<V *>(&TS(i, j, 1 + q * VW)) = v;
            }
         } else {
            for (int e = gtid; e < nx * ny * nz; e += gthreads) {
               int r = e / nz, k = e - r * nz + 1;
               int i = r / ny + 1, j = r - (i - 1) * ny + 1;
               TS(i, j, k) = s[D.cell(i, j, k)];
            }
         }

         // face ghosts (tangential interior), one face per pass
         for (int l = 0; l < 6; l++) {
            const int dir = l >> 1;
            const bool low = !(l & 1);
            const int n = dir == 0 ? nx : (dir == 1 ? ny : nz);
            const int na = dir == 0 ? ny : nx;
            const int nbb = dir == 2 ? ny : nz;
            const int type = sI.f[l].type;
            const int gn = low ? 0 : n + 1;
            for (int e = gtid; e < na * nbb; e += gthreads) {
               const int a = e / nbb + 1, bq = e - (a - 1) * nbb + 1;
               T v;
               if (type == FACE_SAME) {
                  v = src[bv_offset(g, sI.f[l].nb[0], var) +
                          D.fcell(dir, low ? n : 1, a, bq)];
               } else if (type == FACE_BC) {
                  v = s[D.fcell(dir, low ? 1 : n, a, bq)];
               } else if (type == FACE_COARSE) {
                  const int ha = na / 2, hb = nbb / 2;
                  v = quarter(src[bv_offset(g, sI.f[l].nb[0], var) +
                                  D.fcell(dir, low ? n : 1,
                                        (a + 1) / 2 + sI.f[l].jq * ha,
                                        (bq + 1) / 2 + sI.f[l].iq * hb)]);
               } else {
                  const int ha = na / 2, hb = nbb / 2;
                  const int jq = a > ha, iq = bq > hb;
                  const int a2 = a - jq * ha, b2 = bq - iq * hb;
                  const int p = low ? n : 1;
                  const T *f = src + bv_offset(g, sI.f[l].nb[iq * 2 + jq], var);
                  T t = f[D.fcell(dir, p, 2 * a2 - 1, 2 * b2 - 1)] +
                        f[D.fcell(dir, p, 2 * a2 - 1, 2 * b2)];
                  t = t + f[D.fcell(dir, p, 2 * a2, 2 * b2 - 1)];
                  t = t + f[D.fcell(dir, p, 2 * a2, 2 * b2)];
                  v = t;
               }
               int gi, gj, gk;
               if (dir == 0) { gi = gn; gj = a; gk = bq; }
               else if (dir == 1) { gi = a; gj = gn; gk = bq; }
               else { gi = a; gj = bq; gk = gn; }
               TS(gi, gj, gk) = v;
               if (write_ghosts || (kb >> l & 1))
                  d[D.cell(gi, gj, gk)] = v;
            }
         }

         if (ST == 27) {
            // 12 edges and 8 corners: on one level resolved axis by axis
            // (nb27); across level jumps from the block's recipes
            const int ne = 4 * (nx + ny + nz) + 8;
            for (int e = gtid; e < ne; e += gthreads) {
               int gi, gj, gk, ri, t;
               if (e < 4 * nz) {
                  int q = e / nz;
                  gk = e - q * nz + 1;
                  gi = (q & 1) ? nx + 1 : 0;
                  gj = (q & 2) ? ny + 1 : 0;
                  ri = q;
                  t = gk;
               } else if (e < 4 * (nz + ny)) {
                  int e2 = e - 4 * nz, q = e2 / ny;
                  gj = e2 - q * ny + 1;
                  gi = (q & 1) ? nx + 1 : 0;
                  gk = (q & 2) ? nz + 1 : 0;
                  ri = 4 + q;
                  t = gj;
               } else if (e < 4 * (nz + ny + nx)) {
                  int e2 = e - 4 * (nz + ny), q = e2 / nx;
                  gi = e2 - q * nx + 1;
                  gj = (q & 1) ? ny + 1 : 0;
                  gk = (q & 2) ? nz + 1 : 0;
                  ri = 8 + q;
                  t = gi;
               } else {
                  int q = e - 4 * (nx + ny + nz);
                  gi = (q & 1) ? nx + 1 : 0;
                  gj = (q & 2) ? ny + 1 : 0;
                  gk = (q & 4) ? nz + 1 : 0;
                  ri = 12 + q;
                  t = 0;
               }
               if (recipes) {
                  const T v = eval_recipe(recipes[(size_t) b * kGhostRecipes +
                                                  ri],
                                          t, src, stale, g, D, var);
                  TS(gi, gj, gk) = v;
                  if (write_ghosts || (ri < 12 && (kb >> (6 + ri) & 1)))
                     d[D.cell(gi, gj, gk)] = v;
                  continue;
               }
               int dx = gi == 0 ? -1 : (gi == nx + 1 ? 1 : 0);
               int dy = gj == 0 ? -1 : (gj == ny + 1 ? 1 : 0);
               int dz = gk == 0 ? -1 : (gk == nz + 1 ? 1 : 0);
               int si = gi, sj = gj, sk = gk;
               if (dx) {
                  if (sI.bmask & (1 << (dx < 0 ? 0 : 1))) { si = dx < 0 ? 1 : nx; dx = 0; }
                  else si = dx < 0 ? nx : 1;
               }
               if (dy) {
                  if (sI.bmask & (1 << (dy < 0 ? 2 : 3))) { sj = dy < 0 ? 1 : ny; dy = 0; }
                  else sj = dy < 0 ? ny : 1;
               }
               if (dz) {
                  if (sI.bmask & (1 << (dz < 0 ? 4 : 5))) { sk = dz < 0 ? 1 : nz; dz = 0; }
                  else sk = dz < 0 ? nz : 1;
               }
               const int nbs = sI.nb27[(dx + 1) + 3 * (dy + 1) + 9 * (dz + 1)];
               const T v = src[bv_offset(g, nbs, var) + D.cell(si, sj, sk)];
               TS(gi, gj, gk) = v;
               if (write_ghosts)
                  d[D.cell(gi, gj, gk)] = v;
            }
         }
      }
      __syncthreads();

      // stencil, one (j, k) column per thread sweeping i
      if (active)
         for (int col = gtid; col < ny * nz; col += gthreads) {
            const int j = col / nz + 1, k = col - (j - 1) * nz + 1;
            if (ST == 7) {
               T am = TS(0, j, k), ac = TS(1, j, k);
               for (int i = 1; i <= nx; i++) {
                  const T ap = TS(i + 1, j, k);
                  T w = am + TS(i, j - 1, k);
                  w = w + TS(i, j, k - 1);
                  w = w + ac;
                  w = w + TS(i, j, k + 1);
                  w = w + TS(i, j + 1, k);
                  w = w + ap;
                  const T out = div7(w);
                  d[D.cell(i, j, k)] = out;
                  if (sizeof(T) == 4 && do_cs) {
                     fixed52_add((float) out, part);
                     if (nx > 256 && (i & 255) == 0)
                        fixed52_flush(part, lo, hi);
                  }
                  am = ac;
                  ac = ap;
               }
            } else {
               auto S = [&](int p) -> T {
                  T t = TS(p, j - 1, k - 1) + TS(p, j - 1, k);
                  t = t + TS(p, j - 1, k + 1);
                  t = t + TS(p, j, k - 1);
                  t = t + TS(p, j, k);
                  t = t + TS(p, j, k + 1);
                  t = t + TS(p, j + 1, k - 1);
                  t = t + TS(p, j + 1, k);
                  t = t + TS(p, j + 1, k + 1);
                  return t;
               };
               T s0 = S(0), s1 = S(1);
               for (int i = 1; i <= nx; i++) {
                  const T s2 = S(i + 1);
                  const T out = div27((s0 + s1) + s2);
                  d[D.cell(i, j, k)] = out;
                  if (sizeof(T) == 4 && do_cs) {
                     fixed52_add((float) out, part);
                     if (nx > 256 && (i & 255) == 0)
                        fixed52_flush(part, lo, hi);
                  }
                  s0 = s1;
                  s1 = s2;
               }
            }
            if (sizeof(T) == 4 && do_cs)
               fixed52_flush(part, lo, hi);
         }
      __syncthreads();
   }
   if (sizeof(T) == 4 && do_cs) {
      if (cs_var >= 0)
         warp_acc128_flush(lo, hi, acc + 2 * cs_var);
      if (!ok || !fixed52_window(part))
         atomicOr(err, ERR_FIXED_RANGE);
   }
#undef TS
}


// CTAs per SM for one shape; the kernel's dynamic shared memory limit only
// grows, so that every candidate queried stays launchable.
template <typename T, int ST, int BX, int BY, int BZ>
static int per_sm_of(size_t smem, int threads)
{
   int per_sm = 0;
   cudaFuncAttributes fa;
   if (cudaFuncGetAttributes(&fa, batched_stage_kernel<T, ST, BX, BY, BZ>) !=
          cudaSuccess ||
       (size_t) fa.maxDynamicSharedSizeBytes < smem)
      cudaFuncSetAttribute(batched_stage_kernel<T, ST, BX, BY, BZ>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int) smem);
   cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      &per_sm, batched_stage_kernel<T, ST, BX, BY, BZ>, threads, smem);
   return per_sm;
}

template <typename T, int ST>
static int batched_per_sm(const Geom &g, size_t smem, int threads)
{
   switch (dims_kind(g)) {
   case 1: return per_sm_of<T, ST, 8, 8, 8>(smem, threads);
   case 2: return per_sm_of<T, ST, 16, 16, 16>(smem, threads);
   default: return per_sm_of<T, ST, 0, 0, 0>(smem, threads);
   }
}

// Candidates: threads per variable = the (j, k) columns rounded up to
// whole warps (at most 256) or half that (at least one warp), times 1, 2
// or 4 variables per CTA (at most 512 threads and 200 KB of tiles); a
// persistent grid of the CTAs one wave holds.
template <typename T>
void batched_candidates(const Geom &g, int stencil, int n_blocks,
                        std::vector<StageShape> &out)
{
   int dev = 0, sms = 0;
   cudaGetDevice(&dev);
   cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
   out.clear();
   // 8^3 blocks, 7-point: the warp-per-item kernel first; 8^3 and 16^3
   // blocks: the double-buffered tile kernel
   brick_candidates<T>(g, stencil, n_blocks, out);
   tile_candidates<T>(g, stencil, n_blocks, out);
   const int cols = g.ny * g.nz;
   const int full = std::min(256, (cols + 31) / 32 * 32);
   for (int thr : {full, std::max(32, full / 2 / 32 * 32)}) {
      for (int vpc : {1, 2, 4}) {
         if (thr * vpc > 512 || vpc > g.V)
            continue;
         const size_t smem = tile_bytes<T>(g) * vpc;
         if (smem > 200 * 1024)
            continue;
         const int per_sm = stencil == 7
                               ? batched_per_sm<T, 7>(g, smem, thr * vpc)
                               : batched_per_sm<T, 27>(g, smem, thr * vpc);
         if (per_sm <= 0)
            continue;
         const long long items =
            (long long) n_blocks * ((g.V + vpc - 1) / vpc);
         StageShape sh;
         sh.threads = thr;
         sh.vpc = vpc;
         sh.grid = (int) std::max(1LL, std::min<long long>(
                                          (long long) per_sm * sms, items));
         bool dup = false;
         for (const StageShape &o : out)
            dup |= o.kernel == 0 && o.threads == sh.threads &&
                   o.vpc == sh.vpc;
         if (!dup)
            out.push_back(sh);
      }
      if (full == 32)
         break;
   }
}

template <typename T>
int launch_batched_stage(const T *src, T *dst, const Geom &g, int stencil,
                         const BItem *items, const GhostRecipe *recipes,
                         const int *keep, const T *stale, int n_blocks,
                         const StageShape &sh, int write_ghosts, int do_cs,
                         double *partials, double *sums,
                         unsigned long long *acc, unsigned *err,
                         unsigned *ctx_err, long long n_bv,
                         const T *zf_src, T *zf_dst, cudaStream_t s)
{
   if (n_blocks == 0)
      return 0;
   if (sh.kernel == 2) {
      int launches = launch_tile_stage(src, dst, g, stencil, items, recipes,
                                       keep, stale, n_blocks, sh,
                                       write_ghosts, do_cs, acc, err, zf_src,
                                       zf_dst, s);
      if (launches >= 0 && do_cs && sizeof(T) == 8)
         launches += launch_fp64_checksums((const double *) dst, g, items,
                                           n_blocks, partials, sums, s);
      return cudaPeekAtLastError() == cudaSuccess ? launches : -1;
   }
   if (sh.kernel == 1) {
      int launches = launch_brick_stage(src, dst, g, items, n_blocks, sh,
                                        write_ghosts, do_cs, acc, err,
                                        ctx_err, n_bv, zf_src, zf_dst, s);
      if (launches >= 0 && do_cs && sizeof(T) == 8)
         launches += launch_fp64_checksums((const double *) dst, g, items,
                                           n_blocks, partials, sums, s);
      return cudaPeekAtLastError() == cudaSuccess ? launches : -1;
   }
   const size_t smem = tile_bytes<T>(g) * sh.vpc;
   const int thr = sh.threads * sh.vpc;
#define MAMR_GENERIC(ST, BX, BY, BZ)                                          \
   batched_stage_kernel<T, ST, BX, BY, BZ><<<sh.grid, thr, smem, s>>>(         \
      src, dst, g, items, recipes, keep, stale, n_blocks, sh.vpc,             \
      write_ghosts,                                                           \
      sizeof(T) == 4 ? do_cs : 0, acc, err)
   const int kind = dims_kind(g);
   if (stencil == 7) {
      if (kind == 1) MAMR_GENERIC(7, 8, 8, 8);
      else if (kind == 2) MAMR_GENERIC(7, 16, 16, 16);
      else MAMR_GENERIC(7, 0, 0, 0);
   } else {
      if (kind == 1) MAMR_GENERIC(27, 8, 8, 8);
      else if (kind == 2) MAMR_GENERIC(27, 16, 16, 16);
      else MAMR_GENERIC(27, 0, 0, 0);
   }
#undef MAMR_GENERIC
   int launches = 1;
   if (do_cs && sizeof(T) == 8)
      launches += launch_fp64_checksums((const double *) dst, g, items,
                                        n_blocks, partials, sums, s);
   return cudaPeekAtLastError() == cudaSuccess ? launches : -1;
}

// Per-block descriptors of the batched stage kernels from the mesh, one
// thread per block: each face's kind (same level, boundary, coarser with
// the quarter of the coarse face this block covers, finer with its four
// neighbours) and, on single-level meshes, the neighbours across edges and
// corners, reached by hopping along x, then y, then z (a boundary hop
// stays on the block).  A block whose coarser neighbour is inactive or
// does not list it lowers *bad to its index; the descriptor is then left
// with that face as a boundary so that no access leaves the pool.
__global__ void build_items_kernel(const mamr_block *__restrict__ mesh, int n,
                                   const int32_t *__restrict__ slot_pos,
                                   int single, BItem *__restrict__ items,
                                   int *__restrict__ bad)
{
   const int q = blockIdx.x * blockDim.x + threadIdx.x;
   if (q >= n)
      return;
   const mamr_block &bp = mesh[q];
   BItem it;
   it.slot = bp.slot;
   it.bmask = 0;
   for (int l = 0; l < 6; l++) {
      if (!face_desc(mesh, slot_pos, bp, l, it.f[l]))
         atomicMin(bad, q);
      if (bp.nei_level[l] == -2)
         it.bmask |= 1 << l;
   }
   set_jump_bits(it);
   for (int d = 0; d < 27; d++) {
      int cur = bp.slot;
      if (single) {
         const int dd[3] = {d % 3 - 1, (d / 3) % 3 - 1, d / 9 - 1};
         for (int ax = 0; ax < 3 && cur >= 0; ax++) {
            if (!dd[ax])
               continue;
            const mamr_block &cb = mesh[slot_pos[cur]];
            const int l = 2 * ax + (dd[ax] > 0);
            cur = (cb.nei_level[l] == cb.level) ? cb.nei[l][0][0] : -1;
            if (cur >= 0 && slot_pos[cur] < 0)
               cur = -1;
         }
         it.nb27[d] = cur >= 0 ? cur : bp.slot;
      } else {
         it.nb27[d] = 0;
      }
   }
   items[q] = it;
}

// The edge and corner recipes of every block, one thread per (block,
// recipe); a misconnected chain lowers *bad to the block's index and
// leaves a recipe that reads the block's own cell.
__global__ void build_recipes_kernel(const mamr_block *__restrict__ mesh,
                                     int n, const int32_t *__restrict__ slot_pos,
                                     int nx, int ny, int nz,
                                     GhostRecipe *__restrict__ out,
                                     int *__restrict__ keep,
                                     int *__restrict__ bad)
{
   const long long t = blockIdx.x * (long long) blockDim.x + threadIdx.x;
   if (t >= (long long) n * kGhostRecipes)
      return;
   const int q = (int) (t / kGhostRecipes), e = (int) (t % kGhostRecipes);
   GhostRecipe r;
   int kq, kbit;
   if (!resolve_ghost(mesh, slot_pos, q, nx, ny, nz, e, r, kq, kbit)) {
      r.kind = GR_INTERIOR;
      r.vax = -1;
      r.nb[0] = mesh[q].slot;
      r.c[0] = r.c[1] = r.c[2] = 1;
      atomicMin(bad, q);
   } else if (kq >= 0) {
      atomicOr(keep + kq, 1 << kbit);
   }
   out[t] = r;
}

int launch_build_recipes(const mamr_block *mesh, int n,
                         const int32_t *slot_pos, const Geom &g,
                         GhostRecipe *out, int *keep, int *bad,
                         cudaStream_t s)
{
   if (n == 0)
      return 0;
   const long long items = (long long) n * kGhostRecipes;
   if (cudaMemsetAsync(keep, 0, sizeof(int) * (size_t) n, s) != cudaSuccess)
      return -1;
   build_recipes_kernel<<<(unsigned) ((items + 127) / 128), 128, 0, s>>>(
      mesh, n, slot_pos, g.nx, g.ny, g.nz, out, keep, bad);
   return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

int launch_build_items(const mamr_block *mesh, int n, const int32_t *slot_pos,
                       int single, BItem *items, int *bad, cudaStream_t s)
{
   if (n == 0)
      return 0;
   build_items_kernel<<<(n + 127) / 128, 128, 0, s>>>(mesh, n, slot_pos,
                                                      single, items, bad);
   return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

template void batched_candidates<float>(const Geom &, int, int,
                                        std::vector<StageShape> &);
template void batched_candidates<double>(const Geom &, int, int,
                                         std::vector<StageShape> &);
template int launch_batched_stage<float>(const float *, float *, const Geom &,
                                         int, const BItem *,
                                         const GhostRecipe *, const int *,
                                         const float *,
                                         int, const StageShape &, int, int,
                                         double *, double *,
                                         unsigned long long *, unsigned *,
                                         unsigned *, long long,
                                         const float *, float *,
                                         cudaStream_t);
template int launch_batched_stage<double>(const double *, double *,
                                          const Geom &, int, const BItem *,
                                          const GhostRecipe *, const int *,
                                          const double *,
                                          int, const StageShape &, int, int,
                                          double *, double *,
                                          unsigned long long *, unsigned *,
                                          unsigned *, long long,
                                          const double *, double *,
                                          cudaStream_t);

}  // namespace mamr
