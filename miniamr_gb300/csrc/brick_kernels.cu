// Stage kernel for meshes of 8^3 blocks with the 7-point stencil: one or
// two warps per work item -- a block and one or two of its variables -- and
// no CTA-wide barrier, so that every item of an SM streams independently.
// Each item's warps own two sets of tiles in shared memory and fill the
// next item's tiles -- interior rows, and the face ghosts that are copies
// (same-level neighbour, reflection) or single values (coarser neighbour,
// scaled by 1/4 afterwards) -- with cp.async while they compute the current
// item; ghosts from finer neighbours (sums of four cells) are gathered
// after the wait.  With two variables per item the descriptor, the face
// dispatch and the copy addresses serve both variables (their cells are one
// block-variable stride apart), which halves that work per variable.
//
// z-face arrays.  The z ghosts of a block are one value from each of 64
// rows of its neighbour -- a 32-byte sector per value.  So every stage also
// stores each block-variable's k = 1 and k = 8 planes, 64 values each,
// contiguously in a z-face array beside the destination pool, and the next
// stage of the run fetches its z faces from there as 16-byte copies (the
// first stage of a run, whose source has no such array yet, copies them
// value by value).  A tile's z ghosts sit in two planes of 64 values after
// the tile.  The values and the operation
// order are those of the generic stage kernel (batched_kernels.cu): the
// reference's face exchange (ref/comm.c:1465-1965) and 7-point update
// (ref/stencil.c:82-101), with the FP32 fixed-point checksum of every
// result folded in.
#include <algorithm>
#include <vector>

#include "batched.h"
#include "arith.cuh"
#include "cp_async.cuh"
#include "dims.cuh"
#include "tma.cuh"

namespace mamr {

namespace {

template <typename T> struct Vec16;
template <> struct Vec16<float> { using type = float4; };
template <> struct Vec16<double> { using type = double2; };

// Tile of one block-variable: row (i, j), 0 <= i, j <= 9, holds k = 1..8
// (two or four 16-byte vectors); the z ghosts k = 0 and k = 9 sit in two
// planes of 64 values after the rows.  FP32: rows of 8 values (S = 8),
// with the two vectors of a row swapped when j = 4..7, so that the vector
// loads of eight consecutive lanes -- rows j = 1..8, 0..7 or 2..9 of one
// plane -- fall in eight different 16-byte bank groups.  FP64: rows padded
// to S = 10 values, which spreads them the same way.
template <typename T> struct Brick {
   static constexpr int VW = 16 / (int) sizeof(T);   // elements per vector
   static constexpr int R = 8 / VW;                  // vectors per row
   static constexpr bool SWZ = sizeof(T) == 4;
   static constexpr int S = SWZ ? 8 : 10;
   static constexpr int TILE = 100 * S;
   static constexpr int ZST = 128;   // z ghost planes k = 0, 9 after a tile
   static constexpr int SLAB = TILE + ZST;
   static constexpr int DESC = 44;   // ints of a BItem read: slot .. f[5]
   // element k (1 <= k <= 8) of row (i, j)
   __device__ static int at(int i, int j, int k)
   {
      if (SWZ)
         return (i * 10 + j) * 8 +
                ((((k - 1) >> 2) ^ ((j >> 2) & 1)) << 2) + ((k - 1) & 3);
      return (i * 10 + j) * S + k - 1;
   }
   // pool offset of interior cell (i, j, k) (split layout, 1 <= k <= 8)
   __device__ static int gat(int i, int j, int k)
   {
      return (i * 10 + j) * 8 + k - 1;
   }
   // face plane p of direction dir, tangential (a, b)
   __device__ static int face_gat(int dir, int p, int a, int b)
   {
      return dir == 0 ? gat(p, a, b) : (dir == 1 ? gat(a, p, b)
                                                 : gat(a, b, p));
   }
   __device__ static int ghost_at(int dir, int gn, int a, int b)
   {
      return dir == 0 ? at(gn, a, b) : (dir == 1 ? at(a, gn, b)
                                                 : at(a, b, gn));
   }
   static size_t smem_per_item(int vpi)
   {
      return 2 * (vpi * SLAB * sizeof(T) + DESC * sizeof(int));
   }
   // z-face array: planes k = 1 (side 0) and k = 8 (side 1) of a
   // block-variable, 64 values each, at (i-1)*8 + (j-1)
   __device__ static long long zf_at(const Geom &g, int slot, int var,
                                     int side)
   {
      return (((long long) slot * g.V + var) * 2 + side) * 64;
   }
};

template <typename T>
__device__ __forceinline__ void ld4(const T *p, T (&v)[4])
{
   using V = typename Vec16<T>::type;
   if (sizeof(T) == 4) {
      const float4 x = *reinterpret_cast<const float4 *>(p);
      v[0] = x.x; v[1] = x.y; v[2] = x.z; v[3] = x.w;
   } else {
      const V x = *reinterpret_cast<const V *>(p);
      const V y = *reinterpret_cast<const V *>(p + 2);
      v[0] = x.x; v[1] = x.y; v[2] = y.x; v[3] = y.y;
   }
}

template <typename T>
__device__ __forceinline__ void st4(T *p, const T (&v)[4])
{
   if (sizeof(T) == 4) {
      *reinterpret_cast<float4 *>(p) = make_float4(v[0], v[1], v[2], v[3]);
   } else {
      *reinterpret_cast<double2 *>(p) = make_double2(v[0], v[1]);
      *reinterpret_cast<double2 *>(p + 2) = make_double2(v[2], v[3]);
   }
}

// Queues the copies that fill the tiles of item (block sd[0], variables
// var0 .. var0 + nv - 1; tile v at tile + v * SLAB): the interior rows, and
// the face ghosts of same-level, boundary and coarser faces (the coarse
// values unscaled).  sd = the block's BItem, ints 0..DESC-1; sd[1] = its
// bmask, whose bits 8.. and 16.. mark the coarse and fine faces.  The four
// x/y face planes are one pass of 16-byte copies over the item's lanes (a
// lane's chunk decides its face), the two z planes another, so that no
// lane idles through a face it has no chunk of.  Returns whether the tiles
// need brick_fix (a face at a level jump).
template <typename T, int TPI, int VPI>
__device__ __forceinline__ bool brick_issue(const T *__restrict__ src,
                                            const T *__restrict__ zf,
                                            const Geom &g, int var0, int nv,
                                            const int *sd, T *tile, int lane)
{
   using B = Brick<T>;
   constexpr int VW = B::VW, R = B::R;
   const long long bv = g.bv;           // stride of consecutive variables
   const T *own = src + bv_offset(g, sd[0], var0);
   const int bmask = sd[1];
#pragma unroll
   for (int t = 0; t < 64 * R / TPI; t++) {
      const int c = lane + TPI * t, r = c / R, k = 1 + (c % R) * VW;
      const int i = (r >> 3) + 1, j = (r & 7) + 1;
#pragma unroll
      for (int v = 0; v < VPI; v++)
         if (v < nv)
            cp_async16(tile + v * B::SLAB + B::at(i, j, k),
                       own + v * bv + B::gat(i, j, k));
   }
   // x/y faces W, E, S, N: 8 rows of R chunks each
#pragma unroll
   for (int t = 0; t < (32 * R + TPI - 1) / TPI; t++) {
      const int c = lane + TPI * t;
      if (c >= 32 * R)
         break;
      const int l = c / (8 * R), cc = c % (8 * R);
      const int a = cc / R + 1, k = 1 + (cc % R) * VW;
      const int type = sd[2 + 7 * l];
      if (type == FACE_SAME || type == FACE_BC) {
         const bool low = !(l & 1);
         const int gn = low ? 0 : 9;
         // same level: the neighbour's near plane; boundary: reflection
         const int p = (type == FACE_SAME) == low ? 8 : 1;
         const T *sb = type == FACE_SAME ? src + bv_offset(g, sd[3 + 7 * l], var0)
                                         : own;
         const int to = l < 2 ? B::at(gn, a, k) : B::at(a, gn, k);
         const int from = l < 2 ? B::gat(p, a, k) : B::gat(a, p, k);
#pragma unroll
         for (int v = 0; v < VPI; v++)
            if (v < nv)
               cp_async16(tile + v * B::SLAB + to, sb + v * bv + from);
      }
   }
   // z faces D, U: 64 values each, from the z-face arrays as 16-byte copies
   // or, without them, value by value from the pool
   if (zf) {
#pragma unroll
      for (int t = 0; t < (2 * 64 / VW + TPI - 1) / TPI; t++) {
         const int c = lane + TPI * t;
         if (c >= 2 * 64 / VW)
            break;
         const int l = 4 + c / (64 / VW), cc = c % (64 / VW);
         const int type = sd[2 + 7 * l];
         if (type == FACE_SAME || type == FACE_BC) {
            const bool low = l == 4;
            const int p = (type == FACE_SAME) == low ? 8 : 1;
            const int slot = type == FACE_SAME ? sd[3 + 7 * l] : sd[0];
            const T *pl = zf + B::zf_at(g, slot, var0, p == 8) + cc * VW;
            T *to = tile + B::TILE + (low ? 0 : 64) + cc * VW;
#pragma unroll
            for (int v = 0; v < VPI; v++)
               if (v < nv)
                  cp_async16(to + v * B::SLAB, pl + v * 128);
         }
      }
   } else {
#pragma unroll
      for (int t = 0; t < 128 / TPI; t++) {
         const int c = lane + TPI * t, l = 4 + (c >> 6), e = c & 63;
         const int type = sd[2 + 7 * l];
         if (type == FACE_SAME || type == FACE_BC) {
            const bool low = l == 4;
            const int p = (type == FACE_SAME) == low ? 8 : 1;
            const T *sb = type == FACE_SAME
                             ? src + bv_offset(g, sd[3 + 7 * l], var0)
                             : own;
            const int i = (e >> 3) + 1, j = (e & 7) + 1;
#pragma unroll
            for (int v = 0; v < VPI; v++)
               if (v < nv)
                  cp_async_elem(tile + v * B::SLAB + B::TILE + (low ? 0 : 64) +
                                   e,
                                sb + v * bv + B::gat(i, j, p));
         }
      }
   }
   // coarser neighbours: one value per ghost cell (each used by 2 x 2)
   for (unsigned cm = (bmask >> 8) & 63; cm; cm &= cm - 1) {
      const int l = __ffs(cm) - 1;
      const int *f = sd + 2 + 7 * l;
      const int dir = l >> 1;
      const bool low = !(l & 1);
      const int gn = low ? 0 : 9;
      const int zo = B::TILE + (low ? 0 : 64);
      const T *sb = src + bv_offset(g, f[1], var0);
      const int p = low ? 8 : 1, iq = f[5], jq = f[6];
#pragma unroll
      for (int u = 0; u < 64 / TPI; u++) {
         const int e = lane + TPI * u, a = (e >> 3) + 1, b = (e & 7) + 1;
         const int ca = (a + 1) / 2 + 4 * jq, cb = (b + 1) / 2 + 4 * iq;
         const int to = dir < 2 ? B::ghost_at(dir, gn, a, b) : zo + e;
         const T *from =
            dir < 2 ? sb + B::face_gat(dir, p, ca, cb)
                    : (zf ? zf + B::zf_at(g, f[1], var0, p == 8) +
                               (ca - 1) * 8 + (cb - 1)
                          : sb + B::face_gat(dir, p, ca, cb));
         // the variable stride of the source: the pool's, or the z-face
         // array's 128 values per block-variable
         const long long vs = dir == 2 && zf ? 128 : bv;
#pragma unroll
         for (int v = 0; v < VPI; v++)
            if (v < nv)
               cp_async_elem(tile + v * B::SLAB + to, from + v * vs);
      }
   }
   return (bmask & 0x3f3f00) != 0;
}

// After the copies landed: coarse ghosts scaled by 1/4 (each lane the
// elements it copied) and fine ghosts summed from the four finer
// neighbours' cells, in the reference's order.
template <typename T, int TPI, int VPI>
__device__ __forceinline__ void brick_fix(const T *__restrict__ src,
                                          const T *__restrict__ zf,
                                          const Geom &g, int var0, int nv,
                                          const int *sd, T *tile, int lane)
{
   using B = Brick<T>;
   const long long bv = g.bv;
   const int bmask = sd[1];
   for (unsigned cm = (bmask >> 8) & 63; cm; cm &= cm - 1) {
      const int l = __ffs(cm) - 1;
      const int dir = l >> 1, gn = (l & 1) ? 9 : 0;
#pragma unroll
      for (int u = 0; u < 64 / TPI; u++) {
         const int e = lane + TPI * u, a = (e >> 3) + 1, b = (e & 7) + 1;
         const int to = dir < 2 ? B::ghost_at(dir, gn, a, b)
                                : B::TILE + (gn ? 64 : 0) + e;
#pragma unroll
         for (int v = 0; v < VPI; v++)
            if (v < nv) {
               T &x = tile[v * B::SLAB + to];
               x = quarter(x);
            }
      }
   }
   for (unsigned fm = (bmask >> 16) & 63; fm; fm &= fm - 1) {
      const int l = __ffs(fm) - 1;
      const int *f = sd + 2 + 7 * l;
      const int dir = l >> 1;
      const bool low = !(l & 1);
      const int gn = low ? 0 : 9, p = low ? 8 : 1;
#pragma unroll
      for (int u = 0; u < 64 / TPI; u++) {
         const int e = lane + TPI * u, a = (e >> 3) + 1, b = (e & 7) + 1;
         const int to = dir < 2 ? B::ghost_at(dir, gn, a, b)
                                : B::TILE + (low ? 0 : 64) + e;
         const int jq = a > 4, iq = b > 4;
         const int a2 = a - 4 * jq, b2 = b - 4 * iq;
         const int nbs = f[1 + iq * 2 + jq];
         // the four fine cells: from the fine block's z-face array (plane
         // p, 128 values per block-variable) or its pool cells
         const T *q0;
         int o[4];
         long long vs;
         if (dir == 2 && zf) {
            q0 = zf + B::zf_at(g, nbs, var0, p == 8);
            o[0] = (2 * a2 - 2) * 8 + 2 * b2 - 2;
            o[1] = o[0] + 1;
            o[2] = o[0] + 8;
            o[3] = o[0] + 9;
            vs = 128;
         } else {
            q0 = src + bv_offset(g, nbs, var0);
            o[0] = B::face_gat(dir, p, 2 * a2 - 1, 2 * b2 - 1);
            o[1] = B::face_gat(dir, p, 2 * a2 - 1, 2 * b2);
            o[2] = B::face_gat(dir, p, 2 * a2, 2 * b2 - 1);
            o[3] = B::face_gat(dir, p, 2 * a2, 2 * b2);
            vs = bv;
         }
         T w[VPI][4];
#pragma unroll
         for (int v = 0; v < VPI; v++)
            if (v < nv) {
#pragma unroll
               for (int m = 0; m < 4; m++)
                  w[v][m] = q0[v * vs + o[m]];
            }
#pragma unroll
         for (int v = 0; v < VPI; v++)
            if (v < nv) {
               T t = w[v][0] + w[v][1];
               t = t + w[v][2];
               t = t + w[v][3];
               tile[v * B::SLAB + to] = t;
            }
      }
   }
}

// TPI threads (one or two warps) per work item of VPI variables, at most
// 4 items per CTA.  Registers for the CTAs whose tiles fill the shared
// memory: one variable -- 5 CTAs of 4 one-warp items (FP32) or 3 (FP64), 4
// CTAs of 4 two-warp items; two variables -- 3 CTAs.
template <int TPI, int FP32, int VPI> struct BrickBounds {
   static constexpr int THREADS = 4 * TPI;
   static constexpr int CTAS =
      VPI == 2 ? 3 : (TPI == 64 ? 4 : (FP32 ? 5 : 3));
};

// Barrier of the TPI threads that share an item: the warp itself, or a
// named barrier (id 1 + group, at most 4 groups a CTA) over the group's two
// warps.  The ids are immediates: with an id in a register the compiler
// reserves all 16 barriers for the kernel, which caps an SM at 4 of its
// CTAs.
template <int TPI> __device__ __forceinline__ void group_sync(int group)
{
   if (TPI == 32) {
      __syncwarp();
      return;
   }
   switch (group) {
   case 0:
      asm volatile("bar.sync 1, %0;\n" ::"n"(TPI) : "memory");
      break;
   case 1:
      asm volatile("bar.sync 2, %0;\n" ::"n"(TPI) : "memory");
      break;
   case 2:
      asm volatile("bar.sync 3, %0;\n" ::"n"(TPI) : "memory");
      break;
   default:
      asm volatile("bar.sync 4, %0;\n" ::"n"(TPI) : "memory");
      break;
   }
}

template <typename T, int TPI, int VPI>
__global__ void __launch_bounds__(BrickBounds<TPI, sizeof(T) == 4, VPI>::THREADS,
                                  BrickBounds<TPI, sizeof(T) == 4, VPI>::CTAS)
brick_stage_kernel(const T *__restrict__ src, T *__restrict__ dst, Geom g,
                   const BItem *__restrict__ items, int nb, int write_ghosts,
                   int do_cs, unsigned long long *__restrict__ acc,
                   unsigned *__restrict__ err, const T *__restrict__ zf_src,
                   T *__restrict__ zf_dst)
{
   using B = Brick<T>;
   constexpr int DESC = B::DESC;
   constexpr int ND = (DESC + TPI - 1) / TPI;     // descriptor ints a thread
   constexpr int RPT = 64 / TPI;                   // rows of 8 cells a thread
   constexpr int SET = VPI * B::SLAB;              // one item's tiles
   extern __shared__ __align__(16) unsigned char smem_raw[];
   const int lane = threadIdx.x % TPI, group = threadIdx.x / TPI;
   const int gpc = blockDim.x / TPI;
   T *tiles = reinterpret_cast<T *>(smem_raw) + (size_t) group * 2 * SET;
   int *sdesc = reinterpret_cast<int *>(reinterpret_cast<T *>(smem_raw) +
                                        (size_t) gpc * 2 * SET) +
                group * 2 * DESC;
   // work items (block b, variables VPI*pv ..), variable-major; group w
   // takes items w, w + nw, w + 2 nw, ... tracked as (pv, b) without
   // divisions
   const int npv = (g.V + VPI - 1) / VPI;
   const int nw = gridDim.x * gpc;
   const int it0 = blockIdx.x * gpc + group;
   struct Pos {
      int pv, b;
   };
   Pos cur{it0 / nb, it0 % nb};
   if (cur.pv >= npv)
      return;
   const int step_v = nw / nb, step_b = nw - step_v * nb;
   auto advance = [&](Pos q) {
      q.pv += step_v;
      q.b += step_b;
      if (q.b >= nb) {
         q.b -= nb;
         q.pv++;
      }
      return q;
   };
   auto nvars = [&](int pv) { return min(VPI, g.V - pv * VPI); };
   const Dims<8, 8, 8> D(g);
   // this thread's output rows (i0 + m, j), m < RPT
   const int j = (lane & 7) + 1, i0 = RPT * (lane >> 3) + 1;

   int dr[ND];
   auto load_desc = [&](const Pos &q) {
      const int *p = reinterpret_cast<const int *>(items + q.b);
#pragma unroll
      for (int u = 0; u < ND; u++)
         dr[u] = lane + TPI * u < DESC ? __ldg(p + lane + TPI * u) : 0;
   };
   auto put_desc = [&](int *sd) {
#pragma unroll
      for (int u = 0; u < ND; u++)
         if (lane + TPI * u < DESC)
            sd[lane + TPI * u] = dr[u];
      group_sync<TPI>(group);
   };

   load_desc(cur);
   put_desc(sdesc);
   bool fix_cur = brick_issue<T, TPI, VPI>(src, zf_src, g, cur.pv * VPI,
                                           nvars(cur.pv), sdesc, tiles, lane);
   cp_async_commit();
   Pos nxt = advance(cur);
   if (nxt.pv < npv)
      load_desc(nxt);

   unsigned long long lo[VPI], hi[VPI];
#pragma unroll
   for (int v = 0; v < VPI; v++)
      lo[v] = hi[v] = 0;
   Fixed52 part;
   int cs_pv = -1;
   for (int n = 0;; n++) {
      const int cb = n & 1;
      T *tile = tiles + cb * SET;
      const int *sd = sdesc + cb * DESC;
      // the next item: descriptor into shared memory, copies in flight
      bool fix_next = false;
      if (nxt.pv < npv) {
         int *sdn = sdesc + (cb ^ 1) * DESC;
         put_desc(sdn);
         fix_next = brick_issue<T, TPI, VPI>(src, zf_src, g, nxt.pv * VPI,
                                             nvars(nxt.pv), sdn,
                                             tiles + (cb ^ 1) * SET, lane);
         const Pos nn = advance(nxt);
         if (nn.pv < npv)
            load_desc(nn);
      }
      cp_async_commit();
      cp_async_wait_group<1>();
      const int var0 = cur.pv * VPI, nv = nvars(cur.pv);
      if (fix_cur)
         brick_fix<T, TPI, VPI>(src, zf_src, g, var0, nv, sd, tile, lane);
      group_sync<TPI>(group);
      if (sizeof(T) == 4 && do_cs && cur.pv != cs_pv) {
         if (cs_pv >= 0) {
#pragma unroll
            for (int v = 0; v < VPI; v++) {
               if (v < nvars(cs_pv))
                  warp_acc128_flush(lo[v], hi[v], acc + 2 * (cs_pv * VPI + v));
               lo[v] = hi[v] = 0;
            }
         }
         cs_pv = cur.pv;
      }
#pragma unroll
      for (int v = 0; v < VPI; v++) {
         if (v >= nv)
            break;
         const T *tv = tile + v * B::SLAB;
         const T *zst = tv + B::TILE;
         T *d = dst + bv_offset(g, sd[0], var0 + v);
         if (write_ghosts) {
#pragma unroll
            for (int l = 0; l < 6; l++) {
               const int dir = l >> 1, gn = (l & 1) ? 9 : 0;
#pragma unroll
               for (int u = 0; u < 64 / TPI; u++) {
                  const int e = lane + TPI * u, a = (e >> 3) + 1,
                            b = (e & 7) + 1;
                  int gi, gj, gk;
                  if (dir == 0) { gi = gn; gj = a; gk = b; }
                  else if (dir == 1) { gi = a; gj = gn; gk = b; }
                  else { gi = a; gj = b; gk = gn; }
                  d[D.cell(gi, gj, gk)] = dir < 2 ? tv[B::at(gi, gj, gk)]
                                                  : zst[(gn ? 64 : 0) + e];
               }
            }
         }
         // 7-point update of the thread's rows, four k at a time
#pragma unroll
         for (int m = 0; m < RPT; m++) {
            const int i = i0 + m;
#pragma unroll
            for (int h = 0; h < 2; h++) {
               const int k0 = 1 + 4 * h;
               T a[4], jm[4], c[4], jp[4], bq[4];
               ld4(tv + B::at(i - 1, j, k0), a);
               ld4(tv + B::at(i, j - 1, k0), jm);
               ld4(tv + B::at(i, j, k0), c);
               ld4(tv + B::at(i, j + 1, k0), jp);
               ld4(tv + B::at(i + 1, j, k0), bq);
               // k = 0 and k = 9 from the tile's z ghost planes
               const int zi = (i - 1) * 8 + (j - 1);
               const T cm = h == 0 ? zst[zi] : tv[B::at(i, j, k0 - 1)];
               const T cp = h == 1 ? zst[64 + zi] : tv[B::at(i, j, k0 + 4)];
               T w[4], q[4];
#pragma unroll
               for (int t = 0; t < 4; t++) {
                  const T km = t == 0 ? cm : c[t - 1];
                  const T kp = t == 3 ? cp : c[t + 1];
                  T s = a[t] + jm[t];
                  s = s + km;
                  s = s + c[t];
                  s = s + kp;
                  s = s + jp[t];
                  s = s + bq[t];
                  w[t] = s;
               }
               div_const4<7>(w, q);
               st4(d + B::gat(i, j, k0), q);
               if (zf_dst) {
                  // this block's k = 1 / k = 8 plane for the next stage
                  T *zp = zf_dst + B::zf_at(g, sd[0], var0 + v, h);
                  zp[zi] = h == 0 ? q[0] : q[3];
               }
               if (sizeof(T) == 4 && do_cs) {
#pragma unroll
                  for (int t = 0; t < 4; t++)
                     fixed52_add((float) q[t], part);
               }
            }
         }
         if (sizeof(T) == 4 && do_cs)
            fixed52_flush(part, lo[v], hi[v]);
      }
      group_sync<TPI>(group);
      cur = nxt;
      fix_cur = fix_next;
      if (cur.pv >= npv)
         break;
      nxt = advance(nxt);
   }
   if (sizeof(T) == 4 && do_cs) {
      if (cs_pv >= 0) {
#pragma unroll
         for (int v = 0; v < VPI; v++)
            if (v < nvars(cs_pv))
               warp_acc128_flush(lo[v], hi[v], acc + 2 * (cs_pv * VPI + v));
      }
      if (!fixed52_window(part))
         atomicOr(err, ERR_FIXED_RANGE);
   }
}

// ---- the tensor-copy form (FP32) -----------------------------------------
//
// The same work items, ghosts, update, checksum and z-face arrays as the
// kernel above; what differs is how an item's tiles fill.  One lane of the
// item issues, per variable, a tensor copy of the 8 x 8 interior rows (a
// box of the pool seen as the 4-d tensor k: 8, j: 10, i: 10,
// block-variable), a tensor copy of each x or y face plane that is a plain
// copy (a same-level neighbour's near plane, or at the domain boundary the
// block's own) and a bulk copy of each such z plane from the z-face
// arrays, all completing on the item buffer's mbarrier; the lanes only
// gather the level-jump ghosts (and, in a run's first stage, the z planes
// value by value) themselves.  A variable's tiles are its 64 interior rows
// (row (i-1)*8 + j-1, 32 bytes each) and six ghost planes of 64 values:
// x and y planes as 8 rows of 32 bytes (rows j-1 and i-1 of k), z planes
// as (i-1)*8 + j-1.  The tensor copies write the rows with the 32-byte
// swizzle -- the two 16-byte halves of a row swap when bit 7 of its
// shared address is set -- so that the vector loads of eight consecutive
// rows fall on distinct banks; the lanes' own writes into x/y planes use
// the same placement.  Each thread's five neighbour rows (interior or
// ghost plane) are offsets computed once.
struct BrickT {
   static constexpr int INT = 512;             // interior floats, 1 variable
   static constexpr int GP = 64;               // floats of a ghost plane
   static constexpr int VAR = INT + 6 * GP;    // floats of a variable's tiles
   static constexpr int DESC = 44;             // ints of a BItem read
   // element e (0..7) of 32-byte row r of a swizzled region (regions start
   // on 256-byte boundaries, so bit 7 of the address is bit 2 of r)
   __host__ __device__ static constexpr int sw(int r, int e)
   {
      return r * 8 + ((((e >> 2) ^ (r >> 2)) & 1) << 2) + (e & 3);
   }
   // ghost plane l, element (a, b) (1-based; x: (j, k), y: (i, k),
   // z: (i, j))
   __device__ static int gh(int l, int a, int b)
   {
      return INT + l * GP + (l < 4 ? sw(a - 1, b - 1) : (a - 1) * 8 + b - 1);
   }
   // shared memory of gpc items: two buffers of VPI variables' tiles, two
   // descriptors and two mbarriers each, and 256 bytes of alignment slack
   static size_t smem_bytes(int gpc, int vpi)
   {
      return (size_t) gpc * (2 * (size_t) vpi * VAR * 4 + 2 * DESC * 4 + 16) +
             256;
   }
};

// Reduction barrier of an item's threads: whether pred holds in any.
template <int TPI>
__device__ __forceinline__ bool group_any(int group, bool pred)
{
   if (TPI == 32) {
      __syncwarp();
      return __any_sync(0xffffffffu, pred);
   }
   unsigned r = 0;
   const unsigned q = pred ? 1u : 0u;
#define MAMR_BAR_ANY(ID)                                                      \
   asm volatile("{\n\t.reg .pred p, q;\n\tsetp.ne.u32 q, %1, 0;\n\t"         \
                "bar.red.or.pred p, " #ID ", %2, q;\n\t"                      \
                "selp.u32 %0, 1, 0, p;\n\t}"                                  \
                : "=r"(r)                                                     \
                : "r"(q), "n"(TPI)                                            \
                : "memory")
   switch (group) {
   case 0: MAMR_BAR_ANY(1); break;
   case 1: MAMR_BAR_ANY(2); break;
   case 2: MAMR_BAR_ANY(3); break;
   default: MAMR_BAR_ANY(4); break;
   }
#undef MAMR_BAR_ANY
   return r != 0;
}

// Queues the fill of item (block sd[0], variables var0 .. var0 + nv - 1;
// variable v's tiles at tile + v * VAR) on the mbarrier bar: lane 0 posts
// the bytes and issues the tensor and bulk copies; every lane copies its
// share of the coarse faces (unscaled) and, without z-face arrays, of the
// z planes.  Returns whether the tiles need brick_tma_fix.
template <int TPI, int VPI>
__device__ __forceinline__ bool brick_tma_issue(
   const CUtensorMap *tm_int, const CUtensorMap *tm_x, const CUtensorMap *tm_y,
   const float *__restrict__ src, const float *__restrict__ zf, const Geom &g,
   int var0, int nv, const int *sd, float *tile, unsigned bar, int lane)
{
   using B = BrickT;
   const int slot = sd[0], bmask = sd[1];
   if (lane == 0) {
      unsigned per_var = 4u * B::INT;
#pragma unroll
      for (int l = 0; l < 6; l++) {
         const int type = sd[2 + 7 * l];
         if ((type == FACE_SAME || type == FACE_BC) && (l < 4 || zf))
            per_var += 4u * B::GP;
      }
      mbar_expect_tx(bar, per_var * (unsigned) nv);
      for (int v = 0; v < nv; v++) {
         float *tv = tile + v * B::VAR;
         tma_load_4d(tv, tm_int, 0, 1, 1, slot * g.V + var0 + v, bar);
#pragma unroll
         for (int l = 0; l < 6; l++) {
            const int type = sd[2 + 7 * l];
            if (type != FACE_SAME && type != FACE_BC)
               continue;
            const bool low = !(l & 1);
            // same level: the neighbour's near plane; boundary: reflection
            const int p = (type == FACE_SAME) == low ? 8 : 1;
            const int ns = type == FACE_SAME ? sd[3 + 7 * l] : slot;
            float *to = tv + B::INT + l * B::GP;
            if (l < 2)
               tma_load_4d(to, tm_x, 0, 1, p, ns * g.V + var0 + v, bar);
            else if (l < 4)
               tma_load_4d(to, tm_y, 0, p, 1, ns * g.V + var0 + v, bar);
            else if (zf)
               bulk_load(to, zf + Brick<float>::zf_at(g, ns, var0 + v, p == 8),
                         4u * B::GP, bar);
         }
      }
   }
   if (!zf) {
#pragma unroll
      for (int t = 0; t < 128 / TPI; t++) {
         const int c = lane + TPI * t, l = 4 + (c >> 6), e = c & 63;
         const int type = sd[2 + 7 * l];
         if (type == FACE_SAME || type == FACE_BC) {
            const bool low = l == 4;
            const int p = (type == FACE_SAME) == low ? 8 : 1;
            const float *sb = type == FACE_SAME
                                 ? src + bv_offset(g, sd[3 + 7 * l], var0)
                                 : src + bv_offset(g, slot, var0);
            const int i = (e >> 3) + 1, j = (e & 7) + 1;
#pragma unroll
            for (int v = 0; v < VPI; v++)
               if (v < nv)
                  cp_async_elem(tile + v * B::VAR + B::INT + l * B::GP + e,
                                sb + v * g.bv + Brick<float>::gat(i, j, p));
         }
      }
   }
   // coarser neighbours: one value per ghost cell (each used by 2 x 2)
   for (unsigned cm = (bmask >> 8) & 63; cm; cm &= cm - 1) {
      const int l = __ffs(cm) - 1;
      const int *f = sd + 2 + 7 * l;
      const int dir = l >> 1;
      const bool low = !(l & 1);
      const float *sb = src + bv_offset(g, f[1], var0);
      const int p = low ? 8 : 1, iq = f[5], jq = f[6];
#pragma unroll
      for (int u = 0; u < 64 / TPI; u++) {
         const int e = lane + TPI * u, a = (e >> 3) + 1, b = (e & 7) + 1;
         const int ca = (a + 1) / 2 + 4 * jq, cb = (b + 1) / 2 + 4 * iq;
         const float *from =
            dir < 2 ? sb + Brick<float>::face_gat(dir, p, ca, cb)
                    : (zf ? zf + Brick<float>::zf_at(g, f[1], var0, p == 8) +
                               (ca - 1) * 8 + (cb - 1)
                          : sb + Brick<float>::face_gat(dir, p, ca, cb));
         const long long vs = dir == 2 && zf ? 128 : g.bv;
#pragma unroll
         for (int v = 0; v < VPI; v++)
            if (v < nv)
               cp_async_elem(tile + v * B::VAR + B::gh(l, a, b), from + v * vs);
      }
   }
   return (bmask & 0x3f3f00) != 0;
}

// After the copies landed: coarse ghosts scaled by 1/4 and fine ghosts
// summed from the four finer neighbours' cells, in the reference's order
// (as brick_fix).
template <int TPI, int VPI>
__device__ __forceinline__ void brick_tma_fix(const float *__restrict__ src,
                                              const float *__restrict__ zf,
                                              const Geom &g, int var0, int nv,
                                              const int *sd, float *tile,
                                              int lane)
{
   using B = BrickT;
   const int bmask = sd[1];
   for (unsigned cm = (bmask >> 8) & 63; cm; cm &= cm - 1) {
      const int l = __ffs(cm) - 1;
#pragma unroll
      for (int u = 0; u < 64 / TPI; u++) {
         const int e = lane + TPI * u, a = (e >> 3) + 1, b = (e & 7) + 1;
         const int to = B::gh(l, a, b);
#pragma unroll
         for (int v = 0; v < VPI; v++)
            if (v < nv) {
               float &x = tile[v * B::VAR + to];
               x = quarter(x);
            }
      }
   }
   for (unsigned fm = (bmask >> 16) & 63; fm; fm &= fm - 1) {
      const int l = __ffs(fm) - 1;
      const int *f = sd + 2 + 7 * l;
      const int dir = l >> 1;
      const bool low = !(l & 1);
      const int p = low ? 8 : 1;
#pragma unroll
      for (int u = 0; u < 64 / TPI; u++) {
         const int e = lane + TPI * u, a = (e >> 3) + 1, b = (e & 7) + 1;
         const int to = B::gh(l, a, b);
         const int jq = a > 4, iq = b > 4;
         const int a2 = a - 4 * jq, b2 = b - 4 * iq;
         const int nbs = f[1 + iq * 2 + jq];
         const float *q0;
         int o[4];
         long long vs;
         if (dir == 2 && zf) {
            q0 = zf + Brick<float>::zf_at(g, nbs, var0, p == 8);
            o[0] = (2 * a2 - 2) * 8 + 2 * b2 - 2;
            o[1] = o[0] + 1;
            o[2] = o[0] + 8;
            o[3] = o[0] + 9;
            vs = 128;
         } else {
            q0 = src + bv_offset(g, nbs, var0);
            o[0] = Brick<float>::face_gat(dir, p, 2 * a2 - 1, 2 * b2 - 1);
            o[1] = Brick<float>::face_gat(dir, p, 2 * a2 - 1, 2 * b2);
            o[2] = Brick<float>::face_gat(dir, p, 2 * a2, 2 * b2 - 1);
            o[3] = Brick<float>::face_gat(dir, p, 2 * a2, 2 * b2);
            vs = g.bv;
         }
         float w[VPI][4];
#pragma unroll
         for (int v = 0; v < VPI; v++)
            if (v < nv) {
#pragma unroll
               for (int m = 0; m < 4; m++)
                  w[v][m] = q0[v * vs + o[m]];
            }
#pragma unroll
         for (int v = 0; v < VPI; v++)
            if (v < nv) {
               float t = w[v][0] + w[v][1];
               t = t + w[v][2];
               t = t + w[v][3];
               tile[v * B::VAR + to] = t;
            }
      }
   }
}

// CTAs of 128 threads (4 one-warp or 2 two-warp items), 7 per SM: the
// shared memory holds 7 and registers are capped to match.
template <int TPI, int VPI>
__global__ void __launch_bounds__(128, 7)
brick_tma_kernel(const __grid_constant__ CUtensorMap tm_int,
                 const __grid_constant__ CUtensorMap tm_x,
                 const __grid_constant__ CUtensorMap tm_y,
                 const float *__restrict__ src, float *__restrict__ dst,
                 Geom g, const BItem *__restrict__ items, int nb,
                 int write_ghosts, int do_cs,
                 unsigned long long *__restrict__ acc,
                 unsigned *__restrict__ err, unsigned *__restrict__ ctx_err,
                 const float *__restrict__ zf_src, float *__restrict__ zf_dst)
{
   using B = BrickT;
   constexpr int DESC = B::DESC;
   constexpr int ND = (DESC + TPI - 1) / TPI;     // descriptor ints a thread
   constexpr int RPT = 64 / TPI;                   // rows of 8 cells a thread
   constexpr int SET = VPI * B::VAR;               // one item buffer
   extern __shared__ __align__(16) unsigned char smem_raw[];
   float *base = reinterpret_cast<float *>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 255) & ~(uintptr_t) 255);
   const int lane = threadIdx.x % TPI, group = threadIdx.x / TPI;
   const int gpc = blockDim.x / TPI;
   float *tiles = base + (size_t) group * 2 * SET;
   int *sdesc_all = reinterpret_cast<int *>(base + (size_t) gpc * 2 * SET);
   int *sdesc = sdesc_all + group * 2 * DESC;
   unsigned long long *bars =
      reinterpret_cast<unsigned long long *>(sdesc_all + gpc * 2 * DESC) +
      group * 2;
   const unsigned bar0 = smem_addr(bars);
   const int npv = (g.V + VPI - 1) / VPI;
   const int nw = gridDim.x * gpc;
   const int it0 = blockIdx.x * gpc + group;
   struct Pos {
      int pv, b;
   };
   Pos cur{it0 / nb, it0 % nb};
   if (cur.pv >= npv)
      return;
   if (lane == 0) {
      mbar_init(bar0);
      mbar_init(bar0 + 8);
      mbar_init_fence();
   }
   const int step_v = nw / nb, step_b = nw - step_v * nb;
   auto advance = [&](Pos q) {
      q.pv += step_v;
      q.b += step_b;
      if (q.b >= nb) {
         q.b -= nb;
         q.pv++;
      }
      return q;
   };
   auto nvars = [&](int pv) { return min(VPI, g.V - pv * VPI); };
   const Dims<8, 8, 8> D(g);
   // this thread's rows (i0 + m, j), m < RPT: its own row and the four
   // neighbour rows (interior or ghost plane), first halves; the second
   // halves are these ^ 4
   const int j = (lane & 7) + 1, i0 = RPT * (lane >> 3) + 1;
   int oc[RPT], oim[RPT], oip[RPT], ojm[RPT], ojp[RPT];
#pragma unroll
   for (int m = 0; m < RPT; m++) {
      const int i = i0 + m, r = (i - 1) * 8 + (j - 1);
      oc[m] = B::sw(r, 0);
      oim[m] = i == 1 ? B::INT + 0 * B::GP + B::sw(j - 1, 0) : B::sw(r - 8, 0);
      oip[m] = i == 8 ? B::INT + 1 * B::GP + B::sw(j - 1, 0) : B::sw(r + 8, 0);
      ojm[m] = j == 1 ? B::INT + 2 * B::GP + B::sw(i - 1, 0) : B::sw(r - 1, 0);
      ojp[m] = j == 8 ? B::INT + 3 * B::GP + B::sw(i - 1, 0) : B::sw(r + 1, 0);
   }

   int dr[ND];
   auto load_desc = [&](const Pos &q) {
      const int *p = reinterpret_cast<const int *>(items + q.b);
#pragma unroll
      for (int u = 0; u < ND; u++)
         dr[u] = lane + TPI * u < DESC ? __ldg(p + lane + TPI * u) : 0;
   };
   auto put_desc = [&](int *sd) {
#pragma unroll
      for (int u = 0; u < ND; u++)
         if (lane + TPI * u < DESC)
            sd[lane + TPI * u] = dr[u];
      group_sync<TPI>(group);
   };

   load_desc(cur);
   put_desc(sdesc);        // also orders the mbarrier initialisation
   bool fix_cur = brick_tma_issue<TPI, VPI>(
      &tm_int, &tm_x, &tm_y, src, zf_src, g, cur.pv * VPI, nvars(cur.pv),
      sdesc, tiles, bar0, lane);
   cp_async_commit();
   Pos nxt = advance(cur);
   if (nxt.pv < npv)
      load_desc(nxt);

   unsigned long long lo[VPI], hi[VPI];
#pragma unroll
   for (int v = 0; v < VPI; v++)
      lo[v] = hi[v] = 0;
   Fixed52 part;
   int cs_pv = -1;
   unsigned phase = 0;       // bit b: the parity buffer b waits for next
   bool next_issued = false, timed_out = false;
   int brk = 0;              // the buffer whose wait ran out
   for (int n = 0;; n++) {
      const int cb = n & 1;
      float *tile = tiles + cb * SET;
      const int *sd = sdesc + cb * DESC;
      bool fix_next = false;
      next_issued = false;
      if (nxt.pv < npv) {
         int *sdn = sdesc + (cb ^ 1) * DESC;
         put_desc(sdn);
         fix_next = brick_tma_issue<TPI, VPI>(
            &tm_int, &tm_x, &tm_y, src, zf_src, g, nxt.pv * VPI,
            nvars(nxt.pv), sdn, tiles + (cb ^ 1) * SET, bar0 + 8 * (cb ^ 1),
            lane);
         next_issued = true;
         const Pos nn = advance(nxt);
         if (nn.pv < npv)
            load_desc(nn);
      }
      cp_async_commit();
      cp_async_wait_group<1>();
      const bool ok = mbar_wait(bar0 + 8 * cb, (phase >> cb) & 1);
      phase ^= 1u << cb;
      const int var0 = cur.pv * VPI, nv = nvars(cur.pv);
      if (ok && fix_cur)
         brick_tma_fix<TPI, VPI>(src, zf_src, g, var0, nv, sd, tile, lane);
      if (group_any<TPI>(group, !ok)) {
         timed_out = true;
         brk = cb;
         break;
      }
      if (do_cs && cur.pv != cs_pv) {
         if (cs_pv >= 0) {
#pragma unroll
            for (int v = 0; v < VPI; v++) {
               if (v < nvars(cs_pv))
                  warp_acc128_flush(lo[v], hi[v], acc + 2 * (cs_pv * VPI + v));
               lo[v] = hi[v] = 0;
            }
         }
         cs_pv = cur.pv;
      }
#pragma unroll
      for (int v = 0; v < VPI; v++) {
         if (v >= nv)
            break;
         const float *tv = tile + v * B::VAR;
         float *d = dst + bv_offset(g, sd[0], var0 + v);
         if (write_ghosts) {
#pragma unroll
            for (int l = 0; l < 6; l++) {
               const int dir = l >> 1, gn = (l & 1) ? 9 : 0;
#pragma unroll
               for (int u = 0; u < 64 / TPI; u++) {
                  const int e = lane + TPI * u, a = (e >> 3) + 1,
                            b = (e & 7) + 1;
                  int gi, gj, gk;
                  if (dir == 0) { gi = gn; gj = a; gk = b; }
                  else if (dir == 1) { gi = a; gj = gn; gk = b; }
                  else { gi = a; gj = b; gk = gn; }
                  d[D.cell(gi, gj, gk)] = tv[B::gh(l, a, b)];
               }
            }
         }
         // 7-point update of the thread's rows, four k at a time
#pragma unroll
         for (int m = 0; m < RPT; m++) {
            const int i = i0 + m, zi = (i - 1) * 8 + (j - 1);
            float c0[4], c1[4];
            ld4(tv + oc[m], c0);
            ld4(tv + (oc[m] ^ 4), c1);
#pragma unroll
            for (int h = 0; h < 2; h++) {
               const int k0 = 1 + 4 * h, x = h << 2;
               float a[4], jm[4], jp[4], bq[4];
               ld4(tv + (oim[m] ^ x), a);
               ld4(tv + (ojm[m] ^ x), jm);
               ld4(tv + (ojp[m] ^ x), jp);
               ld4(tv + (oip[m] ^ x), bq);
               const float *c = h == 0 ? c0 : c1;
               // k = 0 and k = 9 from the z ghost planes
               const float cm = h == 0 ? tv[B::INT + 4 * B::GP + zi] : c0[3];
               const float cp = h == 1 ? tv[B::INT + 5 * B::GP + zi] : c1[0];
               float w[4], q[4];
#pragma unroll
               for (int t = 0; t < 4; t++) {
                  const float km = t == 0 ? cm : c[t - 1];
                  const float kp = t == 3 ? cp : c[t + 1];
                  float s = a[t] + jm[t];
                  s = s + km;
                  s = s + c[t];
                  s = s + kp;
                  s = s + jp[t];
                  s = s + bq[t];
                  w[t] = s;
               }
               div_const4<7>(w, q);
               st4(d + Brick<float>::gat(i, j, k0), q);
               if (zf_dst) {
                  // this block's k = 1 / k = 8 plane for the next stage
                  float *zp = zf_dst + Brick<float>::zf_at(g, sd[0], var0 + v, h);
                  zp[zi] = h == 0 ? q[0] : q[3];
               }
               if (do_cs) {
#pragma unroll
                  for (int t = 0; t < 4; t++)
                     fixed52_add(q[t], part);
               }
            }
         }
         if (do_cs)
            fixed52_flush(part, lo[v], hi[v]);
      }
      // the buffer's next fill is a tensor copy: order this item's
      // shared-memory accesses before it
      fence_proxy_async_smem();
      group_sync<TPI>(group);
      cur = nxt;
      fix_cur = fix_next;
      if (cur.pv >= npv)
         break;
      nxt = advance(nxt);
   }
   if (timed_out) {
      // let the copies still in flight into this group's buffers land (or
      // run out of time again) before the CTA's shared memory goes
      cp_async_wait_all();
      mbar_wait(bar0 + 8 * brk, ((phase >> brk) & 1) ^ 1);
      if (next_issued)
         mbar_wait(bar0 + 8 * (brk ^ 1), (phase >> (brk ^ 1)) & 1);
      if (lane == 0)
         atomicOr(ctx_err, ERR_WAIT);
   }
   if (do_cs) {
      if (cs_pv >= 0) {
#pragma unroll
         for (int v = 0; v < VPI; v++)
            if (v < nvars(cs_pv))
               warp_acc128_flush(lo[v], hi[v], acc + 2 * (cs_pv * VPI + v));
      }
      if (!fixed52_window(part))
         atomicOr(err, ERR_FIXED_RANGE);
   }
}

}  // namespace

// CTAs per SM with gpc items of TPI threads and VPI variables each; the
// kernel's dynamic shared memory limit is raised once to what 4 items need.
template <typename T, int TPI, int VPI>
static int brick_per_sm(int gpc)
{
   int per_sm = 0;
   cudaFuncSetAttribute(brick_stage_kernel<T, TPI, VPI>,
                        cudaFuncAttributeMaxDynamicSharedMemorySize,
                        (int) (Brick<T>::smem_per_item(VPI) * 4));
   cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      &per_sm, brick_stage_kernel<T, TPI, VPI>, TPI * gpc,
      Brick<T>::smem_per_item(VPI) * gpc);
   return per_sm;
}

// CTAs per SM of the tensor-copy form with gpc items.
template <int TPI, int VPI>
static int brick_tma_per_sm(int gpc)
{
   int per_sm = 0;
   cudaFuncSetAttribute(brick_tma_kernel<TPI, VPI>,
                        cudaFuncAttributeMaxDynamicSharedMemorySize,
                        (int) BrickT::smem_bytes(4, VPI));
   cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      &per_sm, brick_tma_kernel<TPI, VPI>, TPI * gpc,
      BrickT::smem_bytes(gpc, VPI));
   return per_sm;
}

// The tensor maps of the tensor-copy form over an FP32 pool of 8^3 blocks
// in the split layout, seen as the 4-d tensor (k: 8, j: 10, i: 10,
// block-variable: n_bv): boxes of a block-variable's 8 x 8 interior rows,
// of one i-plane's 8 interior rows and of one j-row over the 8 interior i;
// 32-byte swizzle.
static bool brick_tensor_maps(const float *pool, const Geom &g,
                              long long n_bv, CUtensorMap tm[3])
{
   EncodeTiledFn enc = encode_tiled();
   if (!enc || g.kplane < 0 || g.nz != 8 || g.Y != 10 || g.X != 10 ||
       n_bv < 1 || n_bv > (1ll << 31))
      return false;
   const cuuint64_t dims[4] = {8, 10, 10, (cuuint64_t) n_bv};
   const cuuint64_t strides[3] = {8 * 4, 10 * 8 * 4, (cuuint64_t) g.bv * 4};
   const cuuint32_t boxes[3][4] = {{8, 8, 8, 1}, {8, 8, 1, 1}, {8, 1, 8, 1}};
   const cuuint32_t estr[4] = {1, 1, 1, 1};
   for (int q = 0; q < 3; q++)
      if (enc(&tm[q], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4,
              const_cast<float *>(pool), dims, strides, boxes[q], estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_32B,
              CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
         return false;
   return true;
}

// Candidates: one warp per item (two rows of 8 cells a lane) or two warps
// per item (one row a thread), 4 or 2 items per CTA; FP32 also two
// variables per item with two warps, and the tensor-copy form (one warp
// and one variable, or two warps and two variables, per item); a
// persistent grid of the CTAs one wave holds.  Shape fields: threads =
// threads per item, vpc = items per CTA, rows = rows per thread, planes =
// variables per item, tma = 1 for the tensor-copy form.
template <typename T>
void brick_candidates(const Geom &g, int stencil, int n_blocks,
                      std::vector<StageShape> &out)
{
   if (stencil != 7 || dims_kind(g) != 1)
      return;
   int dev = 0, sms = 0;
   cudaGetDevice(&dev);
   cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
   struct Form {
      int tpi, vpi;
   };
   std::vector<Form> forms = {{32, 1}, {64, 1}};
   if (sizeof(T) == 4 && g.V >= 2)
      forms.push_back({64, 2});
   for (const Form &fm : forms)
      for (int gpc : {4, 2}) {
         int per_sm = 0;
         if (fm.vpi == 2) {
            if constexpr (sizeof(T) == 4)
               per_sm = brick_per_sm<T, 64, 2>(gpc);
         } else
            per_sm = fm.tpi == 32 ? brick_per_sm<T, 32, 1>(gpc)
                                  : brick_per_sm<T, 64, 1>(gpc);
         if (per_sm <= 0)
            continue;
         const long long items =
            (long long) n_blocks * ((g.V + fm.vpi - 1) / fm.vpi);
         StageShape sh;
         sh.kernel = 1;
         sh.threads = fm.tpi;
         sh.vpc = gpc;
         sh.rows = 64 / fm.tpi;
         sh.planes = fm.vpi;
         sh.grid = (int) std::max(1LL, std::min<long long>(
                                          (long long) per_sm * sms,
                                          (items + gpc - 1) / gpc));
         out.push_back(sh);
      }
   if constexpr (sizeof(T) == 4) {
      if (!encode_tiled())
         return;
      std::vector<Form> tforms = {{32, 1}};
      if (g.V >= 2)
         tforms.push_back({64, 2});
      for (const Form &fm : tforms) {
            const int gpc = 128 / fm.tpi;
            const int per_sm = fm.vpi == 2 ? brick_tma_per_sm<64, 2>(gpc)
                                           : brick_tma_per_sm<32, 1>(gpc);
            if (per_sm <= 0)
               continue;
            const long long items =
               (long long) n_blocks * ((g.V + fm.vpi - 1) / fm.vpi);
            StageShape sh;
            sh.kernel = 1;
            sh.tma = 1;
            sh.threads = fm.tpi;
            sh.vpc = gpc;
            sh.rows = 64 / fm.tpi;
            sh.planes = fm.vpi;
            sh.grid = (int) std::max(1LL, std::min<long long>(
                                             (long long) per_sm * sms,
                                             (items + gpc - 1) / gpc));
            out.push_back(sh);
         }
   }
}

template <typename T>
int launch_brick_stage(const T *src, T *dst, const Geom &g,
                       const BItem *items, int n_blocks, const StageShape &sh,
                       int write_ghosts, int do_cs, unsigned long long *acc,
                       unsigned *err, unsigned *ctx_err, long long n_bv,
                       const T *zf_src, T *zf_dst, cudaStream_t s)
{
   if (n_blocks == 0)
      return 0;
   const int vpi = sh.planes == 2 ? 2 : 1;
   if (sh.tma) {
      if constexpr (sizeof(T) == 4) {
         CUtensorMap tm[3];
         if (!brick_tensor_maps(src, g, n_bv, tm) ||
             (vpi == 2) != (sh.threads == 64))
            return -1;
         const size_t smem = BrickT::smem_bytes(sh.vpc, vpi);
         if (vpi == 2)
            brick_tma_kernel<64, 2><<<sh.grid, 64 * sh.vpc, smem, s>>>(
               tm[0], tm[1], tm[2], src, dst, g, items, n_blocks,
               write_ghosts, do_cs, acc, err, ctx_err, zf_src, zf_dst);
         else
            brick_tma_kernel<32, 1><<<sh.grid, 32 * sh.vpc, smem, s>>>(
               tm[0], tm[1], tm[2], src, dst, g, items, n_blocks,
               write_ghosts, do_cs, acc, err, ctx_err, zf_src, zf_dst);
         return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
      } else {
         return -1;
      }
   }
   const size_t smem = Brick<T>::smem_per_item(vpi) * sh.vpc;
   const int cs = sizeof(T) == 4 ? do_cs : 0;
   if (vpi == 2) {
      if constexpr (sizeof(T) == 4)
         brick_stage_kernel<T, 64, 2><<<sh.grid, 64 * sh.vpc, smem, s>>>(
            src, dst, g, items, n_blocks, write_ghosts, cs, acc, err, zf_src,
            zf_dst);
      else
         return -1;
   } else if (sh.threads == 64)
      brick_stage_kernel<T, 64, 1><<<sh.grid, 64 * sh.vpc, smem, s>>>(
         src, dst, g, items, n_blocks, write_ghosts, cs, acc, err, zf_src,
         zf_dst);
   else
      brick_stage_kernel<T, 32, 1><<<sh.grid, 32 * sh.vpc, smem, s>>>(
         src, dst, g, items, n_blocks, write_ghosts, cs, acc, err, zf_src,
         zf_dst);
   return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

template void brick_candidates<float>(const Geom &, int, int,
                                      std::vector<StageShape> &);
template void brick_candidates<double>(const Geom &, int, int,
                                       std::vector<StageShape> &);
template int launch_brick_stage<float>(const float *, float *, const Geom &,
                                       const BItem *, int, const StageShape &,
                                       int, int, unsigned long long *,
                                       unsigned *, unsigned *, long long,
                                       const float *, float *, cudaStream_t);
template int launch_brick_stage<double>(const double *, double *,
                                        const Geom &, const BItem *, int,
                                        const StageShape &, int, int,
                                        unsigned long long *, unsigned *,
                                        unsigned *, long long,
                                        const double *, double *,
                                        cudaStream_t);

}  // namespace mamr
