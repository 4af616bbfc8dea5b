// Tile stage kernel for meshes of 8^3 or 16^3 blocks, any number of
// levels, 7- or 27-point: persistent CTAs walk the (block, variable) work
// items, each CTA with two tiles in shared memory -- while it updates one
// item, the copies of the next land in the other (cp.async).  A tile is the
// block-variable with its ghost layer, filled as the batched kernels gather
// it (batched_kernels.cu): interior rows and the faces that are copies
// (same-level neighbour, reflection) or single coarse values as 16-byte or
// element copies; after they land, coarse values are scaled by 1/4, faces
// next to finer blocks summed from four cells, and the 27-point edges and
// corners taken from the neighbour across each ghost axis (one level) or
// from their recipes (level jumps: batched.h).  The update is the plain
// kernel's: FP32 threads each own four k values of one j-row on four
// i-planes (16-byte row loads, each 27-point plane sum formed once), FP64
// threads one (j, k) column; the reference's operation order
// (ref/stencil.c:82-144) and correctly rounded division throughout, the
// FP32 fixed-point checksum fused.  During a run each stage also stores
// the k = 1 and k = N planes of every block-variable it updates in a
// z-face array (batched.h: zface_at), and the next stage takes its z faces
// from there -- the same-level and boundary planes as 16-byte copies into
// a staging area, scattered into the tile after the wait; coarse and fine
// z faces as values of those planes -- instead of one value per 64-byte
// row of the neighbour.
#include <algorithm>
#include <vector>

#include "batched.h"
#include "arith.cuh"
#include "cp_async.cuh"
#include "dims.cuh"
#include "ghost_eval.cuh"

namespace mamr {

namespace {

template <typename T, int N> struct TileK {
   static constexpr int VW = 16 / (int) sizeof(T);   // elements per 16 bytes
   static constexpr int KO = VW - 1;                 // column of k = 0
   static constexpr int Y = N + 2;
   static constexpr int ZS = ((VW - 1 + N + 2 + VW - 1) / VW) * VW;
   static constexpr int TILE = (N + 2) * Y * ZS;     // elements
   static constexpr int CPR = N / VW;                // 16-byte chunks a row
   // FP32: (N/4 plane groups) x N rows x (N/4 quads); FP64: N x N columns
   static constexpr int THREADS = sizeof(T) == 4 ? (N / 4) * N * (N / 4)
                                                 : N * N;
   static constexpr int MINB = sizeof(T) == 4 ? (N == 16 ? 3 : 16)
                                              : (N == 16 ? 2 : 8);
   static constexpr int ZP = N * N;                  // z-plane elements
   __device__ static int at(int i, int j, int k)
   {
      return (i * Y + j) * ZS + KO + k;
   }
   __device__ static int ghost_at(int dir, int gn, int a, int b)
   {
      return dir == 0 ? at(gn, a, b) : (dir == 1 ? at(a, gn, b)
                                                 : at(a, b, gn));
   }
   // two tiles, each with a staging area for its two z planes, and three
   // descriptors
   static size_t smem_bytes()
   {
      return 2 * (size_t) (TILE + 2 * ZP) * sizeof(T) + 3 * sizeof(BItem) +
             16;
   }
};

// Edge or corner cell e of the 4*3N + 8 a 27-point tile needs, in the
// generic kernel's order: its coordinates, recipe index and index along
// the edge.
template <int N>
__device__ __forceinline__ void edge_cell(int e, int &gi, int &gj, int &gk,
                                          int &ri, int &t)
{
   if (e < 4 * N) {
      const int q = e / N;
      gk = e - q * N + 1;
      gi = (q & 1) ? N + 1 : 0;
      gj = (q & 2) ? N + 1 : 0;
      ri = q;
      t = gk;
   } else if (e < 8 * N) {
      const int e2 = e - 4 * N, q = e2 / N;
      gj = e2 - q * N + 1;
      gi = (q & 1) ? N + 1 : 0;
      gk = (q & 2) ? N + 1 : 0;
      ri = 4 + q;
      t = gj;
   } else if (e < 12 * N) {
      const int e2 = e - 8 * N, q = e2 / N;
      gi = e2 - q * N + 1;
      gj = (q & 1) ? N + 1 : 0;
      gk = (q & 2) ? N + 1 : 0;
      ri = 8 + q;
      t = gi;
   } else {
      const int q = e - 12 * N;
      gi = (q & 1) ? N + 1 : 0;
      gj = (q & 2) ? N + 1 : 0;
      gk = (q & 4) ? N + 1 : 0;
      ri = 12 + q;
      t = 0;
   }
}

// Queues the copies that fill tile tb for item (block sd, var); with the
// source's z-face array zf, the same-level and boundary z planes go to the
// staging area zs (plane of side 0, then side 1).
template <typename T, int ST, int N>
__device__ __forceinline__ void tile_issue(const T *__restrict__ src,
                                           const T *__restrict__ stale,
                                           const Geom &g, const BItem &sd,
                                           const GhostRecipe *__restrict__ rc,
                                           int var, T *tb,
                                           const T *__restrict__ zf, T *zs)
{
   using K = TileK<T, N>;
   constexpr int VW = K::VW, CPR = K::CPR, THREADS = K::THREADS;
   const Dims<N, N, N> D(g);
   const int tid = threadIdx.x;
   const T *own = src + bv_offset(g, sd.slot, var);
   for (int c = tid; c < N * N * CPR; c += THREADS) {
      const int r = c / CPR, q = c - r * CPR;
      const int i = r / N + 1, j = r - (i - 1) * N + 1;
      cp_async16(tb + K::at(i, j, 1 + q * VW), own + D.cell(i, j, 1) + q * VW);
   }
#pragma unroll
   for (int l = 0; l < 6; l++) {
      const BFace &f = sd.f[l];
      const int dir = l >> 1;
      const bool low = !(l & 1);
      const int gn = low ? 0 : N + 1;
      if (f.type == FACE_SAME || f.type == FACE_BC) {
         const T *sb = f.type == FACE_SAME ? src + bv_offset(g, f.nb[0], var)
                                          : own;
         // same level: the neighbour's near plane; boundary: reflection
         const int p = (f.type == FACE_SAME) == low ? N : 1;
         if (dir < 2) {
            for (int c = tid; c < N * CPR; c += THREADS) {
               const int a = c / CPR + 1, q = c - (a - 1) * CPR;
               if (dir == 0)
                  cp_async16(tb + K::at(gn, a, 1 + q * VW),
                             sb + D.cell(p, a, 1) + q * VW);
               else
                  cp_async16(tb + K::at(a, gn, 1 + q * VW),
                             sb + D.cell(a, p, 1) + q * VW);
            }
         } else if (zf) {
            const int nbs = f.type == FACE_SAME ? f.nb[0] : sd.slot;
            const T *pl = zf + zface_at(g, nbs, var, p == N);
            for (int c = tid; c < K::ZP / VW; c += THREADS)
               cp_async16(zs + (low ? 0 : K::ZP) + c * VW, pl + c * VW);
         } else {
            for (int e = tid; e < N * N; e += THREADS) {
               const int i = e / N + 1, j = e - (i - 1) * N + 1;
               cp_async_elem(tb + K::at(i, j, gn), sb + D.cell(i, j, p));
            }
         }
      } else if (f.type == FACE_COARSE) {
         // the coarse values, scaled by 1/4 once they have landed (z: from
         // the coarse block's plane in the z-face array)
         const T *sb = src + bv_offset(g, f.nb[0], var);
         const int p = low ? N : 1, h = N / 2;
         const T *pl = dir == 2 && zf ? zf + zface_at(g, f.nb[0], var, p == N)
                                      : nullptr;
         for (int e = tid; e < N * N; e += THREADS) {
            const int a = e / N + 1, b = e - (a - 1) * N + 1;
            const int ca = (a + 1) / 2 + f.jq * h, cb = (b + 1) / 2 + f.iq * h;
            cp_async_elem(tb + K::ghost_at(dir, gn, a, b),
                          pl ? pl + (ca - 1) * N + (cb - 1)
                             : sb + D.fcell(dir, p, ca, cb));
         }
      }
   }
   if (ST == 27) {
      for (int e = tid; e < 12 * N + 8; e += THREADS) {
         int gi, gj, gk, ri, t;
         edge_cell<N>(e, gi, gj, gk, ri, t);
         T *to = tb + K::at(gi, gj, gk);
         if (rc) {
            const GhostRecipe &r = rc[ri];
            if (r.kind == GR_COARSE || r.kind == GR_FINE)
               continue;                       // formed after the wait
            const int c0 = r.vax == 0 ? t : r.c[0];
            const int c1 = r.vax == 1 ? t : r.c[1];
            const int c2 = r.vax == 2 ? t : r.c[2];
            const T *base = r.kind == GR_STALE ? stale : src;
            cp_async_elem(to, base + bv_offset(g, r.nb[0], var) +
                                 D.cell(c0, c1, c2));
         } else {
            // one level: the neighbour across each ghost axis, or the
            // block's own plane where that axis is a boundary
            int dx = gi == 0 ? -1 : (gi == N + 1 ? 1 : 0);
            int dy = gj == 0 ? -1 : (gj == N + 1 ? 1 : 0);
            int dz = gk == 0 ? -1 : (gk == N + 1 ? 1 : 0);
            int si = gi, sj = gj, sk = gk;
            if (dx) {
               if (sd.bmask & (1 << (dx < 0 ? 0 : 1))) { si = dx < 0 ? 1 : N; dx = 0; }
               else si = dx < 0 ? N : 1;
            }
            if (dy) {
               if (sd.bmask & (1 << (dy < 0 ? 2 : 3))) { sj = dy < 0 ? 1 : N; dy = 0; }
               else sj = dy < 0 ? N : 1;
            }
            if (dz) {
               if (sd.bmask & (1 << (dz < 0 ? 4 : 5))) { sk = dz < 0 ? 1 : N; dz = 0; }
               else sk = dz < 0 ? N : 1;
            }
            const int nbs = sd.nb27[(dx + 1) + 3 * (dy + 1) + 9 * (dz + 1)];
            cp_async_elem(to, src + bv_offset(g, nbs, var) +
                                 D.cell(si, sj, sk));
         }
      }
   }
}

// After the copies landed: staged z planes scattered into the tile,
// coarse face values scaled, fine faces summed (z: from the finer blocks'
// planes in the z-face array zf), recipe transforms of the 27-point edges
// formed.
template <typename T, int ST, int N>
__device__ __forceinline__ void tile_fix(const T *__restrict__ src,
                                         const T *__restrict__ stale,
                                         const Geom &g, const BItem &sd,
                                         const GhostRecipe *__restrict__ rc,
                                         int var, T *tb,
                                         const T *__restrict__ zf,
                                         const T *zs)
{
   using K = TileK<T, N>;
   constexpr int THREADS = K::THREADS;
   const Dims<N, N, N> D(g);
   const int tid = threadIdx.x;
   if (zf) {
#pragma unroll
      for (int l = 4; l < 6; l++) {
         const int type = sd.f[l].type;
         if (type != FACE_SAME && type != FACE_BC)
            continue;
         const int gn = l == 4 ? 0 : N + 1;
         for (int e = tid; e < N * N; e += THREADS) {
            const int i = e / N + 1, j = e - (i - 1) * N + 1;
            tb[K::at(i, j, gn)] = zs[(l - 4) * K::ZP + e];
         }
      }
   }
#pragma unroll
   for (int l = 0; l < 6; l++) {
      const BFace &f = sd.f[l];
      if (f.type != FACE_COARSE && f.type != FACE_FINE)
         continue;
      const int dir = l >> 1;
      const bool low = !(l & 1);
      const int gn = low ? 0 : N + 1, p = low ? N : 1, h = N / 2;
      for (int e = tid; e < N * N; e += THREADS) {
         const int a = e / N + 1, b = e - (a - 1) * N + 1;
         T &x = tb[K::ghost_at(dir, gn, a, b)];
         if (f.type == FACE_COARSE) {
            x = quarter(x);
         } else {
            const int jq = a > h, iq = b > h;
            const int a2 = a - jq * h, b2 = b - iq * h;
            const int nbs = f.nb[iq * 2 + jq];
            T s;
            if (dir == 2 && zf) {
               const T *pl = zf + zface_at(g, nbs, var, p == N) +
                             (2 * a2 - 2) * N + 2 * b2 - 2;
               s = pl[0] + pl[1];
               s = s + pl[N];
               s = s + pl[N + 1];
            } else {
               const T *fb = src + bv_offset(g, nbs, var);
               s = fb[D.fcell(dir, p, 2 * a2 - 1, 2 * b2 - 1)] +
                   fb[D.fcell(dir, p, 2 * a2 - 1, 2 * b2)];
               s = s + fb[D.fcell(dir, p, 2 * a2, 2 * b2 - 1)];
               s = s + fb[D.fcell(dir, p, 2 * a2, 2 * b2)];
            }
            x = s;
         }
      }
   }
   if (ST == 27 && rc) {
      for (int e = tid; e < 12 * N + 8; e += THREADS) {
         int gi, gj, gk, ri, t;
         edge_cell<N>(e, gi, gj, gk, ri, t);
         const GhostRecipe &r = rc[ri];
         if (r.kind == GR_COARSE || r.kind == GR_FINE)
            tb[K::at(gi, gj, gk)] = eval_recipe(r, t, src, stale, g, D, var);
      }
   }
}

// The ghost cells of the tile that go to the destination pool: all of
// them at the last stage of a run, else the faces and edges the block's
// keep mask marks (read as previous-stage values by the next stage).
template <typename T, int ST, int N>
__device__ __forceinline__ void tile_ghosts_out(const T *tb, T *d,
                                                const Geom &g, int all,
                                                int kb)
{
   using K = TileK<T, N>;
   constexpr int THREADS = K::THREADS;
   const Dims<N, N, N> D(g);
   const int tid = threadIdx.x;
#pragma unroll
   for (int l = 0; l < 6; l++) {
      if (!all && !(kb >> l & 1))
         continue;
      const int dir = l >> 1, gn = (l & 1) ? N + 1 : 0;
      for (int e = tid; e < N * N; e += THREADS) {
         const int a = e / N + 1, b = e - (a - 1) * N + 1;
         int gi, gj, gk;
         if (dir == 0) { gi = gn; gj = a; gk = b; }
         else if (dir == 1) { gi = a; gj = gn; gk = b; }
         else { gi = a; gj = b; gk = gn; }
         d[D.cell(gi, gj, gk)] = tb[K::at(gi, gj, gk)];
      }
   }
   if (ST == 27 && (all || (kb >> 6))) {
      for (int e = tid; e < 12 * N + 8; e += THREADS) {
         int gi, gj, gk, ri, t;
         edge_cell<N>(e, gi, gj, gk, ri, t);
         if (all || (ri < 12 && (kb >> (6 + ri) & 1)))
            d[D.cell(gi, gj, gk)] = tb[K::at(gi, gj, gk)];
      }
   }
}

// The update of one tile into d (the item's destination block-variable),
// FP32 checksum terms into part; with zfd, its k = 1 and k = N planes also
// into the z-face array (side 0 at zfd, side 1 at zfd + ZP).
template <typename T, int ST, int N>
__device__ __forceinline__ void tile_update(const T *tb, T *d, const Geom &g,
                                            int do_cs, Fixed52 &part,
                                            bool &ok, T *zfd)
{
   using K = TileK<T, N>;
   const Dims<N, N, N> D(g);
   const int tid = threadIdx.x;
#define TL(i, j, k) tb[K::at(i, j, k)]
   if constexpr (sizeof(T) == 4) {
      constexpr int NQ = N / 4, COLS = N * NQ;
      const int t = tid % COLS, grp = tid / COLS;
      const int kq = t % NQ;
      int jr;
      if (NQ == 4) {
         // rows two apart share a phase of 8 lanes: with 24-float rows
         // they fall in opposite 64-byte halves of the bank span
         const int h = (t >> 2) & 1, r = t >> 3;
         jr = (r & 1) + 4 * (r >> 1) + 2 * h;
      } else {
         jr = t / NQ;
      }
      const int j = jr + 1, k = 4 * kq + 1, i0 = 4 * grp;
      auto quad = [&](int i, int jj, T (&v)[4]) {
         const float4 x = *reinterpret_cast<const float4 *>(&TL(i, jj, k));
         v[0] = x.x; v[1] = x.y; v[2] = x.z; v[3] = x.w;
      };
      auto row6 = [&](int i, int jj, T (&r)[6]) {
         T v[4];
         quad(i, jj, v);
         r[0] = TL(i, jj, k - 1);
         r[1] = v[0]; r[2] = v[1]; r[3] = v[2]; r[4] = v[3];
         r[5] = TL(i, jj, k + 4);
      };
      auto emit = [&](int i, const T (&w)[4], auto div4) {
         T q[4];
         div4(w, q);
         *reinterpret_cast<float4 *>(d + D.cell(i, j, k)) =
            make_float4(q[0], q[1], q[2], q[3]);
         if (zfd) {
            if (k == 1)
               zfd[(i - 1) * N + j - 1] = q[0];
            if (k + 3 == N)
               zfd[K::ZP + (i - 1) * N + j - 1] = q[3];
         }
         if (do_cs) {
#pragma unroll
            for (int m = 0; m < 4; m++)
               fixed52_add((float) q[m], part);
         }
      };
      if (ST == 7) {
         T a[4], c[6];
         quad(i0, j, a);
         row6(i0 + 1, j, c);
#pragma unroll
         for (int ii = 1; ii <= 4; ii++) {
            const int i = i0 + ii;
            T jm[4], jp[4], b[6], w[4];
            quad(i, j - 1, jm);
            quad(i, j + 1, jp);
            row6(i + 1, j, b);
#pragma unroll
            for (int m = 0; m < 4; m++) {
               T v = a[m] + jm[m];
               v = v + c[m];
               v = v + c[m + 1];
               v = v + c[m + 2];
               v = v + jp[m];
               v = v + b[m + 1];
               w[m] = v;
            }
            emit(i, w, [](const T (&x)[4], T (&q)[4]) {
               div_const4<7>(x, q);
            });
#pragma unroll
            for (int m = 0; m < 4; m++)
               a[m] = c[m + 1];
#pragma unroll
            for (int m = 0; m < 6; m++)
               c[m] = b[m];
         }
      } else {
         auto S = [&](int p, T (&s4)[4]) {
            T r0[6], r1[6], r2[6];
            row6(p, j - 1, r0);
            row6(p, j, r1);
            row6(p, j + 1, r2);
#pragma unroll
            for (int m = 0; m < 4; m++) {
               T v = r0[m] + r0[m + 1];
               v = v + r0[m + 2];
               v = v + r1[m];
               v = v + r1[m + 1];
               v = v + r1[m + 2];
               v = v + r2[m];
               v = v + r2[m + 1];
               v = v + r2[m + 2];
               s4[m] = v;
            }
         };
         T s0[4], s1[4], s2[4];
         S(i0, s0);
         S(i0 + 1, s1);
#pragma unroll
         for (int ii = 1; ii <= 4; ii++) {
            const int i = i0 + ii;
            S(i + 1, s2);
            T w[4];
#pragma unroll
            for (int m = 0; m < 4; m++)
               w[m] = (s0[m] + s1[m]) + s2[m];
            emit(i, w, [](const T (&x)[4], T (&q)[4]) {
               div_const4<27>(x, q);
            });
#pragma unroll
            for (int m = 0; m < 4; m++) {
               s0[m] = s1[m];
               s1[m] = s2[m];
            }
         }
      }
   } else {
      // FP64: one (j, k) column per thread, swept along i; each 27-point
      // plane sum formed once and used by the three cells that need it
      const int j = tid / N + 1, k = tid - (j - 1) * N + 1;
      if (ST == 7) {
         T am = TL(0, j, k), ac = TL(1, j, k);
#pragma unroll 4
         for (int i = 1; i <= N; i++) {
            const T ap = TL(i + 1, j, k);
            T w = am + TL(i, j - 1, k);
            w = w + TL(i, j, k - 1);
            w = w + ac;
            w = w + TL(i, j, k + 1);
            w = w + TL(i, j + 1, k);
            w = w + ap;
            const T q = div7(w);
            d[D.cell(i, j, k)] = q;
            if (zfd && (k == 1 || k == N))
               zfd[(k == N ? K::ZP : 0) + (i - 1) * N + j - 1] = q;
            am = ac;
            ac = ap;
         }
      } else {
         auto S = [&](int p) -> T {
            T s = TL(p, j - 1, k - 1) + TL(p, j - 1, k);
            s = s + TL(p, j - 1, k + 1);
            s = s + TL(p, j, k - 1);
            s = s + TL(p, j, k);
            s = s + TL(p, j, k + 1);
            s = s + TL(p, j + 1, k - 1);
            s = s + TL(p, j + 1, k);
            s = s + TL(p, j + 1, k + 1);
            return s;
         };
         T s0 = S(0), s1 = S(1);
#pragma unroll 4
         for (int i = 1; i <= N; i++) {
            const T s2 = S(i + 1);
            const T q = div27((s0 + s1) + s2);
            d[D.cell(i, j, k)] = q;
            if (zfd && (k == 1 || k == N))
               zfd[(k == N ? K::ZP : 0) + (i - 1) * N + j - 1] = q;
            s0 = s1;
            s1 = s2;
         }
      }
   }
#undef TL
}

template <typename T, int ST, int N>
__global__ void __launch_bounds__(TileK<T, N>::THREADS, TileK<T, N>::MINB)
tile_stage_kernel(const T *__restrict__ src, T *__restrict__ dst, Geom g,
                  const BItem *__restrict__ items,
                  const GhostRecipe *__restrict__ recipes,
                  const int *__restrict__ keep, const T *__restrict__ stale,
                  int nb, int write_ghosts, int do_cs,
                  unsigned long long *__restrict__ acc,
                  unsigned *__restrict__ err, const T *__restrict__ zf_src,
                  T *__restrict__ zf_dst)
{
   using K = TileK<T, N>;
   constexpr int THREADS = K::THREADS;
   extern __shared__ __align__(16) unsigned char smem_raw[];
   T *tiles = reinterpret_cast<T *>(smem_raw);
   T *stg = tiles + 2 * K::TILE;        // z-plane staging of each tile
   BItem *sI = reinterpret_cast<BItem *>(stg + 4 * K::ZP);
   const int tid = threadIdx.x;
   auto put_desc = [&](int b, BItem &to) {
      const int32_t *from = reinterpret_cast<const int32_t *>(items + b);
      int32_t *t = reinterpret_cast<int32_t *>(&to);
      for (int q = tid; q < (int) (sizeof(BItem) / 4); q += THREADS)
         t[q] = __ldg(from + q);
   };
   // work items (block b, variable var), variable-major; CTA c takes
   // items c, c + grid, ... tracked as (var, b) without divisions
   struct Pos {
      int var, b;
   };
   const int step_v = gridDim.x / nb, step_b = gridDim.x - step_v * nb;
   auto advance = [&](Pos q) {
      q.var += step_v;
      q.b += step_b;
      if (q.b >= nb) {
         q.b -= nb;
         q.var++;
      }
      return q;
   };
   auto recipes_of = [&](int b) {
      return recipes ? recipes + (size_t) b * kGhostRecipes : nullptr;
   };
   unsigned long long lo = 0, hi = 0;
   Fixed52 part;
   bool ok = true;
   int cs_var = -1;
   Pos cur_p{(int) (blockIdx.x / nb), (int) (blockIdx.x % nb)};
   if (cur_p.var >= g.V)
      return;
   put_desc(cur_p.b, sI[0]);
   __syncthreads();
   tile_issue<T, ST, N>(src, stale, g, sI[0], recipes_of(cur_p.b), cur_p.var,
                        tiles, zf_src, stg);
   cp_async_commit();
   for (int n = 0;; n++) {
      const int var = cur_p.var, b = cur_p.b;
      const Pos nx = advance(cur_p);
      const bool more = nx.var < g.V;
      BItem &cur = sI[n % 3];
      T *tb = tiles + (n & 1) * K::TILE;
      const T *zs = stg + (n & 1) * 2 * K::ZP;
      // the next item: descriptor, then its copies into the other tile
      // (every thread finished reading that tile before this barrier)
      if (more)
         put_desc(nx.b, sI[(n + 1) % 3]);
      __syncthreads();
      if (more)
         tile_issue<T, ST, N>(src, stale, g, sI[(n + 1) % 3], recipes_of(nx.b),
                              nx.var, tiles + ((n + 1) & 1) * K::TILE, zf_src,
                              stg + ((n + 1) & 1) * 2 * K::ZP);
      cp_async_commit();
      cp_async_wait_group<1>();
      __syncthreads();
      const GhostRecipe *rc =
         recipes ? recipes + (size_t) b * kGhostRecipes : nullptr;
      tile_fix<T, ST, N>(src, stale, g, cur, rc, var, tb, zf_src, zs);
      __syncthreads();
      T *d = dst + bv_offset(g, cur.slot, var);
      const int kb = keep ? keep[b] : 0;
      if (write_ghosts || kb)
         tile_ghosts_out<T, ST, N>(tb, d, g, write_ghosts, kb);
      if (sizeof(T) == 4 && do_cs && var != cs_var) {
         if (cs_var >= 0) {
            warp_acc128_flush(lo, hi, acc + 2 * cs_var);
            lo = hi = 0;
         }
         cs_var = var;
      }
      tile_update<T, ST, N>(tb, d, g, sizeof(T) == 4 ? do_cs : 0, part, ok,
                            zf_dst ? zf_dst + zface_at(g, cur.slot, var, 0)
                                   : nullptr);
      if (sizeof(T) == 4 && do_cs)
         fixed52_flush(part, lo, hi);
      if (!more)
         break;
      cur_p = nx;
   }
   if (sizeof(T) == 4 && do_cs) {
      if (cs_var >= 0)
         warp_acc128_flush(lo, hi, acc + 2 * cs_var);
      if (!ok || !fixed52_window(part))
         atomicOr(err, ERR_FIXED_RANGE);
   }
}

template <typename T, int ST, int N>
static int tile_per_sm()
{
   using K = TileK<T, N>;
   int per_sm = 0;
   cudaFuncSetAttribute(tile_stage_kernel<T, ST, N>,
                        cudaFuncAttributeMaxDynamicSharedMemorySize,
                        (int) K::smem_bytes());
   cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      &per_sm, tile_stage_kernel<T, ST, N>, K::THREADS, K::smem_bytes());
   return per_sm;
}

}  // namespace

// Candidates: a persistent grid of the CTAs one wave holds, or twice that
// (more items in flight per SM when the CTAs finish unevenly).  Shape
// fields: kernel 2, threads = threads per CTA, vpc 1, rows 0, planes 0.
template <typename T>
void tile_candidates(const Geom &g, int stencil, int n_blocks,
                     std::vector<StageShape> &out)
{
   const int kind = dims_kind(g);
   if (kind == 0)
      return;
   int dev = 0, sms = 0;
   cudaGetDevice(&dev);
   cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
   int per_sm, threads;
   if (kind == 1) {
      per_sm = stencil == 7 ? tile_per_sm<T, 7, 8>() : tile_per_sm<T, 27, 8>();
      threads = TileK<T, 8>::THREADS;
   } else {
      per_sm = stencil == 7 ? tile_per_sm<T, 7, 16>()
                            : tile_per_sm<T, 27, 16>();
      threads = TileK<T, 16>::THREADS;
   }
   if (per_sm <= 0)
      return;
   const long long items = (long long) n_blocks * g.V;
   for (int waves : {1, 2}) {
      StageShape sh;
      sh.kernel = 2;
      sh.threads = threads;
      sh.vpc = 1;
      sh.rows = 0;
      sh.planes = 0;
      sh.grid = (int) std::max(1LL, std::min<long long>(
                                       (long long) waves * per_sm * sms,
                                       items));
      out.push_back(sh);
   }
}

template <typename T>
int launch_tile_stage(const T *src, T *dst, const Geom &g, int stencil,
                      const BItem *items, const GhostRecipe *recipes,
                      const int *keep, const T *stale, int n_blocks,
                      const StageShape &sh, int write_ghosts, int do_cs,
                      unsigned long long *acc, unsigned *err,
                      const T *zf_src, T *zf_dst, cudaStream_t s)
{
   if (n_blocks == 0)
      return 0;
   const int cs = sizeof(T) == 4 ? do_cs : 0;
#define MAMR_TILE(ST, N)                                                      \
   tile_stage_kernel<T, ST, N>                                               \
      <<<sh.grid, TileK<T, N>::THREADS, TileK<T, N>::smem_bytes(), s>>>(      \
         src, dst, g, items, recipes, keep, stale, n_blocks, write_ghosts,    \
         cs, acc, err, zf_src, zf_dst)
   const int kind = dims_kind(g);
   if (kind == 1) {
      if (stencil == 7) MAMR_TILE(7, 8);
      else MAMR_TILE(27, 8);
   } else {
      if (stencil == 7) MAMR_TILE(7, 16);
      else MAMR_TILE(27, 16);
   }
#undef MAMR_TILE
   return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

template void tile_candidates<float>(const Geom &, int, int,
                                     std::vector<StageShape> &);
template void tile_candidates<double>(const Geom &, int, int,
                                      std::vector<StageShape> &);
template int launch_tile_stage<float>(const float *, float *, const Geom &,
                                      int, const BItem *, const GhostRecipe *,
                                      const int *, const float *, int,
                                      const StageShape &, int, int,
                                      unsigned long long *, unsigned *,
                                      const float *, float *, cudaStream_t);
template int launch_tile_stage<double>(const double *, double *,
                                       const Geom &, int, const BItem *,
                                       const GhostRecipe *, const int *,
                                       const double *, int,
                                       const StageShape &, int, int,
                                       unsigned long long *, unsigned *,
                                       const double *, double *,
                                       cudaStream_t);

}  // namespace mamr
