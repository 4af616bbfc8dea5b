// Plain-path kernels: the reference's call sequence, one launch per call,
// every cell bit-identical to the reference in FP64 (compiled with
// -fmad=false; sums in the reference's order; divisions correctly rounded).
#include <algorithm>

#include "mamr_internal.h"
#include "arith.cuh"
#include "dims.cuh"

namespace mamr {

// (normal coordinate nc, tangential a, b) -> (i, j, k) for a face normal to
// dir.  a/b are (j, k) for x faces, (i, k) for y faces, (i, j) for z faces,
// the loop order of ref/comm.c:1473-1534.
__device__ __forceinline__ long long face_cell(const Geom &g, int dir, int nc,
                                               int a, int b)
{
   if (dir == 0) return cell_offset(g, nc, a, b);
   if (dir == 1) return cell_offset(g, a, nc, b);
   return cell_offset(g, a, b, nc);
}

// One CTA per (task, variable).  Tasks of one direction are independent:
// each ghost cell is written by exactly one task and every read is of a
// plane that this direction does not write (ref/comm.c:162-203).  The
// direction and, for 8^3 and 16^3 blocks, the block size are compile-time
// constants, so face addressing folds to a few multiply-adds.
template <typename T, int DIR, int BX, int BY, int BZ>
__global__ void __launch_bounds__(256)
comm_dir_kernel(T *__restrict__ pool, Geom g, int stencil, int code,
                DirTasks t, int var0, int nvar, const T *__restrict__ zc)
{
   const Dims<BX, BY, BZ> D(g);
   constexpr int dir = DIR;
   // one warp per (task, variable): a face is a few hundred cells, so a
   // CTA per task spent more on its own launch than on the copies
   const int lane = threadIdx.x & 31;
   const int n_tasks = t.n_same + t.n_diff + t.n_bc;
   const long long gw =
      (long long) blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
   if (gw >= (long long) n_tasks * nvar)
      return;
   int task = (int) (gw % n_tasks);
   const int var = var0 + (int) (gw / n_tasks);
   const int n = dir == 0 ? D.nx : (dir == 1 ? D.ny : D.nz);
   const int na = dir == 0 ? D.ny : D.nx;
   const int nb = dir == 2 ? D.ny : D.nz;
   auto face_cell = [&](const Geom &, int, int nc, int a, int b) {
      return D.fcell(DIR, nc, a, b);
   };
   // interior plane nc (1 or n) of block `slot`, cell (a, b): from the
   // z-face cache for the interior rows when there is one (z only),
   // else from the pool
   auto plane = [&](const T *blk, int slot, int nc, int a, int b) -> T {
      if (DIR == 2 && zc && a >= 1 && a <= na && b >= 1 && b <= nb)
         return zc[zcache_at(g, slot, var, nc == n ? 1 : 0, a, b)];
      return blk[face_cell(g, dir, nc, a, b)];
   };

   if (task < t.n_same) {
      // ref/comm.c:1473-1534 (code 0)
      SameTask st = t.same[task];
      T *lo = pool + bv_offset(g, st.lo, var);
      T *hi = pool + bv_offset(g, st.hi, var);
      int a0 = 1, a1 = na, b0 = 1, b1 = nb;
      if (code) {
         // code 1/2 (ref/comm.c:1535-1579): whole planes
         a0 = 0; a1 = na + 1; b0 = 0; b1 = nb + 1;
      } else if (stencil != 7) {
         if (dir >= 1) { a0 = 0; a1 = na + 1; }
         if (dir == 2) { b0 = 0; b1 = nb + 1; }
      }
      const int cb = b1 - b0 + 1, cnt = (a1 - a0 + 1) * cb;
      for (int e = lane; e < cnt; e += 32) {
         int a = a0 + e / cb, b = b0 + e % cb;
         lo[face_cell(g, dir, n + 1, a, b)] = plane(hi, st.hi, 1, a, b);
         hi[face_cell(g, dir, 0, a, b)] = plane(lo, st.lo, n, a, b);
      }
      return;
   }
   task -= t.n_same;
   if (task < t.n_diff) {
      // ref/comm.c:1597-1688 (code 0)
      DiffTask dt = t.diff[task];
      T *C = pool + bv_offset(g, dt.coarse, var);
      T *F = pool + bv_offset(g, dt.fine, var);
      const bool low = (dt.l % 2) == 0;
      const int c0 = low ? 0 : n + 1, c1 = low ? 1 : n;
      const int f2 = low ? n + 1 : 0, f3 = low ? n : 1;
      const int ha = na / 2, hb = nb / 2;
      const int oa = dt.jq * ha, ob = dt.iq * hb;
      if (code) {
         // code 1/2 (ref/comm.c:1689-1907), the reference's three
         // direction branches in one form: the fine ghost plane whole,
         // tangential index A reading coarse offset + (A=0: 0, A=na+1:
         // na/2+1, else (A+1)/2); the coarse ghost plane the quarter's 2x2
         // sums plus the fine ghost row / column pair sums on the jq / iq
         // sides and one corner.  Thread (p, q) of (ha+1) x (hb+1) writes
         // coarse cell (p ? p+oa : edge row, q ? q+ob : edge column).
         const int cnt = (na + 2) * (nb + 2);
         for (int e = lane; e < cnt; e += 32) {
            const int A = e / (nb + 2), B = e % (nb + 2);
            const int ca = A == 0 ? oa
                         : (A == na + 1 ? ha + 1 + oa : (A + 1) / 2 + oa);
            const int cb = B == 0 ? ob
                         : (B == nb + 1 ? hb + 1 + ob : (B + 1) / 2 + ob);
            F[face_cell(g, dir, f2, A, B)] =
               quarter(C[face_cell(g, dir, c1, ca, cb)]);
         }
         const int ae = dt.jq ? na + 1 : 0, be = dt.iq ? nb + 1 : 0;
         for (int e = lane; e < (ha + 1) * (hb + 1); e += 32) {
            const int p = e / (hb + 1), q = e % (hb + 1);
            T v;
            if (p && q) {
               v = F[face_cell(g, dir, f3, 2*p - 1, 2*q - 1)] +
                   F[face_cell(g, dir, f3, 2*p - 1, 2*q)];
               v = v + F[face_cell(g, dir, f3, 2*p, 2*q - 1)];
               v = v + F[face_cell(g, dir, f3, 2*p, 2*q)];
            } else if (q) {
               v = F[face_cell(g, dir, f3, ae, 2*q - 1)] +
                   F[face_cell(g, dir, f3, ae, 2*q)];
            } else if (p) {
               v = F[face_cell(g, dir, f3, 2*p - 1, be)] +
                   F[face_cell(g, dir, f3, 2*p, be)];
            } else {
               v = F[face_cell(g, dir, f3, ae, be)];
            }
            C[face_cell(g, dir, c0, p ? p + oa : ae, q ? q + ob : be)] = v;
         }
         return;
      }
      for (int e = lane; e < ha * hb; e += 32) {
         int a = 1 + e / hb, b = 1 + e % hb;
         T q = quarter(plane(C, dt.coarse, c1, a + oa, b + ob));
         F[face_cell(g, dir, f2, 2*a - 1, 2*b - 1)] = q;
         F[face_cell(g, dir, f2, 2*a - 1, 2*b)] = q;
         F[face_cell(g, dir, f2, 2*a, 2*b - 1)] = q;
         F[face_cell(g, dir, f2, 2*a, 2*b)] = q;
         T s = plane(F, dt.fine, f3, 2*a - 1, 2*b - 1) +
               plane(F, dt.fine, f3, 2*a - 1, 2*b);
         s = s + plane(F, dt.fine, f3, 2*a, 2*b - 1);
         s = s + plane(F, dt.fine, f3, 2*a, 2*b);
         C[face_cell(g, dir, c0, a + oa, b + ob)] = s;
      }
      return;
   }
   task -= t.n_diff;
   if (task < t.n_bc) {
      // ref/comm.c:1911-1965
      BcTask bt = t.bc[task];
      T *B = pool + bv_offset(g, bt.slot, var);
      const bool hiside = (bt.l % 2) == 1;
      const int tp = hiside ? n + 1 : 0, fp = hiside ? n : 1;
      const bool full = code != 0 || stencil != 7;
      const int a0 = full ? 0 : 1, a1 = full ? na + 1 : na;
      const int b0 = full ? 0 : 1, b1 = full ? nb + 1 : nb;
      const int cb = b1 - b0 + 1, cnt = (a1 - a0 + 1) * cb;
      for (int e = lane; e < cnt; e += 32) {
         int a = a0 + e / cb, b = b0 + e % cb;
         B[face_cell(g, dir, tp, a, b)] = plane(B, bt.slot, fp, a, b);
      }
   }
}

template <typename T, int DIR>
static void comm_dir_launch(T *pool, const Geom &g, int stencil, int code,
                            const DirTasks &t, int var0, int nvar,
                            unsigned grid, const T *zc, cudaStream_t s)
{
   switch (dims_kind(g)) {
   case 1:
      comm_dir_kernel<T, DIR, 8, 8, 8><<<grid, 256, 0, s>>>(
         pool, g, stencil, code, t, var0, nvar, zc);
      break;
   case 2:
      comm_dir_kernel<T, DIR, 16, 16, 16><<<grid, 256, 0, s>>>(
         pool, g, stencil, code, t, var0, nvar, zc);
      break;
   default:
      comm_dir_kernel<T, DIR, 0, 0, 0><<<grid, 256, 0, s>>>(
         pool, g, stencil, code, t, var0, nvar, zc);
   }
}

template <typename T>
int launch_comm_dir(T *pool, const Geom &g, int dir, int stencil, int code,
                    const DirTasks &t, int var0, int nvar, const T *zc,
                    cudaStream_t s)
{
   int n = t.n_same + t.n_diff + t.n_bc;
   if (n == 0 || nvar == 0)
      return 0;
   // 8 warps a CTA, one (task, variable) a warp
   const unsigned grid = (unsigned) (((long long) n * nvar + 7) / 8);
   // the cache serves the code-0 exchange only
   const T *z = code == 0 ? zc : nullptr;
   if (dir == 0)
      comm_dir_launch<T, 0>(pool, g, stencil, code, t, var0, nvar, grid,
                            nullptr, s);
   else if (dir == 1)
      comm_dir_launch<T, 1>(pool, g, stencil, code, t, var0, nvar, grid,
                            nullptr, s);
   else
      comm_dir_launch<T, 2>(pool, g, stencil, code, t, var0, nvar, grid, z,
                            s);
   return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

// ---------------------------------------------------------------------------
// Stencil: one CTA per active block, the whole block-variable (ghosts
// included) staged in shared memory, each thread sweeping one (j, k) column
// along i (FP32 8^3 and 16^3 blocks: four k values of one j-row on four
// i-planes per thread).  Results are written straight back to the pool: every read comes
// from the staged copy, so the in-place update is the reference's
// work-array Jacobi update (ref/stencil.c:82-99, 103-141).  Staged rows
// are Zs long with k = 1 at a 16-byte boundary, so the interior rows of the
// split layout copy as vectors; 8^3 and 16^3 blocks get compile-time
// dimensions.
template <typename T> struct PlainVec;
template <> struct PlainVec<float> { using V = float4; };
template <> struct PlainVec<double> { using V = double2; };

template <typename T>
__host__ __device__ inline int plain_zs(int nz)
{
   const int vw = 16 / (int) sizeof(T);
   return ((vw - 1 + nz + 2 + vw - 1) / vw) * vw;
}

template <typename T, int ST, int BX, int BY, int BZ>
__global__ void __launch_bounds__(256)
stencil_kernel(T *__restrict__ pool, Geom g, const int32_t *__restrict__ slots,
               int var, T *__restrict__ zc)
{
   extern __shared__ __align__(16) unsigned char smem_raw[];
   T *tile = reinterpret_cast<T *>(smem_raw);
   constexpr int VW = 16 / (int) sizeof(T), KO = VW - 1;
   const Dims<BX, BY, BZ> D(g);
   const int nx = D.nx, ny = D.ny, nz = D.nz, X = D.X, Y = D.Y;
   const int Zs = plain_zs<T>(nz);
   const int slot = slots[blockIdx.x];
   T *base = pool + bv_offset(g, slot, var);
#define TL(i, j, k) tile[((i) * Y + (j)) * Zs + KO + (k)]
   // interior rows (k = 1..nz) of all X*Y rows, then the k ghost planes
   if (nz % VW == 0) {
      using V = typename PlainVec<T>::V;
      const int nv = nz / VW;
      for (int e = threadIdx.x; e < X * Y * nv; e += blockDim.x) {
         const int row = e / nv, q = e - row * nv;
         const V v = __ldg(reinterpret_cast<const V *>(base +
                                                       (size_t) row * nz) + q);
         *reinterpret_cast<V *>(&tile[row * Zs + KO + 1 + q * VW]) = v;
      }
   } else {
      for (int e = threadIdx.x; e < X * Y * nz; e += blockDim.x) {
         const int row = e / nz, k = e - row * nz;
         tile[row * Zs + KO + 1 + k] = base[(size_t) row * nz + k];
      }
   }
   for (int e = threadIdx.x; e < 2 * X * Y; e += blockDim.x) {
      const int row = e % (X * Y), hi = e / (X * Y);
      tile[row * Zs + KO + (hi ? nz + 1 : 0)] =
         base[(size_t) X * Y * nz + (hi ? X * Y : 0) + row];
   }
   __syncthreads();
   if constexpr (sizeof(T) == 4 && BZ > 0 && BZ % 4 == 0 && BX % 4 == 0) {
      // FP32, 8^3 / 16^3: each thread owns four consecutive k values of
      // one j-row on four consecutive i-planes (threads = BX/4 plane
      // groups x BY rows x BZ/4 quads), read as 16-byte row loads plus the
      // two outer neighbours: about 2 shared loads per update instead of
      // 9 (27-point) or 7 (7-point); same operations, same order.
      constexpr int NQ = BZ / 4, COLS = BY * NQ;
      const int t = threadIdx.x % COLS, grp = threadIdx.x / COLS;
      const int kq = t % NQ;
      int jr;
      if (NQ == 4) {
         // rows two apart share a phase of 8 lanes: 2 x 96 bytes puts them
         // in opposite 64-byte halves of the bank span
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
      // row (i, jj) around the quad: k-1 .. k+4
      auto row6 = [&](int i, int jj, T (&r)[6]) {
         T v[4];
         quad(i, jj, v);
         r[0] = TL(i, jj, k - 1);
         r[1] = v[0]; r[2] = v[1]; r[3] = v[2]; r[4] = v[3];
         r[5] = TL(i, jj, k + 4);
      };
      auto store = [&](int i, const T (&w)[4], auto div4) {
         T q[4];
         div4(w, q);
         *reinterpret_cast<float4 *>(base + D.cell(i, j, k)) =
            make_float4(q[0], q[1], q[2], q[3]);
         if (zc) {
            // the planes k = 1 and k = nz for the next z exchange
            if (k == 1)
               zc[zcache_at(g, slot, var, 0, i, j)] = q[0];
            if (k + 3 == nz)
               zc[zcache_at(g, slot, var, 1, i, j)] = q[3];
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
            store(i, w, [](const T (&x)[4], T (&q)[4]) {
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
         // S(p): the 9-point sum on plane p for the four k values
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
            store(i, w, [](const T (&x)[4], T (&q)[4]) {
               div_const4<27>(x, q);
            });
#pragma unroll
            for (int m = 0; m < 4; m++) {
               s0[m] = s1[m];
               s1[m] = s2[m];
            }
         }
      }
      return;
   }
   for (int col = threadIdx.x; col < ny * nz; col += blockDim.x) {
      const int j = col / nz + 1, k = col - (j - 1) * nz + 1;
      if (ST == 7) {
         for (int i = 1; i <= nx; i++) {
            T w = TL(i - 1, j, k) + TL(i, j - 1, k);
            w = w + TL(i, j, k - 1);
            w = w + TL(i, j, k);
            w = w + TL(i, j, k + 1);
            w = w + TL(i, j + 1, k);
            w = w + TL(i + 1, j, k);
            const T out = div7(w);
            base[D.cell(i, j, k)] = out;
            if (zc && (k == 1 || k == nz))
               zc[zcache_at(g, slot, var, k == nz ? 1 : 0, i, j)] = out;
         }
      } else {
         // S(p) = the 9-point left-to-right sum on plane p around (j, k):
         // sb, sm and sf of cell i are S(i-1), S(i), S(i+1), so each S is
         // formed once and reused by three cells -- same operations, same
         // order, a third of the adds.
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
         for (int i = 1; i <= nx; i++) {
            T s2 = S(i + 1);
            const T out = div27((s0 + s1) + s2);
            base[D.cell(i, j, k)] = out;
            if (zc && (k == 1 || k == nz))
               zc[zcache_at(g, slot, var, k == nz ? 1 : 0, i, j)] = out;
            s0 = s1;
            s1 = s2;
         }
      }
   }
#undef TL
}

// Blocks whose whole-block tile does not fit in shared memory (32^3 FP64
// and up): one CTA per block-variable streams the block plane by plane
// along i through a ring of three (ny+2) x (nz+2) planes.  Every read comes
// from the ring, which holds planes i-1, i, i+1 as they were before the
// stage, and plane i is written to the pool only after plane i+1 is in the
// ring, so the in-place update is still the reference's work-array Jacobi
// update (ref/stencil.c:82-99, 103-141) in its operation order.
template <typename T, int ST>
__global__ void __launch_bounds__(256)
stencil_stream_kernel(T *__restrict__ pool, Geom g,
                      const int32_t *__restrict__ slots, int var,
                      T *__restrict__ zc)
{
   extern __shared__ __align__(16) unsigned char smem_raw[];
   T *ring = reinterpret_cast<T *>(smem_raw);
   const int nx = g.nx, ny = g.ny, nz = g.nz, Z = nz + 2;
   const int P = (ny + 2) * Z;
   const int slot = slots[blockIdx.x];
   T *base = pool + bv_offset(g, slot, var);
   auto load = [&](int i) {
      T *pl = ring + (i % 3) * P;
      for (int e = threadIdx.x; e < P; e += blockDim.x) {
         const int j = e / Z, k = e - j * Z;
         pl[e] = base[cell_offset(g, i, j, k)];
      }
   };
   load(0);
   load(1);
   for (int i = 1; i <= nx; i++) {
      load(i + 1);
      __syncthreads();
      const T *pm = ring + ((i - 1) % 3) * P, *pc = ring + (i % 3) * P,
              *pp = ring + ((i + 1) % 3) * P;
      for (int col = threadIdx.x; col < ny * nz; col += blockDim.x) {
         const int j = col / nz + 1, k = col - (j - 1) * nz + 1;
         const int e = j * Z + k;
         T out;
         if (ST == 7) {
            T w = pm[e] + pc[e - Z];
            w = w + pc[e - 1];
            w = w + pc[e];
            w = w + pc[e + 1];
            w = w + pc[e + Z];
            w = w + pp[e];
            out = div7(w);
         } else {
            auto S = [&](const T *pl) -> T {
               T s = pl[e - Z - 1] + pl[e - Z];
               s = s + pl[e - Z + 1];
               s = s + pl[e - 1];
               s = s + pl[e];
               s = s + pl[e + 1];
               s = s + pl[e + Z - 1];
               s = s + pl[e + Z];
               s = s + pl[e + Z + 1];
               return s;
            };
            out = div27((S(pm) + S(pc)) + S(pp));
         }
         base[cell_offset(g, i, j, k)] = out;
         if (zc && (k == 1 || k == nz))
            zc[zcache_at(g, slot, var, k == nz ? 1 : 0, i, j)] = out;
      }
      // the ring slot of plane i-1 is refilled with plane i+2 next
      __syncthreads();
   }
}

// The largest block the streaming kernel's ring fits (shared memory).
bool plain_stencil_fits(const Geom &g, size_t elem)
{
   return 3 * (size_t) (g.ny + 2) * (g.nz + 2) * elem <= kPlainRingBytes;
}

template <typename T, int ST, int BX, int BY, int BZ>
static void stencil_launch(T *pool, const Geom &g, const int32_t *slots,
                           int n, int var, int threads, size_t smem, T *zc,
                           cudaStream_t s)
{
   cudaFuncAttributes fa;
   if (cudaFuncGetAttributes(&fa, stencil_kernel<T, ST, BX, BY, BZ>) !=
          cudaSuccess ||
       (size_t) fa.maxDynamicSharedSizeBytes < smem)
      cudaFuncSetAttribute(stencil_kernel<T, ST, BX, BY, BZ>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int) smem);
   stencil_kernel<T, ST, BX, BY, BZ><<<n, threads, smem, s>>>(pool, g, slots,
                                                              var, zc);
}

template <typename T>
int launch_stencil(T *pool, const Geom &g, int stencil, const int32_t *slots,
                   int n, int var, T *zc, cudaStream_t s)
{
   if (n == 0)
      return 0;
   const size_t smem = (size_t) g.X * g.Y * plain_zs<T>(g.nz) * sizeof(T);
   int threads = g.ny * g.nz;
   threads = threads > 256 ? 256 : ((threads + 31) / 32) * 32;
   if (smem > kPlainTileBytes) {
      // too large to stage whole: stream the block through a plane ring
      const size_t ring = 3 * (size_t) (g.ny + 2) * (g.nz + 2) * sizeof(T);
      auto k7 = stencil_stream_kernel<T, 7>, k27 = stencil_stream_kernel<T, 27>;
      auto kern = stencil == 7 ? k7 : k27;
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int) ring);
      kern<<<n, threads, ring, s>>>(pool, g, slots, var, zc);
      return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
   }
   const int kind = dims_kind(g);
   // FP32 8^3 / 16^3: one thread per (4 i-planes, j-row, 4 k values)
   if (sizeof(T) == 4 && kind != 0)
      threads = (g.nx / 4) * g.ny * (g.nz / 4);
#define MAMR_PLAIN_ST(ST)                                                     \
   if (kind == 1)                                                             \
      stencil_launch<T, ST, 8, 8, 8>(pool, g, slots, n, var, threads, smem,   \
                                     zc, s);                                  \
   else if (kind == 2)                                                        \
      stencil_launch<T, ST, 16, 16, 16>(pool, g, slots, n, var, threads,      \
                                        smem, zc, s);                         \
   else                                                                       \
      stencil_launch<T, ST, 0, 0, 0>(pool, g, slots, n, var, threads, smem,   \
                                     zc, s)
   if (stencil == 7) {
      MAMR_PLAIN_ST(7);
   } else {
      MAMR_PLAIN_ST(27);
   }
#undef MAMR_PLAIN_ST
   return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

// ---------------------------------------------------------------------------
// Checksum, FP64: ref/check_sum.c:44-53 in exactly its order -- each block's
// interior summed serially with k fastest, then the block sums serially in
// sorted_list order.  One thread per block for the first pass.
__global__ void __launch_bounds__(128)
block_sums_fp64(const double *__restrict__ pool, Geom g,
                const int32_t *__restrict__ slots, int n, int var,
                double *__restrict__ partials)
{
   int b = blockIdx.x * blockDim.x + threadIdx.x;
   if (b >= n)
      return;
   const double *base = pool + bv_offset(g, slots[b], var);
   double s = 0.0;
   for (int i = 1; i <= g.nx; i++)
      for (int j = 1; j <= g.ny; j++) {
         const double *row = base + cell_offset(g, i, j, 1);
#pragma unroll 8
         for (int k = 0; k < g.nz; k++)
            s = s + row[k];
      }
   partials[b] = s;
}

__global__ void __launch_bounds__(256)
total_sum_fp64(const double *__restrict__ partials, int n,
               double *__restrict__ out)
{
   __shared__ double buf[2048];
   double s = 0.0;
   for (int base = 0; base < n; base += 2048) {
      int m = n - base < 2048 ? n - base : 2048;
      for (int e = threadIdx.x; e < m; e += blockDim.x)
         buf[e] = partials[base + e];
      __syncthreads();
      if (threadIdx.x == 0)
         for (int e = 0; e < m; e++)
            s = s + buf[e];
      __syncthreads();
   }
   if (threadIdx.x == 0)
      *out = s;
}

int launch_checksum_fp64(const double *pool, const Geom &g,
                         const int32_t *slots, int n, int var,
                         double *d_partials, double *d_out, cudaStream_t s)
{
   int launches = 0;
   if (n > 0) {
      block_sums_fp64<<<(n + 127) / 128, 128, 0, s>>>(pool, g, slots, n, var,
                                                       d_partials);
      launches++;
   }
   total_sum_fp64<<<1, 256, 0, s>>>(d_partials, n, d_out);
   launches++;
   return cudaPeekAtLastError() == cudaSuccess ? launches : -1;
}

// The same for every variable at once: one thread per (variable, block)
// chain, so the latency of the serial FP64 additions overlaps across all
// of them; then each variable's block sums serially in sorted_list order.
// Same additions in the same order as launch_checksum_fp64 per variable.
__global__ void __launch_bounds__(128)
block_sums_vars_fp64(const double *__restrict__ pool, Geom g,
                     const int32_t *__restrict__ slots, int n,
                     double *__restrict__ partials)
{
   const long long e = blockIdx.x * (long long) blockDim.x + threadIdx.x;
   if (e >= (long long) n * g.V)
      return;
   const int var = (int) (e / n), b = (int) (e - (long long) var * n);
   const double *base = pool + bv_offset(g, slots[b], var);
   double s = 0.0;
   for (int i = 1; i <= g.nx; i++)
      for (int j = 1; j <= g.ny; j++) {
         const double *row = base + cell_offset(g, i, j, 1);
#pragma unroll 8
         for (int k = 0; k < g.nz; k++)
            s = s + row[k];
      }
   partials[e] = s;
}

__global__ void total_sums_vars_fp64(const double *__restrict__ partials,
                                     int n, int V, double *__restrict__ sums)
{
   for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < V;
        v += gridDim.x * blockDim.x) {
      const double *p = partials + (size_t) v * n;
      double s = 0.0;
#pragma unroll 8
      for (int b = 0; b < n; b++)
         s = s + p[b];
      sums[v] = s;
   }
}

int launch_checksum_fp64_all(const double *pool, const Geom &g,
                             const int32_t *slots, int n, double *d_partials,
                             double *d_sums, cudaStream_t s)
{
   const long long m = (long long) n * g.V;
   int launches = 0;
   if (m > 0) {
      block_sums_vars_fp64<<<(unsigned) ((m + 127) / 128), 128, 0, s>>>(
         pool, g, slots, n, d_partials);
      launches++;
   }
   total_sums_vars_fp64<<<(g.V + 127) / 128, 128, 0, s>>>(d_partials, n, g.V,
                                                          d_sums);
   launches++;
   return cudaPeekAtLastError() == cudaSuccess ? launches : -1;
}

// Checksum, FP32: every interior cell as a multiple of 2^-52 (truncated
// toward zero), summed exactly in 128-bit two's complement.  Integer
// addition is associative, so the result does not depend on the order in
// which CTAs finish.
// This thread's share of one block-variable's interior terms, added into
// (lo, hi); the CTA's threads stride over the cells.  8^3 and 16^3 blocks
// read their interior rows (contiguous runs of nz values in the split
// layout) as 16-byte vectors with compile-time indexing.
template <int BX, int BY, int BZ>
__device__ __forceinline__ void interior_fixed52(const float *base,
                                                 const Geom &g,
                                                 unsigned long long &lo,
                                                 unsigned long long &hi,
                                                 bool &ok)
{
   Fixed52 part;
   if constexpr (BZ > 0 && BZ % 4 == 0) {
      constexpr int NQ = BZ / 4, Y = BY + 2, QUADS = BX * BY * NQ;
      for (int e = threadIdx.x, t = 1; e < QUADS; e += blockDim.x, t++) {
         const int q = e % NQ, rr = e / NQ;
         const int i = rr / BY + 1, j = rr % BY + 1;
         const float4 v = __ldg(
            reinterpret_cast<const float4 *>(base + (i * Y + j) * BZ) + q);
         fixed52_add(v.x, part);
         fixed52_add(v.y, part);
         fixed52_add(v.z, part);
         fixed52_add(v.w, part);
         if ((t & 63) == 0)                 // 256 terms
            fixed52_flush(part, lo, hi);
      }
   } else {
      const int cells = g.nx * g.ny * g.nz;
      for (int e = threadIdx.x, t = 1; e < cells; e += blockDim.x, t++) {
         int i = e / (g.ny * g.nz) + 1, r = e % (g.ny * g.nz);
         int j = r / g.nz + 1, k = r % g.nz + 1;
         fixed52_add(base[cell_offset(g, i, j, k)], part);
         if ((t & 255) == 0)
            fixed52_flush(part, lo, hi);
      }
   }
   ok &= fixed52_window(part);
   fixed52_flush(part, lo, hi);
}

template <int BX, int BY, int BZ>
__global__ void __launch_bounds__(256)
checksum_fp32_kernel(const float *__restrict__ pool, Geom g,
                     const int32_t *__restrict__ slots, int var,
                     unsigned long long *__restrict__ acc,
                     unsigned *__restrict__ err)
{
   const float *base = pool + bv_offset(g, slots[blockIdx.x], var);
   unsigned long long lo = 0, hi = 0;
   bool ok = true;
   interior_fixed52<BX, BY, BZ>(base, g, lo, hi, ok);
   if (!ok)
      atomicOr(err, ERR_FIXED_RANGE);
   block_acc128_flush(lo, hi, acc);
}

// Every variable at once: CTA (block, variable) adds into acc[2 * var];
// exact integer sums, so the grouping changes no bit.
template <int BX, int BY, int BZ>
__global__ void __launch_bounds__(256)
checksum_fp32_vars_kernel(const float *__restrict__ pool, Geom g,
                          const int32_t *__restrict__ slots,
                          unsigned long long *__restrict__ acc,
                          unsigned *__restrict__ err)
{
   const int var = blockIdx.y;
   const float *base = pool + bv_offset(g, slots[blockIdx.x], var);
   unsigned long long lo = 0, hi = 0;
   bool ok = true;
   interior_fixed52<BX, BY, BZ>(base, g, lo, hi, ok);
   if (!ok)
      atomicOr(err, ERR_FIXED_RANGE);
   block_acc128_flush(lo, hi, acc + 2 * var);
}

int launch_checksum_fp32_all(const float *pool, const Geom &g,
                             const int32_t *slots, int n,
                             unsigned long long *acc, unsigned *err,
                             cudaStream_t s)
{
   if (n == 0)
      return 0;
   const dim3 grid(n, g.V);
   switch (dims_kind(g)) {
   case 1:
      checksum_fp32_vars_kernel<8, 8, 8><<<grid, 128, 0, s>>>(pool, g, slots,
                                                             acc, err);
      break;
   case 2:
      checksum_fp32_vars_kernel<16, 16, 16><<<grid, 256, 0, s>>>(
         pool, g, slots, acc, err);
      break;
   default:
      checksum_fp32_vars_kernel<0, 0, 0><<<grid, 256, 0, s>>>(pool, g, slots,
                                                             acc, err);
   }
   return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

int launch_checksum_fp32(const float *pool, const Geom &g,
                         const int32_t *slots, int n, int var,
                         unsigned long long *acc, unsigned *err,
                         cudaStream_t s)
{
   if (n == 0)
      return 0;
   switch (dims_kind(g)) {
   case 1:
      checksum_fp32_kernel<8, 8, 8><<<n, 128, 0, s>>>(pool, g, slots, var,
                                                      acc, err);
      break;
   case 2:
      checksum_fp32_kernel<16, 16, 16><<<n, 256, 0, s>>>(pool, g, slots, var,
                                                         acc, err);
      break;
   default:
      checksum_fp32_kernel<0, 0, 0><<<n, 256, 0, s>>>(pool, g, slots, var,
                                                      acc, err);
   }
   return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

// ---------------------------------------------------------------------------
// FP32 checksum fallback.  A variable with any cell outside the fixed-point
// window takes the reference's summation order in FP64 with Neumaier
// compensation instead (ref/check_sum.c:44-53): each block's interior
// serially (k fastest) into s + c, rounded once, then the block values
// serially in sorted order, S + C rounded once.  flags[0] is the
// checksum's miss word (the checksum or stage kernel sets it); while it is
// clear the kernel returns at once, so the common case costs one empty
// launch.  One thread per (block, variable) forms the block's compensated
// sum into partials[v * n + b] and records in flags[1 + v] whether variable
// var0 + v has a cell outside the window; the CTA that finishes last (the
// counter flags[1 + nvar]) then adds the block values of each variable that
// missed and stores the result in its checksum slot under the fallback
// mark.
__global__ void __launch_bounds__(128)
fp32_fallback_kernel(const float *__restrict__ pool, Geom g,
                     const int32_t *__restrict__ slots, int n, int var0,
                     int nvar, unsigned *__restrict__ flags,
                     double *__restrict__ partials,
                     unsigned long long *__restrict__ acc)
{
   __shared__ bool last;
   if (*(volatile unsigned *) flags == 0)
      return;
   const long long items = (long long) n * nvar;
   for (long long q = blockIdx.x * (long long) blockDim.x + threadIdx.x;
        q < items; q += (long long) gridDim.x * blockDim.x) {
      const int v = (int) (q / n), b = (int) (q - (long long) v * n);
      const float *base = pool + bv_offset(g, slots[b], var0 + v);
      double s = 0.0, c = 0.0;
      bool miss = false;
      for (int i = 1; i <= g.nx; i++)
         for (int j = 1; j <= g.ny; j++)
            for (int k = 1; k <= g.nz; k++) {
               const float x = base[cell_offset(g, i, j, k)];
               const float a = fabsf(x);
               miss |= !(a < 1024.0f && (a >= 0x1p-52f || a == 0.0f));
               neumaier_add(s, c, (double) x);
            }
      partials[q] = s + c;
      if (miss)
         atomicOr(flags + 1 + v, 1u);
   }
   __threadfence();
   __syncthreads();
   if (threadIdx.x == 0)
      last = atomicAdd(flags + 1 + nvar, 1u) == gridDim.x - 1;
   __syncthreads();
   if (!last)
      return;
   __threadfence();
   for (int v = threadIdx.x; v < nvar; v += blockDim.x) {
      if (((volatile unsigned *) flags)[1 + v] == 0)
         continue;
      double s = 0.0, c = 0.0;
      for (int b = 0; b < n; b++)
         neumaier_add(s, c, ((volatile double *) partials)[(long long) v * n +
                                                           b]);
      acc[2 * v] = (unsigned long long) __double_as_longlong(s + c);
      acc[2 * v + 1] = kChecksumFallbackMark;
   }
}

int launch_fp32_checksum_fallback(const float *pool, const Geom &g,
                                  const int32_t *slots, int n, int var0,
                                  int nvar, unsigned *flags,
                                  double *partials, unsigned long long *acc,
                                  cudaStream_t s)
{
   if (n == 0 || nvar == 0)
      return 0;
   // one CTA per SM: the common case (nothing missed) is a single short
   // wave; the rare recomputation strides over the items
   int dev = 0, sms = 1;
   cudaGetDevice(&dev);
   cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
   const long long items = (long long) n * nvar;
   const unsigned grid = (unsigned) std::max<long long>(
      1, std::min<long long>((items + 127) / 128, sms));
   fp32_fallback_kernel<<<grid, 128, 0, s>>>(pool, g, slots, n, var0, nvar,
                                             flags, partials, acc);
   return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

// ---------------------------------------------------------------------------
// Copies the interior cells of whole blocks (all variables) from pool slots
// to consecutive staging entries, at the same offsets: the split and
// consolidation kernels read nothing else from a staged block.  In the
// device layout the interior rows j = 1..ny of i-plane i are one run of
// ny*nz values from row_offset(i, 1), so a block-variable is nx runs.  One
// CTA row per block, 16-byte vectors when nz values fill whole vectors.
template <typename T>
__global__ void __launch_bounds__(256)
stage_blocks_kernel(T *__restrict__ stage, const T *__restrict__ pool, Geom g,
                    const int32_t *__restrict__ slots)
{
   const T *src = pool + bv_offset(g, slots[blockIdx.y], 0);
   T *dst = stage + bv_offset(g, blockIdx.y, 0);
   const long long step = (long long) gridDim.x * blockDim.x;
   const long long t0 = (long long) blockIdx.x * blockDim.x + threadIdx.x;
   const long long run = (long long) g.ny * g.nz;
   const long long runs = (long long) g.V * g.nx;
   if ((g.nz * sizeof(T)) % 16 == 0) {
      const long long rv = run * (long long) sizeof(T) / 16;   // vectors
      constexpr int VW = 16 / sizeof(T);
      for (long long e = t0; e < runs * rv; e += step) {
         const long long q = e / rv, w = e - q * rv;
         const int var = (int) (q / g.nx), i = (int) (q - (long long) var *
                                                      g.nx) + 1;
         const long long off = var * g.bv + row_offset(g, i, 1) + w * VW;
         *reinterpret_cast<uint4 *>(dst + off) =
            __ldg(reinterpret_cast<const uint4 *>(src + off));
      }
   } else {
      for (long long e = t0; e < runs * run; e += step) {
         const long long q = e / run, w = e - q * run;
         const int var = (int) (q / g.nx), i = (int) (q - (long long) var *
                                                      g.nx) + 1;
         const long long off = var * g.bv + row_offset(g, i, 1) + w;
         dst[off] = src[off];
      }
   }
}

template <typename T>
int launch_stage_blocks(T *stage, const T *pool, const Geom &g,
                        const int32_t *slots, int n, cudaStream_t s)
{
   if (n == 0)
      return 0;
   long long vec = ((long long) g.V * g.nx * g.ny * g.nz * sizeof(T) + 15) /
                   16;
   int gx = (int) std::min<long long>((vec + 255) / 256, 64);
   stage_blocks_kernel<T><<<dim3(gx, n), 256, 0, s>>>(stage, pool, g, slots);
   return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

// ---------------------------------------------------------------------------
// Host layout [n][V][X][Y][Z] doubles <-> pool slots.
//
// Upload: the values are read as 16-byte pairs (rows start on 16 bytes: Z
// is even, so a pair never straddles two rows), consecutive threads taking
// consecutive pairs and each thread four pairs a grid stride apart in
// flight -- enough bytes moving when the values are read in place from
// pinned host memory over the host link.
template <typename T>
__global__ void upload_kernel(T *__restrict__ pool, Geom g,
                              const int32_t *__restrict__ slots,
                              long long n_pairs,
                              const double *__restrict__ dense)
{
   const int XY = g.X * g.Y, HZ = g.Z / 2;
   const double2 *src = reinterpret_cast<const double2 *>(dense);
   const long long stride = (long long) gridDim.x * blockDim.x;
   auto put = [&](long long pr, double2 v) {
      const long long row = pr / HZ;
      const int k = 2 * (int) (pr - row * HZ);
      const long long bvi = row / XY;
      const int r = (int) (row - bvi * XY);
      const int b = (int) (bvi / g.V), var = (int) (bvi - (long long) b * g.V);
      const int i = r / g.Y, j = r - i * g.Y;
      T *base = pool + bv_offset(g, slots[b], var);
      base[cell_offset(g, i, j, k)] = (T) v.x;
      base[cell_offset(g, i, j, k + 1)] = (T) v.y;
   };
   for (long long p = blockIdx.x * (long long) blockDim.x + threadIdx.x;
        p < n_pairs; p += 4 * stride) {
      double2 v[4];
#pragma unroll
      for (int u = 0; u < 4; u++)
         if (p + u * stride < n_pairs)
            v[u] = src[p + u * stride];
#pragma unroll
      for (int u = 0; u < 4; u++)
         if (p + u * stride < n_pairs)
            put(p + u * stride, v[u]);
   }
}

template <typename T>
__global__ void download_kernel(const T *__restrict__ pool, Geom g,
                                const int32_t *__restrict__ slots,
                                long long total, double *__restrict__ dense)
{
   for (long long e = blockIdx.x * (long long) blockDim.x + threadIdx.x;
        e < total; e += (long long) gridDim.x * blockDim.x) {
      long long row = e / g.Z;
      int k = (int) (e - row * g.Z);
      long long bvi = row / (g.X * g.Y);
      int r = (int) (row - bvi * (g.X * g.Y));
      int b = (int) (bvi / g.V), var = (int) (bvi - (long long) b * g.V);
      int i = r / g.Y, j = r - i * g.Y;
      dense[e] = (double) pool[bv_offset(g, slots[b], var) +
                               cell_offset(g, i, j, k)];
   }
}

template <typename T>
int launch_upload(T *pool, const Geom &g, const int32_t *slots, int n,
                  const double *dense, cudaStream_t s)
{
   const long long pairs = (long long) n * g.V * g.X * g.Y * (g.Z / 2);
   if (pairs == 0)
      return 0;
   if ((reinterpret_cast<uintptr_t>(dense) & 15) || (g.Z & 1))
      return -1;   // the 16-byte pairs need both
   long long blocks = (pairs + 1023) / 1024;
   upload_kernel<T><<<(int) (blocks < 152 * 16 ? blocks : 152 * 16), 256, 0,
                      s>>>(pool, g, slots, pairs, dense);
   return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

template <typename T>
int launch_download(const T *pool, const Geom &g, const int32_t *slots,
                    int n, double *dense, cudaStream_t s)
{
   long long total = (long long) n * g.V * g.X * g.Y * g.Z;
   if (total == 0)
      return 0;
   long long blocks = (total + 255) / 256;
   download_kernel<T><<<(int) (blocks < 152 * 64 ? blocks : 152 * 64), 256,
                        0, s>>>(pool, g, slots, total, dense);
   return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

#define INSTANTIATE(T)                                                        \
   template int launch_comm_dir<T>(T *, const Geom &, int, int, int,          \
                                   const DirTasks &, int, int, const T *,     \
                                   cudaStream_t);                             \
   template int launch_stencil<T>(T *, const Geom &, int, const int32_t *,    \
                                  int, int, T *, cudaStream_t);               \
   template int launch_stage_blocks<T>(T *, const T *, const Geom &,          \
                                       const int32_t *, int, cudaStream_t);   \
   template int launch_upload<T>(T *, const Geom &, const int32_t *, int,     \
                                 const double *, cudaStream_t);               \
   template int launch_download<T>(const T *, const Geom &, const int32_t *,  \
                                   int, double *, cudaStream_t);
INSTANTIATE(double)
INSTANTIATE(float)

}  // namespace mamr
