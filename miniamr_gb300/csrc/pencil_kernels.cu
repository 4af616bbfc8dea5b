// Pencil stage kernel for single-level meshes of 16^3-cell blocks.
//
// One CTA walks a pencil -- the column of blocks along z at one (x, y) of
// the block lattice -- for one variable, keeping a ring of three tiles in
// shared memory: tile s (being updated), s+1 (loaded, its k = 1 plane is
// tile s's upper ghost plane) and s+2 (in flight, cp.async).  The ghost
// planes normal to z -- including their x/y edges and corners -- therefore
// come from neighbouring tiles already on chip; only the x and y face rows
// (and, for the 27-point stencil, the four z-running edge rows) are fetched
// from the neighbouring pencils, as 64-byte rows that those pencils' own
// CTAs read at about the same time, so they hit in L2.
//
// Shared-memory traffic bounds the FP32 kernel, so the tile is laid out
// and walked to keep it low: every thread of an FP32 CTA updates two
// j-rows of four k values on four i-planes (four rows loaded per two
// output rows).  Each i-plane of a tile is padded by 16 bytes, which puts
// rows four planes apart in opposite halves of a 128-byte bank span; an
// 8-lane phase of a warp pairs such rows, so the warp's 16-byte row loads
// are free of bank conflicts while every address stays a per-thread base
// plus a constant.
//
// Values and operation order are exactly those of the plain path: ghosts
// as comm() leaves them on a single-level mesh (axis-by-axis neighbour or
// reflection), the reference's summation order, correctly rounded
// division, and the FP32 checksum as exact 128-bit fixed point.
#include <algorithm>
#include <vector>

#include <cuda.h>
#include <mutex>

#include "batched.h"
#include "arith.cuh"
#include "cp_async.cuh"
#include "tma.cuh"

namespace mamr {

namespace {

constexpr int NB = 16;              // cells per block edge
constexpr int G = NB + 2;           // with ghosts
constexpr int RS = NB;              // shared row: the 16 interior k values
constexpr int KC = G * G;           // rows of a tile (i, j incl. ghosts)

// Tile geometry in elements of T: row (i, j) starts at joff() + i * PW +
// j * RS.  TM = 0 (rows filled by cp.async): planes padded by 16 bytes.
// TM = 1 (interior planes filled by the tensor engine, FP32): planes of 20
// row slots (1280 bytes, a multiple of 128) with row j in slot j + 1, so
// that each plane's 16 interior rows start on a 128-byte boundary, as a
// bulk tensor copy's shared-memory destination must.
template <typename T, int TM = 0> struct TileGeom {
   static constexpr int PW = TM ? 20 * RS : G * RS + 16 / (int) sizeof(T);
   static constexpr int TILE = G * PW;
   __host__ __device__ static constexpr int joff() { return TM ? RS : 0; }
};
// Offset of row (i, j) from row (0, 0).
template <typename T, int TM = 0>
__device__ __forceinline__ int trow(int i, int j)
{
   return i * TileGeom<T, TM>::PW + j * RS;
}

// Work split: JP j-rows and IH i-planes per thread (JP x IH = 1x4, 2x4 or
// 1x8; the autotuner picks), so 1024 / (JP * IH) threads per tile; FP32
// tiles allow three CTAs per SM, FP64 one.  More planes per thread share
// each 9-term plane sum among more outputs (IH + 2 sums per IH planes).
template <typename T, int JP, int IH> struct Shape {
   static constexpr int THREADS = 1024 / (JP * IH);
   static constexpr int CTAS = sizeof(T) == 4 ? 3 : 1;
};

// Four consecutive k values (16-byte aligned).
template <typename T> struct Quad;
template <> struct Quad<float> {
   __device__ static void ld(const float *p, float (&v)[4])
   {
      float4 q = *reinterpret_cast<const float4 *>(p);
      v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
   }
   __device__ static void st(float *p, const float (&v)[4])
   {
      *reinterpret_cast<float4 *>(p) = make_float4(v[0], v[1], v[2], v[3]);
   }
};
template <> struct Quad<double> {
   __device__ static void ld(const double *p, double (&v)[4])
   {
      double2 a = *reinterpret_cast<const double2 *>(p);
      double2 b = *reinterpret_cast<const double2 *>(p + 2);
      v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
   }
   __device__ static void st(double *p, const double (&v)[4])
   {
      *reinterpret_cast<double2 *>(p) = make_double2(v[0], v[1]);
      *reinterpret_cast<double2 *>(p + 2) = make_double2(v[2], v[3]);
   }
};

// Ring of three tiles, two lower z-ghost columns (tiles s and s+1) and
// one upper column, one element per row; the upper column sits an odd
// number of words after the lower ones so that the two read in one
// instruction use disjoint banks.  After a 128-byte alignment pad.
template <typename T, int TM = 0>
constexpr size_t pencil_smem_bytes()
{
   // + the ring's three 8-byte barriers of the tensor-copy form
   return (size_t) (3 * TileGeom<T, TM>::TILE + 3 * KC + 1) * sizeof(T) +
          128 + (TM ? 32 : 0);
}

constexpr int DESC = sizeof(TileDesc) / sizeof(int32_t);

// Global row (i, j) of a 16^3 block-variable (split layout: rows of the
// 16 interior k values, ghost rows included).
__device__ __forceinline__ int grow(int i, int j) { return (i * G + j) * NB; }

// Queues the cp.async copies of tile `s` of the pencil into ring buffer t:
// the interior rows, the four x/y face rows (neighbour or reflection) and,
// for 27 points, the four z-running edge rows.  A thread's chunks sit at
// fixed (j, k) positions, so every address is a per-tile base plus a
// constant.
template <typename T, int ST, int THREADS>
__device__ __forceinline__ void issue_tile(const T *__restrict__ src,
                                           const Geom &g, const TileDesc *it,
                                           int var, T *t)
{
   constexpr int VW = 16 / (int) sizeof(T);   // elements per 16 bytes
   constexpr int CPR = NB / VW;               // 16-byte chunks per row
   constexpr int RPP = NB * CPR;              // chunks per 16-row plane
   constexpr int PW = TileGeom<T>::PW;
   constexpr int PSTEP = THREADS / RPP;       // planes per sweep
   static_assert(THREADS % RPP == 0, "thread count vs plane chunks");
   const int tid = threadIdx.x;
   const int q = tid % CPR, a = (tid / CPR) % NB + 1, p0 = tid / RPP;
   const int slot = it->slot, bmask = it->bmask;
   const T *own = src + bv_offset(g, slot, var);
   {
      const T *from = own + grow(p0 + 1, a) + q * VW;
      T *to = t + trow<T>(p0 + 1, a) + q * VW;
#pragma unroll
      for (int m = 0; m < NB / PSTEP; m++)
         cp_async16(to + m * PSTEP * PW, from + m * PSTEP * grow(1, 0));
   }
#pragma unroll
   for (int m = 0; m < 4 / PSTEP; m++) {
      const int f = p0 + m * PSTEP;            // face W, E, S, N
      const bool bnd = (bmask >> f) & 1;
      // nb9 index of the W, E, S, N neighbour: 3, 5, 1, 7
      const int nbi = (f < 2) ? (f == 0 ? 3 : 5) : (f == 2 ? 1 : 7);
      const T *blk = bnd ? own : src + bv_offset(g, it->nb9[nbi], var);
      const bool low = (f & 1) == 0;
      // neighbour: its plane next to us; boundary: our own first plane
      const int sp = bnd ? (low ? 1 : NB) : (low ? NB : 1);
      const int gp = low ? 0 : G - 1;
      const int from = f < 2 ? grow(sp, a) : grow(a, sp);
      const int to = f < 2 ? trow<T>(gp, a) : trow<T>(a, gp);
      cp_async16(t + to + q * VW, blk + from + q * VW);
   }
   if (ST == 27 && tid < 4 * CPR) {
      const int e = tid / CPR;
      const int gi = (e & 1) ? G - 1 : 0, gj = (e & 2) ? G - 1 : 0;
      int dx = (e & 1) ? 1 : -1, dy = (e & 2) ? 1 : -1, si, sj;
      if (bmask & (1 << ((e & 1) ? 1 : 0))) { si = (e & 1) ? NB : 1; dx = 0; }
      else si = (e & 1) ? 1 : NB;
      if (bmask & (1 << ((e & 2) ? 3 : 2))) { sj = (e & 2) ? NB : 1; dy = 0; }
      else sj = (e & 2) ? 1 : NB;
      const int nb = it->nb9[(dx + 1) + 3 * (dy + 1)];
      cp_async16(t + trow<T>(gi, gj) + q * VW,
                 src + bv_offset(g, nb, var) + grow(si, sj) + q * VW);
   }
   cp_async_commit();
}

// Row (i, j) of tile t as six k values: k-1 .. k+4 around the thread's
// quad k .. k+3 (k = 4*kq + 1).  The four lanes of a row hold the row's 16
// values between them; the outer neighbours k-1 and k+4 come from the
// adjacent lanes by shuffle, and from the z ghost columns at the row ends.
// Every lane of the warp must call this together.
// `tq` is the thread's quad in tile t (row 0 of plane 0 plus 4*kq) and
// `eg` its ghost column (the lower column for kq < 3, the upper for kq = 3).
template <typename T, int TM>
__device__ __forceinline__ void row6(const T *tq, const T *eg, int i, int j,
                                     int kq, T (&r)[6])
{
   T v[4];
   Quad<T>::ld(tq + trow<T, TM>(i, j), v);
   const T left = __shfl_up_sync(0xffffffffu, v[3], 1);
   const T right = __shfl_down_sync(0xffffffffu, v[0], 1);
   const T edge = eg[i * G + j];
   r[0] = kq == 0 ? edge : left;
   r[1] = v[0]; r[2] = v[1]; r[3] = v[2]; r[4] = v[3];
   r[5] = kq == 3 ? edge : right;
}

template <typename T>
__device__ __forceinline__ void checksum4(const T (&out)[4], bool &ok,
                                          Fixed52 &part)
{
#pragma unroll
   for (int m = 0; m < 4; m++)
      fixed52_add((float) out[m], part);
}

__device__ __forceinline__ float div_rn_inline(float x, float c)
{
   return __fdiv_rn(x, c);
}
__device__ __forceinline__ double div_rn_inline(double x, double c)
{
   return __ddiv_rn(x, c);
}

// Accumulators of a thread's pass over its outputs of a tile.
struct PassState {
   bool slow;                       // some sum fell outside div_window
   bool ok;                         // every FP32 checksum term in range
   Fixed52 part;                    // this tile's FP32 checksum terms
   unsigned long long lo, hi;       // FP32 fixed-point checksum
};

// Quotients of four sums, stored at p (global).  The fast pass stores the
// three-step quotient and records whether any sum lay outside the window
// where it is exact; the fix-up pass (run only then) stores the IEEE
// quotient for those sums and moves their checksum terms accordingly.
template <int C, bool FIX, typename T>
__device__ __forceinline__ void emit4(const T (&w)[4], T *p, int do_cs,
                                      PassState &st)
{
   if (!FIX) {
      T q[4];
#pragma unroll
      for (int m = 0; m < 4; m++) {
         q[m] = div_fast<C>(w[m]);
         st.slow |= !div_window(w[m]);
      }
      Quad<T>::st(p, q);
      if (sizeof(T) == 4 && do_cs)
         checksum4(q, st.ok, st.part);
   } else {
#pragma unroll
      for (int m = 0; m < 4; m++)
         if (!div_window(w[m])) {
            const T qf = div_fast<C>(w[m]);
            const T qc = div_rn_inline(w[m], (T) C);
            p[m] = qc;
            if (sizeof(T) == 4 && do_cs) {
               fixed52_add((float) qc, st.part);
               fixed52_add((float) qf, st.part, true);
            }
         }
   }
}

// One pass over the thread's outputs of a tile: JP rows (jrow ..) of four
// k values on planes 4*ih+1 .. 4*ih+4.  `tq` is the thread's quad of row
// (4*ih, jrow) in the tile, `eg` its ghost column from the same row, `d`
// the matching global position.  Every lane of the warp runs it together.
template <typename T, int ST, int JP, int IH, bool FIX, int TM>
__device__ __forceinline__ void tile_pass(const T *tq, const T *eg, T *d,
                                          int kq, int do_cs, PassState &st)
{
   if (ST == 7) {
      // (i-1, j) quads and (i, j) rows of the thread's JP rows
      T am[JP][4], r[JP][6];
#pragma unroll
      for (int jj = 0; jj < JP; jj++) {
         Quad<T>::ld(tq + trow<T, TM>(0, jj), am[jj]);
         row6<T, TM>(tq, eg, 1, jj, kq, r[jj]);
      }
#pragma unroll
      for (int ii = 1; ii <= IH; ii++) {
         T qm[4], qp[4], c[JP][6];
         Quad<T>::ld(tq + trow<T, TM>(ii, -1), qm);
         Quad<T>::ld(tq + trow<T, TM>(ii, JP), qp);
#pragma unroll
         for (int jj = 0; jj < JP; jj++)
            row6<T, TM>(tq, eg, ii + 1, jj, kq, c[jj]);
#pragma unroll
         for (int jj = 0; jj < JP; jj++) {
            T w[4];
#pragma unroll
            for (int m = 0; m < 4; m++) {
               const T sm = jj == 0 ? qm[m] : r[jj > 0 ? jj - 1 : 0][m + 1];
               const T sp = jj == JP - 1 ? qp[m]
                                         : r[jj < JP - 1 ? jj + 1 : 0][m + 1];
               T v = am[jj][m] + sm;
               v = v + r[jj][m];
               v = v + r[jj][m + 1];
               v = v + r[jj][m + 2];
               v = v + sp;
               v = v + c[jj][m + 1];
               w[m] = v;
            }
            emit4<7, FIX>(w, d + grow(ii, jj), do_cs, st);
         }
#pragma unroll
         for (int jj = 0; jj < JP; jj++) {
#pragma unroll
            for (int m = 0; m < 4; m++)
               am[jj][m] = r[jj][m + 1];
#pragma unroll
            for (int m = 0; m < 6; m++)
               r[jj][m] = c[jj][m];
         }
      }
   } else {
      // S(p): the reference's 9-term sum on plane p, for the thread's JP
      // rows and 4 k values
      auto S = [&](int pl, T (&s4)[JP][4]) {
         T rw[JP + 2][6];
#pragma unroll
         for (int dd = 0; dd < JP + 2; dd++)
            row6<T, TM>(tq, eg, pl, dd - 1, kq, rw[dd]);
#pragma unroll
         for (int jj = 0; jj < JP; jj++)
#pragma unroll
            for (int m = 0; m < 4; m++) {
               const T *a = rw[jj], *b = rw[jj + 1], *c = rw[jj + 2];
               T v = a[m] + a[m + 1];
               v = v + a[m + 2];
               v = v + b[m];
               v = v + b[m + 1];
               v = v + b[m + 2];
               v = v + c[m];
               v = v + c[m + 1];
               v = v + c[m + 2];
               s4[jj][m] = v;
            }
      };
      T s0[JP][4], s1[JP][4], s2[JP][4];
      S(0, s0);
      S(1, s1);
#pragma unroll
      for (int ii = 1; ii <= IH; ii++) {
         S(ii + 1, s2);
#pragma unroll
         for (int jj = 0; jj < JP; jj++) {
            T w[4];
#pragma unroll
            for (int m = 0; m < 4; m++)
               w[m] = (s0[jj][m] + s1[jj][m]) + s2[jj][m];
            emit4<27, FIX>(w, d + grow(ii, jj), do_cs, st);
         }
#pragma unroll
         for (int jj = 0; jj < JP; jj++)
#pragma unroll
            for (int m = 0; m < 4; m++) {
               s0[jj][m] = s1[jj][m];
               s1[jj][m] = s2[jj][m];
            }
      }
   }
}

// The fix-up pass out of line, so that its registers do not weigh on the
// fast pass; called only when a warp met a sum outside the window.
template <typename T, int ST, int JP, int IH, int TM>
__device__ __noinline__ PassState tile_fix(const T *tq, const T *eg, T *d,
                                           int kq, int do_cs, PassState st)
{
   tile_pass<T, ST, JP, IH, true, TM>(tq, eg, d, kq, do_cs, st);
   return st;
}

}  // namespace

template <typename T, int ST, int JP, int IH>
__global__ void __launch_bounds__(Shape<T, JP, IH>::THREADS,
                                  Shape<T, JP, IH>::CTAS)
pencil_stage_kernel(const T *__restrict__ src, T *__restrict__ dst, Geom g,
                    const TileDesc *__restrict__ chain,
                    const int2 *__restrict__ pencils, int n_pencils,
                    int write_ghosts, int do_cs,
                    unsigned long long *__restrict__ acc,
                    unsigned *__restrict__ err)
{
   constexpr int THREADS = Shape<T, JP, IH>::THREADS;
   extern __shared__ __align__(16) unsigned char smem_raw[];
   __shared__ TileDesc s_desc[PENCIL_MAX];
   T *tiles = reinterpret_cast<T *>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~(uintptr_t) 127);
   constexpr int TILE = TileGeom<T>::TILE;
   T *klos = tiles + 3 * TILE;          // lower columns of tiles s, s+1
   T *khi = klos + 2 * KC + 1;          // upper column of tile s
   const int tid = threadIdx.x, lane = tid & 31;
   // Lanes: kq fastest.  For two rows per thread, lane bit 2 selects the
   // i-plane group (4 planes apart) and bits 3-4 the row pair, so an
   // 8-lane phase loads two rows in opposite halves of a bank span.
   const int kq = lane & 3;
   const int jrow = JP == 2
      ? 2 * (((lane >> 3) & 3) + 4 * ((tid >> 5) & 1)) + 1
      : ((tid >> 2) & 15) + 1;
   const int ih = JP == 2 ? ((lane >> 2) & 1) + 2 * (tid >> 6) : tid >> 6;
   static_assert(JP == 1 || IH == 4, "two rows per thread need 4 planes");

   // the ghost-column rows this thread copies each step, walked i fastest
   // (fewer bank conflicts): (tile offset << 9) | column index
   constexpr int NFILL = (KC + THREADS - 1) / THREADS;
   int fill[NFILL];
#pragma unroll
   for (int m = 0; m < NFILL; m++) {
      const int q = tid + m * THREADS, i = q % G, j = q / G;
      fill[m] = q < KC ? (trow<T>(i, j) << 9) | (i * G + j) : -1;
   }

   for (int w = blockIdx.x; w < n_pencils * g.V; w += gridDim.x) {
      const int var = w / n_pencils, p = w - var * n_pencils;
      const int2 pc = pencils[p];
      const int len = pc.y;
      {
         const int32_t *from = reinterpret_cast<const int32_t *>(chain + pc.x);
         int32_t *to = reinterpret_cast<int32_t *>(s_desc);
         for (int q = tid; q < len * DESC; q += THREADS)
            to[q] = from[q];
      }
      __syncthreads();
      issue_tile<T, ST, THREADS>(src, g, s_desc, var, tiles);
      if (len > 1)
         issue_tile<T, ST, THREADS>(src, g, s_desc + 1, var, tiles + TILE);
      PassState st;
      st.ok = true;
      st.lo = st.hi = 0;
      for (int s = 0; s < len; s++) {
         const T *t = tiles + (s % 3) * TILE;
         const T *tn = tiles + ((s + 1) % 3) * TILE;
         T *kcur = klos + (s & 1) * KC;
         T *knext = klos + ((s + 1) & 1) * KC;
         cp_async_wait_all();
         __syncthreads();
         // z ghost columns: upper of tile s = tile s+1's k = 1 (our own
         // k = 16 at the top); lower of tile s+1 = our k = 16; the bottom
         // tile reflects its own k = 1
#pragma unroll
         for (int m = 0; m < NFILL; m++) {
            if (fill[m] < 0)
               continue;
            const int r = fill[m] >> 9, e = fill[m] & 511;
            const T top = t[r + NB - 1];
            khi[e] = s + 1 < len ? tn[r] : top;
            if (s + 1 < len)
               knext[e] = top;
            if (s == 0)
               kcur[e] = t[r];
         }
         __syncthreads();
         if (s + 2 < len)
            issue_tile<T, ST, THREADS>(src, g, s_desc + s + 2, var,
                                       tiles + ((s + 2) % 3) * TILE);
         // the thread's quad of row (4*ih, jrow) and its ghost column
         const T *tq = t + trow<T>(IH * ih, jrow) + 4 * kq;
         const T *eg = (kq == 3 ? khi : kcur) + IH * ih * G + jrow;
         const int slot = s_desc[s].slot;
         T *d = dst + bv_offset(g, slot, var) + grow(IH * ih, jrow) + 4 * kq;
         st.slow = false;
         tile_pass<T, ST, JP, IH, false, 0>(tq, eg, d, kq, do_cs, st);
         if (__any_sync(0xffffffffu, st.slow))
            st = tile_fix<T, ST, JP, IH, 0>(tq, eg, d, kq, do_cs, st);
         if (sizeof(T) == 4 && do_cs)
            fixed52_flush(st.part, st.lo, st.hi);
         if (write_ghosts) {
            T *base = dst + bv_offset(g, slot, var);
            // the ghost cells comm() writes: face interiors for 7 points,
            // the whole shell for 27 points
            const int n_shell = G * G * G - NB * NB * NB;
            for (int e = tid; e < n_shell; e += THREADS) {
               // enumerate the shell: planes i = 0 and G-1 entirely, then
               // rows j = 0 and G-1 of the inner planes, then k = 0, G-1
               int gi, gj, gk;
               if (e < 2 * G * G) {
                  gi = e < G * G ? 0 : G - 1;
                  const int r = e % (G * G);
                  gj = r / G; gk = r % G;
               } else if (e < 2 * G * G + 2 * NB * G) {
                  const int r = e - 2 * G * G;
                  gj = r < NB * G ? 0 : G - 1;
                  const int r2 = r % (NB * G);
                  gi = r2 / G + 1; gk = r2 % G;
               } else {
                  const int r = e - 2 * G * G - 2 * NB * G;
                  gk = r < NB * NB ? 0 : G - 1;
                  const int r2 = r % (NB * NB);
                  gi = r2 / NB + 1; gj = r2 % NB + 1;
               }
               const int outside = (gi == 0 || gi == G - 1) +
                                   (gj == 0 || gj == G - 1) +
                                   (gk == 0 || gk == G - 1);
               if (ST == 7 && outside != 1)
                  continue;
               const int ee = gi * G + gj;
               const T v = gk == 0 ? kcur[ee]
                         : (gk == G - 1 ? khi[ee]
                                        : t[trow<T>(gi, gj) + gk - 1]);
               base[cell_offset(g, gi, gj, gk)] = v;
            }
         }
      }
      if (sizeof(T) == 4 && do_cs) {
         if (!st.ok || !fixed52_window(st.part))
            atomicOr(err, ERR_FIXED_RANGE);
         block_acc128_flush(st.lo, st.hi, acc + 2 * var);
      }
      __syncthreads();
   }
}

// ---- the tensor-copy form (FP32, one j-row per thread) -------------------
//
// The same walk, update and ghost handling; only the filling of a tile
// differs: its 16 interior planes and the two x-face planes (each 16 rows
// of 64 bytes, contiguous in the pool and in the tile) arrive by bulk
// tensor copies (cp.async.bulk.tensor, 18 per tile, issued by one warp)
// that complete on the ring slot's mbarrier, and only the y-face rows and
// the 27-point z-running edge rows remain per-thread 16-byte copies.  The
// pool is the 4-d tensor (k: 16, j: 18, i: 18, block-variable) of the
// split layout (rows of 64 bytes, planes of 1152 bytes, block-variables bv
// elements apart); a box is one plane's 16 interior rows.

__device__ __forceinline__ void tma_plane(float *dst, const CUtensorMap *tm,
                                          int i, int bvi, unsigned bar)
{
   const unsigned d = (unsigned) __cvta_generic_to_shared(dst);
   asm volatile("cp.async.bulk.tensor.4d.shared::cluster.global.tile"
                ".mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
                "[%6];"
                ::"r"(d), "l"(reinterpret_cast<unsigned long long>(tm)),
                "r"(0), "r"(1), "r"(i), "r"(bvi), "r"(bar)
                : "memory");
}

// Bytes one tile's tensor copies deliver: 18 planes of 16 rows x 64 bytes.
constexpr unsigned kTmaTileBytes = 18u * NB * NB * 4u;

template <int ST, int THREADS>
__device__ __forceinline__ void issue_tile_tma(const CUtensorMap *tm,
                                               const float *__restrict__ src,
                                               const Geom &g,
                                               const TileDesc *it, int var,
                                               float *t, unsigned bar)
{
   using TG = TileGeom<float, 1>;
   constexpr int VW = 4, CPR = NB / VW;
   const int tid = threadIdx.x;
   const int slot = it->slot, bmask = it->bmask;
   if (tid < 32) {
      if (tid == 0)
         asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], "
                      "%1;" ::"r"(bar), "r"(kTmaTileBytes)
                      : "memory");
      __syncwarp();
      if (tid < NB) {
         tma_plane(t + TG::joff() + trow<float, 1>(tid + 1, 1), tm, tid + 1,
                   slot * g.V + var, bar);
      } else if (tid < NB + 2) {
         // x faces: the W / E neighbour's near plane, or (boundary) this
         // block's own first / last plane
         const int f = tid - NB;
         const bool low = f == 0, bnd = (bmask >> f) & 1;
         const int sp = bnd ? (low ? 1 : NB) : (low ? NB : 1);
         const int nb = bnd ? slot : it->nb9[low ? 3 : 5];
         tma_plane(t + TG::joff() + trow<float, 1>(low ? 0 : G - 1, 1), tm, sp,
                   nb * g.V + var, bar);
      }
   }
   // y faces S, N: 16 rows each, as 16-byte copies
   const float *own = src + bv_offset(g, slot, var);
   for (int c = tid; c < 2 * NB * CPR; c += THREADS) {
      const int f = 2 + c / (NB * CPR), r = c % (NB * CPR);
      const int a = r / CPR + 1, q = r % CPR;
      const bool low = f == 2, bnd = (bmask >> f) & 1;
      const float *blk = bnd ? own
                             : src + bv_offset(g, it->nb9[low ? 1 : 7], var);
      const int sp = bnd ? (low ? 1 : NB) : (low ? NB : 1);
      cp_async16(t + TG::joff() + trow<float, 1>(a, low ? 0 : G - 1) + q * VW,
                 blk + grow(a, sp) + q * VW);
   }
   if (ST == 27 && tid < 4 * CPR) {
      const int e = tid / CPR, q = tid % CPR;
      const int gi = (e & 1) ? G - 1 : 0, gj = (e & 2) ? G - 1 : 0;
      int dx = (e & 1) ? 1 : -1, dy = (e & 2) ? 1 : -1, si, sj;
      if (bmask & (1 << ((e & 1) ? 1 : 0))) { si = (e & 1) ? NB : 1; dx = 0; }
      else si = (e & 1) ? 1 : NB;
      if (bmask & (1 << ((e & 2) ? 3 : 2))) { sj = (e & 2) ? NB : 1; dy = 0; }
      else sj = (e & 2) ? 1 : NB;
      const int nb = it->nb9[(dx + 1) + 3 * (dy + 1)];
      cp_async16(t + TG::joff() + trow<float, 1>(gi, gj) + q * VW,
                 src + bv_offset(g, nb, var) + grow(si, sj) + q * VW);
   }
   cp_async_commit();
}

template <int ST, int IH>
__global__ void __launch_bounds__(1024 / IH, 3)
pencil_tma_kernel(const __grid_constant__ CUtensorMap tm,
                  const float *__restrict__ src, float *__restrict__ dst,
                  Geom g, const TileDesc *__restrict__ chain,
                  const int2 *__restrict__ pencils, int n_pencils,
                  int write_ghosts, int do_cs,
                  unsigned long long *__restrict__ acc,
                  unsigned *__restrict__ err, unsigned *__restrict__ ctx_err)
{
   using T = float;
   constexpr int JP = 1, THREADS = 1024 / IH;
   using TG = TileGeom<float, 1>;
   constexpr int TILE = TG::TILE, JO = TG::joff();
   extern __shared__ __align__(16) unsigned char smem_raw[];
   __shared__ TileDesc s_desc[PENCIL_MAX];
   T *tiles = reinterpret_cast<T *>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~(uintptr_t) 127);
   T *klos = tiles + 3 * TILE;          // lower columns of tiles s, s+1
   T *khi = klos + 2 * KC + 1;          // upper column of tile s
   unsigned long long *bars = reinterpret_cast<unsigned long long *>(
      (reinterpret_cast<uintptr_t>(khi + KC) + 7) & ~(uintptr_t) 7);
   const unsigned bar0 = (unsigned) __cvta_generic_to_shared(bars);
   const int tid = threadIdx.x;
   const int kq = tid & 3, jrow = ((tid >> 2) & 15) + 1, ih = tid >> 6;
   if (tid == 0) {
      for (int b = 0; b < 3; b++)
         asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(
                         bar0 + 8 * b)
                      : "memory");
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
   }
   __syncthreads();
   unsigned phase = 0;                  // bit b: parity slot b waits for
   bool timed_out = false;

   constexpr int NFILL = (KC + THREADS - 1) / THREADS;
   int fill[NFILL];
#pragma unroll
   for (int m = 0; m < NFILL; m++) {
      const int q = tid + m * THREADS, i = q % G, j = q / G;
      fill[m] = q < KC ? ((JO + trow<T, 1>(i, j)) << 9) | (i * G + j) : -1;
   }

   for (int w = blockIdx.x; w < n_pencils * g.V; w += gridDim.x) {
      const int var = w / n_pencils, p = w - var * n_pencils;
      const int2 pc = pencils[p];
      const int len = pc.y;
      {
         const int32_t *from = reinterpret_cast<const int32_t *>(chain + pc.x);
         int32_t *to = reinterpret_cast<int32_t *>(s_desc);
         for (int q = tid; q < len * DESC; q += THREADS)
            to[q] = from[q];
      }
      __syncthreads();
      issue_tile_tma<ST, THREADS>(&tm, src, g, s_desc, var, tiles, bar0);
      if (len > 1)
         issue_tile_tma<ST, THREADS>(&tm, src, g, s_desc + 1, var,
                                     tiles + TILE, bar0 + 8);
      PassState st;
      st.ok = true;
      st.lo = st.hi = 0;
      for (int s = 0; s < len; s++) {
         const int sl = s % 3;
         const T *t = tiles + sl * TILE;
         const T *tn = tiles + ((s + 1) % 3) * TILE;
         T *kcur = klos + (s & 1) * KC;
         T *knext = klos + ((s + 1) & 1) * KC;
         if (!mbar_wait(bar0 + 8 * sl, (phase >> sl) & 1))
            timed_out = true;
         phase ^= 1u << sl;
         cp_async_wait_all();
         __syncthreads();
#pragma unroll
         for (int m = 0; m < NFILL; m++) {
            if (fill[m] < 0)
               continue;
            const int r = fill[m] >> 9, e = fill[m] & 511;
            const T top = t[r + NB - 1];
            khi[e] = s + 1 < len ? tn[r] : top;
            if (s + 1 < len)
               knext[e] = top;
            if (s == 0)
               kcur[e] = t[r];
         }
         __syncthreads();
         if (s + 2 < len) {
            const int sl2 = (s + 2) % 3;
            issue_tile_tma<ST, THREADS>(&tm, src, g, s_desc + s + 2, var,
                                        tiles + sl2 * TILE, bar0 + 8 * sl2);
         }
         const T *tq = t + JO + trow<T, 1>(IH * ih, jrow) + 4 * kq;
         const T *eg = (kq == 3 ? khi : kcur) + IH * ih * G + jrow;
         const int slot = s_desc[s].slot;
         T *d = dst + bv_offset(g, slot, var) + grow(IH * ih, jrow) + 4 * kq;
         st.slow = false;
         tile_pass<T, ST, JP, IH, false, 1>(tq, eg, d, kq, do_cs, st);
         if (__any_sync(0xffffffffu, st.slow))
            st = tile_fix<T, ST, JP, IH, 1>(tq, eg, d, kq, do_cs, st);
         if (do_cs)
            fixed52_flush(st.part, st.lo, st.hi);
         if (write_ghosts) {
            T *base = dst + bv_offset(g, slot, var);
            const int n_shell = G * G * G - NB * NB * NB;
            for (int e = tid; e < n_shell; e += THREADS) {
               int gi, gj, gk;
               if (e < 2 * G * G) {
                  gi = e < G * G ? 0 : G - 1;
                  const int r = e % (G * G);
                  gj = r / G; gk = r % G;
               } else if (e < 2 * G * G + 2 * NB * G) {
                  const int r = e - 2 * G * G;
                  gj = r < NB * G ? 0 : G - 1;
                  const int r2 = r % (NB * G);
                  gi = r2 / G + 1; gk = r2 % G;
               } else {
                  const int r = e - 2 * G * G - 2 * NB * G;
                  gk = r < NB * NB ? 0 : G - 1;
                  const int r2 = r % (NB * NB);
                  gi = r2 / NB + 1; gj = r2 % NB + 1;
               }
               const int outside = (gi == 0 || gi == G - 1) +
                                   (gj == 0 || gj == G - 1) +
                                   (gk == 0 || gk == G - 1);
               if (ST == 7 && outside != 1)
                  continue;
               const int ee = gi * G + gj;
               const T v = gk == 0 ? kcur[ee]
                         : (gk == G - 1 ? khi[ee]
                                        : t[JO + trow<T, 1>(gi, gj) + gk - 1]);
               base[cell_offset(g, gi, gj, gk)] = v;
            }
         }
      }
      if (do_cs) {
         if (!st.ok || !fixed52_window(st.part))
            atomicOr(err, ERR_FIXED_RANGE);
         block_acc128_flush(st.lo, st.hi, acc + 2 * var);
      }
      __syncthreads();
   }
   if (timed_out)
      atomicOr(ctx_err, ERR_WAIT);
}

// FP64 checksum of every (block, variable) of the pool in the reference's
// order: one thread per block-variable sums its interior serially.
__global__ void __launch_bounds__(128)
block_sums_all_fp64(const double *__restrict__ pool, Geom g,
                    const BItem *__restrict__ items, int nb,
                    double *__restrict__ partials)
{
   const long long e = blockIdx.x * (long long) blockDim.x + threadIdx.x;
   if (e >= (long long) nb * g.V)
      return;
   const int var = (int) (e / nb), b = (int) (e - (long long) var * nb);
   const double *base = pool + bv_offset(g, items[b].slot, var);
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

__global__ void finalize_all_fp64(const double *__restrict__ partials,
                                  int nb, int V, double *__restrict__ sums)
{
   for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < V;
        v += gridDim.x * blockDim.x) {
      const double *p = partials + (size_t) v * nb;
      double s = 0.0;
#pragma unroll 8
      for (int b = 0; b < nb; b++)
         s = s + p[b];
      sums[v] = s;
   }
}

int launch_fp64_checksums(const double *pool, const Geom &g,
                          const BItem *items, int n_blocks, double *partials,
                          double *sums, cudaStream_t s)
{
   const long long n = (long long) n_blocks * g.V;
   if (n == 0)
      return 0;
   block_sums_all_fp64<<<(unsigned) ((n + 127) / 128), 128, 0, s>>>(
      pool, g, items, n_blocks, partials);
   finalize_all_fp64<<<(g.V + 127) / 128, 128, 0, s>>>(partials, n_blocks,
                                                        g.V, sums);
   return 2;
}

// cuTensorMapEncodeTiled through the runtime's driver entry point.
EncodeTiledFn encode_tiled()
{
   static std::once_flag once;
   static EncodeTiledFn fn = nullptr;
   std::call_once(once, [] {
      void *p = nullptr;
      cudaDriverEntryPointQueryResult q;
      if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p,
                                           12000, cudaEnableDefault,
                                           &q) == cudaSuccess &&
          q == cudaDriverEntryPointSuccess)
         fn = reinterpret_cast<EncodeTiledFn>(p);
   });
   return fn;
}

// The tensor map of an FP32 pool of 16^3 blocks in the split layout:
// (k: 16, j: 18, i: 18, block-variable: n_bv), boxes of one plane's 16
// interior rows.
static bool pool_tensor_map(const float *pool, const Geom &g, long long n_bv,
                            CUtensorMap *tm)
{
   EncodeTiledFn enc = encode_tiled();
   if (!enc || g.kplane < 0 || n_bv < 1 || n_bv > (1ll << 31))
      return false;
   const cuuint64_t dims[4] = {(cuuint64_t) NB, (cuuint64_t) G,
                               (cuuint64_t) G, (cuuint64_t) n_bv};
   const cuuint64_t strides[3] = {NB * 4u, (cuuint64_t) G * NB * 4u,
                                  (cuuint64_t) g.bv * 4u};
   const cuuint32_t box[4] = {NB, NB, 1, 1};
   const cuuint32_t estr[4] = {1, 1, 1, 1};
   return enc(tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4,
              const_cast<float *>(pool), dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
              CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int ST, int IH>
static int pencil_tma_per_sm()
{
   int per_sm = 0;
   cudaFuncSetAttribute(pencil_tma_kernel<ST, IH>,
                        cudaFuncAttributeMaxDynamicSharedMemorySize,
                        (int) pencil_smem_bytes<float, 1>());
   cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      &per_sm, pencil_tma_kernel<ST, IH>, 1024 / IH,
      pencil_smem_bytes<float, 1>());
   return per_sm;
}

template <typename T, int ST, int JP, int IH>
static int pencil_per_sm()
{
   int per_sm = 0;
   cudaFuncSetAttribute(pencil_stage_kernel<T, ST, JP, IH>,
                        cudaFuncAttributeMaxDynamicSharedMemorySize,
                        (int) pencil_smem_bytes<T>());
   cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      &per_sm, pencil_stage_kernel<T, ST, JP, IH>,
      Shape<T, JP, IH>::THREADS, pencil_smem_bytes<T>());
   return per_sm > 0 ? per_sm : 1;
}

// Candidates: (rows, planes) per thread = (2, 4), (1, 4), (1, 8), each
// with a persistent grid (the CTAs one wave holds, looping over work
// items) or one CTA per work item (the hardware balances the tail).
template <typename T>
void pencil_candidates(int stencil, int n_work, std::vector<StageShape> &out)
{
   int dev = 0, sms = 0;
   cudaGetDevice(&dev);
   cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
   out.clear();
   const int shapes[3][2] = {{2, 4}, {1, 4}, {1, 8}};
   for (const auto &sp : shapes) {
      const int jp = sp[0], ih = sp[1];
      int per_sm;
      if (stencil == 7)
         per_sm = jp == 2 ? pencil_per_sm<T, 7, 2, 4>()
                : ih == 4 ? pencil_per_sm<T, 7, 1, 4>()
                          : pencil_per_sm<T, 7, 1, 8>();
      else
         per_sm = jp == 2 ? pencil_per_sm<T, 27, 2, 4>()
                : ih == 4 ? pencil_per_sm<T, 27, 1, 4>()
                          : pencil_per_sm<T, 27, 1, 8>();
      const long long wave = (long long) per_sm * sms;
      StageShape a;
      a.rows = jp;
      a.planes = ih;
      a.vpc = 1;
      a.threads = 1024 / (jp * ih);
      a.grid = (int) std::max(1LL, std::min<long long>(wave, n_work));
      out.push_back(a);
      if (n_work > wave) {
         a.grid = n_work;
         out.push_back(a);
      }
   }
   // FP32: the tensor-copy form, one j-row and 8 planes per thread (with
   // 4 planes it measured 8-10 % slower still, and is not offered)
   if (sizeof(T) == 4 && encode_tiled()) {
      for (int ih : {8}) {
         const int per_sm = stencil == 7 ? pencil_tma_per_sm<7, 8>()
                                         : pencil_tma_per_sm<27, 8>();
         if (per_sm <= 0)
            continue;
         const long long wave = (long long) per_sm * sms;
         StageShape a;
         a.kernel = 3;
         a.rows = 1;
         a.planes = ih;
         a.vpc = 1;
         a.threads = 1024 / ih;
         a.grid = (int) std::max(1LL, std::min<long long>(wave, n_work));
         out.push_back(a);
         if (n_work > wave) {
            a.grid = n_work;
            out.push_back(a);
         }
      }
   }
}

template <typename T>
int launch_pencil_stage(const T *src, T *dst, const Geom &g, int stencil,
                        const BItem *items, int n_blocks,
                        const TileDesc *chain, const int2 *pencils,
                        int n_pencils, const StageShape &sh, int write_ghosts,
                        int do_cs, double *partials, double *sums,
                        unsigned long long *acc, unsigned *err,
                        unsigned *ctx_err, long long n_bv, cudaStream_t s)
{
   if (n_pencils == 0)
      return 0;
   if (sh.kernel == 3) {
      if constexpr (sizeof(T) == 4) {
         CUtensorMap tm;
         if (!pool_tensor_map(src, g, n_bv, &tm))
            return -1;
         const size_t smem = pencil_smem_bytes<float, 1>();
#define MAMR_PENCIL_TMA(ST, IH)                                               \
   pencil_tma_kernel<ST, IH><<<sh.grid, 1024 / IH, smem, s>>>(                \
      tm, src, dst, g, chain, pencils, n_pencils, write_ghosts, do_cs, acc,   \
      err, ctx_err)
         if (sh.planes != 8)
            return -1;
         if (stencil == 7)
            MAMR_PENCIL_TMA(7, 8);
         else
            MAMR_PENCIL_TMA(27, 8);
#undef MAMR_PENCIL_TMA
         return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
      } else {
         return -1;
      }
   }
   const size_t smem = pencil_smem_bytes<T>();
   const int fused_cs = (sizeof(T) == 4) ? do_cs : 0;
   const int grid = sh.grid;
#define MAMR_PENCIL(ST, JP, IH)                                               \
   pencil_stage_kernel<T, ST, JP, IH>                                        \
      <<<grid, Shape<T, JP, IH>::THREADS, smem, s>>>(                         \
         src, dst, g, chain, pencils, n_pencils, write_ghosts, fused_cs, acc, \
         err)
   if (stencil == 7) {
      if (sh.rows == 2) MAMR_PENCIL(7, 2, 4);
      else if (sh.planes == 8) MAMR_PENCIL(7, 1, 8);
      else MAMR_PENCIL(7, 1, 4);
   } else {
      if (sh.rows == 2) MAMR_PENCIL(27, 2, 4);
      else if (sh.planes == 8) MAMR_PENCIL(27, 1, 8);
      else MAMR_PENCIL(27, 1, 4);
   }
#undef MAMR_PENCIL
   int launches = 1;
   if (do_cs && sizeof(T) == 8)
      launches += launch_fp64_checksums((const double *) dst, g, items,
                                        n_blocks, partials, sums, s);
   return cudaPeekAtLastError() == cudaSuccess ? launches : -1;
}

template void pencil_candidates<float>(int, int, std::vector<StageShape> &);
template void pencil_candidates<double>(int, int, std::vector<StageShape> &);
template int launch_pencil_stage<float>(const float *, float *, const Geom &,
                                        int, const BItem *, int,
                                        const TileDesc *, const int2 *, int,
                                        const StageShape &, int, int, double *,
                                        double *, unsigned long long *,
                                        unsigned *, unsigned *, long long,
                                        cudaStream_t);
template int launch_pencil_stage<double>(const double *, double *,
                                         const Geom &, int, const BItem *,
                                         int, const TileDesc *, const int2 *,
                                         int, const StageShape &, int, int,
                                         double *, double *,
                                         unsigned long long *, unsigned *,
                                         unsigned *, long long, cudaStream_t);

}  // namespace mamr
