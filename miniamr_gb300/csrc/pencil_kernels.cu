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
// Values and operation order are exactly those of the plain path: ghosts
// as comm() leaves them on a single-level mesh (axis-by-axis neighbour or
// reflection), the reference's summation order, correctly rounded
// division, and the FP32 checksum as exact 128-bit fixed point.
#include "batched.h"
#include "arith.cuh"

namespace mamr {

namespace {

constexpr int NB = 16;              // cells per block edge
constexpr int G = NB + 2;           // with ghosts
constexpr int RS = NB;              // shared row: the 16 interior k values
constexpr int KC = G * G;           // one k-column array (i, j incl. ghosts)
constexpr int TILE_ROWS = G * G;
constexpr int THREADS = 256;

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem)
{
   unsigned s = (unsigned) __cvta_generic_to_shared(smem);
   asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s),
                "l"(gmem));
}
__device__ __forceinline__ void cp_async_commit()
{
   asm volatile("cp.async.commit_group;\n" ::);
}
__device__ __forceinline__ void cp_async_wait_all()
{
   asm volatile("cp.async.wait_all;\n" ::: "memory");
}

template <typename T> struct Quad;   // four consecutive k values
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

template <typename T>
constexpr size_t pencil_smem_bytes()
{
   return (size_t) 3 * (TILE_ROWS * RS + 2 * KC) * sizeof(T);
}

constexpr int DESC = sizeof(TileDesc) / sizeof(int32_t);

// Queues the cp.async copies of tile `s` of the pencil into ring buffer t:
// the interior rows, the four x/y face rows (neighbour or reflection) and,
// for 27 points, the four z-running edge rows.
template <typename T, int ST>
__device__ __forceinline__ void issue_tile(const T *__restrict__ src,
                                           const Geom &g, const TileDesc *it,
                                           int var, T *t)
{
   constexpr int VW = 16 / (int) sizeof(T);   // elements per 16 bytes
   constexpr int CPR = NB / VW;               // 16-byte chunks per row
   const int tid = threadIdx.x;
   const int slot = it->slot, bmask = it->bmask;
   const T *own = src + bv_offset(g, slot, var);
   for (int c = tid; c < NB * NB * CPR; c += THREADS) {
      const int q = c % CPR, r = c / CPR;
      const int j = r % NB + 1, i = r / NB + 1;
      cp_async16(t + (i * G + j) * RS + q * VW,
                 own + row_offset(g, i, j) + q * VW);
   }
   for (int c = tid; c < 4 * NB * CPR; c += THREADS) {
      const int f = c / (NB * CPR), r = c % (NB * CPR);
      const int a = r / CPR + 1, q = r % CPR;
      const bool bnd = (bmask >> f) & 1;
      // nb9 index of the W, E, S, N neighbour: 3, 5, 1, 7
      const int nbi = (f < 2) ? (f == 0 ? 3 : 5) : (f == 2 ? 1 : 7);
      const T *blk = bnd ? own : src + bv_offset(g, it->nb9[nbi], var);
      const bool low = (f & 1) == 0;
      // neighbour: its plane next to us; boundary: our own first plane
      const int sp = bnd ? (low ? 1 : NB) : (low ? NB : 1);
      const int gp = low ? 0 : G - 1;
      const T *from;
      T *to;
      if (f < 2) {
         from = blk + row_offset(g, sp, a);
         to = t + (gp * G + a) * RS;
      } else {
         from = blk + row_offset(g, a, sp);
         to = t + (a * G + gp) * RS;
      }
      cp_async16(to + q * VW, from + q * VW);
   }
   if (ST == 27) {
      for (int c = tid; c < 4 * CPR; c += THREADS) {
         const int e = c / CPR, q = c % CPR;
         const int gi = (e & 1) ? G - 1 : 0, gj = (e & 2) ? G - 1 : 0;
         int dx = (e & 1) ? 1 : -1, dy = (e & 2) ? 1 : -1, si, sj;
         if (bmask & (1 << ((e & 1) ? 1 : 0))) { si = (e & 1) ? NB : 1; dx = 0; }
         else si = (e & 1) ? 1 : NB;
         if (bmask & (1 << ((e & 2) ? 3 : 2))) { sj = (e & 2) ? NB : 1; dy = 0; }
         else sj = (e & 2) ? 1 : NB;
         const int nb = it->nb9[(dx + 1) + 3 * (dy + 1)];
         cp_async16(t + (gi * G + gj) * RS + q * VW,
                    src + bv_offset(g, nb, var) + row_offset(g, si, sj) +
                       q * VW);
      }
   }
   cp_async_commit();
}

// Row (i, j) of a tile as six k values: k-1 .. k+4 around the thread's
// quad k .. k+3 (k = 4*kq + 1).  The four lanes of a row hold the row's 16
// values between them; the outer neighbours k-1 and k+4 come from the
// adjacent lanes by shuffle, and from the z ghost columns at the row ends.
// Every lane of the warp must call this together.
template <typename T>
__device__ __forceinline__ void row6(const T *t, const T *klo, const T *khi,
                                     int i, int j, int kq, T (&r)[6])
{
   const int e = i * G + j;
   T v[4];
   Quad<T>::ld(t + e * RS + 4 * kq, v);
   const T left = __shfl_up_sync(0xffffffffu, v[3], 1);
   const T right = __shfl_down_sync(0xffffffffu, v[0], 1);
   const T edge = kq == 0 ? klo[e] : khi[e];
   r[0] = kq == 0 ? edge : left;
   r[1] = v[0]; r[2] = v[1]; r[3] = v[2]; r[4] = v[3];
   r[5] = kq == 3 ? edge : right;
}

}  // namespace

template <typename T, int ST>
__global__ void __launch_bounds__(THREADS, sizeof(T) == 4 ? 3 : 1)
pencil_stage_kernel(const T *__restrict__ src, T *__restrict__ dst, Geom g,
                    const TileDesc *__restrict__ chain,
                    const int2 *__restrict__ pencils, int n_pencils,
                    int write_ghosts, int do_cs,
                    unsigned long long *__restrict__ acc,
                    unsigned *__restrict__ err)
{
   extern __shared__ __align__(16) unsigned char smem_raw[];
   __shared__ TileDesc s_desc[PENCIL_MAX];
   T *tiles = reinterpret_cast<T *>(smem_raw);
   T *klos = tiles + 3 * TILE_ROWS * RS;
   T *khis = klos + 3 * KC;
   const int tid = threadIdx.x;
   const int kq = tid & 3, j = ((tid >> 2) & 15) + 1, ih = tid >> 6;

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
      issue_tile<T, ST>(src, g, s_desc, var, tiles);
      if (len > 1)
         issue_tile<T, ST>(src, g, s_desc + 1, var, tiles + TILE_ROWS * RS);
      unsigned long long lo = 0, hi = 0;
      bool ok = true;
      for (int s = 0; s < len; s++) {
         const int b = s % 3, bn = (s + 1) % 3;
         T *t = tiles + b * TILE_ROWS * RS;
         T *klo = klos + b * KC, *khi = khis + b * KC;
         cp_async_wait_all();
         __syncthreads();
         // z ghost columns: tile s+1's k=1 (or our own k=16 at the top
         // boundary); tile s+1's lower column is our k=16; the bottom tile
         // reflects its own k=1
         for (int e = tid; e < KC; e += THREADS) {
            const T *tn = tiles + bn * TILE_ROWS * RS;
            if (s + 1 < len) {
               khi[e] = tn[e * RS];
               klos[bn * KC + e] = t[e * RS + NB - 1];
            } else {
               khi[e] = t[e * RS + NB - 1];
            }
            if (s == 0)
               klo[e] = t[e * RS];
         }
         __syncthreads();
         if (s + 2 < len)
            issue_tile<T, ST>(src, g, s_desc + s + 2, var,
                              tiles + ((s + 2) % 3) * TILE_ROWS * RS);

         const int slot = s_desc[s].slot;
         T *d = dst + bv_offset(g, slot, var);
         T out[4];
         if (ST == 7) {
            T am[4], r[6], c[6];
            Quad<T>::ld(t + ((4 * ih) * G + j) * RS + 4 * kq, am);
            row6(t, klo, khi, 4 * ih + 1, j, kq, r);
#pragma unroll
            for (int ii = 1; ii <= 4; ii++) {
               const int i = 4 * ih + ii;
               T sm[4], sp[4];
               Quad<T>::ld(t + (i * G + j - 1) * RS + 4 * kq, sm);
               Quad<T>::ld(t + (i * G + j + 1) * RS + 4 * kq, sp);
               row6(t, klo, khi, i + 1, j, kq, c);
               T w[4];
#pragma unroll
               for (int m = 0; m < 4; m++) {
                  T v = am[m] + sm[m];
                  v = v + r[m];
                  v = v + r[m + 1];
                  v = v + r[m + 2];
                  v = v + sp[m];
                  v = v + c[m + 1];
                  w[m] = v;
               }
               div_const4<7>(w, out);
               Quad<T>::st(d + row_offset(g, i, j) + 4 * kq, out);
               if (sizeof(T) == 4 && do_cs)
#pragma unroll
                  for (int m = 0; m < 4; m++) {
                     long long q;
                     ok &= fixed52((float) out[m], q);
                     acc128_add(lo, hi, q);
                  }
#pragma unroll
               for (int m = 0; m < 4; m++) {
                  am[m] = r[m + 1];
               }
#pragma unroll
               for (int m = 0; m < 6; m++)
                  r[m] = c[m];
            }
         } else {
            // S(p): the reference's 9-term sum on plane p, for 4 k values
            auto S4 = [&](int pl, T (&s4)[4]) {
               T a[6], bb[6], cc[6];
               row6(t, klo, khi, pl, j - 1, kq, a);
               row6(t, klo, khi, pl, j, kq, bb);
               row6(t, klo, khi, pl, j + 1, kq, cc);
#pragma unroll
               for (int m = 0; m < 4; m++) {
                  T v = a[m] + a[m + 1];
                  v = v + a[m + 2];
                  v = v + bb[m];
                  v = v + bb[m + 1];
                  v = v + bb[m + 2];
                  v = v + cc[m];
                  v = v + cc[m + 1];
                  v = v + cc[m + 2];
                  s4[m] = v;
               }
            };
            T s0[4], s1[4], s2[4];
            S4(4 * ih, s0);
            S4(4 * ih + 1, s1);
#pragma unroll
            for (int ii = 1; ii <= 4; ii++) {
               const int i = 4 * ih + ii;
               S4(i + 1, s2);
               T w[4];
#pragma unroll
               for (int m = 0; m < 4; m++)
                  w[m] = (s0[m] + s1[m]) + s2[m];
               div_const4<27>(w, out);
               Quad<T>::st(d + row_offset(g, i, j) + 4 * kq, out);
               if (sizeof(T) == 4 && do_cs)
#pragma unroll
                  for (int m = 0; m < 4; m++) {
                     long long q;
                     ok &= fixed52((float) out[m], q);
                     acc128_add(lo, hi, q);
                  }
#pragma unroll
               for (int m = 0; m < 4; m++) {
                  s0[m] = s1[m];
                  s1[m] = s2[m];
               }
            }
         }
         if (write_ghosts) {
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
               const T v = gk == 0 ? klo[ee]
                         : (gk == G - 1 ? khi[ee] : t[ee * RS + gk - 1]);
               d[cell_offset(g, gi, gj, gk)] = v;
            }
         }
      }
      if (sizeof(T) == 4 && do_cs) {
         if (!ok)
            atomicOr(err, ERR_FIXED_RANGE);
         block_acc128_flush(lo, hi, acc + 2 * var);
      }
      __syncthreads();
   }
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

template <typename T, int ST>
static cudaError_t pencil_attr()
{
   return cudaFuncSetAttribute(pencil_stage_kernel<T, ST>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int) pencil_smem_bytes<T>());
}

template <typename T>
int pencil_grid(int stencil, int n_work)
{
   int per_sm = 0, dev = 0, sms = 0;
   cudaGetDevice(&dev);
   cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
   if (stencil == 7) {
      pencil_attr<T, 7>();
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(
         &per_sm, pencil_stage_kernel<T, 7>, THREADS, pencil_smem_bytes<T>());
   } else {
      pencil_attr<T, 27>();
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(
         &per_sm, pencil_stage_kernel<T, 27>, THREADS, pencil_smem_bytes<T>());
   }
   long long grid = (long long) (per_sm > 0 ? per_sm : 1) * sms;
   return (int) (grid < n_work ? grid : (n_work > 0 ? n_work : 1));
}

template <typename T>
int launch_pencil_stage(const T *src, T *dst, const Geom &g, int stencil,
                        const BItem *items, int n_blocks,
                        const TileDesc *chain, const int2 *pencils,
                        int n_pencils, int grid, int write_ghosts, int do_cs,
                        double *partials, double *sums,
                        unsigned long long *acc, unsigned *err,
                        cudaStream_t s)
{
   if (n_pencils == 0)
      return 0;
   const size_t smem = pencil_smem_bytes<T>();
   const int fused_cs = (sizeof(T) == 4) ? do_cs : 0;
   if (stencil == 7)
      pencil_stage_kernel<T, 7><<<grid, THREADS, smem, s>>>(
         src, dst, g, chain, pencils, n_pencils, write_ghosts, fused_cs, acc,
         err);
   else
      pencil_stage_kernel<T, 27><<<grid, THREADS, smem, s>>>(
         src, dst, g, chain, pencils, n_pencils, write_ghosts, fused_cs, acc,
         err);
   int launches = 1;
   if (do_cs && sizeof(T) == 8) {
      const long long n = (long long) n_blocks * g.V;
      block_sums_all_fp64<<<(unsigned) ((n + 127) / 128), 128, 0, s>>>(
         (const double *) dst, g, items, n_blocks, partials);
      finalize_all_fp64<<<(g.V + 127) / 128, 128, 0, s>>>(partials, n_blocks,
                                                           g.V, sums);
      launches += 2;
   }
   return cudaPeekAtLastError() == cudaSuccess ? launches : -1;
}

template int pencil_grid<float>(int, int);
template int pencil_grid<double>(int, int);
template int launch_pencil_stage<float>(const float *, float *, const Geom &,
                                        int, const BItem *, int,
                                        const TileDesc *, const int2 *, int,
                                        int, int, int, double *, double *,
                                        unsigned long long *, unsigned *,
                                        cudaStream_t);
template int launch_pencil_stage<double>(const double *, double *,
                                         const Geom &, int, const BItem *,
                                         int, const TileDesc *, const int2 *,
                                         int, int, int, int, double *,
                                         double *, unsigned long long *,
                                         unsigned *, cudaStream_t);

}  // namespace mamr
