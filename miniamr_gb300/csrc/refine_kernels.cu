// Cell data of split_blocks() and consolidate_blocks() (ref/block.c:158-173,
// 411-431): one CTA per (job, variable) covering all eight octants, a
// thread per row of cells, 16-byte row loads and stores for the 8^3 and
// 16^3 block sizes (their dimensions are compile-time constants).
//
// Reads go through read_base: a negative slot names an entry of the
// staging copy taken before a job list whose later jobs overwrite a slot
// that an earlier job reads (segments.h).
#include "mamr_internal.h"
#include "arith.cuh"
#include "dims.cuh"

namespace mamr {

namespace {

template <typename T>
__device__ __forceinline__ const T *read_base(const T *pool, const T *stage,
                                              const Geom &g, int slot, int var)
{
   return slot >= 0 ? pool + bv_offset(g, slot, var)
                    : stage + bv_offset(g, -slot - 1, var);
}

template <typename T> struct Vec;
template <> struct Vec<float> {
   using V = float4;
   static constexpr int W = 4;
   __device__ static void ld(const float *p, float *v)
   {
      const float4 x = *reinterpret_cast<const float4 *>(p);
      v[0] = x.x; v[1] = x.y; v[2] = x.z; v[3] = x.w;
   }
   __device__ static void st(float *p, const float *v)
   {
      *reinterpret_cast<float4 *>(p) = make_float4(v[0], v[1], v[2], v[3]);
   }
};
template <> struct Vec<double> {
   using V = double2;
   static constexpr int W = 2;
   __device__ static void ld(const double *p, double *v)
   {
      const double2 x = *reinterpret_cast<const double2 *>(p);
      v[0] = x.x; v[1] = x.y;
   }
   __device__ static void st(double *p, const double *v)
   {
      *reinterpret_cast<double2 *>(p) = make_double2(v[0], v[1]);
   }
};

// The sum of eight children as consolidation defines it for FP32 pools:
// the compensated FP64 sum of arith.cuh's sum8, rounded once to FP32.
// When the children's binary exponents span at most 26 (and stay clear of
// the ends of the range), every partial sum in FP64 is exact -- 24-bit
// significands over 26 binades plus 3 carry bits fit 53 bits -- so the
// compensation is zero and sum8 returns the correctly rounded sum.  That
// sum is then formed as an exact integer (the significands aligned to the
// smallest exponent) and rounded by one conversion; the power-of-two
// scaling after it is exact because the result stays a normal float.
// Anything else takes sum8 itself.  Both give the same bits.
__device__ __forceinline__ float sum8_children(const float (&t)[8])
{
   unsigned emax = 0, emin = 255, special = 0;
#pragma unroll
   for (int q = 0; q < 8; q++) {
      const unsigned u = __float_as_uint(t[q]), e = (u >> 23) & 0xffu;
      special |= e == 255u;
      if (u << 1) {
         const unsigned eb = e ? e : 1u;
         emax = eb > emax ? eb : emax;
         emin = eb < emin ? eb : emin;
      }
   }
   if (!special && emax <= emin + 26u && emin >= 30u && emax <= 220u) {
      long long s = 0;
#pragma unroll
      for (int q = 0; q < 8; q++) {
         const unsigned u = __float_as_uint(t[q]), e = (u >> 23) & 0xffu;
         if (!(u << 1))
            continue;
         const long long m =
            (long long) ((u & 0x7fffffu) | (e ? 0x800000u : 0u))
            << ((e ? e : 1u) - emin);
         s += (u >> 31) ? -m : m;
      }
      // value = s * 2^(emin - 150)
      return __fmul_rn(__ll2float_rn(s), __uint_as_float((emin - 23u) << 23));
   }
   return sum8(t);
}
__device__ __forceinline__ double sum8_children(const double (&t)[8])
{
   return sum8(t);
}

// A child cell (ci, cj, ck) of octant o takes parent cell
// ((ci+1)/2 + i1, (cj+1)/2 + j1, (ck+1)/2 + k1) / 8 -- exact.
template <typename T, int BX, int BY, int BZ>
__global__ void __launch_bounds__(256)
split_jobs_kernel(T *__restrict__ pool, const T *__restrict__ stage, Geom g,
                  const mamr_split_job *__restrict__ jobs, T *__restrict__ zf)
{
   const Dims<BX, BY, BZ> D(g);
   const int job = blockIdx.x, var = blockIdx.y;
   const T *P = read_base(pool, stage, g, jobs[job].parent, var);
   const int hx = D.nx / 2, hy = D.ny / 2, hz = D.nz / 2;
   const int per_child = D.nx * D.ny;
   if constexpr (BX > 0 && (BZ / 2) % Vec<T>::W == 0) {
      // 8^3 and 16^3: the thread's rows r = threadIdx.x + u * NT in groups
      // of G, each group's parent half-rows loaded before any of its child
      // rows is stored (no row a segment's jobs read is written in it), so
      // that G loads are in flight instead of one
      constexpr int W = Vec<T>::W, H = BZ / 2;
      constexpr int NT = BX == 8 ? 128 : 256;   // launch_split's CTA size
      constexpr int RPT = 8 * BX * BY / NT, G = RPT < 4 ? RPT : 4;
      static_assert((BX == 8 || BX == 16) && RPT * NT == 8 * BX * BY &&
                    RPT % G == 0, "split rows per thread");
      const int32_t *ch = jobs[job].child;
#pragma unroll 1
      for (int u0 = 0; u0 < RPT; u0 += G) {
         T p[G][H];
#pragma unroll
         for (int u = 0; u < G; u++) {
            const int r = threadIdx.x + (u0 + u) * NT;
            const int o = r / per_child, rr = r - o * per_child;
            const int ci = rr / D.ny + 1, cj = rr - (ci - 1) * D.ny + 1;
            const T *prow = P + D.cell((ci + 1) / 2 + (o & 1) * hx,
                                       (cj + 1) / 2 + ((o >> 1) & 1) * hy,
                                       1 + (o >> 2) * hz);
#pragma unroll
            for (int q = 0; q < H; q += W)
               Vec<T>::ld(prow + q, p[u] + q);
         }
#pragma unroll
         for (int u = 0; u < G; u++) {
            const int r = threadIdx.x + (u0 + u) * NT;
            const int o = r / per_child, rr = r - o * per_child;
            const int ci = rr / D.ny + 1, cj = rr - (ci - 1) * D.ny + 1;
            T *crow = pool + bv_offset(g, ch[o], var) + D.cell(ci, cj, 1);
#pragma unroll
            for (int q = 0; q < H; q += W) {
               T c[2 * W];
#pragma unroll
               for (int m = 0; m < W; m++)
                  c[2 * m] = c[2 * m + 1] = eighth(p[u][q + m]);
               Vec<T>::st(crow + 2 * q, c);
               Vec<T>::st(crow + 2 * q + W, c + W);
            }
            if (zf) {
               T *z = zf + zface_at(g, ch[o], var, 0) + (ci - 1) * D.ny +
                      (cj - 1);
               z[0] = eighth(p[u][0]);
               z[D.nx * D.ny] = eighth(p[u][H - 1]);
            }
         }
      }
      return;
   }
   for (int r = threadIdx.x; r < 8 * per_child; r += blockDim.x) {
      const int o = r / per_child, rr = r - o * per_child;
      const int ci = rr / D.ny + 1, cj = rr - (ci - 1) * D.ny + 1;
      const int i1 = (o & 1) * hx, j1 = ((o >> 1) & 1) * hy,
                k1 = (o >> 2) * hz;
      const T *prow = P + D.cell((ci + 1) / 2 + i1, (cj + 1) / 2 + j1,
                                 1 + k1);
      T *crow = pool + bv_offset(g, jobs[job].child[o], var) +
                D.cell(ci, cj, 1);
      if (BZ && (BZ / 2) % Vec<T>::W == 0) {
         constexpr int W = Vec<T>::W;
#pragma unroll
         for (int q = 0; q < BZ / 2; q += W) {
            T p[W], c[2 * W];
            Vec<T>::ld(prow + q, p);
#pragma unroll
            for (int m = 0; m < W; m++)
               c[2 * m] = c[2 * m + 1] = eighth(p[m]);
            Vec<T>::st(crow + 2 * q, c);
            Vec<T>::st(crow + 2 * q + W, c + W);
         }
      } else {
         for (int ck = 1; ck <= D.nz; ck++)
            crow[ck - 1] = eighth(prow[(ck + 1) / 2 - 1]);
      }
      if (zf) {
         // the child's k = 1 and k = nz planes for the z-face array
         T *z = zf + zface_at(g, jobs[job].child[o], var, 0) +
                (ci - 1) * D.ny + (cj - 1);
         z[0] = eighth(prow[0]);
         z[D.nx * D.ny] = eighth(prow[D.nz / 2 - 1]);
      }
   }
}

// A coarse cell (i + i1, j + j1, k + k1) of the target is the sum of the
// 2x2x2 cells (2i-1.., 2j-1.., 2k-1..) of child o in the reference's term
// order: (i2,j2,k2), (i2+1,j2,k2), (i2,j2+1,k2), (i2+1,j2+1,k2), then the
// same four at k2+1.
template <typename T, int BX, int BY, int BZ>
__global__ void __launch_bounds__(256)
consolidate_jobs_kernel(T *__restrict__ pool, const T *__restrict__ stage,
                        Geom g, const mamr_consolidate_job *__restrict__ jobs,
                        T *__restrict__ zf)
{
   const Dims<BX, BY, BZ> D(g);
   const int job = blockIdx.x, var = blockIdx.y;
   T *P = pool + bv_offset(g, jobs[job].target, var);
   const int hx = D.nx / 2, hy = D.ny / 2, hz = D.nz / 2;
   const int per_child = hx * hy;
   for (int r = threadIdx.x; r < 8 * per_child; r += blockDim.x) {
      const int o = r / per_child, rr = r - o * per_child;
      const int i = rr / hy + 1, j = rr - (i - 1) * hy + 1;
      const int i1 = (o & 1) * hx, j1 = ((o >> 1) & 1) * hy,
                k1 = (o >> 2) * hz;
      const T *C = read_base(pool, stage, g, jobs[job].child[o], var);
      const T *f00 = C + D.cell(2 * i - 1, 2 * j - 1, 1);
      const T *f10 = C + D.cell(2 * i, 2 * j - 1, 1);
      const T *f01 = C + D.cell(2 * i - 1, 2 * j, 1);
      const T *f11 = C + D.cell(2 * i, 2 * j, 1);
      T *prow = P + D.cell(i + i1, j + j1, 1 + k1);
      T zv = 0;   // the target's k = 1 (k1 = 0) or k = nz value of the row
      if (BZ && (BZ / 2) % Vec<T>::W == 0) {
         constexpr int W = Vec<T>::W;
#pragma unroll
         for (int q = 0; q < BZ / 2; q += W) {
            T a[2 * W], b[2 * W], c[2 * W], d[2 * W], out[W];
            Vec<T>::ld(f00 + 2 * q, a); Vec<T>::ld(f00 + 2 * q + W, a + W);
            Vec<T>::ld(f10 + 2 * q, b); Vec<T>::ld(f10 + 2 * q + W, b + W);
            Vec<T>::ld(f01 + 2 * q, c); Vec<T>::ld(f01 + 2 * q + W, c + W);
            Vec<T>::ld(f11 + 2 * q, d); Vec<T>::ld(f11 + 2 * q + W, d + W);
#pragma unroll
            for (int m = 0; m < W; m++) {
               const T t[8] = {a[2 * m], b[2 * m], c[2 * m], d[2 * m],
                               a[2 * m + 1], b[2 * m + 1], c[2 * m + 1],
                               d[2 * m + 1]};
               out[m] = sum8_children(t);
            }
            Vec<T>::st(prow + q, out);
            if (q == 0 && k1 == 0)
               zv = out[0];
            if (q + W == BZ / 2 && k1 != 0)
               zv = out[W - 1];
         }
      } else {
         for (int k = 1; k <= hz; k++) {
            const int k2 = 2 * k - 1;
            const T t[8] = {f00[k2 - 1], f10[k2 - 1], f01[k2 - 1],
                            f11[k2 - 1], f00[k2], f10[k2], f01[k2], f11[k2]};
            const T v = sum8_children(t);
            prow[k - 1] = v;
            if ((k == 1 && k1 == 0) || (k == hz && k1 != 0))
               zv = v;
         }
      }
      if (zf)
         zf[zface_at(g, jobs[job].target, var, k1 != 0) +
            (i + i1 - 1) * D.ny + (j + j1 - 1)] = zv;
   }
}

}  // namespace

template <typename T>
int launch_split(T *pool, const T *stage, const Geom &g,
                 const mamr_split_job *jobs, int n, T *zf, cudaStream_t s)
{
   if (n == 0)
      return 0;
   const dim3 grid(n, g.V);
   switch (dims_kind(g)) {
   case 1:
      split_jobs_kernel<T, 8, 8, 8><<<grid, 128, 0, s>>>(pool, stage, g, jobs,
                                                         zf);
      break;
   case 2:
      split_jobs_kernel<T, 16, 16, 16><<<grid, 256, 0, s>>>(pool, stage, g,
                                                            jobs, zf);
      break;
   default:
      split_jobs_kernel<T, 0, 0, 0><<<grid, 256, 0, s>>>(pool, stage, g, jobs,
                                                         zf);
   }
   return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

template <typename T>
int launch_consolidate(T *pool, const T *stage, const Geom &g,
                       const mamr_consolidate_job *jobs, int n, T *zf,
                       cudaStream_t s)
{
   if (n == 0)
      return 0;
   const dim3 grid(n, g.V);
   switch (dims_kind(g)) {
   case 1:
      consolidate_jobs_kernel<T, 8, 8, 8><<<grid, 128, 0, s>>>(pool, stage, g,
                                                               jobs, zf);
      break;
   case 2:
      consolidate_jobs_kernel<T, 16, 16, 16><<<grid, 256, 0, s>>>(
         pool, stage, g, jobs, zf);
      break;
   default:
      consolidate_jobs_kernel<T, 0, 0, 0><<<grid, 256, 0, s>>>(pool, stage, g,
                                                               jobs, zf);
   }
   return cudaPeekAtLastError() == cudaSuccess ? 1 : -1;
}

template int launch_split<float>(float *, const float *, const Geom &,
                                 const mamr_split_job *, int, float *,
                                 cudaStream_t);
template int launch_split<double>(double *, const double *, const Geom &,
                                  const mamr_split_job *, int, double *,
                                  cudaStream_t);
template int launch_consolidate<float>(float *, const float *, const Geom &,
                                       const mamr_consolidate_job *, int,
                                       float *, cudaStream_t);
template int launch_consolidate<double>(double *, const double *,
                                        const Geom &,
                                        const mamr_consolidate_job *, int,
                                        double *, cudaStream_t);

}  // namespace mamr
