// Arithmetic building blocks shared by the plain and batched kernels.
#pragma once

#include <cuda_runtime.h>

namespace mamr {

// ---- correctly rounded division by the stencil constants -----------------
//
// FP64: x / 7 and x / 27 as the reference computes them (IEEE division,
// round to nearest), in three FP64 operations instead of a full divide.
// Method: Markstein (1990), correction of a quotient by its exact
// remainder.  With y = RN(1/c): q0 = RN(x*y); r = fma(-q0, c, x), exact
// whenever q0 is a faithful rounding of x/c; then RN(q0 + r*y) = RN(x/c)
// (Markstein's theorem; Muller et al., Handbook of Floating-Point
// Arithmetic, section on division with a known reciprocal).  q0 is faithful
// here because |y*c - 1| = 2^-54 for both constants (checked with exact
// rational arithmetic), so |x*y - x/c| < ulp(x/c)/2.  The argument needs x,
// q0 and r away from underflow and overflow, so x outside biased exponents
// (100, 2000) -- zero, tiny, huge, inf, nan -- takes the IEEE division.
// mamr_selftest_division compares against IEEE division on the GPU.
// The fast quotient is computed for every argument; arguments outside the
// window take the IEEE division in a separate, rarely entered branch so
// that the long IEEE sequence is never if-converted into the common path.
__device__ __forceinline__ bool div_window(double x)
{
   const unsigned e = ((unsigned) __double2hiint(x) >> 20) & 0x7ffu;
   return e - 101u < 1899u;                   // 100 < e < 2000
}
__device__ __forceinline__ bool div_window(float x)
{
   // 60 < e < 250 on the magnitude's bits (NaN and inf fall outside)
   return (__float_as_uint(x) & 0x7fffffffu) - (61u << 23) < (189u << 23);
}

template <int C>
__device__ __forceinline__ double div_fast(double x)
{
   const double y = C == 7 ? 0x1.2492492492492p-3    // RN(1/7)
                           : 0x1.2f684bda12f68p-5;   // RN(1/27)
   const double q0 = __dmul_rn(x, y);
   const double r = __fma_rn(-q0, (double) C, x);
   return __fma_rn(r, y, q0);
}

// FP32: the same three-step quotient with y = RN_f32(1/c).  The general
// bound does not cover c = 7 in FP32 (|y*7 - 1| = 1.5 * 2^-25), so this
// form was instead checked exhaustively against IEEE FP32 division on
// every float in [1, 2) for both constants (mamr_selftest_division; zero
// differences).  All three steps scale exactly by powers of two, so the
// result holds for every x whose quotient and remainder stay normal:
// biased exponents (60, 250); the rest takes the IEEE division.
template <int C>
__device__ __forceinline__ float div_fast(float x)
{
   const float y = C == 7 ? 0x1.24924ap-3f : 0x1.2f684cp-5f;
   const float q0 = __fmul_rn(x, y);
   const float r = __fmaf_rn(-q0, (float) C, x);
   return __fmaf_rn(r, y, q0);
}

static __device__ __noinline__ double div_ieee(double x, double c)
{
   return __ddiv_rn(x, c);
}
static __device__ __noinline__ float div_ieee(float x, float c)
{
   return __fdiv_rn(x, c);
}

template <int C, typename T>
__device__ __forceinline__ T div_const(T x)
{
   T q = div_fast<C>(x);
   if (__builtin_expect(!div_window(x), 0))
      q = div_ieee(x, (T) C);
   return q;
}

// Four quotients at once: one test for the rare slow path.
template <int C, typename T>
__device__ __forceinline__ void div_const4(const T (&x)[4], T (&q)[4])
{
   bool slow = false;
#pragma unroll
   for (int m = 0; m < 4; m++) {
      q[m] = div_fast<C>(x[m]);
      slow |= !div_window(x[m]);
   }
   if (__builtin_expect(slow, 0)) {
#pragma unroll
      for (int m = 0; m < 4; m++)
         if (!div_window(x[m]))
            q[m] = div_ieee(x[m], (T) C);
   }
}

__device__ __forceinline__ double div7(double x) { return div_const<7>(x); }
__device__ __forceinline__ double div27(double x) { return div_const<27>(x); }
__device__ __forceinline__ float div7(float x) { return div_const<7>(x); }
__device__ __forceinline__ float div27(float x) { return div_const<27>(x); }

// Exact scalings: x/4 and x/8 equal x*0.25 and x*0.125 in IEEE arithmetic.
__device__ __forceinline__ double quarter(double x) { return x * 0.25; }
__device__ __forceinline__ float quarter(float x) { return x * 0.25f; }
__device__ __forceinline__ double eighth(double x) { return x * 0.125; }
__device__ __forceinline__ float eighth(float x) { return x * 0.125f; }

// ---- coarsening sum of 8 children ----------------------------------------
// FP64: left to right, as ref/block.c:419-426.
__device__ __forceinline__ double sum8(const double *t)
{
   double s = t[0] + t[1];
   s = s + t[2];
   s = s + t[3];
   s = s + t[4];
   s = s + t[5];
   s = s + t[6];
   s = s + t[7];
   return s;
}

// FP32 pools: Neumaier-compensated FP64 sum in the same term order, rounded
// once to FP32.
__device__ __forceinline__ float sum8(const float *t)
{
   double s = (double) t[0], comp = 0.0;
#pragma unroll
   for (int q = 1; q < 8; q++) {
      double v = (double) t[q];
      double u = s + v;
      if (fabs(s) >= fabs(v))
         comp = comp + ((s - u) + v);
      else
         comp = comp + ((v - u) + s);
      s = u;
   }
   return (float) (s + comp);
}

// ---- exact fixed-point checksum of FP32 cells ------------------------------
// A cell v contributes trunc(v * 2^52) (toward zero), summed exactly in
// 128-bit two's complement.  The exact window is v == 0 or
// 2^-52 <= |v| < 2^10: larger or non-finite cells do not fit the
// accumulator, smaller non-zero ones would vanish.  A variable with a cell
// outside it takes the compensated FP64 sum instead (fp32_fallback_* in
// plain_kernels.cu); fixed52_add reports the miss.
//
// The term is formed with FP32 additions only (an FP64 or 64-bit integer
// conversion would run on this part's slow FP64 pipe): with x = |v| and
// magic constants M = 2^11, 2^-11, 2^-29, a round-toward-zero addition
// t = RZ(r + M) keeps r's bits down to ulp(M) = 2^-12, 2^-34, 2^-52 in the
// mantissa of t (r < 2^22 ulp(M), so t stays in M's binade), and
// r - (t - M) is the exact remainder.  So
//   floor(x * 2^52) = I1 * 2^40 + I2 * 2^18 + I3,
//   Ik = mantissa of tk = bits(tk) - bits(Mk)  (I1, I2 < 2^22, I3 < 2^18),
// and trunc(v * 2^52) = sign(v) * floor(x * 2^52).  The three pieces are
// summed in 32-bit words (mod 2^32, the sign as a factor of +-1, bits(Mk)
// removed once per term through the sum of the signs) and folded into the
// 128-bit accumulator by fixed52_flush at least every 512 terms, before
// |sum of I1| can reach 2^31.
struct Fixed52 {
   unsigned a1 = 0, a2 = 0, a3 = 0;   // sums of sign * bits(tk), mod 2^32
   int cnt = 0;                       // sum of the signs
   // window statistics of the terms added: the largest bits(|v|) and the
   // smallest bits(|v|) - 1 (a zero wraps to the top and counts as inside)
   unsigned umax = 0u, umin1 = 0xffffffffu;
};

// Adds the term of v (negate: its opposite, a term taken back, which the
// window statistics leave out).  Whether every term lay in the exact window
// is asked once, of the statistics (fixed52_window), not per term.
__device__ __forceinline__ void fixed52_add(float v, Fixed52 &p,
                                            bool negate = false)
{
   const float x = fabsf(v);
   const float t1 = __fadd_rz(x, 0x1p11f);
   const float r1 = __fsub_rn(x, __fsub_rn(t1, 0x1p11f));
   const float t2 = __fadd_rz(r1, 0x1p-11f);
   const float r2 = __fsub_rn(r1, __fsub_rn(t2, 0x1p-11f));
   const float t3 = __fadd_rz(r2, 0x1p-29f);
   int s = ((int) __float_as_uint(v) >> 31) | 1;
   if (negate)
      s = -s;
   p.a1 += (unsigned) s * __float_as_uint(t1);
   p.a2 += (unsigned) s * __float_as_uint(t2);
   p.a3 += (unsigned) s * __float_as_uint(t3);
   p.cnt += s;
   if (!negate) {
      const unsigned u = __float_as_uint(x);
      p.umax = max(p.umax, u);
      p.umin1 = min(p.umin1, u - 1u);
   }
}

// Whether every term added lay in the exact window: v == 0 or
// 2^-52 <= |v| < 2^10 (NaN and infinities have larger bits than 2^10).
__device__ __forceinline__ bool fixed52_window(const Fixed52 &p)
{
   return p.umax < __float_as_uint(1024.0f) &&
          p.umin1 >= __float_as_uint(0x1p-52f) - 1u;
}

// The compensated (Neumaier) FP64 step the checksum fallback uses: adds x
// to the running sum s with its correction c.  Once the sum is not finite
// the correction is left alone (it would turn an infinite sum into NaN),
// so an infinite cell gives an infinite sum, as plain summation does.
__host__ __device__ __forceinline__ void neumaier_add(double &s, double &c,
                                                      double x)
{
   const double t = s + x;
   if (isfinite(t)) {
      if (fabs(s) >= fabs(x))
         c = c + ((s - t) + x);
      else
         c = c + ((x - t) + s);
   }
   s = t;
}

// 128-bit two's complement accumulator held as (lo, hi): adds the
// sign-extended q with one carry chain.
__device__ __forceinline__ void acc128_add(unsigned long long &lo,
                                           unsigned long long &hi,
                                           long long q)
{
   const unsigned long long s = (unsigned long long) (q >> 63);
   asm("add.cc.u64 %0, %0, %2;\n\taddc.u64 %1, %1, %3;"
       : "+l"(lo), "+l"(hi)
       : "l"((unsigned long long) q), "l"(s));
}

// Folds the piece sums into (lo, hi) and clears them.
__device__ __forceinline__ void fixed52_flush(Fixed52 &p,
                                              unsigned long long &lo,
                                              unsigned long long &hi)
{
   const unsigned c = (unsigned) p.cnt;
   const long long i1 = (int) (p.a1 - c * __float_as_uint(0x1p11f));
   const long long i2 = (int) (p.a2 - c * __float_as_uint(0x1p-11f));
   const long long i3 = (int) (p.a3 - c * __float_as_uint(0x1p-29f));
   // i1 * 2^40 needs 128 bits; i2 * 2^18 + i3 fits in 64
   asm("add.cc.u64 %0, %0, %2;\n\taddc.u64 %1, %1, %3;"
       : "+l"(lo), "+l"(hi)
       : "l"((unsigned long long) i1 << 40),
         "l"((unsigned long long) (i1 >> 24)));
   acc128_add(lo, hi, i2 * (1ll << 18) + i3);
   p.a1 = p.a2 = p.a3 = 0;     // the window statistics carry on
   p.cnt = 0;
}

__device__ __forceinline__ void acc128_merge(unsigned long long &lo,
                                             unsigned long long &hi,
                                             unsigned long long lo2,
                                             unsigned long long hi2)
{
   unsigned long long n = lo + lo2;
   hi = hi + hi2 + (n < lo ? 1ull : 0ull);
   lo = n;
}

// Adds a warp's 128-bit fixed-point partial sums into acc[0..1] (every
// lane of the warp calls it).
__device__ __forceinline__ void warp_acc128_flush(unsigned long long lo,
                                                  unsigned long long hi,
                                                  unsigned long long *acc)
{
#pragma unroll
   for (int off = 16; off; off >>= 1) {
      unsigned long long l2 = __shfl_down_sync(0xffffffffu, lo, off);
      unsigned long long h2 = __shfl_down_sync(0xffffffffu, hi, off);
      acc128_merge(lo, hi, l2, h2);
   }
   if ((threadIdx.x & 31) == 0) {
      unsigned long long old = atomicAdd(acc, lo);
      unsigned long long hadd = hi + ((old + lo < old) ? 1ull : 0ull);
      if (hadd)
         atomicAdd(acc + 1, hadd);
   }
}

// Adds the CTA's accumulators into the global 128-bit acc[0..1].  Two
// atomics per CTA: the low word, then the high word plus the carry the low
// add produced.  The carries and the high words add up to the exact 128-bit
// total whatever order the CTAs arrive in.  blockDim.x must be a multiple
// of 32 and at most 1024.
__device__ __forceinline__ void block_acc128_flush(unsigned long long lo,
                                                   unsigned long long hi,
                                                   unsigned long long *acc)
{
   __shared__ unsigned long long s_lo[32], s_hi[32];
#pragma unroll
   for (int off = 16; off; off >>= 1) {
      unsigned long long l2 = __shfl_down_sync(0xffffffffu, lo, off);
      unsigned long long h2 = __shfl_down_sync(0xffffffffu, hi, off);
      acc128_merge(lo, hi, l2, h2);
   }
   const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
   if (lane == 0) {
      s_lo[w] = lo;
      s_hi[w] = hi;
   }
   __syncthreads();
   if (threadIdx.x == 0) {
      unsigned long long L = 0, H = 0;
      for (int q = 0; q < (int) (blockDim.x >> 5); q++)
         acc128_merge(L, H, s_lo[q], s_hi[q]);
      unsigned long long old = atomicAdd(acc, L);
      unsigned long long hadd = H + ((old + L < old) ? 1ull : 0ull);
      if (hadd)
         atomicAdd(acc + 1, hadd);
   }
   __syncthreads();
}

}  // namespace mamr
