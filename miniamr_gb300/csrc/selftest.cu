// Device self-test of the division routines the kernels rely on.
//
// FP32: the kernels' x/7 and x/27 (a three-operation remainder-corrected
// quotient q0 = x*y, r = fma(-q0, c, x), q = fma(r, y, q0), y = RN(1/c),
// inside its exponent window) against the IEEE division __fdiv_rn for every
// float in [1, 2) -- both sides scale exactly with the exponent, so that
// binade decides the whole window -- and on hashed floats of every class.
// FP64: the kernels' div7/div27 against __ddiv_rn on hashed bit patterns
// covering all exponents (zeros, subnormals, inf and nan included).
#include "mamr_internal.h"
#include "arith.cuh"

namespace {

__device__ __forceinline__ unsigned mix32(unsigned z)
{
   z ^= z >> 16; z *= 0x7feb352du; z ^= z >> 15; z *= 0x846ca68bu;
   return z ^ (z >> 16);
}

__global__ void check_f32(unsigned long long *bad)
{
   unsigned long long b7 = 0, b27 = 0;
   for (unsigned m = blockIdx.x * blockDim.x + threadIdx.x; m < (1u << 24);
        m += gridDim.x * blockDim.x) {
      // first 2^23: the binade [1, 2); then hashed bit patterns
      const unsigned bits = m < (1u << 23) ? (0x3f800000u | m) : mix32(m);
      const float x = __uint_as_float(bits);
      b7 += __float_as_uint(mamr::div7(x)) !=
            __float_as_uint(__fdiv_rn(x, 7.0f));
      b27 += __float_as_uint(mamr::div27(x)) !=
             __float_as_uint(__fdiv_rn(x, 27.0f));
   }
   if (b7) atomicAdd(bad + 0, b7);
   if (b27) atomicAdd(bad + 1, b27);
}

__device__ __forceinline__ unsigned long long mix64(unsigned long long z)
{
   z += 0x9E3779B97F4A7C15ull;
   z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
   z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
   return z ^ (z >> 31);
}

__global__ void check_f64(long long n, unsigned long long *bad)
{
   unsigned long long b7 = 0, b27 = 0;
   for (long long q = blockIdx.x * (long long) blockDim.x + threadIdx.x;
        q < n; q += (long long) gridDim.x * blockDim.x) {
      unsigned long long bits = mix64((unsigned long long) q);
      // half the samples keep full random bits; half are pulled into
      // [2^-40, 2^10), the range stencil averages live in
      if (q & 1)
         bits = (bits & 0x800fffffffffffffull) |
                ((unsigned long long) (983 + (bits >> 52) % 50) << 52);
      const double x = __longlong_as_double((long long) bits);
      b7 += __double_as_longlong(mamr::div7(x)) !=
            __double_as_longlong(__ddiv_rn(x, 7.0));
      b27 += __double_as_longlong(mamr::div27(x)) !=
             __double_as_longlong(__ddiv_rn(x, 27.0));
   }
   if (b7) atomicAdd(bad + 2, b7);
   if (b27) atomicAdd(bad + 3, b27);
}

}  // namespace

extern "C" int mamr_selftest_division(int64_t n_fp64, int64_t *mismatches)
{
   if (!mismatches || n_fp64 < 0)
      return mamr::report_error(MAMR_EINVAL, "selftest: bad arguments");
   unsigned long long *d = nullptr;
   cudaError_t e = cudaMalloc(&d, 4 * sizeof(unsigned long long));
   if (e == cudaSuccess)
      e = cudaMemset(d, 0, 4 * sizeof(unsigned long long));
   if (e == cudaSuccess) {
      check_f32<<<152 * 8, 256>>>(d);
      if (n_fp64)
         check_f64<<<152 * 8, 256>>>(n_fp64, d);
      e = cudaDeviceSynchronize();
   }
   unsigned long long h[4] = {0, 0, 0, 0};
   if (e == cudaSuccess)
      e = cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
   if (d)
      cudaFree(d);
   if (e != cudaSuccess)
      return mamr::report_error(MAMR_ECUDA, "selftest: %s",
                                cudaGetErrorString(e));
   for (int q = 0; q < 4; q++)
      mismatches[q] = (int64_t) h[q];
   return MAMR_OK;
}
