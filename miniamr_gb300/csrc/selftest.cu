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

// ---- FP64 pipe throughput --------------------------------------------------
// The bit-exact FP64 paths are bound by the FP64 pipe, not by HBM.  This
// probe measures what that pipe sustains: every thread runs 8 independent
// chains of dependent FP64 adds (or FMAs), enough warps in flight to cover
// the pipe's latency, a fixed number of iterations (no data-dependent
// loop), and the result is stored only under a condition the values never
// meet, so that nothing is optimised away.
namespace {

constexpr int kProbeIters = 2048;

template <bool FMA>
__global__ void __launch_bounds__(256) fp64_probe(double seed, double *sink)
{
   double a[8];
#pragma unroll
   for (int q = 0; q < 8; q++)
      a[q] = seed + (threadIdx.x + q) * 1e-9;
   const double c = 1e-300, m = 1.0 - 1e-16;
#pragma unroll 4
   for (int it = 0; it < kProbeIters; it++)
#pragma unroll
      for (int q = 0; q < 8; q++)
         a[q] = FMA ? __fma_rn(a[q], m, c) : __dadd_rn(a[q], c);
   double t = a[0];
#pragma unroll
   for (int q = 1; q < 8; q++)
      t = __dadd_rn(t, a[q]);
   if (t == 12345.678)
      *sink = t;
}

template <bool FMA>
float time_probe(int grid, double *sink, cudaStream_t s, cudaEvent_t e0,
                 cudaEvent_t e1)
{
   fp64_probe<FMA><<<grid, 256, 0, s>>>(1.0, sink);           // warm-up
   cudaEventRecord(e0, s);
   fp64_probe<FMA><<<grid, 256, 0, s>>>(1.0, sink);
   cudaEventRecord(e1, s);
   float ms = 0.f;
   if (cudaEventSynchronize(e1) != cudaSuccess ||
       cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess)
      return -1.f;
   return ms;
}

}  // namespace

extern "C" int mamr_probe_fp64_rate(double *add_per_s, double *fma_per_s)
{
   if (!add_per_s || !fma_per_s)
      return mamr::report_error(MAMR_EINVAL, "fp64 probe: null argument");
   int dev = 0, sms = 0;
   cudaError_t e = cudaGetDevice(&dev);
   if (e == cudaSuccess)
      e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
   double *sink = nullptr;
   cudaStream_t s = nullptr;
   cudaEvent_t e0 = nullptr, e1 = nullptr;
   if (e == cudaSuccess)
      e = cudaMalloc(&sink, sizeof(double));
   if (e == cudaSuccess)
      e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
   if (e == cudaSuccess)
      e = cudaEventCreate(&e0);
   if (e == cudaSuccess)
      e = cudaEventCreate(&e1);
   float ms_add = -1.f, ms_fma = -1.f;
   const int grid = sms * 8;
   if (e == cudaSuccess) {
      ms_add = time_probe<false>(grid, sink, s, e0, e1);
      ms_fma = time_probe<true>(grid, sink, s, e0, e1);
      e = cudaGetLastError();
   }
   if (e0) cudaEventDestroy(e0);
   if (e1) cudaEventDestroy(e1);
   if (s) cudaStreamDestroy(s);
   if (sink) cudaFree(sink);
   if (e != cudaSuccess || ms_add <= 0.f || ms_fma <= 0.f)
      return mamr::report_error(MAMR_ECUDA, "fp64 probe: %s",
                                cudaGetErrorString(e));
   const double ops = (double) grid * 256 * kProbeIters * 8;
   *add_per_s = ops / (ms_add * 1e-3);
   *fma_per_s = ops / (ms_fma * 1e-3);
   return MAMR_OK;
}
