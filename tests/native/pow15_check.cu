// Checks the device hg_pow15_25 and hg_pow15_or_25 (Goldschmidt square root from the hardware
// estimate) against the host method (correctly rounded sqrt, double-double,
// the midpoint family set exactly), written out here with CUDA's sqrt and rsqrt, on random x with uniformly
// random mantissas and exponents in [-100, 100] plus mantissas next to a
// binade edge; then a sample of device results against pow in extended
// (quad) precision on the host.  Prints
//   "<samples> <mismatches vs host method> <max seed error, log2> <quad samples> <quad mismatches> <cuda error>".
// Bounded grid-stride loops, one atomic counter per quantity.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cmath>
#include <cuda_runtime.h>
#include "hg_crmath.cuh"
#if defined(__aarch64__)
typedef long double q_t;
#define QPOW powl
#else
#include <quadmath.h>
typedef __float128 q_t;
#define QPOW powq
#endif

__device__ unsigned long long mix(unsigned long long x) {
  x ^= x >> 33; x *= 0xff51afd7ed558ccdull; x ^= x >> 33; x *= 0xc4ceb9fe1a85ec53ull; x ^= x >> 33;
  return x;
}
__device__ double make(unsigned long long r, int mode) {
  unsigned long long mant = r & 0x000FFFFFFFFFFFFFull;
  if (mode == 1) mant = 0x000FFFFFFFFFFFFFull - (r & 0xFF);
  if (mode == 2) mant = (r & 0xFF);
  const long long e = 1023 + (long long)((r >> 52) % 201) - 100;
  return __longlong_as_double((long long)(((unsigned long long)e << 52) | mant));
}
__device__ void host_method(double x, double& p15, double& p25) {
  const double s = sqrt(x);
  const double rho = fma(-s, s, x);
  const double d = rho * (0.5 * rsqrt(x));
  const double hi = x * s;
  double lo = fma(x, s, -hi);
  lo = fma(x, d, lo);
  p15 = hi + lo;
  const double h2 = x * hi;
  double l2 = fma(x, hi, -h2);
  l2 = fma(x, lo, l2);
  p25 = h2 + l2;
  // x = 2^(2q) (1 - 2^-53): the powers lie just above rounding midpoints
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  if ((b & 0x000FFFFFFFFFFFFFull) == 0x000FFFFFFFFFFFFFull && ((b >> 52) & 1u) == 0) {
    const int q = ((int)(b >> 52) - 1022) / 2;
    p15 = __longlong_as_double((long long)(((unsigned long long)(3 * q + 1022) << 52) | 0x000FFFFFFFFFFFFFull));
    p25 = __longlong_as_double((long long)(((unsigned long long)(5 * q + 1022) << 52) | 0x000FFFFFFFFFFFFEull));
  }
}
__global__ void check(unsigned long long n, unsigned long long seed, unsigned long long* bad,
                      unsigned long long* worst_seed, double* sample, int n_sample) {
  unsigned long long local = 0, worst = 0;
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;
       i += (unsigned long long)gridDim.x * blockDim.x) {
    const double x = make(mix(i + seed), (int)(i % 3));
    double a, b, c, d;
    hg_pow15_25(x, a, b);
    host_method(x, c, d);
    const double a1 = hg_pow15_or_25(x, false), b1 = hg_pow15_or_25(x, true);
    if (__double_as_longlong(a) != __double_as_longlong(c) || __double_as_longlong(b) != __double_as_longlong(d) ||
        __double_as_longlong(a1) != __double_as_longlong(c) || __double_as_longlong(b1) != __double_as_longlong(d))
      ++local;
    double y0;
    asm("rsqrt.approx.f64 %0, %1;" : "=d"(y0) : "d"(x));
    const double err = fabs(fma(y0 * y0, x, -1.0));  // ~2 x relative error of the estimate
    const unsigned long long eb = (unsigned long long)__double_as_longlong(err);
    if (eb > worst) worst = eb;
    if (i < (unsigned long long)n_sample) {
      sample[3 * i] = x;
      sample[3 * i + 1] = a;
      sample[3 * i + 2] = b;
    }
  }
  if (local) atomicAdd(bad, local);
  atomicMax(worst_seed, worst);
}
int main(int argc, char** argv) {
  const unsigned long long n = argc > 1 ? strtoull(argv[1], 0, 10) : (1ull << 30);
  const int n_sample = argc > 2 ? atoi(argv[2]) : (1 << 18);
  unsigned long long *bad, *worst;
  double* sample;
  cudaMalloc(&bad, 8);
  cudaMalloc(&worst, 8);
  cudaMalloc(&sample, sizeof(double) * 3 * n_sample);
  cudaMemset(bad, 0, 8);
  cudaMemset(worst, 0, 8);
  check<<<152 * 16, 256>>>(n, 777, bad, worst, sample, n_sample);
  unsigned long long hb = 0, hw = 0;
  cudaMemcpy(&hb, bad, 8, cudaMemcpyDeviceToHost);
  cudaMemcpy(&hw, worst, 8, cudaMemcpyDeviceToHost);
  double* hs = (double*)malloc(sizeof(double) * 3 * n_sample);
  cudaMemcpy(hs, sample, sizeof(double) * 3 * n_sample, cudaMemcpyDeviceToHost);
  const cudaError_t e = cudaGetLastError();
  long qbad = 0;
  for (int i = 0; i < n_sample; ++i) {
    const double x = hs[3 * i];
    if (hs[3 * i + 1] != (double)QPOW((q_t)x, (q_t)1.5)) ++qbad;
    if (hs[3 * i + 2] != (double)QPOW((q_t)x, (q_t)2.5)) ++qbad;
  }
  double w;
  memcpy(&w, &hw, 8);
  printf("%llu %llu %.2f %d %ld %s\n", n, hb, log2(w > 0 ? w : 1e-300), n_sample, qbad,
         e == cudaSuccess ? "ok" : cudaGetErrorString(e));
  return e == cudaSuccess ? 0 : 1;
}
