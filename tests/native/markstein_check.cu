// Checks hg_div_rn (quotient from the correctly rounded reciprocal) against
// IEEE division on the GPU: random operands with uniformly random mantissas
// and exponents in [-40, 40], plus operands whose mantissas sit next to a
// binade edge.  Prints "<samples> <mismatches>".  Bounded grid-stride loop,
// one atomic counter.
#include <cstdio>
#include <cstdlib>
#include <cuda_runtime.h>
#include "hg_crmath.cuh"

__device__ unsigned long long mix(unsigned long long x) {
  x ^= x >> 33; x *= 0xff51afd7ed558ccdull; x ^= x >> 33; x *= 0xc4ceb9fe1a85ec53ull; x ^= x >> 33;
  return x;
}
__device__ double make(unsigned long long r, int mode) {
  unsigned long long mant = r & 0x000FFFFFFFFFFFFFull;
  if (mode == 1) mant = 0x000FFFFFFFFFFFFFull - (r & 0xFF);  // just below the next power of two
  if (mode == 2) mant = (r & 0xFF);                          // just above a power of two
  const long long e = 1023 + (long long)((r >> 52) % 81) - 40;
  const unsigned long long sign = (r >> 63) << 63;
  return __longlong_as_double((long long)(sign | ((unsigned long long)e << 52) | mant));
}
__global__ void check(unsigned long long n, unsigned long long seed, unsigned long long* bad) {
  unsigned long long local = 0;
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;
       i += (unsigned long long)gridDim.x * blockDim.x) {
    const unsigned long long r1 = mix(i * 2 + seed), r2 = mix(i * 2 + 1 + seed * 7);
    const int ma = (int)(i % 3), mb = (int)((i / 3) % 3);
    const double a = make(r1, ma), b = make(r2, mb);
    const double q = a / b;
    const double m = hg_div_rn(a, b, hg_rcp_rn(b));
    if (__double_as_longlong(q) != __double_as_longlong(m)) ++local;
  }
  if (local) atomicAdd(bad, local);
}
int main(int argc, char** argv) {
  const unsigned long long n = argc > 1 ? strtoull(argv[1], 0, 10) : (1ull << 30);
  unsigned long long* bad;
  cudaMalloc(&bad, 8);
  cudaMemset(bad, 0, 8);
  check<<<152 * 16, 256>>>(n, 12345, bad);
  unsigned long long h = 0;
  cudaMemcpy(&h, bad, 8, cudaMemcpyDeviceToHost);
  const cudaError_t e = cudaGetLastError();
  printf("%llu %llu %s\n", n, h, cudaGetErrorString(e));
  cudaFree(bad);
  return e == cudaSuccess ? 0 : 1;
}
