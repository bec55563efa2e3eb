// Standalone FP64 pipe probe (not part of the library): DFMA throughput with 32/8/1 active lanes
// per warp at 4..32 warps/SM, DMUL, sqrt, IEEE division and __drcp_rn rates, and the cycles per warp
// instruction of 1..8 dependent chains per thread at one warp per SM sub-partition.  Bounded loops,
// writes only out[0].  Build: nvcc -gencode arch=compute_103a,code=sm_103a -O3 -o probe fp64_pipe_probe.cu
#include <cstdio>
#include <cuda_runtime.h>
__global__ void k_fma(double* out, int iters, double a, double b, int active) {
  double x[8];
  for (int i = 0; i < 8; ++i) x[i] = threadIdx.x * 1e-9 + i;
  if ((threadIdx.x & 31) < active) {
    for (int it = 0; it < iters; ++it)
#pragma unroll
      for (int i = 0; i < 8; ++i) x[i] = fma(x[i], a, b);
  }
  double s = 0; for (int i = 0; i < 8; ++i) s += x[i];
  if (s == 1.2345) out[0] = s;
}
__global__ void k_mul(double* out, int iters, double a, double b) {
  double x[8];
  for (int i = 0; i < 8; ++i) x[i] = threadIdx.x * 1e-9 + i;
  for (int it = 0; it < iters; ++it)
#pragma unroll
    for (int i = 0; i < 8; ++i) x[i] = x[i] * a;
  double s = 0; for (int i = 0; i < 8; ++i) s += x[i];
  if (s == 1.2345) out[0] = s;
}
__global__ void k_sqrt(double* out, int iters) {
  double x[8];
  for (int i = 0; i < 8; ++i) x[i] = 1.0 + threadIdx.x * 1e-9 + i;
  for (int it = 0; it < iters; ++it)
#pragma unroll
    for (int i = 0; i < 8; ++i) x[i] = sqrt(x[i]) + 1.0;
  double s = 0; for (int i = 0; i < 8; ++i) s += x[i];
  if (s == 1.2345) out[0] = s;
}
__global__ void k_div(double* out, int iters, double a) {
  double x[8];
  for (int i = 0; i < 8; ++i) x[i] = 1.0 + threadIdx.x * 1e-9 + i;
  for (int it = 0; it < iters; ++it)
#pragma unroll
    for (int i = 0; i < 8; ++i) x[i] = a / x[i] + 1.0;
  double s = 0; for (int i = 0; i < 8; ++i) s += x[i];
  if (s == 1.2345) out[0] = s;
}
__global__ void k_rcp(double* out, int iters) {
  double x[8];
  for (int i = 0; i < 8; ++i) x[i] = 1.0 + threadIdx.x * 1e-9 + i;
  for (int it = 0; it < iters; ++it)
#pragma unroll
    for (int i = 0; i < 8; ++i) x[i] = __drcp_rn(x[i]) + 1.0;
  double s = 0; for (int i = 0; i < 8; ++i) s += x[i];
  if (s == 1.2345) out[0] = s;
}
// K independent dependent chains per thread, one warp per SM sub-partition
// (blocks of four warps, one block per SM through shared memory); cycles
// per warp instruction from clock64 of block 0.  MUL: dmul then dadd.
template <int K, bool MUL>
__global__ void k_chains(double* out, int iters, double a, double b, long long* cyc) {
  extern __shared__ double pad[];
  double x[K];
  for (int i = 0; i < K; ++i) x[i] = threadIdx.x * 1e-9 + i + 1.0;
  const long long t0 = clock64();
  for (int it = 0; it < iters; ++it)
#pragma unroll
    for (int i = 0; i < K; ++i) x[i] = MUL ? x[i] * a + b : fma(x[i], a, b);
  const long long t1 = clock64();
  double s = 0;
  for (int i = 0; i < K; ++i) s += x[i];
  if (s == 1.2345) out[0] = s + pad[0];
  if (threadIdx.x == 0 && blockIdx.x == 0) cyc[0] = t1 - t0;
}
template <int K, bool MUL>
void chains(double* out, long long* cyc, int sms, int smem_sm) {
  const int iters = 4096;
  const size_t smem = smem_sm / 2 + 1024;
  cudaFuncSetAttribute(k_chains<K, MUL>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  for (int r = 0; r < 2; ++r) k_chains<K, MUL><<<sms, 128, smem>>>(out, iters, 0.999999, 1e-7, cyc);
  long long c = 0;
  cudaMemcpy(&c, cyc, 8, cudaMemcpyDeviceToHost);
  printf("%s chains %d: %.1f cycles per warp instruction\n", MUL ? "dmul+dadd" : "dfma", K,
         (double)c / iters / K / (MUL ? 2 : 1));
}
int main() {
  int sms; cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
  int clk; cudaDeviceGetAttribute(&clk, cudaDevAttrClockRate, 0);
  printf("SMs %d clock(kHz) %d\n", sms, clk);
  double* out; cudaMalloc(&out, 64);
  cudaEvent_t a, b; cudaEventCreate(&a); cudaEventCreate(&b);
  const int iters = 2048;
  for (int wpsm : {4, 8, 16, 32}) {
    int blocks = sms * wpsm / 4, threads = 128;
    for (int active : {32, 8, 1}) {
      k_fma<<<blocks, threads>>>(out, 16, 0.9999, 1e-7, active);
      cudaEventRecord(a); k_fma<<<blocks, threads>>>(out, iters, 0.9999, 1e-7, active); cudaEventRecord(b);
      cudaEventSynchronize(b); float ms; cudaEventElapsedTime(&ms, a, b);
      double lane_ops = 8.0 * iters * threads * (double)blocks * active / 32.0;
      double warp_instr = 8.0 * iters * threads / 32.0 * blocks;
      printf("fma warps/SM %2d active %2d: %.3f ms  lane-FMA/s %.3e  TFLOP/s(lanes) %.3f  warp-instr/clk/SM %.4f\n",
             wpsm, active, ms, lane_ops / (ms * 1e-3), 2 * lane_ops / (ms * 1e-3) / 1e12,
             warp_instr / (ms * 1e-3) / (clk * 1e3) / sms);
    }
  }
  int blocks = sms * 4, threads = 128;
  float ms;
  k_mul<<<blocks, threads>>>(out, 16, 0.9999, 1e-7);
  cudaEventRecord(a); k_mul<<<blocks, threads>>>(out, iters, 0.9999, 1e-7); cudaEventRecord(b); cudaEventSynchronize(b);
  cudaEventElapsedTime(&ms, a, b); printf("dmul: %.3e lane-op/s\n", 8.0 * iters * threads * blocks / (ms * 1e-3));
  cudaEventRecord(a); k_sqrt<<<blocks, threads>>>(out, iters / 8); cudaEventRecord(b); cudaEventSynchronize(b);
  cudaEventElapsedTime(&ms, a, b); printf("sqrt+add: %.3e lane-op/s\n", 8.0 * iters / 8 * threads * blocks / (ms * 1e-3));
  cudaEventRecord(a); k_div<<<blocks, threads>>>(out, iters / 8, 3.0); cudaEventRecord(b); cudaEventSynchronize(b);
  cudaEventElapsedTime(&ms, a, b); printf("div+add: %.3e lane-op/s\n", 8.0 * iters / 8 * threads * blocks / (ms * 1e-3));
  cudaEventRecord(a); k_rcp<<<blocks, threads>>>(out, iters / 8); cudaEventRecord(b); cudaEventSynchronize(b);
  cudaEventElapsedTime(&ms, a, b); printf("rcp+add: %.3e lane-op/s\n", 8.0 * iters / 8 * threads * blocks / (ms * 1e-3));
  int smem_sm = 0;
  cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, 0);
  long long* cyc;
  cudaMalloc(&cyc, 64);
  chains<1, false>(out, cyc, sms, smem_sm);
  chains<2, false>(out, cyc, sms, smem_sm);
  chains<4, false>(out, cyc, sms, smem_sm);
  chains<8, false>(out, cyc, sms, smem_sm);
  chains<1, true>(out, cyc, sms, smem_sm);
  chains<2, true>(out, cyc, sms, smem_sm);
  chains<4, true>(out, cyc, sms, smem_sm);
  printf("err: %s\n", cudaGetErrorString(cudaGetLastError()));
  return 0;
}
