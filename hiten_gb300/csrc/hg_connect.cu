// Section-point matching for heteroclinic connections
// (connections/backends.py:31-235): radius pairs between two 2-D point sets
// with each query point's nearest partner, and each set's nearest neighbour.
//
// Both searches are all-pairs.  GB300 retires FP32 ~60x faster than FP64, so
// every pair is first screened in FP32 with a margin that provably covers
// the FP32 rounding, and only the survivors are decided in FP64 with the
// reference's exact comparisons (dx*dx + dy*dy <= r^2, strict < for minima,
// the lower index winning ties).  Results are therefore those of the FP64
// loops.  Error bounds (u = 2^-24, R = max |coordinate| of both sets,
// a_f = fl32(a)): |a_f - a| <= u R; dx_f = fl32(a_f - b_f) satisfies
// |dx_f - dx| <= u|dx_f|(1 + 2u) + 2uR =: eta; d2_f = fl32(fl32(dx_f^2) +
// fl32(dy_f^2)) satisfies |d2_f - d2| <= 2^-21.8 d2_f + 2^-21.9 R(|dx_f| +
// |dy_f|) + 2^-45 R^2, bounded here by
//   e = 2^-20 (d2_f + R(|dx_f| + |dy_f|)) + 2^-43 R^2   (evaluated in FP32,
// the factor-two slack absorbing its own rounding).  Radius screen: a pair
// needs |dx|, |dy| <= eps, hence |dx_f|, |dy_f| <= T = (eps + 2^-22 R)(1 + 2^-20).
#include <cuda_runtime.h>
#include <math.h>

#include "hitengpu.h"

namespace {

constexpr int kTile = 256;
constexpr int kBlock = 128;

struct P2 {
  double x, y;
};

__device__ __forceinline__ float err_bound(float d2f, float adx, float ady, float R, float R2c) {
  return 0x1p-20f * (d2f + R * (adx + ady)) + R2c;
}

// For each query point: number of reference points within eps (exact FP64
// test), and the nearest of them (strict <: the lowest index wins ties).
__global__ void __launch_bounds__(kBlock) radius_best_kernel(int nq, const double* __restrict__ qx,
                                                              const double* __restrict__ qy, int nr,
                                                              const double* __restrict__ rx,
                                                              const double* __restrict__ ry, double r2, float T,
                                                              int* __restrict__ count, int* __restrict__ best_idx,
                                                              double* __restrict__ best_d2) {
  __shared__ float sfx[kTile], sfy[kTile];
  __shared__ double sdx[kTile], sdy[kTile];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = i < nq;
  const double xi = active ? qx[i] : 0.0, yi = active ? qy[i] : 0.0;
  const float xf = (float)xi, yf = (float)yi;
  int c = 0, bj = -1;
  double bd = 0.0;
  for (int base = 0; base < nr; base += kTile) {
    const int n = min(kTile, nr - base);
    __syncthreads();
    for (int t = threadIdx.x; t < n; t += blockDim.x) {
      const double a = rx[base + t], b = ry[base + t];
      sdx[t] = a;
      sdy[t] = b;
      sfx[t] = (float)a;
      sfy[t] = (float)b;
    }
    __syncthreads();
    if (active) {
      for (int t = 0; t < n; ++t) {
        const float dxf = xf - sfx[t], dyf = yf - sfy[t];
        if (fabsf(dxf) > T || fabsf(dyf) > T) continue;
        const double dx = xi - sdx[t], dy = yi - sdy[t];
        const double d2 = dx * dx + dy * dy;
        if (d2 <= r2) {
          ++c;
          if (bj < 0 || d2 < bd) {
            bd = d2;
            bj = base + t;
          }
        }
      }
    }
  }
  if (active) {
    count[i] = c;
    best_idx[i] = bj;
    best_d2[i] = bj < 0 ? 0.0 : bd;
  }
}

// Nearest neighbour of every point within its own set (excluding itself;
// strict <, the lowest index wins ties).  Pass 1 finds m = min_j (d2_f + e),
// an upper bound on the true minimum; pass 2 decides in FP64 among the j
// with d2_f - e <= m, which contain every j whose true distance can be
// minimal.
__global__ void __launch_bounds__(kBlock) nearest_kernel(int n, const double* __restrict__ px,
                                                          const double* __restrict__ py, float R, float R2c,
                                                          int* __restrict__ out) {
  __shared__ float sfx[kTile], sfy[kTile];
  __shared__ double sdx[kTile], sdy[kTile];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = i < n;
  const double xi = active ? px[i] : 0.0, yi = active ? py[i] : 0.0;
  const float xf = (float)xi, yf = (float)yi;
  float m = INFINITY;
  for (int pass = 0; pass < 2; ++pass) {
    int bj = -1;
    double bd = 1e300;
    for (int base = 0; base < n; base += kTile) {
      const int cnt = min(kTile, n - base);
      __syncthreads();
      for (int t = threadIdx.x; t < cnt; t += blockDim.x) {
        const double a = px[base + t], b = py[base + t];
        sdx[t] = a;
        sdy[t] = b;
        sfx[t] = (float)a;
        sfy[t] = (float)b;
      }
      __syncthreads();
      if (active) {
        for (int t = 0; t < cnt; ++t) {
          const int j = base + t;
          if (j == i) continue;
          const float dxf = xf - sfx[t], dyf = yf - sfy[t];
          const float d2f = __fadd_rn(__fmul_rn(dxf, dxf), __fmul_rn(dyf, dyf));
          const float e = err_bound(d2f, fabsf(dxf), fabsf(dyf), R, R2c);
          if (pass == 0) {
            m = fminf(m, __fadd_ru(d2f, e));
          } else if (__fsub_rd(d2f, e) <= m) {
            const double dx = xi - sdx[t], dy = yi - sdy[t];
            const double d2 = dx * dx + dy * dy;
            if (d2 < bd) {
              bd = d2;
              bj = j;
            }
          }
        }
      }
    }
    if (pass == 1 && active) out[i] = bj;
  }
}

int check(const char* what) {
  (void)what;
  return cudaGetLastError() == cudaSuccess ? HG_OK : HG_ERR_CUDA;
}

}  // namespace

extern "C" {

int hg_radius_best(int nq, const double* qx, const double* qy, int nr, const double* rx, const double* ry, double eps,
                   double coord_max, int* count, int* best_idx, double* best_d2, void* stream) {
  if (nq < 0 || nr < 0 || !(eps >= 0.0) || !(coord_max >= 0.0)) return HG_ERR_ARGS;
  if (nq == 0) return HG_OK;
  if (!qx || !qy || !count || !best_idx || !best_d2 || (nr > 0 && (!rx || !ry))) return HG_ERR_ARGS;
  const double T = (eps + 0x1p-22 * coord_max) * (1.0 + 0x1p-20);
  const float Tf = nextafterf((float)T, INFINITY);
  radius_best_kernel<<<(nq + kBlock - 1) / kBlock, kBlock, 0, (cudaStream_t)stream>>>(
      nq, qx, qy, nr, rx, ry, eps * eps, Tf, count, best_idx, best_d2);
  return check("radius_best_kernel");
}

int hg_nearest_neighbor(int n, const double* x, const double* y, double coord_max, int* out, void* stream) {
  if (n < 0 || !(coord_max >= 0.0)) return HG_ERR_ARGS;
  if (n == 0) return HG_OK;
  if (!x || !y || !out) return HG_ERR_ARGS;
  const float R = nextafterf((float)coord_max, INFINITY);
  const float R2c = nextafterf((float)(0x1p-43 * coord_max * coord_max), INFINITY);
  nearest_kernel<<<(n + kBlock - 1) / kBlock, kBlock, 0, (cudaStream_t)stream>>>(n, x, y, R, R2c, out);
  return check("nearest_kernel");
}

}  // extern "C"
