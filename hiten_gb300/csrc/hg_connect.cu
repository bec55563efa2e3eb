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
#include <stdint.h>
#include <math.h>

#include <algorithm>

#include "hitengpu.h"

namespace {

constexpr int kTile = 256;
constexpr int kBlock = 128;

// One tile of reference points in shared memory: their FP32 copies for the
// screen (converted once per call by to_float2_kernel: a double-to-float
// conversion holds GB300's FP64 pipe, so converting in every block's tile load
// costs as much as the screen).  The exact FP64 decisions read the rare
// surviving points from global memory.
struct Tile {
  float2 f[kTile];
};

__device__ __forceinline__ void load_tile(Tile& T, const float2* __restrict__ pf, int base, int n) {
  for (int t = threadIdx.x; t < n; t += blockDim.x) T.f[t] = pf[base + t];
}

__global__ void to_float2_kernel(int n, const double* __restrict__ x, const double* __restrict__ y,
                                 float2* __restrict__ out) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = make_float2((float)x[i], (float)y[i]);
}

// (d2, j) lexicographic minimum of two candidates (j < 0: none).  A scan in
// increasing j that keeps the first strict minimum ends at the lowest index
// of the minimal distance, which is this minimum over any split of the scan.
__device__ __forceinline__ void take_best(double& bd, int& bj, double d2, int j) {
  if (j >= 0 && (bj < 0 || d2 < bd || (d2 == bd && j < bj))) {
    bd = d2;
    bj = j;
  }
}

// The S lanes of a query are consecutive lanes of one warp: lane s of the
// query scans tile entries s, s + S, s + 2S, ...; every lane of the warp
// reaches the shuffles (no early exit).
template <int S>
__device__ __forceinline__ void combine_best(double& bd, int& bj) {
#pragma unroll
  for (int o = 1; o < S; o <<= 1) {
    const double d2 = __shfl_xor_sync(0xFFFFFFFFu, bd, o);
    const int j = __shfl_xor_sync(0xFFFFFFFFu, bj, o);
    take_best(bd, bj, d2, j);
  }
}

// Radius scan of one tile (entries s, s + S, ...): the FP32 box screen, then
// the exact FP64 test and the running strict minimum.
template <int S>
__device__ __forceinline__ void tile_radius(const Tile& T, const double* __restrict__ rx, const double* __restrict__ ry,
                                            int n, int s, int base, double xi, double yi, float xf, float yf, float Tf,
                                            double r2, int& c, double& bd, int& bj) {
#pragma unroll 4
  for (int t = s; t < n; t += S) {
    const float2 pf = T.f[t];
    const float dxf = xf - pf.x, dyf = yf - pf.y;
    if (fmaxf(fabsf(dxf), fabsf(dyf)) > Tf) continue;
    const double dx = xi - rx[base + t], dy = yi - ry[base + t];
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

// For each query point: number of reference points within eps (exact FP64
// test), and the nearest of them (strict <: the lowest index wins ties).
template <int S>
__global__ void __launch_bounds__(kBlock, 16) radius_best_kernel(int nq, const double* __restrict__ qx,
                                                              const double* __restrict__ qy, int nr,
                                                              const double* __restrict__ rx,
                                                              const double* __restrict__ ry,
                                                              const float2* __restrict__ rf, double r2, float T,
                                                              int* __restrict__ count, int* __restrict__ best_idx,
                                                              double* __restrict__ best_d2) {
  __shared__ Tile tile;
  const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int s = (int)(g % S);
  const long long i = g / S;
  const bool active = i < nq;
  const double xi = active ? qx[i] : 0.0, yi = active ? qy[i] : 0.0;
  const float xf = (float)xi, yf = (float)yi;
  int c = 0, bj = -1;
  double bd = 0.0;
  for (int base = 0; base < nr; base += kTile) {
    const int n = min(kTile, nr - base);
    __syncthreads();
    load_tile(tile, rf, base, n);
    __syncthreads();
    if (active) {
      if (n == kTile)
        tile_radius<S>(tile, rx, ry, kTile, s, base, xi, yi, xf, yf, T, r2, c, bd, bj);
      else
        tile_radius<S>(tile, rx, ry, n, s, base, xi, yi, xf, yf, T, r2, c, bd, bj);
    }
  }
#pragma unroll
  for (int o = 1; o < S; o <<= 1) c += __shfl_xor_sync(0xFFFFFFFFu, c, o);
  combine_best<S>(bd, bj);
  if (active && s == 0) {
    count[i] = c;
    best_idx[i] = bj;
    best_d2[i] = bj < 0 ? 0.0 : bd;
  }
}

// Pass-1 screen of the nearest-neighbour search.  With D the smallest FP32
// distance d2_f of the query (pass 0), the true minimum is at most
// M = D + E(D), where E(x) = 2^-20 (x + R (sqrt(2x)/(1 - u) + 2^-62)) + R2c
// bounds e for any pair with d2_f = x (|dx_f| + |dy_f| <= sqrt(2 (dx_f^2 +
// dy_f^2)) <= sqrt(2 d2_f)/(1 - u), the 2^-62 covering FP32 underflow of the
// squares).  A point can be the exact minimiser only if d2_f - E(d2_f) <= M,
// i.e. sqrt(d2_f) <= (c1 + sqrt(c1^2 + 4a(c0 + M)))/(2a) with a = 1 - 2^-20,
// c1 = 2^-20 R sqrt2/(1 - u), c0 = 2^-82 R + R2c.  Everything is evaluated
// rounding upward (each quantity only grows), so the returned FP32 threshold
// admits every possible minimiser.
__device__ __forceinline__ float nearest_threshold(float D, double R, double R2c) {
  if (!(D < INFINITY)) return INFINITY;
  const double u1 = 1.0 / (1.0 - 0x1p-24) * (1.0 + 0x1p-50);  // >= 1/(1 - u)
  const double d = (double)D;
  const double c1 = __dmul_ru(__dmul_ru(0x1p-20 * R, 1.4142135623730952), u1);  // sqrt2 rounded up
  const double c0 = __dadd_ru(0x1p-82 * R, R2c);
  const double E = __dadd_ru(__dadd_ru(0x1p-20 * d, __dmul_ru(c1, __dsqrt_ru(d))), c0);
  const double M = __dadd_ru(d, E);
  const double a = 1.0 - 0x1p-20;
  const double disc = __dadd_ru(__dmul_ru(c1, c1), __dmul_ru(4.0 * a, __dadd_ru(c0, M)));
  const double smax = __ddiv_ru(__dadd_ru(c1, __dsqrt_ru(disc)), 2.0 * a);
  return __double2float_ru(__dmul_ru(smax, smax));
}

// Pass-0 scan of one tile: the smallest FP32 distance over entries s, s + S,
// ... (self excluded when the query's own index lies in the tile).
template <int S, bool SELF>
__device__ __forceinline__ float tile_min(const Tile& T, int cnt, int s, int self, float xf, float yf, float D) {
#pragma unroll 4
  for (int t = s; t < cnt; t += S) {
    if (SELF && t == self) continue;
    const float2 pf = T.f[t];
    const float dxf = xf - pf.x, dyf = yf - pf.y;
    D = fminf(D, __fadd_rn(__fmul_rn(dxf, dxf), __fmul_rn(dyf, dyf)));
  }
  return D;
}

// Pass-1 scan of one tile: exact FP64 distances of the entries under thr.
template <int S, bool SELF>
__device__ __forceinline__ void tile_best(const Tile& T, const double* __restrict__ px, const double* __restrict__ py,
                                          int cnt, int s, int self, int base, double xi, double yi, float xf, float yf,
                                          float thr, double& bd, int& bj) {
#pragma unroll 4
  for (int t = s; t < cnt; t += S) {
    const float2 pf = T.f[t];
    const float dxf = xf - pf.x, dyf = yf - pf.y;
    if (!(__fadd_rn(__fmul_rn(dxf, dxf), __fmul_rn(dyf, dyf)) <= thr) || (SELF && t == self)) continue;
    const double dx = xi - px[base + t], dy = yi - py[base + t];
    const double d2 = dx * dx + dy * dy;
    if (bj < 0 ? d2 < 1e300 : d2 < bd) {
      bd = d2;
      bj = base + t;
    }
  }
}

// Nearest neighbour of every point within its own set (excluding itself;
// strict <, the lowest index wins ties).  Pass 0 finds the smallest FP32
// distance, pass 1 decides in FP64 among the points under the threshold
// above, which contain every point whose true distance can be minimal.
// The query's own index is tested only in the tile that holds it; full tiles
// run a fixed trip count.
template <int S>
__global__ void __launch_bounds__(kBlock, 16) nearest_kernel(int n, const double* __restrict__ px,
                                                              const double* __restrict__ py,
                                                              const float2* __restrict__ pf, double R, double R2c,
                                                              int* __restrict__ out) {
  __shared__ Tile tile;
  const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int s = (int)(g % S);
  const long long i = g / S;
  const bool active = i < n;
  const double xi = active ? px[i] : 0.0, yi = active ? py[i] : 0.0;
  const float xf = (float)xi, yf = (float)yi;
  float D = INFINITY;
  for (int base = 0; base < n; base += kTile) {
    const int cnt = min(kTile, n - base);
    __syncthreads();
    load_tile(tile, pf, base, cnt);
    __syncthreads();
    if (active) {
      const long long self = i - base;
      if (self >= 0 && self < cnt)
        D = tile_min<S, true>(tile, cnt, s, (int)self, xf, yf, D);
      else if (cnt == kTile)
        D = tile_min<S, false>(tile, kTile, s, -1, xf, yf, D);
      else
        D = tile_min<S, false>(tile, cnt, s, -1, xf, yf, D);
    }
  }
#pragma unroll
  for (int o = 1; o < S; o <<= 1) D = fminf(D, __shfl_xor_sync(0xFFFFFFFFu, D, o));
  const float thr = nearest_threshold(D, R, R2c);
  int bj = -1;
  double bd = 0.0;
  for (int base = 0; base < n; base += kTile) {
    const int cnt = min(kTile, n - base);
    __syncthreads();
    load_tile(tile, pf, base, cnt);
    __syncthreads();
    if (active) {
      const long long self = i - base;
      if (self >= 0 && self < cnt)
        tile_best<S, true>(tile, px, py, cnt, s, (int)self, base, xi, yi, xf, yf, thr, bd, bj);
      else if (cnt == kTile)
        tile_best<S, false>(tile, px, py, kTile, s, -1, base, xi, yi, xf, yf, thr, bd, bj);
      else
        tile_best<S, false>(tile, px, py, cnt, s, -1, base, xi, yi, xf, yf, thr, bd, bj);
    }
  }
  combine_best<S>(bd, bj);
  if (active && s == 0) out[i] = bj;
}

// Lanes per query: the largest of 8, 4, 2, 1 whose grid still fits in one
// wave of resident blocks (more lanes per query shorten each lane's scan;
// a second partial wave would cost a whole extra scan).
template <class K>
int lanes_per_query(K k8, long long n) {
  int dev = 0, sms = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k8, kBlock, 0) != cudaSuccess)
    return 1;
  const long long resident = (long long)sms * per_sm * kBlock;
  for (int S = 8; S > 1; S >>= 1)
    if (n * S <= resident) return S;
  return 1;
}

int check(const char* what) {
  (void)what;
  return cudaGetLastError() == cudaSuccess ? HG_OK : HG_ERR_CUDA;
}

// Segment refinement of the connection pairs (connections/backends.py:237-320,
// _closest_points_on_segments_2d, and the interpolation of :480-520): pair k
// joins a0 = pu[I], a1 = pu[IU] with b0 = ps[J], b1 = ps[JS]; where ok[k] its
// closest-point parameters s, t (the reference's scalar arithmetic and
// clamping order, every product and sum rounded on its own) give the states
// (1 - s) Xu[I] + s Xu[IU], (1 - t) Xs[J] + t Xs[JS] and the midpoint of the
// two closest points; elsewhere Xu[I], Xs[J] and pu[I].  An index outside its
// set writes NaN (it cannot come from the searches).
__global__ void refine_pairs_kernel(int n, const int* __restrict__ I, const int* __restrict__ IU,
                                    const int* __restrict__ J, const int* __restrict__ JS,
                                    const unsigned char* __restrict__ ok, int nu, const double* __restrict__ pu,
                                    const double* __restrict__ Xu, int ns, const double* __restrict__ ps,
                                    const double* __restrict__ Xs, double* __restrict__ xu, double* __restrict__ xs,
                                    double* __restrict__ pt) {
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const int i = I[k], j = J[k];
    const bool use = ok[k] != 0;
    const int iu = use ? IU[k] : i, js = use ? JS[k] : j;
    if (i < 0 || i >= nu || iu < 0 || iu >= nu || j < 0 || j >= ns || js < 0 || js >= ns) {
      for (int c = 0; c < 6; ++c) xu[6 * k + c] = xs[6 * k + c] = nan("");
      pt[2 * k] = pt[2 * k + 1] = nan("");
      continue;
    }
    if (!use) {
      for (int c = 0; c < 6; ++c) {
        xu[6 * k + c] = Xu[6LL * i + c];
        xs[6 * k + c] = Xs[6LL * j + c];
      }
      pt[2 * k] = pu[2LL * i];
      pt[2 * k + 1] = pu[2LL * i + 1];
      continue;
    }
    const double a0x = pu[2LL * i], a0y = pu[2LL * i + 1], a1x = pu[2LL * iu], a1y = pu[2LL * iu + 1];
    const double b0x = ps[2LL * j], b0y = ps[2LL * j + 1], b1x = ps[2LL * js], b1y = ps[2LL * js + 1];
    const double ux = a1x - a0x, uy = a1y - a0y, vx = b1x - b0x, vy = b1y - b0y;
    const double wx = a0x - b0x, wy = a0y - b0y;
    const double A = ux * ux + uy * uy, B = ux * vx + uy * vy, Cc = vx * vx + vy * vy;
    const double D = ux * wx + uy * wy, E = vx * wx + vy * wy;
    const double den = A * Cc - B * B;
    double s = 0.0, t = 0.0;
    if (den > 0.0) {
      s = (B * E - Cc * D) / den;
      t = (A * E - B * D) / den;
    }
    if (s < 0.0) {
      s = 0.0;
      if (Cc > 0.0) t = E / Cc;
    } else if (s > 1.0) {
      s = 1.0;
      if (Cc > 0.0) t = (E + B) / Cc;
    }
    if (t < 0.0) {
      t = 0.0;
      if (A > 0.0) {
        s = -D / A;
        s = s < 0.0 ? 0.0 : (s > 1.0 ? 1.0 : s);
      }
    } else if (t > 1.0) {
      t = 1.0;
      if (A > 0.0) {
        s = (B - D) / A;
        s = s < 0.0 ? 0.0 : (s > 1.0 ? 1.0 : s);
      }
    }
    for (int c = 0; c < 6; ++c) {
      xu[6 * k + c] = (1.0 - s) * Xu[6LL * i + c] + s * Xu[6LL * iu + c];
      xs[6 * k + c] = (1.0 - t) * Xs[6LL * j + c] + t * Xs[6LL * js + c];
    }
    pt[2 * k] = 0.5 * ((a0x + s * ux) + (b0x + t * vx));
    pt[2 * k + 1] = 0.5 * ((a0y + s * uy) + (b0y + t * vy));
  }
}

long long points_ws_bytes(long long n) { return ((n * (long long)sizeof(float2)) + 255) & ~255LL; }

// FP32 copy of a point set: into the caller's workspace when one is given
// (*owned = false), else into stream-ordered scratch that the caller frees on
// the stream after the search (*owned = true); nullptr on failure.
float2* float2_copy(int n, const double* x, const double* y, void* ws, long long ws_bytes, bool* owned,
                    cudaStream_t st) {
  void* p = ws;
  *owned = false;
  if (p) {
    if (ws_bytes < points_ws_bytes(n) || ((uintptr_t)p & 15) != 0) return nullptr;
  } else {
    if (cudaMallocAsync(&p, (size_t)n * sizeof(float2), st) != cudaSuccess) return nullptr;
    *owned = true;
  }
  const int blocks = (int)std::min<long long>(((long long)n + 255) / 256, 4096);
  to_float2_kernel<<<blocks, 256, 0, st>>>(n, x, y, (float2*)p);
  return (float2*)p;
}

}  // namespace

extern "C" {

long long hg_points_workspace_bytes(int n) { return n < 0 ? -1 : points_ws_bytes(n); }

int hg_radius_best(int nq, const double* qx, const double* qy, int nr, const double* rx, const double* ry, double eps,
                   double coord_max, int* count, int* best_idx, double* best_d2, void* workspace,
                   long long workspace_bytes, void* stream) {
  if (nq < 0 || nr < 0 || !(eps >= 0.0) || !(coord_max >= 0.0)) return HG_ERR_ARGS;
  if (workspace && (workspace_bytes < points_ws_bytes(nr) || ((uintptr_t)workspace & 15) != 0)) return HG_ERR_ARGS;
  if (nq == 0) return HG_OK;
  if (!qx || !qy || !count || !best_idx || !best_d2 || (nr > 0 && (!rx || !ry))) return HG_ERR_ARGS;
  const double T = (eps + 0x1p-22 * coord_max) * (1.0 + 0x1p-20);
  const float Tf = nextafterf((float)T, INFINITY);
  const cudaStream_t st = (cudaStream_t)stream;
  bool owned = false;
  float2* rf = nr > 0 ? float2_copy(nr, rx, ry, workspace, workspace_bytes, &owned, st) : nullptr;
  if (nr > 0 && !rf) return HG_ERR_CUDA;
  const int S = lanes_per_query(radius_best_kernel<8>, nq);
  const long long blocks = ((long long)nq * S + kBlock - 1) / kBlock;
  if (S == 8)
    radius_best_kernel<8><<<(unsigned)blocks, kBlock, 0, st>>>(nq, qx, qy, nr, rx, ry, rf, eps * eps, Tf, count, best_idx, best_d2);
  else if (S == 4)
    radius_best_kernel<4><<<(unsigned)blocks, kBlock, 0, st>>>(nq, qx, qy, nr, rx, ry, rf, eps * eps, Tf, count, best_idx, best_d2);
  else if (S == 2)
    radius_best_kernel<2><<<(unsigned)blocks, kBlock, 0, st>>>(nq, qx, qy, nr, rx, ry, rf, eps * eps, Tf, count, best_idx, best_d2);
  else
    radius_best_kernel<1><<<(unsigned)blocks, kBlock, 0, st>>>(nq, qx, qy, nr, rx, ry, rf, eps * eps, Tf, count, best_idx, best_d2);
  if (owned) cudaFreeAsync(rf, st);
  return check("radius_best_kernel");
}

int hg_nearest_neighbor(int n, const double* x, const double* y, double coord_max, int* out, void* workspace,
                        long long workspace_bytes, void* stream) {
  if (n < 0 || !(coord_max >= 0.0)) return HG_ERR_ARGS;
  if (workspace && (workspace_bytes < points_ws_bytes(n) || ((uintptr_t)workspace & 15) != 0)) return HG_ERR_ARGS;
  if (n == 0) return HG_OK;
  if (!x || !y || !out) return HG_ERR_ARGS;
  // R and 2^-43 R^2 as FP32 values rounded up (the bound's constants), passed in FP64
  const double R = (double)nextafterf((float)coord_max, INFINITY);
  const double R2c = (double)nextafterf((float)(0x1p-43 * coord_max * coord_max), INFINITY);
  const cudaStream_t st = (cudaStream_t)stream;
  bool owned = false;
  float2* pf = float2_copy(n, x, y, workspace, workspace_bytes, &owned, st);
  if (!pf) return HG_ERR_CUDA;
  const int S = lanes_per_query(nearest_kernel<8>, n);
  const long long blocks = ((long long)n * S + kBlock - 1) / kBlock;
  if (S == 8)
    nearest_kernel<8><<<(unsigned)blocks, kBlock, 0, st>>>(n, x, y, pf, R, R2c, out);
  else if (S == 4)
    nearest_kernel<4><<<(unsigned)blocks, kBlock, 0, st>>>(n, x, y, pf, R, R2c, out);
  else if (S == 2)
    nearest_kernel<2><<<(unsigned)blocks, kBlock, 0, st>>>(n, x, y, pf, R, R2c, out);
  else
    nearest_kernel<1><<<(unsigned)blocks, kBlock, 0, st>>>(n, x, y, pf, R, R2c, out);
  if (owned) cudaFreeAsync(pf, st);
  return check("nearest_kernel");
}

int hg_connection_refine(int n, const int* I, const int* IU, const int* J, const int* JS, const unsigned char* ok,
                         int nu, const double* pu, const double* Xu, int ns, const double* ps, const double* Xs,
                         double* xu, double* xs, double* pt, void* stream) {
  if (n < 0 || nu < 0 || ns < 0) return HG_ERR_ARGS;
  if (n == 0) return HG_OK;
  if (!I || !IU || !J || !JS || !ok || !pu || !Xu || !ps || !Xs || !xu || !xs || !pt) return HG_ERR_ARGS;
  const int blocks = (int)std::min<long long>(((long long)n + 127) / 128, 4096);
  refine_pairs_kernel<<<blocks, 128, 0, (cudaStream_t)stream>>>(n, I, IU, J, JS, ok, nu, pu, Xu, ns, ps, Xs, xu, xs,
                                                                 pt);
  return check("refine_pairs_kernel");
}

}  // extern "C"
