// Device-side primitives shared by the assembly and product kernels.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace ahx {

constexpr double kFourPi = 4.0 * 3.14159265358979323846;

// Collocation points in permuted (cluster) order, structure of arrays.
struct PointsSoA {
  const double* x;
  const double* y;
  const double* z;
};

// Laplace single-layer entry K(i,j) = 1/(4 pi |x_i - x_j|), diag = 1/(4 pi h).
// Evaluated with explicitly rounded operations (no contraction to FMA) so that
// every entry equals the host evaluation bit for bit.
__device__ __forceinline__ double lap_entry(const PointsSoA& P, uint32_t i, uint32_t j,
                                            double xi, double yi, double zi, double diag) {
  if (i == j) return diag;
  const double dx = __dsub_rn(xi, P.x[j]);
  const double dy = __dsub_rn(yi, P.y[j]);
  const double dz = __dsub_rn(zi, P.z[j]);
  const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
  return __ddiv_rn(1.0, __dmul_rn(kFourPi, __dsqrt_rn(r2)));
}

// The same kernel inside the ACA steps, evaluated as (1/(4 pi)) * rsqrt(r^2):
// within an ulp of lap_entry and several times fewer FP64 instructions (the
// FP64 pipe is what bounds the assembly on this GPU).  Dense leaves use
// lap_entry.
__device__ __forceinline__ double lap_entry_aca(const PointsSoA& P, uint32_t i, uint32_t j,
                                                double xi, double yi, double zi, double diag) {
  if (i == j) return diag;
  const double dx = xi - P.x[j];
  const double dy = yi - P.y[j];
  const double dz = zi - P.z[j];
  const double r2 = fma(dz, dz, fma(dy, dy, dx * dx));
  return (1.0 / kFourPi) * rsqrt(r2);
}

// a > b for non-negative doubles, on the integer pipe (IEEE order of the bit patterns)
__device__ __forceinline__ bool gt_nonneg(double a, double b) {
  return __double_as_longlong(a) > __double_as_longlong(b);
}

// ---------------------------------------------------------------------------
// Cooperative groups of G threads working on one block.  G == 32: one warp
// (several groups per CTA).  G > 32: the whole CTA.  All reductions are
// all-reduces whose result is bitwise identical on every thread (xor
// butterflies are symmetric; the cross-warp stage combines warp results in a
// fixed order), so control decisions taken on reduced values stay uniform.

struct ArgMax {
  double v;      // |value| (>= 0); 0 means "no candidate"
  uint32_t idx;  // smallest index among equal maxima
  double sv;     // signed value at idx
};

__device__ __forceinline__ void argmax_merge(ArgMax& a, const ArgMax& b) {
  const long long bv = __double_as_longlong(b.v), av = __double_as_longlong(a.v);
  if (bv > av || (bv == av && b.idx < a.idx)) a = b;
}

struct ArgMinI {
  int v;         // value (INT_MAX: none)
  uint32_t idx;  // smallest index among equal minima
};

__device__ __forceinline__ void argmin_merge(ArgMinI& a, const ArgMinI& b) {
  if (b.v < a.v || (b.v == a.v && b.idx < a.idx)) a = b;
}

template <int G>
struct Group;

template <>
struct Group<32> {
  uint32_t rank;  // 0..31
  __device__ explicit Group(uint32_t r) : rank(r) {}
  __device__ static void sync() { __syncwarp(); }
  __device__ static double sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
  }
  __device__ static void sum2(double& a, double& b) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      a += __shfl_xor_sync(0xffffffffu, a, o);
      b += __shfl_xor_sync(0xffffffffu, b, o);
    }
  }
  __device__ static void sum3(double& a, double& b, double& c) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      a += __shfl_xor_sync(0xffffffffu, a, o);
      b += __shfl_xor_sync(0xffffffffu, b, o);
      c += __shfl_xor_sync(0xffffffffu, c, o);
    }
  }
  __device__ static ArgMax argmax(ArgMax a) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      ArgMax b;
      b.v = __shfl_xor_sync(0xffffffffu, a.v, o);
      b.idx = __shfl_xor_sync(0xffffffffu, a.idx, o);
      b.sv = __shfl_xor_sync(0xffffffffu, a.sv, o);
      argmax_merge(a, b);
    }
    return a;
  }
  __device__ static ArgMinI argmin(ArgMinI a) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      ArgMinI b;
      b.v = __shfl_xor_sync(0xffffffffu, a.v, o);
      b.idx = __shfl_xor_sync(0xffffffffu, a.idx, o);
      argmin_merge(a, b);
    }
    return a;
  }
  __device__ static uint32_t umin(uint32_t v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = min(v, (uint32_t)__shfl_xor_sync(0xffffffffu, v, o));
    return v;
  }
  __device__ static int imax(int v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
  }
};

// Whole-CTA group of G threads (G a multiple of 32, <= 1024).  Uses a small
// shared scratch area; every call begins and ends with a CTA barrier.
template <int G>
struct Group {
  static constexpr int W = G / 32;
  uint32_t rank;
  double* red;  // shared scratch of 3*W doubles + 2*W words (see ctor users)
  __device__ Group(uint32_t r, double* scratch) : rank(r), red(scratch) {}
  __device__ static void sync() { __syncthreads(); }
  __device__ double sum(double v) const {
    v = Group<32>::sum(v);
    __syncthreads();
    if ((rank & 31) == 0) red[rank >> 5] = v;
    __syncthreads();
    double s = red[0];
    for (int w = 1; w < W; ++w) s += red[w];
    return s;
  }
  __device__ void sum2(double& a, double& b) const {
    Group<32>::sum2(a, b);
    __syncthreads();
    if ((rank & 31) == 0) {
      red[rank >> 5] = a;
      red[W + (rank >> 5)] = b;
    }
    __syncthreads();
    a = red[0];
    b = red[W];
    for (int w = 1; w < W; ++w) {
      a += red[w];
      b += red[W + w];
    }
  }
  __device__ void sum3(double& a, double& b, double& c) const {
    Group<32>::sum3(a, b, c);
    __syncthreads();
    if ((rank & 31) == 0) {
      red[rank >> 5] = a;
      red[W + (rank >> 5)] = b;
      red[2 * W + (rank >> 5)] = c;
    }
    __syncthreads();
    a = red[0];
    b = red[W];
    c = red[2 * W];
    for (int w = 1; w < W; ++w) {
      a += red[w];
      b += red[W + w];
      c += red[2 * W + w];
    }
  }
  __device__ ArgMax argmax(ArgMax a) const {
    a = Group<32>::argmax(a);
    __syncthreads();
    uint32_t* ri = reinterpret_cast<uint32_t*>(red + 2 * W);
    if ((rank & 31) == 0) {
      red[rank >> 5] = a.v;
      red[W + (rank >> 5)] = a.sv;
      ri[rank >> 5] = a.idx;
    }
    __syncthreads();
    ArgMax r{red[0], ri[0], red[W]};
    for (int w = 1; w < W; ++w) argmax_merge(r, ArgMax{red[w], ri[w], red[W + w]});
    return r;
  }
  __device__ ArgMinI argmin(ArgMinI a) const {
    a = Group<32>::argmin(a);
    __syncthreads();
    int* rv = reinterpret_cast<int*>(red);
    uint32_t* ri = reinterpret_cast<uint32_t*>(red) + W;
    if ((rank & 31) == 0) {
      rv[rank >> 5] = a.v;
      ri[rank >> 5] = a.idx;
    }
    __syncthreads();
    ArgMinI r{rv[0], ri[0]};
    for (int w = 1; w < W; ++w) argmin_merge(r, ArgMinI{rv[w], ri[w]});
    return r;
  }
  __device__ uint32_t umin(uint32_t v) const {
    v = Group<32>::umin(v);
    __syncthreads();
    uint32_t* ri = reinterpret_cast<uint32_t*>(red);
    if ((rank & 31) == 0) ri[rank >> 5] = v;
    __syncthreads();
    uint32_t r = ri[0];
    for (int w = 1; w < W; ++w) r = min(r, ri[w]);
    return r;
  }
  __device__ int imax(int v) const {
    v = Group<32>::imax(v);
    __syncthreads();
    int* ri = reinterpret_cast<int*>(red);
    if ((rank & 31) == 0) ri[rank >> 5] = v;
    __syncthreads();
    int r = ri[0];
    for (int w = 1; w < W; ++w) r = max(r, ri[w]);
    return r;
  }
};

}  // namespace ahx
