// FP64-class H-matrix product on the FP32 pipes: Y += A X with the FP64 leaves
// held as pairs of floats (hi + lo, 48 significant bits) and double-float
// arithmetic (Dekker's exact product and Knuth's two-sum, T. J. Dekker, "A
// floating-point technique for extending the available precision", Numer.
// Math. 18 (1971); D. E. Knuth, TAOCP vol. 2, 4.2.2).  GB300 runs FP32 at 64x
// its FP64 rate, so the twelve FP32 operations of one double-float
// multiply-add are still several times faster than one FP64 FMA.  Used for the
// outer residual r = b - A x of mixed-precision iterative refinement, where
// the product must be accurate to well below the 1e-8 target; products of
// values in [2^-100, 2^100] keep about 2^-44 relative accuracy per leaf row.
//
// Same leaf schedule as the FP64 kernel (one CTA per leaf, descending cost,
// PG right-hand sides per pass, staged X rows); sums of partial results stay
// in double-float and reach Y as one FP64 atomic add of hi + lo.
#include <algorithm>

#include "ahx_matvec.cuh"

namespace ahx {
namespace {

constexpr int kThreads = 128;
constexpr int kCh = 128;  // X rows per staged chunk
constexpr int kKt = 32;   // low-rank columns per pass
constexpr int kNorm = 32; // terms between renormalisations of an accumulator
// loads in flight per thread in the streaming loops: deeper for narrow passes
template <int PG>
constexpr int kPF = PG <= 2 ? 4 : 1;


struct dfloat {
  float hi, lo;
};

// c += a * b.  p + e is the exact product of the hi parts (FMA), the cross
// terms enter e rounded; two-sum adds p to c.hi exactly, its error and e go
// to c.lo (unnormalised between renormalisations).
__device__ __forceinline__ void df_madd(dfloat& c, const dfloat a, const dfloat b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  const float s = __fadd_rn(c.hi, p);
  const float bb = __fsub_rn(s, c.hi);
  const float err = __fadd_rn(__fsub_rn(c.hi, __fsub_rn(s, bb)), __fsub_rn(p, bb));
  c.hi = s;
  c.lo = __fadd_rn(c.lo, __fadd_rn(e, err));
}

// c = two-sum(c.hi, c.lo): |lo| <= ulp(hi) / 2 again
__device__ __forceinline__ void df_norm(dfloat& c) {
  const float s = __fadd_rn(c.hi, c.lo);
  const float bb = __fsub_rn(s, c.hi);
  c.lo = __fadd_rn(__fsub_rn(c.hi, __fsub_rn(s, bb)), __fsub_rn(c.lo, bb));
  c.hi = s;
}

// c += a
__device__ __forceinline__ void df_add(dfloat& c, const dfloat a) {
  const float s = __fadd_rn(c.hi, a.hi);
  const float bb = __fsub_rn(s, c.hi);
  const float err = __fadd_rn(__fsub_rn(c.hi, __fsub_rn(s, bb)), __fsub_rn(a.hi, bb));
  c.hi = s;
  c.lo = __fadd_rn(c.lo, __fadd_rn(a.lo, err));
  df_norm(c);
}

// float -> double exactly, by integer operations only (keeps the conversion off
// the FP64 unit): normal, subnormal, infinite and NaN inputs
__device__ __forceinline__ double widen(float f) {
  const uint32_t u = __float_as_uint(f);
  const uint64_t sign = (uint64_t)(u & 0x80000000u) << 32;
  const uint32_t e = (u >> 23) & 0xffu, m = u & 0x7fffffu;
  uint64_t bits;
  if (e == 0xffu) {
    bits = sign | (0x7ffull << 52) | ((uint64_t)m << 29);
  } else if (e != 0u) {
    bits = sign | ((uint64_t)(e + 896u) << 52) | ((uint64_t)m << 29);
  } else if (m != 0u) {  // subnormal: m 2^-149 with its leading bit at position t
    const uint32_t t = 31u - (uint32_t)__clz((int)m);
    bits = sign | ((uint64_t)(t + 874u) << 52) | (((uint64_t)m << (52u - t)) & 0xfffffffffffffull);
  } else {
    bits = sign;
  }
  return __longlong_as_double((long long)bits);
}

// one FP64 atomic per output (the sum of the two widened halves rounds once)
__device__ __forceinline__ void emit(double* y, dfloat v) { atomicAdd(y, widen(v.hi) + widen(v.lo)); }

__device__ __forceinline__ dfloat ld(const float2* p) {
  const float2 v = __ldg(p);
  return dfloat{v.x, v.y};
}

template <int PG>
__device__ __forceinline__ void stage_x(dfloat (*Xs)[PG + 1], const DfArgs& a, uint32_t r0, uint32_t pg,
                                        uint32_t b2, uint32_t jb, uint32_t jn) {
  for (uint32_t e = threadIdx.x; e < jn * PG; e += kThreads) {
    const uint32_t j = e % jn, r = e / jn;
    Xs[j][r] = r < pg ? ld(a.X + (uint64_t)(r0 + r) * a.ldX + b2 + jb + j) : dfloat{0.f, 0.f};
  }
}

template <int PG>
__device__ __forceinline__ void emit_row(double* y, uint64_t ldY, const dfloat (&acc)[PG], uint32_t pg) {
#pragma unroll
  for (int r = 0; r < PG; ++r)
    if ((uint32_t)r < pg) emit(y + (uint64_t)r * ldY, acc[r]);
}

template <int PG>
__global__ void __launch_bounds__(kThreads, 8) mv_df_kernel(DfArgs a) {
  __shared__ dfloat Xs[kCh][PG + 1];
  __shared__ dfloat Ts[kKt][PG];
  const MvLeaf L = a.leaves[a.order[blockIdx.x]];
  const uint32_t tid = threadIdx.x;
  for (uint32_t r0 = 0; r0 < a.p; r0 += PG) {
    const uint32_t pg = min((uint32_t)PG, a.p - r0);
    if (L.rank < 0) {
      // one row per thread; the next column's element is loaded ahead
      const float2* D = a.arena + L.off;
      for (uint32_t ib = 0; ib < L.n1; ib += kThreads) {
        const uint32_t i = ib + tid;
        dfloat acc[PG];
#pragma unroll
        for (int r = 0; r < PG; ++r) acc[r] = dfloat{0.f, 0.f};
        for (uint32_t jb = 0; jb < L.n2; jb += kCh) {
          const uint32_t jn = min((uint32_t)kCh, L.n2 - jb);
          __syncthreads();
          stage_x<PG>(Xs, a, r0, pg, L.b2, jb, jn);
          __syncthreads();
          if (i < L.n1) {
            const float2* col = D + i + (uint64_t)jb * L.n1;
            for (uint32_t j0 = 0; j0 < jn; j0 += kNorm) {
              const uint32_t je = min(j0 + kNorm, jn);
              // the next PF columns' elements in flight (PF = 4 for narrow passes:
              // few operations per element, so more loads must overlap)
              dfloat buf[kPF<PG>];
#pragma unroll
              for (int u = 0; u < kPF<PG>; ++u)
                buf[u] = j0 + u < je ? ld(col + (uint64_t)(j0 + u) * L.n1) : dfloat{0.f, 0.f};
              for (uint32_t j = j0; j < je; ++j) {
                const dfloat av = buf[0];
#pragma unroll
                for (int u = 0; u + 1 < kPF<PG>; ++u) buf[u] = buf[u + 1];
                const uint32_t jf = j + kPF<PG>;
                buf[kPF<PG> - 1] = jf < je ? ld(col + (uint64_t)jf * L.n1) : dfloat{0.f, 0.f};
#pragma unroll
                for (int r = 0; r < PG; ++r) df_madd(acc[r], av, Xs[j][r]);
              }
#pragma unroll
              for (int r = 0; r < PG; ++r) df_norm(acc[r]);
            }
          }
        }
        if (i < L.n1) emit_row<PG>(a.Y + (uint64_t)r0 * a.ldY + L.b1 + i, a.ldY, acc, pg);
      }
    } else if (L.rank > 0) {
      const uint32_t k = (uint32_t)L.rank;
      const float2* U = a.arena + L.off;
      const float2* V = U + (uint64_t)L.n1 * k;
      for (uint32_t lb = 0; lb < k; lb += kKt) {
        const uint32_t kn = min((uint32_t)kKt, k - lb);
        // phase 1: Ts[l][r] = sum_j V[j, lb+l] X[b2+j, r0+r].  Thread (l, js): column
        // l of V, rows j = js mod S (consecutive threads, consecutive rows), all PG
        // right-hand sides; the S partial sums of each output meet in shared memory.
        const uint32_t KP = kn <= 1 ? 1u : 1u << (32 - __clz((int)(kn - 1)));  // kn rounded up to 2^m
        const uint32_t S = kThreads / KP, l = tid / S, js = tid % S;
        dfloat acc[PG];
#pragma unroll
        for (int r = 0; r < PG; ++r) acc[r] = dfloat{0.f, 0.f};
        const float2* vc = V + (uint64_t)(lb + l) * L.n2;
        for (uint32_t jb = 0; jb < L.n2; jb += kCh) {
          const uint32_t jn = min((uint32_t)kCh, L.n2 - jb);
          __syncthreads();
          stage_x<PG>(Xs, a, r0, pg, L.b2, jb, jn);
          __syncthreads();
          if (l < kn) {
            for (uint32_t j0 = js; j0 < jn; j0 += kNorm * S) {
              const uint32_t je = min(j0 + kNorm * S, jn);
              dfloat buf[kPF<PG>];
#pragma unroll
              for (int u = 0; u < kPF<PG>; ++u)
                buf[u] = j0 + u * S < je ? ld(vc + jb + j0 + u * S) : dfloat{0.f, 0.f};
              for (uint32_t j = j0; j < je; j += S) {
                const dfloat vv = buf[0];
#pragma unroll
                for (int u = 0; u + 1 < kPF<PG>; ++u) buf[u] = buf[u + 1];
                const uint32_t jf = j + kPF<PG> * S;
                buf[kPF<PG> - 1] = jf < je ? ld(vc + jb + jf) : dfloat{0.f, 0.f};
#pragma unroll
                for (int r = 0; r < PG; ++r) df_madd(acc[r], vv, Xs[j][r]);
              }
#pragma unroll
              for (int r = 0; r < PG; ++r) df_norm(acc[r]);
            }
          }
        }
        __syncthreads();  // staged rows no longer needed: Xs holds the partial sums
        {
          dfloat* buf = &Xs[0][0];
#pragma unroll
          for (int r = 0; r < PG; ++r) buf[((uint32_t)r * KP + l) * S + js] = acc[r];
          __syncthreads();
          for (uint32_t o = tid; o < kn * PG; o += kThreads) {
            const uint32_t r = o / kn, ll = o % kn;
            const dfloat* src = buf + (r * KP + ll) * S;
            dfloat t = src[0];
            for (uint32_t q = 1; q < S; ++q) df_add(t, src[q]);
            Ts[ll][r] = t;
          }
        }
        __syncthreads();
        // phase 2: Y[b1+i, r] += sum_l U[i, lb+l] Ts[l][r], one row per thread
        for (uint32_t ib = 0; ib < L.n1; ib += kThreads) {
          const uint32_t i = ib + tid;
          if (i < L.n1) {
            dfloat acc[PG];
#pragma unroll
            for (int r = 0; r < PG; ++r) acc[r] = dfloat{0.f, 0.f};
            const float2* uc = U + (uint64_t)lb * L.n1 + i;
            for (uint32_t l = 0; l < kn; ++l) {
              const dfloat uv = ld(uc + (uint64_t)l * L.n1);
#pragma unroll
              for (int r = 0; r < PG; ++r) df_madd(acc[r], uv, Ts[l][r]);
            }
            emit_row<PG>(a.Y + (uint64_t)r0 * a.ldY + L.b1 + i, a.ldY, acc, pg);
          }
        }
        __syncthreads();
      }
    }
  }
}

// dst[r + c * rows] = split(scale * src[r + c * ld])
__global__ void split_kernel(const double* __restrict__ src, uint64_t ld, uint64_t rows, uint32_t cols,
                             double scale, float2* __restrict__ dst) {
  const uint64_t total = rows * cols;
  for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < total;
       e += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t c = e / rows, r = e - c * rows;
    const double v = scale * src[r + c * ld];
    const float hi = __double2float_rn(v);
    dst[e] = make_float2(hi, __double2float_rn(v - (double)hi));
  }
}

}  // namespace

cudaError_t launch_split_df(const double* src, uint64_t ld, uint64_t rows, uint32_t cols, double scale,
                            void* dst, cudaStream_t s) {
  const uint64_t total = rows * cols;
  if (!total) return cudaSuccess;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const uint64_t want = (total + 255) / 256;
  const uint32_t grid = (uint32_t)std::min<uint64_t>(want, (uint64_t)std::max(sms, 1) * 16);
  split_kernel<<<grid, 256, 0, s>>>(src, ld, rows, cols, scale, static_cast<float2*>(dst));
  return cudaGetLastError();
}

cudaError_t launch_matvec_df(const DfArgs& a, cudaStream_t s) {
  if (a.nleaves == 0 || a.p == 0) return cudaSuccess;
  const uint32_t grid = a.nleaves;
  if (a.p == 1) mv_df_kernel<1><<<grid, kThreads, 0, s>>>(a);
  else if (a.p == 2) mv_df_kernel<2><<<grid, kThreads, 0, s>>>(a);
  else if (a.p <= 4) mv_df_kernel<4><<<grid, kThreads, 0, s>>>(a);
  else if (a.p <= 8) mv_df_kernel<8><<<grid, kThreads, 0, s>>>(a);
  else mv_df_kernel<16><<<grid, kThreads, 0, s>>>(a);
  count_product_launches(1);
  return cudaGetLastError();
}

}  // namespace ahx
