// Complex H-matrix product Y += d op(A) X with op = A (mltaGeHVec / mltaGeHGeM),
// A^H (mltaGeHhVec / mltaGeHhGeM) or A^T (mltaGeHtVec / mltaGeHtGeM) for the
// complex leaves of H/mltaGeHVec.cpp:16-150 and H/mblock.cpp:126-215: a low-rank
// leaf U V^H applies as U (V^H x), V (U^H x) or conj(V) (U^T x); a dense leaf D
// as D x, D^H x or D^T x (Include/mblock.h:99-130).
//
// One CTA per leaf, leaves in descending cost order.  Right-hand sides in
// groups of PG; the input rows of a leaf are staged in shared memory; the
// low-rank inner products T = Q^H X (Q the input-side factor) split every
// output over several threads and sum the parts in a fixed order; the output
// side has one row per thread (coalesced factor reads).  Complex128 leaves
// accumulate in FP64, complex64 leaves in FP32; contributions reach Y through
// FP64 atomics (leaves share rows).
#include <algorithm>

#include "ahx_matvec.cuh"

namespace ahx {
namespace {

constexpr int kThreads = 128;
constexpr int kCh = 64;  // input rows per staged chunk

template <typename R>
struct C2 {
  R re, im;
};

// acc += a x
template <typename R>
__device__ __forceinline__ void cfma(C2<R>& acc, const C2<R>& a, const C2<R>& x) {
  acc.re = fma(a.re, x.re, acc.re);
  acc.re = fma(-a.im, x.im, acc.re);
  acc.im = fma(a.re, x.im, acc.im);
  acc.im = fma(a.im, x.re, acc.im);
}

__device__ __forceinline__ C2<double> ldz(const double2* p, bool cj) {
  const double2 v = __ldg(p);
  return C2<double>{v.x, cj ? -v.y : v.y};
}
__device__ __forceinline__ C2<float> ldz(const float2* p, bool cj) {
  const float2 v = __ldg(p);
  return C2<float>{v.x, cj ? -v.y : v.y};
}

// Xs[j][r] = X[row0 + j, r0 + r] for j < jn (zero for r >= pg)
template <typename R, int PG>
__device__ __forceinline__ void stage(C2<R> (*Xs)[PG], const ZArgs& a, uint32_t r0, uint32_t pg, uint32_t row0,
                                      uint32_t jn) {
  for (uint32_t e = threadIdx.x; e < jn * PG; e += kThreads) {
    const uint32_t j = e % jn, r = e / jn;
    C2<R> v{(R)0, (R)0};
    if (r < pg) {
      const double2 x = a.X[(uint64_t)(r0 + r) * a.ldX + row0 + j];
      v = C2<R>{(R)x.x, (R)x.y};
    }
    Xs[j][r] = v;
  }
}

// Y[row, r0 + r] += d acc[r]
template <typename R, int PG>
__device__ __forceinline__ void emit(const ZArgs& a, uint32_t r0, uint32_t pg, uint64_t row, const C2<R>* acc) {
#pragma unroll
  for (int r = 0; r < PG; ++r) {
    if ((uint32_t)r < pg) {
      const double ar = (double)acc[r].re, ai = (double)acc[r].im;
      double* y = &a.Y[(uint64_t)(r0 + r) * a.ldY + row].x;
      atomicAdd(y, a.dre * ar - a.dim * ai);
      atomicAdd(y + 1, a.dre * ai + a.dim * ar);
    }
  }
}

template <typename S, typename R, int PG, int OP>
__global__ void __launch_bounds__(kThreads) zmv_kernel(ZArgs a) {
  __shared__ C2<R> Xs[kCh][PG];
  __shared__ C2<R> Ts[kThreads];       // kThreads / PG columns x PG right-hand sides
  __shared__ C2<R> red[kThreads * PG];  // per-slice partial inner products
  const MvLeaf L = a.leaves[a.order[blockIdx.x]];
  const S* base = reinterpret_cast<const S*>(a.arena) + L.off;
  const uint32_t tid = threadIdx.x;
  constexpr bool kFwd = OP == kZOpN;
  // output rows (ro, nr) and input rows (co, nc) of op(A)
  const uint32_t ro = kFwd ? L.b1 : L.b2, nr = kFwd ? L.n1 : L.n2;
  const uint32_t co = kFwd ? L.b2 : L.b1, nc = kFwd ? L.n2 : L.n1;
  for (uint32_t r0 = 0; r0 < a.p; r0 += PG) {
    const uint32_t pg = min((uint32_t)PG, a.p - r0);
    if (L.rank < 0) {
      // dense: thread per output row; the forward product reads D by rows
      // (coalesced across threads), the adjoint ones read column ro + i of D
      for (uint32_t ib = 0; ib < nr; ib += kThreads) {
        const uint32_t i = ib + tid;
        C2<R> acc[PG];
#pragma unroll
        for (int r = 0; r < PG; ++r) acc[r] = C2<R>{(R)0, (R)0};
        for (uint32_t jb = 0; jb < nc; jb += kCh) {
          const uint32_t jn = min((uint32_t)kCh, nc - jb);
          __syncthreads();
          stage<R, PG>(Xs, a, r0, pg, co + jb, jn);
          __syncthreads();
          if (i < nr) {
            for (uint32_t j = 0; j < jn; ++j) {
              const C2<R> av = kFwd ? ldz(base + i + (uint64_t)(jb + j) * L.n1, false)
                                    : ldz(base + (jb + j) + (uint64_t)i * L.n1, OP == kZOpH);
#pragma unroll
              for (int r = 0; r < PG; ++r) cfma(acc[r], av, Xs[j][r]);
            }
          }
        }
        if (i < nr) emit<R, PG>(a, r0, pg, ro + i, acc);
      }
    } else if (L.rank > 0) {
      const uint32_t k = (uint32_t)L.rank;
      // P: output-side factor (nr rows), Q: input-side factor (nc rows)
      const S* P = kFwd ? base : base + (uint64_t)L.n1 * k;
      const S* Q = kFwd ? base + (uint64_t)L.n1 * k : base;
      constexpr bool kConjP = OP == kZOpT, kConjQ = OP != kZOpT;
      constexpr uint32_t kKt = kThreads / PG;
      for (uint32_t lb = 0; lb < k; lb += kKt) {
        const uint32_t kn = min(kKt, k - lb);
        // thread = (column l, row slice sub): each factor entry is loaded once and
        // multiplied with all PG right-hand sides; the slices are summed in order
        const uint32_t ns = kThreads / kn;
        const uint32_t l = tid % kn, sub = tid / kn;
        C2<R> t[PG];
#pragma unroll
        for (int r = 0; r < PG; ++r) t[r] = C2<R>{(R)0, (R)0};
        for (uint32_t jb = 0; jb < nc; jb += kCh) {
          const uint32_t jn = min((uint32_t)kCh, nc - jb);
          __syncthreads();
          stage<R, PG>(Xs, a, r0, pg, co + jb, jn);
          __syncthreads();
          if (sub < ns) {
            const S* qc = Q + (uint64_t)(lb + l) * nc + jb;
            for (uint32_t j = sub; j < jn; j += ns) {
              const C2<R> q = ldz(qc + j, kConjQ);
#pragma unroll
              for (int r = 0; r < PG; ++r) cfma(t[r], q, Xs[j][r]);
            }
          }
        }
        if (sub < ns) {
#pragma unroll
          for (int r = 0; r < PG; ++r) red[(sub * kn + l) * PG + r] = t[r];
        }
        __syncthreads();
        if (tid < kn * PG) {
          const uint32_t l2 = tid / PG, r2 = tid % PG;
          C2<R> s = red[l2 * PG + r2];
          for (uint32_t q = 1; q < ns; ++q) {
            s.re += red[(q * kn + l2) * PG + r2].re;
            s.im += red[(q * kn + l2) * PG + r2].im;
          }
          Ts[tid] = s;  // Ts[l * PG + r]
        }
        __syncthreads();
        for (uint32_t ib = 0; ib < nr; ib += kThreads) {
          const uint32_t i = ib + tid;
          if (i < nr) {
            C2<R> acc[PG];
#pragma unroll
            for (int rr = 0; rr < PG; ++rr) acc[rr] = C2<R>{(R)0, (R)0};
            const S* pc = P + (uint64_t)lb * nr + i;
            for (uint32_t ll = 0; ll < kn; ++ll) {
              const C2<R> pv = ldz(pc + (uint64_t)ll * nr, kConjP);
#pragma unroll
              for (int rr = 0; rr < PG; ++rr) cfma(acc[rr], pv, Ts[ll * PG + rr]);
            }
            emit<R, PG>(a, r0, pg, ro + i, acc);
          }
        }
        __syncthreads();
      }
    }
  }
}

template <typename S, typename R, int OP>
void launch_op(const ZArgs& a, cudaStream_t s) {
  const uint32_t grid = a.nleaves;
  if (a.p == 1) zmv_kernel<S, R, 1, OP><<<grid, kThreads, 0, s>>>(a);
  else if (a.p == 2) zmv_kernel<S, R, 2, OP><<<grid, kThreads, 0, s>>>(a);
  else if (a.p <= 4) zmv_kernel<S, R, 4, OP><<<grid, kThreads, 0, s>>>(a);
  // wider groups (16) measured slower: fewer columns per pass, lower occupancy
  else zmv_kernel<S, R, 8, OP><<<grid, kThreads, 0, s>>>(a);
}

template <typename S, typename R>
void launch_typed(const ZArgs& a, cudaStream_t s) {
  if (a.op == kZOpH) launch_op<S, R, kZOpH>(a, s);
  else if (a.op == kZOpT) launch_op<S, R, kZOpT>(a, s);
  else launch_op<S, R, kZOpN>(a, s);
}

__global__ void z_to_c64_kernel(const double2* __restrict__ src, uint64_t n, float2* __restrict__ dst) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const double2 v = src[i];
    dst[i] = make_float2((float)v.x, (float)v.y);
  }
}

}  // namespace

cudaError_t launch_matvec_z(const ZArgs& a, cudaStream_t s) {
  if (a.op < kZOpN || a.op > kZOpT) return cudaErrorInvalidValue;
  if (a.nleaves == 0 || a.p == 0) return cudaSuccess;
  if (a.single) launch_typed<float2, float>(a, s);
  else launch_typed<double2, double>(a, s);
  count_product_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_z_to_c64(const double2* src, uint64_t n, float2* dst, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  const unsigned grid = (unsigned)std::min<uint64_t>((n + 255) / 256, 152ull * 16);
  z_to_c64_kernel<<<grid, 256, 0, s>>>(src, n, dst);
  return cudaGetLastError();
}

}  // namespace ahx
