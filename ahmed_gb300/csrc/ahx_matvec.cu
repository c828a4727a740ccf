// Batched H-matrix product Y += d A X (mltaGeHVec / mltaGeHGeM semantics:
// H/mltaGeHVec.cpp:16-59, H/mblock.cpp:126-154, Include/mblock.h:99-109).
//
// One CTA per leaf, leaves launched in descending cost order so that the
// large coarse-level leaves start first.  Right-hand sides are processed in
// groups of PG; the X rows of a leaf are staged in shared memory (coalesced
// column-major loads); dense leaves and the U-phase of low-rank leaves have
// one output row per thread (coalesced arena reads, broadcast shared reads);
// the V-phase T = V^T X splits each output over several threads and sums the
// partial results in a fixed order (run-to-run deterministic per leaf).
// Contributions are added to Y with FP64 atomics (leaves sharing rows).
#include <cuda_bf16.h>

#include "ahx_matvec.cuh"

namespace ahx {
namespace {

constexpr int kThreads = 128;
constexpr int kCh = 128;  // X rows per staged chunk
constexpr int kKt = 32;   // low-rank columns per pass

template <typename S, typename A>
__device__ __forceinline__ A ldcvt(const S* p);
template <>
__device__ __forceinline__ double ldcvt<double, double>(const double* p) { return __ldg(p); }
template <>
__device__ __forceinline__ float ldcvt<float, float>(const float* p) { return __ldg(p); }
template <>
__device__ __forceinline__ float ldcvt<__nv_bfloat16, float>(const __nv_bfloat16* p) {
  return __bfloat162float(__ldg(p));
}

template <typename A, int PG>
__device__ __forceinline__ void stage_x(A (*Xs)[PG + 1], const MvArgs& a, uint32_t r0, uint32_t pg,
                                        uint32_t b2, uint32_t jb, uint32_t jn) {
  for (uint32_t e = threadIdx.x; e < jn * PG; e += kThreads) {
    const uint32_t j = e % jn, r = e / jn;
    Xs[j][r] = r < pg ? (A)a.X[(uint64_t)(r0 + r) * a.ldX + b2 + jb + j] : (A)0;
  }
}

// TR: the transposed product Y += d A^T X (mltaGeHtVec / mltaGeHhVec for real
// leaves, H/mltaGeHVec.cpp:62-150): a low-rank leaf U V^T acts as V U^T (the
// roles of the factors and of the row / column ranges swap); a dense leaf D
// acts as D^T, one warp per column of D.
template <typename SL, typename SD, typename A, int PG, bool TR>
__global__ void __launch_bounds__(kThreads) mv_kernel(MvArgs a) {
  __shared__ A Xs[kCh][PG + 1];
  __shared__ A Ts[kKt][PG];
  __shared__ A red[kThreads];
  MvLeaf L = a.leaves[a.order[blockIdx.x]];
  const uint32_t tid = threadIdx.x;
  const double d = a.d;
  uint64_t voff = L.off + (uint64_t)L.n1 * (L.rank > 0 ? (uint32_t)L.rank : 0u);  // V of U V^T
  if (TR && L.rank > 0) {
    const uint64_t uo = voff;
    voff = L.off;
    L.off = uo;
    const uint32_t b = L.b1, n = L.n1;
    L.b1 = L.b2;
    L.n1 = L.n2;
    L.b2 = b;
    L.n2 = n;
  }
  if (TR && L.rank < 0) {
    // Y[b2 + j] += d sum_i D[i + j n1] X[b1 + i]: one output column j of D per
    // thread, the X rows of D's row range staged in shared memory (as the plain
    // path stages the column range); a thread reads its column of D in order
    const SD* Ad = L.dense_in_lr_arena ? reinterpret_cast<const SD*>(reinterpret_cast<const SL*>(a.arena_lr) + L.off)
                                       : reinterpret_cast<const SD*>(a.arena_dn) + L.off;
    for (uint32_t r0 = 0; r0 < a.p; r0 += PG) {
      const uint32_t pg = min((uint32_t)PG, a.p - r0);
      for (uint32_t jb = 0; jb < L.n2; jb += kThreads) {
        const uint32_t j = jb + tid;
        A acc[PG];
#pragma unroll
        for (int r = 0; r < PG; ++r) acc[r] = 0;
        for (uint32_t ib = 0; ib < L.n1; ib += kCh) {
          const uint32_t in = min((uint32_t)kCh, L.n1 - ib);
          __syncthreads();
          stage_x<A, PG>(Xs, a, r0, pg, L.b1, ib, in);
          __syncthreads();
          if (j < L.n2) {
            const SD* col = Ad + (uint64_t)j * L.n1 + ib;
            for (uint32_t i = 0; i < in; ++i) {
              const A av = ldcvt<SD, A>(col + i);
#pragma unroll
              for (int r = 0; r < PG; ++r) acc[r] = fma(av, Xs[i][r], acc[r]);
            }
          }
        }
        if (j < L.n2) {
#pragma unroll
          for (int r = 0; r < PG; ++r)
            if ((uint32_t)r < pg) atomicAdd(a.Y + (uint64_t)(r0 + r) * a.ldY + L.b2 + j, d * (double)acc[r]);
        }
      }
    }
    return;
  }
  for (uint32_t r0 = 0; r0 < a.p; r0 += PG) {
    const uint32_t pg = min((uint32_t)PG, a.p - r0);
    if (L.rank < 0) {
      const SD* Ad = L.dense_in_lr_arena ? reinterpret_cast<const SD*>(
                                               reinterpret_cast<const SL*>(a.arena_lr) + L.off)
                                         : reinterpret_cast<const SD*>(a.arena_dn) + L.off;
      for (uint32_t ib = 0; ib < L.n1; ib += kThreads) {
        const uint32_t i = ib + tid;
        A acc[PG];
#pragma unroll
        for (int r = 0; r < PG; ++r) acc[r] = 0;
        for (uint32_t jb = 0; jb < L.n2; jb += kCh) {
          const uint32_t jn = min((uint32_t)kCh, L.n2 - jb);
          __syncthreads();
          stage_x<A, PG>(Xs, a, r0, pg, L.b2, jb, jn);
          __syncthreads();
          if (i < L.n1) {
            const SD* col = Ad + i + (uint64_t)jb * L.n1;
            for (uint32_t j = 0; j < jn; ++j) {
              const A av = ldcvt<SD, A>(col + (uint64_t)j * L.n1);
#pragma unroll
              for (int r = 0; r < PG; ++r) acc[r] = fma(av, Xs[j][r], acc[r]);
            }
          }
        }
        if (i < L.n1) {
#pragma unroll
          for (int r = 0; r < PG; ++r)
            if ((uint32_t)r < pg) atomicAdd(a.Y + (uint64_t)(r0 + r) * a.ldY + L.b1 + i, d * (double)acc[r]);
        }
      }
    } else if (L.rank > 0) {
      const uint32_t k = (uint32_t)L.rank;
      const SL* U = reinterpret_cast<const SL*>(a.arena_lr) + L.off;
      const SL* V = reinterpret_cast<const SL*>(a.arena_lr) + voff;
      for (uint32_t lb = 0; lb < k; lb += kKt) {
        const uint32_t kn = min((uint32_t)kKt, k - lb);
        const uint32_t nout = kn * PG;
        // phase 1: Ts[l][r] = sum_j V[j, lb+l] X[b2+j, r0+r]
        const uint32_t ns = nout >= kThreads ? 1u : kThreads / nout;  // threads per output
        const uint32_t nq = (nout + kThreads - 1) / kThreads;         // outputs per thread
        A tacc[(kKt * PG + kThreads - 1) / kThreads];
#pragma unroll
        for (int q = 0; q < (kKt * PG + kThreads - 1) / kThreads; ++q) tacc[q] = 0;
        const uint32_t sub = tid / nout, o1 = tid % nout;
        for (uint32_t jb = 0; jb < L.n2; jb += kCh) {
          const uint32_t jn = min((uint32_t)kCh, L.n2 - jb);
          __syncthreads();
          stage_x<A, PG>(Xs, a, r0, pg, L.b2, jb, jn);
          __syncthreads();
          if (ns > 1) {
            if (sub < ns) {
              const uint32_t l = o1 / PG, r = o1 % PG;
              const SL* vc = V + (uint64_t)(lb + l) * L.n2 + jb;
              for (uint32_t j = sub; j < jn; j += ns) tacc[0] = fma(ldcvt<SL, A>(vc + j), Xs[j][r], tacc[0]);
            }
          } else {
#pragma unroll
            for (int q = 0; q < (kKt * PG + kThreads - 1) / kThreads; ++q) {
              const uint32_t o = tid + q * kThreads;
              if (q < (int)nq && o < nout) {
                const uint32_t l = o / PG, r = o % PG;
                const SL* vc = V + (uint64_t)(lb + l) * L.n2 + jb;
                A s = tacc[q];
                for (uint32_t j = 0; j < jn; ++j) s = fma(ldcvt<SL, A>(vc + j), Xs[j][r], s);
                tacc[q] = s;
              }
            }
          }
        }
        __syncthreads();
        if (ns > 1) {
          red[tid] = tacc[0];
          __syncthreads();
          if (tid < nout) {
            A s = red[tid];
            for (uint32_t q = 1; q < ns; ++q) s += red[tid + q * nout];
            Ts[tid / PG][tid % PG] = s;
          }
        } else {
#pragma unroll
          for (int q = 0; q < (kKt * PG + kThreads - 1) / kThreads; ++q) {
            const uint32_t o = tid + q * kThreads;
            if (q < (int)nq && o < nout) Ts[o / PG][o % PG] = tacc[q];
          }
        }
        __syncthreads();
        // phase 2: Y[b1+i, r] += d sum_l U[i, lb+l] Ts[l][r]
        for (uint32_t ib = 0; ib < L.n1; ib += kThreads) {
          const uint32_t i = ib + tid;
          if (i < L.n1) {
            A acc[PG];
#pragma unroll
            for (int r = 0; r < PG; ++r) acc[r] = 0;
            const SL* uc = U + (uint64_t)lb * L.n1 + i;
            for (uint32_t l = 0; l < kn; ++l) {
              const A uv = ldcvt<SL, A>(uc + (uint64_t)l * L.n1);
#pragma unroll
              for (int r = 0; r < PG; ++r) acc[r] = fma(uv, Ts[l][r], acc[r]);
            }
#pragma unroll
            for (int r = 0; r < PG; ++r)
              if ((uint32_t)r < pg) atomicAdd(a.Y + (uint64_t)(r0 + r) * a.ldY + L.b1 + i, d * (double)acc[r]);
          }
        }
        __syncthreads();
      }
    }
  }
}

template <typename SL, typename SD, typename A, bool TR>
cudaError_t launch_typed(const MvArgs& a, cudaStream_t s) {
  if (a.nleaves == 0 || a.p == 0) return cudaSuccess;
  const uint32_t grid = a.nleaves;
  if (a.p == 1) mv_kernel<SL, SD, A, 1, TR><<<grid, kThreads, 0, s>>>(a);
  else if (a.p == 2) mv_kernel<SL, SD, A, 2, TR><<<grid, kThreads, 0, s>>>(a);
  else if (a.p <= 4) mv_kernel<SL, SD, A, 4, TR><<<grid, kThreads, 0, s>>>(a);
  else if (a.p <= 8) mv_kernel<SL, SD, A, 8, TR><<<grid, kThreads, 0, s>>>(a);
  else mv_kernel<SL, SD, A, 16, TR><<<grid, kThreads, 0, s>>>(a);
  count_product_launches(1);
  return cudaGetLastError();
}

}  // namespace

// the plain (FP64) form; the mixed forms run the tensor-core sweeps
cudaError_t launch_matvec(int prec, const MvArgs& a, cudaStream_t s) {
  if (prec != kFP64) return cudaErrorInvalidValue;
  return a.transposed ? launch_typed<double, double, double, true>(a, s)
                      : launch_typed<double, double, double, false>(a, s);
}

}  // namespace ahx
