// Mixed-precision H-matrix product as two linear sweeps over a re-laid-out
// arena: Y += d A X with mltaGeHGeM semantics (H/mltaGeHVec.cpp:38-59,
// H/mblock.cpp:141-154, Include/mblock.h:105-109).
//
// Each CTA owns a contiguous byte range of a stream (balanced by bytes).  One
// producer warp moves the range unit by unit into a ring of shared-memory slots
// with cp.async.bulk (completion on a "full" mbarrier per slot); the consumer
// warps take the units round-robin, compute from shared memory and release the
// slot on its "empty" mbarrier.  Every wait is bounded: on timeout the kernel
// raises the plan's error word, the producer waits (bounded) for the copies it
// issued, and all warps return.
#include <algorithm>
#include <map>
#include <numeric>

#include <cuda_bf16.h>

#include "ahx_matvec.cuh"

namespace ahx {
namespace {

constexpr int kWarps = 6;                 // compute warps per CTA, each with two slots
constexpr int kStages = 2 * kWarps;
constexpr int kThreads = 32 * kWarps;
constexpr uint32_t kSlotStride = kSlotBytes + kSideBytes;  // leaf bytes, then X / T rows
constexpr size_t kSmemBytes = (size_t)kStages * kSlotStride + kStages * sizeof(uint64_t);
constexpr uint32_t kWaitLimit = 1u << 22;
constexpr uint32_t kMaxEnts = 32;  // entries per rows unit (one per lane)

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

// bounded wait for the phase with the given parity; false (and the error word set) on timeout
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, int* err) {
  for (uint32_t it = 0; it < kWaitLimit; ++it)
    if (mbar_try_wait(bar, parity)) return true;
  atomicExch(err, 1);
  return false;
}

__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
      "l"(src), "r"(bytes), "r"(bar)
      : "memory");
}

// generic-proxy reads of a slot are ordered before the next bulk copy into it
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

template <typename S>
__device__ __forceinline__ float cvt(S v);
template <>
__device__ __forceinline__ float cvt<float>(float v) { return v; }
template <>
__device__ __forceinline__ float cvt<__nv_bfloat16>(__nv_bfloat16 v) { return __bfloat162float(v); }

__device__ __forceinline__ void red4(float* p, float a, float b, float c, float d) {
  asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(p), "f"(a), "f"(b), "f"(c), "f"(d)
               : "memory");
}

// Per-warp double buffering.  Warp w of a CTA takes the units q = w, w + W, ...
// of the CTA's range; its i-th unit lands in slot 2w + (i & 1) (fill i >> 1),
// so each slot is filled and read strictly in order by one warp and the parity
// waits are exact.  A unit's descriptor D is loaded one unit ahead of use
// (load(q) -> D), the copies are queued by issue(D, slot, bar) right after the
// slot's previous unit was computed, and body(D, slot, lane) computes.
template <class Desc, class Load, class Issue, class Body>
__device__ void warp_stream(uint32_t u0, uint32_t u1, int* err, Load load, Issue issue, Body body) {
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + (size_t)kStages * kSlotStride);
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) {
    mbar_init(smem_u32(&bars[2 * warp]), 1);
    mbar_init(smem_u32(&bars[2 * warp + 1]), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncwarp();
  const uint32_t nq = u1 > u0 ? u1 - u0 : 0;
  const uint32_t mine = nq > warp ? (nq - warp + kWarps - 1) / kWarps : 0;  // units of this warp
  unsigned char* const slotA = smem + (size_t)(2 * warp) * kSlotStride;
  unsigned char* const slotB = smem + (size_t)(2 * warp + 1) * kSlotStride;
  const uint32_t barA = smem_u32(&bars[2 * warp]), barB = smem_u32(&bars[2 * warp + 1]);
  Desc dA, dB;
  if (mine > 0) {
    dA = load(u0 + warp);
    issue(dA, slotA, barA);
  }
  if (mine > 1) {
    dB = load(u0 + warp + kWarps);
    issue(dB, slotB, barB);
  }
  uint32_t issued = mine < 2 ? mine : 2;
  // one step: unit i in (slot, bar, desc); refill with unit i + 2
  auto step = [&](uint32_t i, unsigned char* slot, uint32_t bar, Desc& d) -> bool {
    Desc nxt;
    const bool more = i + 2 < mine;
    if (more) nxt = load(u0 + warp + (i + 2) * kWarps);  // in flight while unit i is computed
    if (!mbar_wait(bar, (i >> 1) & 1, err)) return false;
    body(d, slot, lane);
    __syncwarp();
    if (more) {
      fence_proxy_async();
      d = nxt;
      issue(d, slot, bar);
      ++issued;
    }
    return true;
  };
  bool ok = true;
  for (uint32_t i = 0; ok && i < mine; i += 2) {
    ok = step(i, slotA, barA, dA);
    if (ok && i + 1 < mine) ok = step(i + 1, slotB, barB, dB);
  }
  if (!ok) {
    // never leave while a copy into this CTA's shared memory is in flight
    for (uint32_t i = issued > 2 ? issued - 2 : 0; i < issued; ++i)
      mbar_wait((i & 1) ? barB : barA, (i >> 1) & 1, err);
  }
}

struct VDesc {
  StreamVUnit u;
};

// One V unit, KV >= kn columns: T[t_row + l][r] = sum_{j < jn} Vc[l * jn + j] X[xrow + j][r]
// lane = jj * RG + rg: rg picks 4 right-hand sides, jj a row phase.
template <typename SL, int P, int KV>
__device__ __forceinline__ void v_unit(const StreamVUnit& U, const unsigned char* slot, uint32_t lane,
                                       float* __restrict__ T) {
  constexpr int RG = P / 4;
  constexpr int NJ = 32 / RG;
  const SL* Vc = reinterpret_cast<const SL*>(slot);
  const float* xs = reinterpret_cast<const float*>(slot + U.bytes);
  const uint32_t rg = lane % RG, jj = lane / RG;
  float acc[KV][4];
#pragma unroll
  for (int l = 0; l < KV; ++l) acc[l][0] = acc[l][1] = acc[l][2] = acc[l][3] = 0.f;
#pragma unroll 2
  for (uint32_t j = jj; j < U.jn; j += NJ) {
    const float4 x = *reinterpret_cast<const float4*>(xs + j * P + 4 * rg);
#pragma unroll
    for (int l = 0; l < KV; ++l) {
      const float v = (uint32_t)l < U.kn ? cvt<SL>(Vc[(uint32_t)l * U.jn + j]) : 0.f;
      acc[l][0] = fmaf(v, x.x, acc[l][0]);
      acc[l][1] = fmaf(v, x.y, acc[l][1]);
      acc[l][2] = fmaf(v, x.z, acc[l][2]);
      acc[l][3] = fmaf(v, x.w, acc[l][3]);
    }
  }
#pragma unroll
  for (int s = RG; s < 32; s <<= 1) {
#pragma unroll
    for (int l = 0; l < KV; ++l) {
#pragma unroll
      for (int c = 0; c < 4; ++c) acc[l][c] += __shfl_xor_sync(0xffffffffu, acc[l][c], s);
    }
  }
  if (jj == 0) {
#pragma unroll
    for (int l = 0; l < KV; ++l)
      if ((uint32_t)l < U.kn)
        *reinterpret_cast<float4*>(T + (uint64_t)(U.t_row + l) * P + 4 * rg) =
            make_float4(acc[l][0], acc[l][1], acc[l][2], acc[l][3]);
  }
}

template <typename SL, int P>
__global__ void __launch_bounds__(kThreads, 1) v_sweep_kernel(MvPlan pl) {
  const uint32_t u0 = pl.vranges[blockIdx.x], u1 = pl.vranges[blockIdx.x + 1];
  warp_stream<VDesc>(
      u0, u1, pl.err, [&](uint32_t u) { return VDesc{pl.vunits[u]}; },
      [&](const VDesc& D, unsigned char* slot, uint32_t bar) {
        if ((threadIdx.x & 31) == 0) {
          // V chunk first, then its X rows right behind it (16-byte aligned)
          const uint32_t xb = D.u.jn * P * 4;
          mbar_expect_tx(bar, D.u.bytes + xb);
          bulk_g2s(smem_u32(slot), pl.vstream + D.u.src, D.u.bytes, bar);
          bulk_g2s(smem_u32(slot + D.u.bytes), pl.xr + (uint64_t)D.u.xrow * P, xb, bar);
        }
      },
      [&](const VDesc& D, const unsigned char* slot, uint32_t lane) {
        const uint32_t kq = (D.u.kn + 3) / 4;
        if (kq <= 1) v_unit<SL, P, 4>(D.u, slot, lane, pl.t);
        else if (kq == 2) v_unit<SL, P, 8>(D.u, slot, lane, pl.t);
        else if (kq == 3) v_unit<SL, P, 12>(D.u, slot, lane, pl.t);
        else v_unit<SL, P, 16>(D.u, slot, lane, pl.t);
      });
}

// T[t_row + l] = sum over the V chunks c of T[t_row + c k + l]
template <int P>
__global__ void t_reduce_kernel(const TReduce* __restrict__ items, uint32_t n, float* __restrict__ T) {
  const uint32_t it = blockIdx.x;
  if (it >= n) return;
  const TReduce R = items[it];
  for (uint32_t e = threadIdx.x; e < R.k * P; e += blockDim.x) {
    const uint32_t l = e / P, r = e % P;
    float s = T[(uint64_t)(R.t_row + l) * P + r];
    for (uint32_t c = 1; c < R.nchunk; ++c) s += T[(uint64_t)(R.t_row + c * R.k + l) * P + r];
    T[(uint64_t)(R.t_row + l) * P + r] = s;
  }
}

// One rows unit.  lane = rq * 16 + rr: rr picks rows rr, rr + 16, ... (S row slots,
// S = ceil(nrows / 16)), rq picks half of the P right-hand sides.
template <typename SL, int P, int S>
__device__ __forceinline__ void rows_unit(const StreamUnit& U, const StreamEnt& myent,
                                          const unsigned char* slot, uint32_t lane, float* __restrict__ yr) {
  constexpr int H = P / 2;  // right-hand sides per lane (P >= 4 -> H >= 2)
  const uint32_t nr = U.nrows;
  const uint32_t rr = lane & 15, rq = lane >> 4;
  bool ok[S];
#pragma unroll
  for (int k = 0; k < S; ++k) ok[k] = rr + 16 * k < nr;
  float a[S][H];
#pragma unroll
  for (int k = 0; k < S; ++k)
#pragma unroll
    for (int r = 0; r < H; ++r) a[k][r] = 0.f;
  const float* side = reinterpret_cast<const float*>(slot + kSlotBytes) + rq * H;
  for (uint32_t e = 0; e < U.ne; ++e) {
    const uint32_t boff = __shfl_sync(0xffffffffu, myent.boff, e);
    const uint32_t kind = __shfl_sync(0xffffffffu, myent.kind, e);
    const uint32_t ncols = __shfl_sync(0xffffffffu, myent.ncols, e);
    if (kind == 0) {
      const float* A = reinterpret_cast<const float*>(slot + boff) + rr;
#pragma unroll 4
      for (uint32_t j = 0; j < ncols; ++j) {
        float u[S];
#pragma unroll
        for (int k = 0; k < S; ++k) u[k] = ok[k] ? A[j * nr + 16 * k] : 0.f;
        const float* xrow = side + j * P;
#pragma unroll
        for (int q = 0; q < H / 4 + (H % 4 ? 1 : 0); ++q) {
          float x[4];
          if (H >= 4) {
            const float4 v = *reinterpret_cast<const float4*>(xrow + 4 * q);
            x[0] = v.x; x[1] = v.y; x[2] = v.z; x[3] = v.w;
          } else {
            const float2 v = *reinterpret_cast<const float2*>(xrow);
            x[0] = v.x; x[1] = v.y; x[2] = 0.f; x[3] = 0.f;
          }
#pragma unroll
          for (int c = 0; c < 4 && 4 * q + c < H; ++c)
#pragma unroll
            for (int k = 0; k < S; ++k) a[k][4 * q + c] = fmaf(u[k], x[c], a[k][4 * q + c]);
        }
      }
    } else {
      const SL* Uc = reinterpret_cast<const SL*>(slot + boff) + rr;
#pragma unroll 4
      for (uint32_t l = 0; l < ncols; ++l) {
        float u[S];
#pragma unroll
        for (int k = 0; k < S; ++k) u[k] = ok[k] ? cvt<SL>(Uc[l * nr + 16 * k]) : 0.f;
        const float* trow = side + l * P;
#pragma unroll
        for (int q = 0; q < H / 4 + (H % 4 ? 1 : 0); ++q) {
          float x[4];
          if (H >= 4) {
            const float4 v = *reinterpret_cast<const float4*>(trow + 4 * q);
            x[0] = v.x; x[1] = v.y; x[2] = v.z; x[3] = v.w;
          } else {
            const float2 v = *reinterpret_cast<const float2*>(trow);
            x[0] = v.x; x[1] = v.y; x[2] = 0.f; x[3] = 0.f;
          }
#pragma unroll
          for (int c = 0; c < 4 && 4 * q + c < H; ++c)
#pragma unroll
            for (int k = 0; k < S; ++k) a[k][4 * q + c] = fmaf(u[k], x[c], a[k][4 * q + c]);
        }
      }
    }
    side += ncols * P;
  }
#pragma unroll
  for (int k = 0; k < S; ++k) {
    if (!ok[k]) continue;
    float* y = yr + (uint64_t)(U.row0 + rr + 16 * k) * P + rq * H;
    if (H >= 4) {
#pragma unroll
      for (int q = 0; q < H / 4; ++q) red4(y + 4 * q, a[k][4 * q], a[k][4 * q + 1], a[k][4 * q + 2], a[k][4 * q + 3]);
    } else {
      atomicAdd(y, a[k][0]);
      atomicAdd(y + 1, a[k][1]);
    }
  }
}

// A rows unit as one warp holds it: the unit (all lanes) and entry `lane` (lane < ne)
struct RDesc {
  StreamUnit u;
  StreamEnt e;
};

// rows sweep: Yr[row0 + i] += sum over the unit's chunks (dense A X, low rank U T)
template <typename SL, int P>
__global__ void __launch_bounds__(kThreads, 1) rows_sweep_kernel(MvPlan pl) {
  const uint32_t u0 = pl.rranges[blockIdx.x], u1 = pl.rranges[blockIdx.x + 1];
  warp_stream<RDesc>(
      u0, u1, pl.err,
      [&](uint32_t u) {
        RDesc D;
        D.u = pl.units[u];
        const uint32_t lane = threadIdx.x & 31;
        if (lane < D.u.ne) D.e = pl.ents[D.u.e0 + lane];
        else D.e = StreamEnt{0u, 0u, 0u, 0u};
        return D;
      },
      [&](const RDesc& D, unsigned char* slot, uint32_t bar) {
        const uint32_t lane = threadIdx.x & 31;
        // side rows of every entry, packed after the leaf bytes in entry order
        const uint32_t mybytes = D.e.ncols * P * 4;
        uint32_t off = mybytes;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const uint32_t v = __shfl_up_sync(0xffffffffu, off, o);
          if (lane >= (uint32_t)o) off += v;
        }
        const uint32_t total = __shfl_sync(0xffffffffu, off, 31);
        off -= mybytes;  // exclusive prefix
        if (lane == 0) {
          mbar_expect_tx(bar, D.u.bytes + total);
          bulk_g2s(smem_u32(slot), pl.rstream + D.u.src, D.u.bytes, bar);
        }
        __syncwarp();
        if (lane < D.u.ne) {
          const float* src = (D.e.kind == 0 ? pl.xr : pl.t) + (uint64_t)D.e.xrow * P;
          bulk_g2s(smem_u32(slot + kSlotBytes + off), src, mybytes, bar);
        }
      },
      [&](const RDesc& D, const unsigned char* slot, uint32_t lane) {
        const uint32_t S = (D.u.nrows + 15) / 16;
        if (S <= 1) rows_unit<SL, P, 1>(D.u, D.e, slot, lane, pl.yr);
        else if (S == 2) rows_unit<SL, P, 2>(D.u, D.e, slot, lane, pl.yr);
        else if (S == 3) rows_unit<SL, P, 3>(D.u, D.e, slot, lane, pl.yr);
        else rows_unit<SL, P, 4>(D.u, D.e, slot, lane, pl.yr);
      });
}

// Xr[i * P + r] = X[(r0 + r) * ldX + i] for r < pg, 0 for pg <= r < P
template <int P>
__global__ void xr_kernel(const double* __restrict__ X, uint64_t ldX, uint64_t n, uint32_t r0,
                          uint32_t pg, float* __restrict__ xr) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    float v[P];
#pragma unroll
    for (int r = 0; r < P; ++r) v[r] = (uint32_t)r < pg ? (float)X[(uint64_t)(r0 + r) * ldX + i] : 0.f;
    float4* o = reinterpret_cast<float4*>(xr + i * P);
#pragma unroll
    for (int q = 0; q < P / 4; ++q) o[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
  }
}

// Y[(r0 + r) * ldY + i] += d * Yr[i * P + r]
template <int P>
__global__ void yr_kernel(const float* __restrict__ yr, uint64_t n, uint32_t r0, uint32_t pg,
                          double d, double* __restrict__ Y, uint64_t ldY) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const float4* src = reinterpret_cast<const float4*>(yr + i * P);
#pragma unroll
    for (int q = 0; q < P / 4; ++q) {
      const float4 v = src[q];
      const float w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const uint32_t r = 4 * q + c;
        if (r < pg) Y[(uint64_t)(r0 + r) * ldY + i] += d * (double)w[c];
      }
    }
  }
}

__global__ void stream_copy_kernel(const StreamCopy* __restrict__ tasks, const double* __restrict__ a64,
                                   unsigned char* __restrict__ dst) {
  const StreamCopy c = tasks[blockIdx.x];
  const uint64_t cnt = (uint64_t)c.nrows * c.ncols;
  for (uint64_t e = threadIdx.x; e < cnt; e += blockDim.x) {
    const uint32_t i = (uint32_t)(e % c.nrows), j = (uint32_t)(e / c.nrows);
    const double v = a64[c.src + (uint64_t)j * c.src_ld + i];
    if (c.dtype == 0) reinterpret_cast<float*>(dst + c.dst)[e] = (float)v;
    else reinterpret_cast<__nv_bfloat16*>(dst + c.dst)[e] = __double2bfloat16(v);
  }
}

unsigned grid_rows(uint64_t n) { return (unsigned)std::min<uint64_t>((n + 255) / 256, 152ull * 8); }

template <typename SL, int P>
cudaError_t run_group(const MvPlan& pl, double d, uint32_t r0, uint32_t pg, const double* X,
                      uint64_t ldX, double* Y, uint64_t ldY, cudaStream_t s) {
  static bool attr_set = false;
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(v_sweep_kernel<SL, P>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)kSmemBytes);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(rows_sweep_kernel<SL, P>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)kSmemBytes);
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  xr_kernel<P><<<grid_rows(pl.n), 256, 0, s>>>(X, ldX, pl.n, r0, pg, pl.xr);
  cudaError_t e = cudaMemsetAsync(pl.yr, 0, pl.n * P * sizeof(float), s);
  if (e != cudaSuccess) return e;
  if (pl.nvunits) v_sweep_kernel<SL, P><<<pl.grid, kThreads, kSmemBytes, s>>>(pl);
  if (pl.ntreduce) t_reduce_kernel<P><<<pl.ntreduce, 128, 0, s>>>(pl.treduce, pl.ntreduce, pl.t);
  if (pl.nunits) rows_sweep_kernel<SL, P><<<pl.grid, kThreads, kSmemBytes, s>>>(pl);
  yr_kernel<P><<<grid_rows(pl.n), 256, 0, s>>>(pl.yr, pl.n, r0, pg, d, Y, ldY);
  return cudaGetLastError();
}

template <typename SL>
cudaError_t run_typed(const MvPlan& pl, double d, uint32_t p, const double* X, uint64_t ldX,
                      double* Y, uint64_t ldY, cudaStream_t s) {
  for (uint32_t r0 = 0; r0 < p; r0 += 16) {
    const uint32_t pg = std::min(16u, p - r0);
    cudaError_t e;
    if (pg <= 4) e = run_group<SL, 4>(pl, d, r0, pg, X, ldX, Y, ldY, s);
    else if (pg <= 8) e = run_group<SL, 8>(pl, d, r0, pg, X, ldX, Y, ldY, s);
    else e = run_group<SL, 16>(pl, d, r0, pg, X, ldX, Y, ldY, s);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

uint32_t align16(uint64_t b) { return (uint32_t)((b + 15) & ~uint64_t(15)); }

}  // namespace

void build_stream_layout(const std::vector<PlanLeaf>& leaves, int lr_dtype, StreamLayout& L) {
  L = StreamLayout();
  const uint32_t lsz = lr_dtype == 0 ? 4 : 2;
  std::vector<uint32_t> trow(leaves.size(), 0), nchunk(leaves.size(), 0);
  // V stream, leaf by leaf
  for (size_t q = 0; q < leaves.size(); ++q) {
    const PlanLeaf& P = leaves[q];
    if (P.rank <= 0) continue;
    const uint32_t k = (uint32_t)P.rank;
    // rows per V unit: the chunk and its X rows (64 B per row at P = 16) fill a slot
    const uint32_t kfirst = std::min(kVRank, k);
    const uint32_t vrows = std::max(8u, std::min(256u, ((kSlotStride - 16) / (kfirst * lsz + 64)) & ~7u));
    const uint32_t nc = (P.n2 + vrows - 1) / vrows;
    trow[q] = L.t_rows;
    nchunk[q] = nc;
    if (nc > 1) L.treduce.push_back(TReduce{L.t_rows, k, nc, 0u});
    for (uint32_t c = 0; c < nc; ++c) {
      const uint32_t j0 = c * vrows, jn = std::min(vrows, P.n2 - j0);
      for (uint32_t l0 = 0; l0 < k; l0 += kVRank) {
        const uint32_t kn = std::min(kVRank, k - l0);
        const uint32_t nb = align16((uint64_t)jn * kn * lsz);
        StreamVUnit u;
        u.src = L.vbytes;
        u.bytes = nb;
        u.jn = jn;
        u.kn = kn;
        u.xrow = P.b2 + j0;
        u.t_row = L.t_rows + c * k + l0;
        u.pad = 0;
        L.vunits.push_back(u);
        StreamCopy cp;
        cp.src = P.off + (uint64_t)P.n1 * k + (uint64_t)l0 * P.n2 + j0;
        cp.dst = L.vbytes;
        cp.src_ld = P.n2;
        cp.nrows = jn;
        cp.ncols = kn;
        cp.dtype = (uint32_t)lr_dtype;
        L.vcopies.push_back(cp);
        L.vbytes += nb;
        L.payload_bytes += (uint64_t)jn * kn * lsz;
      }
    }
    L.t_rows += nc * k;
  }
  // rows stream: block rows (row clusters identified by (b1, n1)), 64-row tiles
  std::map<std::pair<uint32_t, uint32_t>, std::vector<size_t>> rowsets;
  for (size_t q = 0; q < leaves.size(); ++q)
    if (leaves[q].rank != 0) rowsets[{leaves[q].b1, leaves[q].n1}].push_back(q);
  for (auto& kv : rowsets) {
    const uint32_t b1 = kv.first.first, n1 = kv.first.second;
    for (uint32_t r0 = 0; r0 < n1; r0 += kTileRows) {
      const uint32_t nr = std::min(kTileRows, n1 - r0);
      StreamUnit u{};
      uint32_t side_rows = 0;
      auto open = [&]() {
        side_rows = 0;
        u.src = L.rbytes;
        u.bytes = 0;
        u.row0 = b1 + r0;
        u.nrows = nr;
        u.e0 = (uint32_t)L.ents.size();
        u.ne = 0;
      };
      auto close = [&]() {
        if (u.ne == 0) return;
        L.units.push_back(u);
        L.rbytes += u.bytes;
      };
      open();
      for (size_t q : kv.second) {
        const PlanLeaf& P = leaves[q];
        const bool dense = P.rank < 0;
        const uint32_t esz = dense ? 4 : lsz;
        const uint32_t ncol_all = dense ? P.n2 : (uint32_t)P.rank;
        const uint32_t maxc = std::min(kSideRows, std::max(1u, (uint32_t)(kSlotBytes / ((uint64_t)nr * esz)) & ~3u));
        for (uint32_t c0 = 0; c0 < ncol_all; c0 += maxc) {
          const uint32_t nc = std::min(maxc, ncol_all - c0);
          const uint32_t nb = align16((uint64_t)nr * nc * esz);
          if (u.bytes + nb > kSlotBytes || side_rows + nc > kSideRows || u.ne == kMaxEnts) {
            close();
            open();
          }
          side_rows += nc;
          StreamEnt E;
          E.boff = u.bytes;
          E.kind = dense ? 0u : 1u;
          E.ncols = nc;
          E.xrow = dense ? P.b2 + c0 : trow[q] + c0;
          L.ents.push_back(E);
          StreamCopy cp;
          cp.src = P.off + r0 + (uint64_t)c0 * P.n1;
          cp.dst = L.rbytes + u.bytes;
          cp.src_ld = P.n1;
          cp.nrows = nr;
          cp.ncols = nc;
          cp.dtype = dense ? 0u : (uint32_t)lr_dtype;
          L.rcopies.push_back(cp);
          u.bytes += nb;
          u.ne++;
          L.payload_bytes += (uint64_t)nr * nc * esz;
        }
      }
      close();
    }
  }
}

void balance_ranges(const std::vector<uint64_t>& bytes, uint32_t grid, std::vector<uint32_t>& first) {
  first.assign(grid + 1, 0);
  const uint64_t total = std::accumulate(bytes.begin(), bytes.end(), (uint64_t)0);
  uint64_t acc = 0;
  uint32_t g = 1;
  for (uint32_t u = 0; u < bytes.size() && g < grid; ++u) {
    acc += bytes[u];
    while (g < grid && acc >= (total * g) / grid) first[g++] = u + 1;
  }
  while (g <= grid) first[g++] = (uint32_t)bytes.size();
  first[grid] = (uint32_t)bytes.size();
}

cudaError_t launch_stream_copies(const StreamCopy* copies, uint32_t n, const double* arena64,
                                 unsigned char* dst, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  stream_copy_kernel<<<n, 256, 0, s>>>(copies, arena64, dst);
  return cudaGetLastError();
}

cudaError_t launch_matvec_mixed(int prec, const MvPlan& pl, double d, uint32_t p, const double* X,
                                uint64_t ldX, double* Y, uint64_t ldY, cudaStream_t s) {
  if (p == 0 || pl.n == 0) return cudaSuccess;
  switch (prec) {
    case kFP32: return run_typed<float>(pl, d, p, X, ldX, Y, ldY, s);
    case kBF16FP32: return run_typed<__nv_bfloat16>(pl, d, p, X, ldX, Y, ldY, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace ahx
