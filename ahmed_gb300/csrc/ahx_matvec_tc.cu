// Mixed-precision H-matrix product on the tensor cores: Y += d A X with
// mltaGeHGeM semantics (H/mltaGeHVec.cpp:38-59, H/mblock.cpp:141-154,
// Include/mblock.h:105-109) as two linear sweeps over fragment-ordered leaf
// streams (layout described in ahx_matvec.cuh).
//
// One CTA per SM with kTcGroups groups.  Each group owns a contiguous range of
// units (balanced over all groups of the launch by bytes), a ring of kTcRing
// shared-memory slots, a producer warp and one or two consumer warps.  The
// producer fills the ring: per unit one bulk copy (cp.async.bulk, mbarrier completion) of the
// descriptor, one of the B fragments (L2 evict-first) and one per A-row run
// (L2 evict-last: X and T rows are re-read by many units).  The consumer
// warps of a group wait on the slot's full barrier, run the unit's mma.sync
// k-loop into register accumulators and release the slot on its empty
// barrier.  Accumulators persist across consecutive units of one output tile
// (one flush per tile run).  Every wait is bounded: on timeout the kernel
// raises the plan's error word, the producer waits (bounded) for the copies it
// queued, and all warps return.
#include <algorithm>
#include <atomic>
#include <cstdlib>
#include <map>
#include <numeric>
#include <type_traits>

#include <cuda_bf16.h>

#include "ahx_matvec.cuh"
#include "ahx_ptx.cuh"

namespace ahx {
namespace {

using namespace ptx;

constexpr int kG = (int)kTcGroups;
constexpr int kR = (int)kTcRing;
// slots, their mbarriers, and 2 KB that the extra-tile reads of the last slot may touch
constexpr size_t kSmem = (size_t)kG * kR * kTcSlot + (size_t)2 * kG * kR * sizeof(uint64_t) + 2048;

// Launch shapes for P right-hand sides.  Per group one producer warp and two
// consumer warps.  At 64 right-hand sides the two consumers split the m-tiles
// (16 right-hand sides each) of every unit; below, in the rows sweep each
// consumer takes every other unit of the group with the whole tile, and in
// the V sweep the two split the unit's n-tiles (distinct T rows).  The
// units of a group form SEQ sequences (unit i belongs to sequence i % SEQ),
// each with its own kR / SEQ slots, so every slot is filled and read strictly
// in order by one sequence and a parity wait never runs two phases ahead.
// Warps 0 .. kG * W - 1 consume (group = warp / W), warps kG * W + g produce.
template <int P, bool ROWS>
struct Cfg {
  static constexpr bool MSPLIT = P >= 64;                  // consumers split the m-tiles
  static constexpr bool NSPLIT = !MSPLIT && !ROWS;         // consumers split the n-tiles (V sweep)
  static constexpr int W = 2;                              // consumer warps per group
  static constexpr int SEQ = (MSPLIT || NSPLIT) ? 1 : W;   // unit sequences per group
  static constexpr int MTW = P / 16 / (MSPLIT ? 2 : 1);    // m-tiles per consumer warp
  static constexpr int NTW = NSPLIT ? 4 : 0;               // n-tiles per consumer warp (0: all)
  static constexpr int kEmpty = SEQ == 1 ? 2 : 1;          // releases per unit
  static constexpr int kConsumers = kG * W;
  static constexpr int kThreads = 32 * (kConsumers + kG);
  // registers per thread the CTA can give (multiple of 8)
  static constexpr int kRegs = (65536 / kThreads) & ~7 > 255 ? 255 : (65536 / kThreads) & ~7;
  static_assert(kR % SEQ == 0, "slots split evenly between sequences");
};

// slot and fill number of group-local unit i with SEQ sequences
template <int SEQ>
__device__ __forceinline__ void slot_of(uint32_t i, uint32_t& slot, uint32_t& fill) {
  constexpr uint32_t RS = kR / SEQ;
  const uint32_t q = i % SEQ, k = i / SEQ;
  slot = q * RS + k % RS;
  fill = k / RS;
}

__device__ __forceinline__ float sel4(const float (&v)[4], uint32_t i) {
  return i == 0 ? v[0] : i == 1 ? v[1] : i == 2 ? v[2] : v[3];
}

// Lanes t + 4 (4 q + j), j = 0..3, exchange their accumulator quadruples so
// that lane j ends with element j of each: w[j'] = v_{lane j'}[j].  For an
// m16n8 C fragment (v = C[g][2t], C[g][2t+1], C[g+8][2t], C[g+8][2t+1]) lane j
// then holds 4 consecutive rows p = 4 q + 8 (j >> 1) + 0..3 of column 2 t + (j & 1).
__device__ __forceinline__ void transpose4(const float (&v)[4], float (&w)[4], uint32_t j) {
  const float own = sel4(v, j);
  const float x1 = __shfl_xor_sync(0xffffffffu, sel4(v, j ^ 1u), 4);
  const float x2 = __shfl_xor_sync(0xffffffffu, sel4(v, j ^ 2u), 8);
  const float x3 = __shfl_xor_sync(0xffffffffu, sel4(v, j ^ 3u), 12);
#pragma unroll
  for (uint32_t i = 0; i < 4; ++i)
    w[i] = i == j ? own : i == (j ^ 1u) ? x1 : i == (j ^ 2u) ? x2 : x3;
}

// Accumulators of one consumer warp: acc[mt][n] is the m16n8 C fragment of
// m-tile mt, n-tile n.
template <int MTW, bool SPLIT>
struct Accs {
  float acc[MTW][8][4];
  __device__ __forceinline__ void zero() {
#pragma unroll
    for (int m = 0; m < MTW; ++m)
#pragma unroll
      for (int n = 0; n < 8; ++n)
#pragma unroll
        for (int i = 0; i < 4; ++i) acc[m][n][i] = 0.f;
  }
  __device__ __forceinline__ void total(int mt, int n, float (&v)[4]) const {
#pragma unroll
    for (int i = 0; i < 4; ++i) v[i] = acc[mt][n][i];
  }
};

// Fragments of one k-block held in registers.
template <int MTW, int NT>
struct TfFrag {
  float a[MTW][4];  // A (FP32 words; TF32-rounded already unless split)
  uint2 b[NT];      // B fragment words
};

template <int P, int MTW, int NT>
__device__ __forceinline__ void tf32_load(TfFrag<MTW, NT>& F, const uint2* fb, const float* side, uint32_t kb,
                                          uint32_t nt, uint32_t mt0, uint32_t lane) {
  constexpr uint32_t S = P + 8;
  const uint32_t g = lane >> 2, t = lane & 3;
  const float* sr = side + (kb * 8 + t) * S + 16 * mt0 + g;
#pragma unroll
  for (int mt = 0; mt < MTW; ++mt) {
    F.a[mt][0] = sr[16 * mt];
    F.a[mt][1] = sr[16 * mt + 8];
    F.a[mt][2] = sr[4 * S + 16 * mt];
    F.a[mt][3] = sr[4 * S + 16 * mt + 8];
  }
#pragma unroll
  for (int n = 0; n < NT; ++n) F.b[n] = fb[(kb * nt + n) * 32];
}

// SPLIT: the three products of a k-block (hi*hi + hi*lo + lo*hi) go into a
// fresh tile that is added to acc with round-to-nearest FP32 adds, so the
// tensor core's own accumulation spans 24 products.  Otherwise one pass on A
// and B already rounded to TF32.
template <int MTW, int NT, bool SPLIT>
__device__ __forceinline__ void tf32_compute(const TfFrag<MTW, NT>& F, Accs<MTW, SPLIT>& A) {
  uint32_t ah[MTW][4], al[MTW][4];
#pragma unroll
  for (int mt = 0; mt < MTW; ++mt)
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      if (SPLIT) {
        ah[mt][i] = to_tf32(F.a[mt][i]);
        al[mt][i] = to_tf32(F.a[mt][i] - __uint_as_float(ah[mt][i]));
      } else {
        ah[mt][i] = __float_as_uint(F.a[mt][i]);
        al[mt][i] = 0u;
      }
    }
#pragma unroll
  for (int n = 0; n < NT; ++n) {
    if (SPLIT) {
      const float b0 = __uint_as_float(F.b[n].x), b1 = __uint_as_float(F.b[n].y);
      const uint32_t bh0 = to_tf32(b0), bh1 = to_tf32(b1);
      const uint32_t bl0 = to_tf32(b0 - __uint_as_float(bh0)), bl1 = to_tf32(b1 - __uint_as_float(bh1));
#pragma unroll
      for (int mt = 0; mt < MTW; ++mt) {
        float c[4] = {0.f, 0.f, 0.f, 0.f};
        mma_tf32(c, al[mt], bh0, bh1);
        mma_tf32(c, ah[mt], bl0, bl1);
        mma_tf32(c, ah[mt], bh0, bh1);
#pragma unroll
        for (int i = 0; i < 4; ++i) A.acc[mt][n][i] += c[i];
      }
    } else {
#pragma unroll
      for (int mt = 0; mt < MTW; ++mt) mma_tf32(A.acc[mt][n], ah[mt], F.b[n].x, F.b[n].y);
    }
  }
}

// C += A B over k < kp for FP32 B fragments (k-blocks of 8) and FP32 A rows
// side[k][p] (stride P + 8), m-tiles mt0 .. mt0 + MTW - 1, NT n-tiles.
template <int P, int MTW, bool SPLIT, int NT>
__device__ __forceinline__ void tf32_group_nt(const unsigned char* frag, const float* side, uint32_t kp,
                                              uint32_t nt, uint32_t mt0, uint32_t n0, Accs<MTW, SPLIT>& A,
                                              uint32_t lane) {
  const uint2* fb = reinterpret_cast<const uint2*>(frag) + n0 * 32 + lane;
  for (uint32_t kb = 0; kb < kp / 8; ++kb) {
    TfFrag<MTW, NT> F;
    tf32_load<P, MTW, NT>(F, fb, side, kb, nt, mt0, lane);
    tf32_compute<MTW, NT, SPLIT>(F, A);
  }
}

template <int MTW, int NT>
struct BfFrag {
  uint32_t a[MTW][4];
  uint2 b[NT];
};

template <int P, int MTW, int NT>
__device__ __forceinline__ void bf16_load(BfFrag<MTW, NT>& F, const uint2* fb, uint32_t sbase, uint32_t kb, uint32_t nt,
                                          uint32_t lane) {
  constexpr uint32_t SB = (P + 8) * 2;
  const uint32_t m = lane >> 3, r = lane & 7;
  const uint32_t ra = sbase + (kb * 16 + (m >> 1) * 8 + r) * SB + (m & 1) * 16;
#pragma unroll
  for (int mt = 0; mt < MTW; ++mt) ldsm_x4_t(F.a[mt], ra + mt * 32);
#pragma unroll
  for (int n = 0; n < NT; ++n) F.b[n] = fb[(kb * nt + n) * 32];
}

template <int MTW, int NT>
__device__ __forceinline__ void bf16_compute(const BfFrag<MTW, NT>& F, Accs<MTW, false>& A) {
#pragma unroll
  for (int n = 0; n < NT; ++n)
#pragma unroll
    for (int mt = 0; mt < MTW; ++mt) mma_bf16_k16(A.acc[mt][n], F.a[mt], F.b[n].x, F.b[n].y);
}

// C += A B over k < kp for BF16 B fragments (k-blocks of 16, then one of 8
// when kp % 16 == 8) and BF16 A rows side[k][p] (stride P + 8) read with
// ldmatrix.trans, m-tiles mt0 .. mt0 + MTW - 1, NT n-tiles.
template <int P, int MTW, int NT>
__device__ __forceinline__ void bf16_group_nt(const unsigned char* frag, const unsigned char* side, uint32_t kp,
                                              uint32_t nt, uint32_t mt0, uint32_t n0, Accs<MTW, false>& A,
                                              uint32_t lane) {
  constexpr uint32_t SB = (P + 8) * 2;
  const uint32_t kfull = kp >> 4;
  const uint32_t m = lane >> 3, r = lane & 7;
  const uint32_t sbase = smem_u32(side) + mt0 * 32;
  const uint2* fb = reinterpret_cast<const uint2*>(frag) + n0 * 32 + lane;
  // one register set: a second (loads of block kb + 1 under the mma of kb)
  // exceeds the register budget at 64 right-hand sides
  for (uint32_t kb = 0; kb < kfull; ++kb) {
    BfFrag<MTW, NT> F;
    bf16_load<P, MTW, NT>(F, fb, sbase, kb, nt, lane);
    bf16_compute<MTW, NT>(F, A);
  }
  if (kp & 8) {
    const uint32_t* ft = reinterpret_cast<const uint32_t*>(frag + (size_t)kfull * nt * 256) + n0 * 32 + lane;
    const uint32_t ra = sbase + (kfull * 16 + r) * SB + (m & 1) * 16;
    uint32_t a0[MTW], a1[MTW], b[NT];
#pragma unroll
    for (int mt = 0; mt < MTW; ++mt) ldsm_x2_t(a0[mt], a1[mt], ra + mt * 32);
#pragma unroll
    for (int n = 0; n < NT; ++n) b[n] = ft[n * 32];
#pragma unroll
    for (int n = 0; n < NT; ++n)
#pragma unroll
      for (int mt = 0; mt < MTW; ++mt) mma_bf16_k8(A.acc[mt][n], a0[mt], a1[mt], b[n]);
  }
}

// The k-loops run NT n-tiles with no per-tile branches, so the independent
// mma chains of a k-block interleave: NT = 4 or 8 below 64 right-hand sides
// (two code paths: more would thrash the instruction cache), NT = 8 at 64
// (one code path keeps the register budget).
// Tiles n >= nt read B words past the group's fragments (inside the slot, or
// inside the padding after the last slot) into accumulators that are never
// flushed: those tiles hold no output rows.
// NT > 0: a fixed count of n-tiles starting at n-tile n0 (warps that split a
// unit's n-tiles); NT == 0: the unit's own count, rounded up to 4 or 8.
template <int P, int MTW, bool SPLIT, int NT = 0>
__device__ __forceinline__ void tf32_group(const unsigned char* frag, const float* side, uint32_t kp, uint32_t nt,
                                           uint32_t mt0, uint32_t n0, Accs<MTW, SPLIT>& acc, uint32_t lane) {
  if (NT > 0 || P >= 64) {
    tf32_group_nt<P, MTW, SPLIT, (NT > 0 ? NT : 8)>(frag, side, kp, nt, mt0, n0, acc, lane);
    return;
  }
  if (nt <= 4) tf32_group_nt<P, MTW, SPLIT, 4>(frag, side, kp, nt, mt0, 0, acc, lane);
  else tf32_group_nt<P, MTW, SPLIT, 8>(frag, side, kp, nt, mt0, 0, acc, lane);
}

template <int P, int MTW, int NT = 0>
__device__ __forceinline__ void bf16_group(const unsigned char* frag, const unsigned char* side, uint32_t kp,
                                           uint32_t nt, uint32_t mt0, uint32_t n0, Accs<MTW, false>& acc,
                                           uint32_t lane) {
  if (NT > 0 || P >= 64) {
    bf16_group_nt<P, MTW, (NT > 0 ? NT : 8)>(frag, side, kp, nt, mt0, n0, acc, lane);
    return;
  }
  if (nt <= 4) bf16_group_nt<P, MTW, 4>(frag, side, kp, nt, mt0, 0, acc, lane);
  else bf16_group_nt<P, MTW, 8>(frag, side, kp, nt, mt0, 0, acc, lane);
}

// ---------------------------------------------------------------------------
// Narrow form (one right-hand side): the same fragment-ordered streams read by
// FP32 FMAs instead of mma.sync, so a single-vector product does 1/16 of the
// arithmetic of a 16-wide pass.  X and T rows have the stride kSN (elements)
// and only column 0 is read; lane (g, t) of a fragment holds column 8 n + g of
// the k-block's rows listed at frag_pos, and the four lanes t of one g sum
// their partial dot products at the end.
constexpr uint32_t kSN = 8;

__device__ __forceinline__ float bf_lo(uint32_t w) { return __uint_as_float(w << 16); }
__device__ __forceinline__ float bf_hi(uint32_t w) { return __uint_as_float(w & 0xffff0000u); }

// FP32 B words (k-blocks of 8: b.x = B[8 kb + t][.], b.y = B[8 kb + t + 4][.]), FP32 A rows
template <int NT>
__device__ __forceinline__ void narrow_f32(const unsigned char* frag, const float* side, uint32_t kp, uint32_t nt,
                                           uint32_t n0, float (&acc)[NT], uint32_t lane) {
  const uint32_t t = lane & 3;
  const uint2* fb = reinterpret_cast<const uint2*>(frag) + n0 * 32 + lane;
  for (uint32_t kb = 0; kb < (kp >> 3); ++kb) {
    const float a0 = side[(kb * 8 + t) * kSN], a1 = side[(kb * 8 + t + 4) * kSN];
#pragma unroll
    for (int n = 0; n < NT; ++n)
      if (n0 + n < nt) {
        const uint2 b = fb[(kb * nt + n) * 32];
        acc[n] = fmaf(a1, __uint_as_float(b.y), fmaf(a0, __uint_as_float(b.x), acc[n]));
      }
  }
}

// BF16 B words (k-blocks of 16: b.x = B[16 kb + 2t, + 1][.], b.y = B[16 kb + 2t + 8, + 9][.];
// a last block of 8 when kp % 16 == 8), BF16 A rows
template <int NT>
__device__ __forceinline__ void narrow_bf16(const unsigned char* frag, const __nv_bfloat16* side, uint32_t kp,
                                            uint32_t nt, uint32_t n0, float (&acc)[NT], uint32_t lane) {
  const uint32_t t = lane & 3;
  const uint16_t* sh = reinterpret_cast<const uint16_t*>(side);
  const uint32_t kfull = kp >> 4;
  const uint2* fb = reinterpret_cast<const uint2*>(frag) + n0 * 32 + lane;
  for (uint32_t kb = 0; kb < kfull; ++kb) {
    const uint32_t k = kb * 16 + 2 * t;
    const float a0 = bf_lo(sh[k * kSN]), a1 = bf_lo(sh[(k + 1) * kSN]);
    const float a2 = bf_lo(sh[(k + 8) * kSN]), a3 = bf_lo(sh[(k + 9) * kSN]);
#pragma unroll
    for (int n = 0; n < NT; ++n)
      if (n0 + n < nt) {
        const uint2 b = fb[(kb * nt + n) * 32];
        float c = fmaf(a0, bf_lo(b.x), acc[n]);
        c = fmaf(a1, bf_hi(b.x), c);
        c = fmaf(a2, bf_lo(b.y), c);
        acc[n] = fmaf(a3, bf_hi(b.y), c);
      }
  }
  if (kp & 8) {
    const uint32_t* ft = reinterpret_cast<const uint32_t*>(frag + (size_t)kfull * nt * 256) + n0 * 32 + lane;
    const uint32_t k = kfull * 16 + 2 * t;
    const float a0 = bf_lo(sh[k * kSN]), a1 = bf_lo(sh[(k + 1) * kSN]);
#pragma unroll
    for (int n = 0; n < NT; ++n)
      if (n0 + n < nt) {
        const uint32_t b = ft[n * 32];
        acc[n] = fmaf(a1, bf_hi(b), fmaf(a0, bf_lo(b), acc[n]));
      }
  }
}

// lane 4 g (t = 0) receives the sum over t of column g's partial sums
__device__ __forceinline__ float narrow_sum(float v) {
  v += __shfl_xor_sync(0xffffffffu, v, 1);
  return v + __shfl_xor_sync(0xffffffffu, v, 2);
}

// ---------------------------------------------------------------------------
// Rings.  Group g of the CTA owns kR slots; slot s has a "full" mbarrier
// (count 1: the producer's arrive.expect_tx; the bulk copies complete its
// transaction count) and an "empty" mbarrier (count WPU: one arrive per
// consumer warp once it has read the slot).  The k-th fill of a slot waits for
// completion k - 1 of its empty barrier.
struct Ring {
  unsigned char* smem;
  __device__ unsigned char* slot(uint32_t g, uint32_t s) const { return smem + (size_t)(g * kR + s) * kTcSlot; }
  __device__ uint32_t full(uint32_t g, uint32_t s) const {
    return smem_u32(smem + (size_t)kG * kR * kTcSlot + (g * kR + s) * 8);
  }
  __device__ uint32_t empty(uint32_t g, uint32_t s) const {
    return smem_u32(smem + (size_t)kG * kR * kTcSlot + (kG * kR + g * kR + s) * 8);
  }
};

template <int EMPTY>
__device__ __forceinline__ Ring ring_init() {
  extern __shared__ __align__(128) unsigned char smem[];
  Ring R{smem};
  if (threadIdx.x == 0) {
    for (uint32_t g = 0; g < (uint32_t)kG; ++g)
      for (uint32_t s = 0; s < (uint32_t)kR; ++s) {
        mbar_init(R.full(g, s), 1);
        mbar_init(R.empty(g, s), EMPTY);
      }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  return R;
}

// Unit descriptors of a group are fetched 32 at a time (one coalesced load
// per warp): lane l holds the 32-byte descriptor of unit 32 b + l of the
// current batch b (c0, c1) and of the next one (n0, n1).
struct DescBatch {
  const uint4* base;  // descriptors of the group's first unit onwards
  uint32_t n, cb;
  uint4 c0, c1, n0, n1;
  __device__ void fetch(uint32_t b, uint4& w0, uint4& w1) const {
    const uint32_t i = b * 32 + (threadIdx.x & 31);
    if (i < n) {
      w0 = __ldg(base + 2 * (size_t)i);
      w1 = __ldg(base + 2 * (size_t)i + 1);
    } else {
      w0 = w1 = make_uint4(0u, 0u, 0u, 0u);
    }
  }
  __device__ void init(const void* descs, uint32_t u0, uint32_t count) {
    base = reinterpret_cast<const uint4*>(descs) + 2 * (size_t)u0;
    n = count;
    cb = 0;
    fetch(0, c0, c1);
    fetch(1, n0, n1);
  }
  // call with i = 32 cb + 32 when unit i is next: the next batch becomes current
  __device__ void advance() {
    c0 = n0;
    c1 = n1;
    ++cb;
    fetch(cb + 1, n0, n1);
  }
  // the eight words of unit i's descriptor (i in the current or next batch), in every lane
  __device__ void get(uint32_t i, uint32_t (&w)[8]) const {
    const bool c = (i >> 5) == cb;
    const int src = (int)(i & 31);
    const uint4 a = c ? c0 : n0, b = c ? c1 : n1;
    w[0] = __shfl_sync(0xffffffffu, a.x, src);
    w[1] = __shfl_sync(0xffffffffu, a.y, src);
    w[2] = __shfl_sync(0xffffffffu, a.z, src);
    w[3] = __shfl_sync(0xffffffffu, a.w, src);
    w[4] = __shfl_sync(0xffffffffu, b.x, src);
    w[5] = __shfl_sync(0xffffffffu, b.y, src);
    w[6] = __shfl_sync(0xffffffffu, b.z, src);
    w[7] = __shfl_sync(0xffffffffu, b.w, src);
  }
};

// Producer warp of group g: fills the group's ring in unit order.  issue(i, w,
// slot, bar) queues unit i's copies (w: its descriptor words).  A slot is
// reused after all consumer warps released it (sleeping bounded wait).  Before
// returning the warp waits (bounded) until every copy it queued has landed.
template <int SEQ, class Issue>
__device__ void produce(const Ring& R, const void* descs, const uint32_t* ranges, uint32_t g, int* err,
                        Issue issue) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t u0 = ranges[blockIdx.x * kG + g], u1 = ranges[blockIdx.x * kG + g + 1];
  const uint32_t n = u1 > u0 ? u1 - u0 : 0;
  uint32_t issued = 0;
  if (n > 0) {
    DescBatch B;
    B.init(descs, u0, n);
    for (uint32_t i = 0; i < n; ++i) {
      if (i > 0 && (i & 31) == 0) B.advance();
      uint32_t w[8];
      B.get(i, w);
      uint32_t s, k;
      slot_of<SEQ>(i, s, k);
      uint32_t ok = 1;
      if (k > 0 && lane == 0) ok = mbar_wait_sleep(R.empty(g, s), (k - 1) & 1, err) ? 1u : 0u;
      ok = __shfl_sync(0xffffffffu, ok, 0);
      if (!ok) break;
      issue(i, u0 + i, w, B, R.slot(g, s), R.full(g, s));
      ++issued;
    }
  }
  // every queued copy has landed before the CTA may exit
  if (lane == 0)
    for (uint32_t i = issued > (uint32_t)kR ? issued - kR : 0; i < issued; ++i) {
      uint32_t s, k;
      slot_of<SEQ>(i, s, k);
      mbar_wait_sleep(R.full(g, s), k & 1, err);
    }
  __syncwarp();
}

// Consumer warp of group g reading sequence seq: takes the units seq,
// seq + SEQ, ... of the group's range, runs body(head, data, lane) on each and
// releases its slot.
template <int SEQ, class Head, class Body>
__device__ void consume(const Ring& R, const uint32_t* ranges, uint32_t g, uint32_t seq, int* err, Body body) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t u0 = ranges[blockIdx.x * kG + g], u1 = ranges[blockIdx.x * kG + g + 1];
  const uint32_t n = u1 > u0 ? u1 - u0 : 0;
  for (uint32_t i = seq; i < n; i += SEQ) {
    uint32_t s, k;
    slot_of<SEQ>(i, s, k);
    if (!mbar_wait_sleep(R.full(g, s), k & 1, err)) return;
    const unsigned char* slot = R.slot(g, s);
    const Head H = *reinterpret_cast<const Head*>(slot);
    body(H, slot + kTcHead, lane);
    __syncwarp();
    // the arrive (release) orders this warp's reads of the slot before the
    // producer's acquire of the empty phase and its next bulk copy
    if (lane == 0) mbar_arrive(R.empty(g, s));
  }
}

static_assert(sizeof(TcVUnit) == kTcHead && sizeof(TcRowUnit) == kTcHead, "descriptor = slot head");

// ---- V sweep: T rows (T^T = X^T V per column cluster)
template <int P, bool BF, bool NARROW = false>
__global__ void __launch_bounds__((Cfg<P, false>::kThreads), 1) __maxnreg__((Cfg<P, false>::kRegs))
    tc_v_kernel(TcPlan pl) {
  using TT = typename std::conditional<BF, __nv_bfloat16, float>::type;
  using C = Cfg<P, false>;
  constexpr int MTW = C::MTW;
  constexpr uint32_t SX = (NARROW ? kSN : P + 8) * sizeof(TT);  // X row bytes (V's type)
  const Ring R = ring_init<C::kEmpty>();
  const uint32_t warp = threadIdx.x >> 5;
  if (warp >= (uint32_t)C::kConsumers) {
    const unsigned char* xs = reinterpret_cast<const unsigned char*>(BF ? pl.xb : (void*)pl.xf);
    const uint64_t pf = policy_evict_first(), pk = policy_evict_last();
    produce<C::SEQ>(R, pl.vunits, pl.vranges, warp - C::kConsumers, pl.err,
            [&](uint32_t, uint32_t u, const uint32_t (&w)[8], const DescBatch&, unsigned char* slot, uint32_t bar) {
              if ((threadIdx.x & 31) == 0) {
                // TcVUnit words: src (0, 1), bytes 2, xrow 3, kp | ncols << 16 4, trow 5, flags 6
                const uint64_t src = (uint64_t)w[0] | ((uint64_t)w[1] << 32);
                const uint32_t bytes = w[2], xb = (w[4] & 0xffffu) * SX;
                mbar_expect_tx(bar, kTcHead + bytes + xb);
                bulk_g2s(smem_u32(slot), pl.vunits + u, kTcHead, bar);
                bulk_g2s_hint(smem_u32(slot + kTcHead), pl.vstream + src, bytes, bar, pf);
                bulk_g2s_hint(smem_u32(slot + kTcHead + bytes), xs + (uint64_t)w[3] * SX, xb, bar, pk);
              }
            });
    return;
  }
  const uint32_t g = warp / C::W, h = warp % C::W;
  const uint32_t lane = threadIdx.x & 31, j = (lane >> 2) & 3, q = lane >> 4, t = lane & 3;
  TT* T = reinterpret_cast<TT*>(pl.t);
  if constexpr (NARROW) {
    // the two consumers split each unit's n-tiles (4 each); T rows of stride kSN
    const uint32_t n0 = h * 4;
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
    consume<C::SEQ, TcVUnit>(R, pl.vranges, g, 0, pl.err, [&](const TcVUnit& U, const unsigned char* data, uint32_t) {
      if (U.flags & 1u) acc[0] = acc[1] = acc[2] = acc[3] = 0.f;
      const uint32_t nt = (U.ncols + 7u) >> 3;
      if (n0 >= nt) return;
      if constexpr (BF) narrow_bf16<4>(data, reinterpret_cast<const __nv_bfloat16*>(data + U.bytes), U.kp, nt, n0, acc, lane);
      else narrow_f32<4>(data, reinterpret_cast<const float*>(data + U.bytes), U.kp, nt, n0, acc, lane);
      if (U.flags & 2u) {
#pragma unroll
        for (int n = 0; n < 4; ++n)
          if (n0 + n < nt) {
            const float v = narrow_sum(acc[n]);
            const uint32_t col = 8 * (n0 + n) + (lane >> 2);
            if (t == 0 && col < U.ncols) T[(uint64_t)(U.trow + col) * kSN] = (TT)v;
          }
      }
    });
    return;
  }
  Accs<MTW, !BF> acc;
  acc.zero();
  const uint32_t mt0 = C::MSPLIT ? h * MTW : 0, n0 = C::NSPLIT ? h * C::NTW : 0;
  consume<C::SEQ, TcVUnit>(R, pl.vranges, g, 0, pl.err, [&](const TcVUnit& U, const unsigned char* data, uint32_t) {
    if (U.flags & 1u) acc.zero();
    const uint32_t nt = (U.ncols + 7u) >> 3;
    if (n0 >= nt) return;  // no columns for this warp in this unit
    if constexpr (BF) bf16_group<P, MTW, C::NTW>(data, data + U.bytes, U.kp, nt, mt0, n0, acc, lane);
    else tf32_group<P, MTW, true, C::NTW>(data, reinterpret_cast<const float*>(data + U.bytes), U.kp, nt, mt0, n0,
                                          acc, lane);
    if (U.flags & 2u) {
#pragma unroll
      for (int mt = 0; mt < MTW; ++mt)
#pragma unroll
        for (int n = 0; n < (C::NTW ? C::NTW : 8); ++n) {
          if (n0 + n < nt) {
            float v[4], w[4];
            acc.total(mt, n, v);
            transpose4(v, w, j);
            const uint32_t col = 8 * (n0 + n) + 2 * t + (j & 1);
            if (col < U.ncols) {
              TT* dst = T + (uint64_t)(U.trow + col) * (P + 8) + 16 * (mt0 + mt) + 8 * (j >> 1) + 4 * q;
              if (BF) {
                __nv_bfloat162 lo = __floats2bfloat162_rn(w[0], w[1]);
                __nv_bfloat162 hi = __floats2bfloat162_rn(w[2], w[3]);
                uint2 pk;
                pk.x = *reinterpret_cast<uint32_t*>(&lo);
                pk.y = *reinterpret_cast<uint32_t*>(&hi);
                *reinterpret_cast<uint2*>(dst) = pk;
              } else {
                *reinterpret_cast<float4*>(dst) = make_float4(w[0], w[1], w[2], w[3]);
              }
            }
          }
        }
    }
  });
}

// NARROW: T rows of stride kSN, column 0 only
template <int P, bool BF, bool NARROW = false>
__global__ void tc_treduce_kernel(const TcTReduce* __restrict__ items, uint32_t n, void* tv) {
  using TT = typename std::conditional<BF, __nv_bfloat16, float>::type;
  constexpr uint32_t W = NARROW ? 1 : P, S = NARROW ? kSN : P + 8;
  TT* T = reinterpret_cast<TT*>(tv);
  const uint32_t it = blockIdx.x;
  if (it >= n) return;
  const TcTReduce R = items[it];
  for (uint32_t e = threadIdx.x; e < R.ncols * W; e += blockDim.x) {
    const uint32_t c = e / W, p = e % W;
    float s = (float)T[(uint64_t)(R.dst + c) * S + p];
    for (uint32_t k = 0; k < R.nsrc; ++k) s += (float)T[(uint64_t)(R.src + k * R.ncols + c) * S + p];
    T[(uint64_t)(R.dst + c) * S + p] = (TT)s;
  }
}

// ---- rows sweep: Yr[row0 + n][p] += sum over the tile's groups
template <int P, bool BF, bool NARROW = false>
__global__ void __launch_bounds__((Cfg<P, true>::kThreads), 1) __maxnreg__((Cfg<P, true>::kRegs))
    tc_rows_kernel(TcPlan pl) {
  using TT = typename std::conditional<BF, __nv_bfloat16, float>::type;
  using C = Cfg<P, true>;
  constexpr int MTW = C::MTW;
  constexpr uint32_t SE = NARROW ? kSN : P + 8;  // row stride (elements) of T and X rows
  constexpr uint32_t S0 = SE * sizeof(TT);       // T row bytes
  constexpr uint32_t S1 = SE * 4;                // FP32 X row bytes
  constexpr uint32_t ES0 = sizeof(TT);
  const Ring R = ring_init<C::kEmpty>();
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (warp >= (uint32_t)C::kConsumers) {
    const unsigned char* tsrc = reinterpret_cast<const unsigned char*>(pl.t);
    const unsigned char* xsrc = reinterpret_cast<const unsigned char*>(pl.xf);
    const uint64_t pf = policy_evict_first(), pk = policy_evict_last();
    // side entries of the unit two ahead are loaded while the current one is queued
    TcSide sA{0u, 0u, 0u, 0u}, sB{0u, 0u, 0u, 0u};
    auto side_load = [&](uint32_t i, const DescBatch& Bt, uint32_t nunits) {
      TcSide e{0u, 0u, 0u, 0u};
      if (i < nunits) {
        uint32_t w[8];
        Bt.get(i, w);
        if (lane < (w[5] & 0xffffu)) e = pl.sides[w[4] + lane];
      }
      return e;
    };
    bool primed = false;
    produce<C::SEQ>(R, pl.runits, pl.rranges, warp - C::kConsumers, pl.err,
            [&](uint32_t i, uint32_t u, const uint32_t (&w)[8], const DescBatch& Bt, unsigned char* slot,
                uint32_t bar) {
              if (!primed) {
                sA = side_load(0, Bt, Bt.n);
                sB = side_load(1, Bt, Bt.n);
                primed = true;
              }
              // TcRowUnit words: src (0, 1), bytes 2, row0 3, e0 4, ne | nr << 16 5,
              // kp0 | kp1 << 16 6, flags 7
              TcSide e;
              if (i & 1) {
                e = sB;
                sB = side_load(i + 2, Bt, Bt.n);
              } else {
                e = sA;
                sA = side_load(i + 2, Bt, Bt.n);
              }
              const uint64_t src = (uint64_t)w[0] | ((uint64_t)w[1] << 32);
              const uint32_t bytes = w[2], ne = w[5] & 0xffffu, kp0 = w[6] & 0xffffu;
              const bool g0 = e.group == 0;
              const uint32_t mine = lane < ne ? e.nrows * (g0 ? S0 : S1) : 0u;
              uint32_t total = mine;
#pragma unroll
              for (int o = 16; o > 0; o >>= 1) total += __shfl_xor_sync(0xffffffffu, total, o);
              if (lane == 0) {
                mbar_expect_tx(bar, kTcHead + bytes + total);
                bulk_g2s(smem_u32(slot), pl.runits + u, kTcHead, bar);
                bulk_g2s_hint(smem_u32(slot + kTcHead), pl.rstream + src, bytes, bar, pf);
              }
              __syncwarp();
              if (mine) {
                const uint32_t dst = kTcHead + bytes + (g0 ? e.dst_k * S0 : kp0 * S0 + e.dst_k * S1);
                const unsigned char* sp = g0 ? tsrc + (uint64_t)e.src_row * S0 : xsrc + (uint64_t)e.src_row * S1;
                bulk_g2s_hint(smem_u32(slot + dst), sp, mine, bar, pk);
              }
            });
    return;
  }
  const uint32_t g = warp / C::W, h = warp % C::W;
  const uint32_t mt0 = C::MSPLIT ? h * MTW : 0;
  const uint32_t j = (lane >> 2) & 3, q = lane >> 4, t = lane & 3;
  if constexpr (NARROW) {
    // each consumer takes every other unit (whole tiles); Yr has one float per row
    float acc[8];
#pragma unroll
    for (int n = 0; n < 8; ++n) acc[n] = 0.f;
    uint32_t cur_row0 = 0, cur_nr = 0;
    auto flush = [&]() {
      const uint32_t nt = (cur_nr + 7u) >> 3;
#pragma unroll
      for (int n = 0; n < 8; ++n) {
        if ((uint32_t)n < nt) {
          const float v = narrow_sum(acc[n]);
          const uint32_t row = 8 * n + (lane >> 2);
          if (t == 0 && row < cur_nr) atomicAdd(pl.yr + cur_row0 + row, v);
        }
        acc[n] = 0.f;
      }
    };
    consume<C::SEQ, TcRowUnit>(R, pl.rranges, g, h, pl.err, [&](const TcRowUnit& U, const unsigned char* data, uint32_t) {
      if (cur_nr && (U.row0 != cur_row0 || U.nr != cur_nr)) flush();
      cur_row0 = U.row0;
      cur_nr = U.nr;
      const uint32_t nt = (U.nr + 7u) >> 3;
      const unsigned char* side0 = data + U.bytes;
      if (U.kp0) {
        if constexpr (BF) narrow_bf16<8>(data, reinterpret_cast<const __nv_bfloat16*>(side0), U.kp0, nt, 0, acc, lane);
        else narrow_f32<8>(data, reinterpret_cast<const float*>(side0), U.kp0, nt, 0, acc, lane);
      }
      if (U.kp1)
        narrow_f32<8>(data + (size_t)U.kp0 * nt * 8 * sizeof(TT), reinterpret_cast<const float*>(side0 + (size_t)U.kp0 * S0),
                      U.kp1, nt, 0, acc, lane);
    });
    if (cur_nr) flush();
    return;
  }
  Accs<MTW, !BF> acc;
  acc.zero();
  // consecutive units of one tile accumulate; a change of tile (or the end)
  // flushes the accumulators into Yr with vector atomic adds
  uint32_t cur_row0 = 0, cur_nr = 0;
  auto flush = [&]() {
    const uint32_t nt = (cur_nr + 7u) >> 3;
#pragma unroll
    for (int mt = 0; mt < MTW; ++mt)
#pragma unroll
      for (int n = 0; n < 8; ++n) {
        if ((uint32_t)n < nt) {
          float v[4], w[4];
          acc.total(mt, n, v);
          transpose4(v, w, j);
          const uint32_t row = 8 * n + 2 * t + (j & 1);
          if (row < cur_nr)
            red4(pl.yr + (uint64_t)(cur_row0 + row) * P + 16 * (mt0 + mt) + 8 * (j >> 1) + 4 * q, w[0], w[1], w[2],
                 w[3]);
        }
      }
    acc.zero();
  };
  consume<C::SEQ, TcRowUnit>(R, pl.rranges, g, C::MSPLIT ? 0 : h, pl.err,
                     [&](const TcRowUnit& U, const unsigned char* data, uint32_t) {
    if (cur_nr && (U.row0 != cur_row0 || U.nr != cur_nr)) flush();
    cur_row0 = U.row0;
    cur_nr = U.nr;
    const uint32_t nt = (U.nr + 7u) >> 3;
    const unsigned char* side0 = data + U.bytes;
    if (U.kp0) {
      if constexpr (BF) bf16_group<P, MTW>(data, side0, U.kp0, nt, mt0, 0, acc, lane);
      else tf32_group<P, MTW, true>(data, reinterpret_cast<const float*>(side0), U.kp0, nt, mt0, 0, acc, lane);
    }
    if (U.kp1)
      tf32_group<P, MTW, !BF>(data + (size_t)U.kp0 * nt * 8 * ES0,
                              reinterpret_cast<const float*>(side0 + (size_t)U.kp0 * S0), U.kp1, nt, mt0, 0, acc,
                              lane);
  });
  if (cur_nr) flush();
}

// X (FP64, column-major, ld ldX) -> X rows: FP32 (stride P + 8; TF32-rounded
// when BF) and, when BF, BF16 (stride P + 8); columns pg .. P - 1 are zero.
template <int P, bool BF>
__global__ void tc_xr_kernel(const double* __restrict__ X, uint64_t ldX, uint64_t n, uint32_t r0, uint32_t pg,
                             float* __restrict__ xf, __nv_bfloat16* __restrict__ xb) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
#pragma unroll
    for (int c = 0; c < P; c += 8) {
      float v[8];
#pragma unroll
      for (int r = 0; r < 8; ++r)
        v[r] = (uint32_t)(c + r) < pg ? (float)X[(uint64_t)(r0 + c + r) * ldX + i] : 0.f;
      float4* of = reinterpret_cast<float4*>(xf + i * (P + 8) + c);
      if (BF) {
        float u[8];
#pragma unroll
        for (int r = 0; r < 8; ++r) u[r] = __uint_as_float(to_tf32(v[r]));
        of[0] = make_float4(u[0], u[1], u[2], u[3]);
        of[1] = make_float4(u[4], u[5], u[6], u[7]);
        __nv_bfloat162 b[4];
#pragma unroll
        for (int r = 0; r < 4; ++r) b[r] = __floats2bfloat162_rn(v[2 * r], v[2 * r + 1]);
        *reinterpret_cast<uint4*>(xb + i * (P + 8) + c) = *reinterpret_cast<uint4*>(b);
      } else {
        of[0] = make_float4(v[0], v[1], v[2], v[3]);
        of[1] = make_float4(v[4], v[5], v[6], v[7]);
      }
    }
  }
}

// Y[(r0 + p) * ldY + i] += d * Yr[i * P + p], p < pg
template <int P>
__global__ void tc_yr_kernel(const float* __restrict__ yr, uint64_t n, uint32_t r0, uint32_t pg, double d,
                             double* __restrict__ Y, uint64_t ldY) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const float4* src = reinterpret_cast<const float4*>(yr + i * P);
#pragma unroll
    for (int c = 0; c < P / 4; ++c) {
      const float4 v = src[c];
      const float w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
      for (int r = 0; r < 4; ++r)
        if ((uint32_t)(4 * c + r) < pg) Y[(uint64_t)(r0 + 4 * c + r) * ldY + i] += d * (double)w[r];
    }
  }
}

// narrow X rows (stride kSN): column 0 = X[r0 * ldX + i] (TF32-rounded FP32 and
// BF16 when BF), the rest zero
template <bool BF>
__global__ void tc_xr_narrow_kernel(const double* __restrict__ X, uint64_t n, float* __restrict__ xf,
                                    __nv_bfloat16* __restrict__ xb) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const float v = (float)X[i];
    float4* of = reinterpret_cast<float4*>(xf + i * kSN);
    of[0] = make_float4(BF ? __uint_as_float(to_tf32(v)) : v, 0.f, 0.f, 0.f);
    of[1] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (BF) {
      __nv_bfloat162 b[4];
      b[0] = __floats2bfloat162_rn(v, 0.f);
      b[1] = b[2] = b[3] = __floats2bfloat162_rn(0.f, 0.f);
      *reinterpret_cast<uint4*>(xb + i * kSN) = *reinterpret_cast<uint4*>(b);
    }
  }
}

// Y[i] += d * Yr[i] (narrow Yr: one float per row)
__global__ void tc_yr_narrow_kernel(const float* __restrict__ yr, uint64_t n, double d, double* __restrict__ Y) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    Y[i] += d * (double)yr[i];
}

// byte position of B[k][n] in fragment order (see TcFragTask)
__host__ __device__ __forceinline__ uint64_t frag_pos(uint32_t k, uint32_t n, uint32_t kp, uint32_t nt, uint32_t dtype) {
  const uint32_t g = n & 7, ntile = n >> 3;
  if (dtype != 1) {
    const uint32_t kb = k >> 3, kk = k & 7;
    const uint32_t lane = g * 4 + (kk & 3);
    return ((uint64_t)(kb * nt + ntile) * 32 + lane) * 8 + (kk >> 2) * 4;
  }
  const uint32_t kfull = kp >> 4;
  if ((k >> 4) < kfull) {
    const uint32_t kb = k >> 4, kk = k & 15;
    const uint32_t lane = g * 4 + ((kk & 7) >> 1);
    return ((uint64_t)(kb * nt + ntile) * 32 + lane) * 8 + (kk >> 3) * 4 + (kk & 1) * 2;
  }
  const uint32_t kk = k - kfull * 16;
  const uint32_t lane = g * 4 + (kk >> 1);
  return (uint64_t)kfull * nt * 256 + ((uint64_t)ntile * 32 + lane) * 4 + (kk & 1) * 2;
}

__global__ void tc_build_kernel(const TcFragTask* __restrict__ tasks, const TcSeg* __restrict__ segs,
                                const double* __restrict__ a64, unsigned char* __restrict__ dst) {
  const TcFragTask T = tasks[blockIdx.x];
  unsigned char* out = dst + T.dst;
  for (uint32_t s = 0; s < T.nseg; ++s) {
    const TcSeg S = segs[T.seg0 + s];
    const uint32_t inner = T.mode == 0 ? T.nvalid : T.kvalid;  // contiguous index
    const uint64_t cnt = (uint64_t)S.ncols * inner;
    for (uint64_t e = threadIdx.x; e < cnt; e += blockDim.x) {
      const uint32_t c = (uint32_t)(e / inner), r = (uint32_t)(e % inner);
      const double v = a64[S.base + (uint64_t)c * S.ld + r];
      const uint32_t k = T.mode == 0 ? S.start + c : r;
      const uint32_t n = T.mode == 0 ? r : S.start + c;
      const uint64_t pos = frag_pos(k, n, T.kp, T.nt, T.dtype);
      if (T.dtype == 0) *reinterpret_cast<float*>(out + pos) = (float)v;
      else if (T.dtype == 2) *reinterpret_cast<uint32_t*>(out + pos) = to_tf32((float)v);
      else *reinterpret_cast<__nv_bfloat16*>(out + pos) = __double2bfloat16(v);
    }
  }
}

unsigned grid_rows(uint64_t n) { return (unsigned)std::min<uint64_t>((n + 255) / 256, 152ull * 8); }

std::atomic<uint64_t> g_product_launches{0};

template <int P, bool BF, bool NARROW = false>
cudaError_t set_attributes() {
  cudaError_t e =
      cudaFuncSetAttribute(tc_v_kernel<P, BF, NARROW>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmem);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(tc_rows_kernel<P, BF, NARROW>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmem);
}

// one right-hand side (column r0 of X and Y): the narrow sweeps
template <bool BF>
cudaError_t run_tc_narrow(const TcPlan& pl, double d, uint32_t r0, const double* X, uint64_t ldX, double* Y,
                          uint64_t ldY, cudaStream_t s) {
  tc_xr_narrow_kernel<BF><<<grid_rows(pl.n), 256, 0, s>>>(X + (uint64_t)r0 * ldX, pl.n, pl.xf,
                                                         reinterpret_cast<__nv_bfloat16*>(pl.xb));
  g_product_launches += 2 + (pl.nvunits ? 1 : 0) + (pl.ntreduce ? 1 : 0) + (pl.nrunits ? 1 : 0);
  cudaError_t e = cudaMemsetAsync(pl.yr, 0, pl.n * sizeof(float), s);
  if (e != cudaSuccess) return e;
  if (pl.nvunits) tc_v_kernel<16, BF, true><<<pl.grid, Cfg<16, false>::kThreads, kSmem, s>>>(pl);
  if (pl.ntreduce) tc_treduce_kernel<16, BF, true><<<pl.ntreduce, 128, 0, s>>>(pl.treduce, pl.ntreduce, pl.t);
  if (pl.nrunits) tc_rows_kernel<16, BF, true><<<pl.grid, Cfg<16, true>::kThreads, kSmem, s>>>(pl);
  tc_yr_narrow_kernel<<<grid_rows(pl.n), 256, 0, s>>>(pl.yr, pl.n, d, Y + (uint64_t)r0 * ldY);
  return cudaGetLastError();
}

template <int P, bool BF>
cudaError_t run_tc_group(const TcPlan& pl, double d, uint32_t r0, uint32_t pg, const double* X, uint64_t ldX,
                         double* Y, uint64_t ldY, cudaStream_t s) {
  tc_xr_kernel<P, BF><<<grid_rows(pl.n), 256, 0, s>>>(X, ldX, pl.n, r0, pg, pl.xf,
                                                       reinterpret_cast<__nv_bfloat16*>(pl.xb));
  g_product_launches += 2 + (pl.nvunits ? 1 : 0) + (pl.ntreduce ? 1 : 0) + (pl.nrunits ? 1 : 0);
  cudaError_t e = cudaMemsetAsync(pl.yr, 0, pl.n * P * sizeof(float), s);
  if (e != cudaSuccess) return e;
  if (pl.nvunits) tc_v_kernel<P, BF><<<pl.grid, Cfg<P, false>::kThreads, kSmem, s>>>(pl);
  if (pl.ntreduce) tc_treduce_kernel<P, BF><<<pl.ntreduce, 128, 0, s>>>(pl.treduce, pl.ntreduce, pl.t);
  if (pl.nrunits) tc_rows_kernel<P, BF><<<pl.grid, Cfg<P, true>::kThreads, kSmem, s>>>(pl);
  tc_yr_kernel<P><<<grid_rows(pl.n), 256, 0, s>>>(pl.yr, pl.n, r0, pg, d, Y, ldY);
  return cudaGetLastError();
}

// AHX_NARROW=0 runs single-vector products through the 16-wide sweeps
bool narrow_enabled() {
  static const bool on = [] {
    const char* e = std::getenv("AHX_NARROW");
    return !(e && e[0] == '0');
  }();
  return on;
}

template <bool BF>
cudaError_t run_tc(const TcPlan& pl, double d, uint32_t p, const double* X, uint64_t ldX, double* Y,
                   uint64_t ldY, cudaStream_t s) {
  for (uint32_t r0 = 0; r0 < p; r0 += pl.pmax) {
    const uint32_t pg = std::min(pl.pmax, p - r0);
    cudaError_t e;
    // one right-hand side: FP32 FMAs on the fragments (narrow sweeps); FP32
    // storage runs 16 right-hand sides per pass (its 3-pass products would make
    // wider passes tensor-bound); BF16 up to 64
    if (pg == 1 && narrow_enabled()) e = run_tc_narrow<BF>(pl, d, r0, X, ldX, Y, ldY, s);
    else if (!BF || pg <= 16) e = run_tc_group<16, BF>(pl, d, r0, pg, X, ldX, Y, ldY, s);
    else if (pg <= 32) e = run_tc_group<32, true>(pl, d, r0, pg, X, ldX, Y, ldY, s);
    else e = run_tc_group<64, true>(pl, d, r0, pg, X, ldX, Y, ldY, s);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

uint32_t round8(uint32_t x) { return (x + 7u) & ~7u; }

// index of the entry containing column c (starts ascending, starts[0] = 0)
size_t entry_of(const std::vector<uint32_t>& starts, uint32_t c) {
  return (size_t)(std::upper_bound(starts.begin(), starts.end(), c) - starts.begin()) - 1;
}

}  // namespace

uint64_t product_launches() { return g_product_launches.load(); }

// shared-memory opt-in of every sweep kernel of the current device (before any
// launch, so that products can be captured in CUDA graphs)
cudaError_t tc_init_attributes() {
  cudaError_t e;
  if ((e = set_attributes<16, false>()) != cudaSuccess) return e;
  if ((e = set_attributes<16, true>()) != cudaSuccess) return e;
  if ((e = set_attributes<32, true>()) != cudaSuccess) return e;
  if ((e = set_attributes<16, false, true>()) != cudaSuccess) return e;
  if ((e = set_attributes<16, true, true>()) != cudaSuccess) return e;
  return set_attributes<64, true>();
}
void count_product_launches(uint64_t n) { g_product_launches += n; }

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

void build_tc_layout(const std::vector<PlanLeaf>& leaves, bool lr_bf16, uint32_t pmax, uint32_t nparts,
                     TcLayout& L, uint32_t unit_bytes) {
  L = TcLayout();
  const uint32_t cap = std::min(unit_bytes, kTcSlotData);
  const uint32_t es = lr_bf16 ? 2u : 4u;
  const uint32_t s_t = (pmax + 8) * es;  // T rows and the V sweep's X rows (factor type)
  const uint32_t s_x = (pmax + 8) * 4;   // FP32 X rows of dense leaves
  const uint32_t kblk0 = lr_bf16 ? 16u : 8u;
  std::vector<uint32_t> trow(leaves.size(), 0);

  // ---- V stream: low-rank leaves grouped by column cluster, <= 64 columns per unit
  struct VGroup {
    size_t u0, u1;
    uint32_t trow, ncols;
  };
  std::vector<VGroup> vgroups;
  std::map<std::pair<uint32_t, uint32_t>, std::vector<size_t>> colsets;
  for (size_t q = 0; q < leaves.size(); ++q)
    if (leaves[q].rank > 0) colsets[{leaves[q].b2, leaves[q].n2}].push_back(q);
  std::vector<uint64_t> vcost;
  for (auto& kv : colsets) {
    const uint32_t b2 = kv.first.first, n2 = kv.first.second;
    const std::vector<size_t>& ls = kv.second;
    std::vector<uint32_t> coloff(ls.size());
    uint32_t kc = 0;
    for (size_t i = 0; i < ls.size(); ++i) {
      coloff[i] = kc;
      kc += (uint32_t)leaves[ls[i]].rank;
    }
    const uint32_t tb = L.t_rows;
    L.t_rows += kc;
    for (size_t i = 0; i < ls.size(); ++i) trow[ls[i]] = tb + coloff[i];
    for (uint32_t c0 = 0; c0 < kc; c0 += 64) {
      const uint32_t nc = std::min(64u, kc - c0), nt = (nc + 7) / 8;
      const uint32_t rowb = nt * 8 * es + s_t;
      const uint32_t q = cap / rowb;  // rows per unit: multiples of 16, or of 8 for small caps
      const uint32_t chunk = q >= 16 ? q & ~15u : std::max(8u, q & ~7u);
      VGroup G{L.vunits.size(), 0, tb + c0, nc};
      for (uint32_t j0 = 0; j0 < n2; j0 += chunk) {
        const uint32_t jn = std::min(chunk, n2 - j0), kp = round8(jn);
        TcVUnit u{};
        u.src = L.vbytes;
        u.bytes = kp * nt * 8 * es;
        u.xrow = b2 + j0;
        u.kp = (uint16_t)kp;
        u.ncols = (uint16_t)nc;
        u.trow = tb + c0;
        TcFragTask T{};
        T.dst = L.vbytes;
        T.dtype = lr_bf16 ? 1u : 0u;
        T.kp = kp;
        T.nt = nt;
        T.kvalid = jn;
        T.nvalid = nc;
        T.seg0 = (uint32_t)L.segs.size();
        T.mode = 1;
        for (size_t i = 0; i < ls.size(); ++i) {
          const uint32_t k = (uint32_t)leaves[ls[i]].rank;
          const uint32_t lo = std::max(coloff[i], c0), hi = std::min(coloff[i] + k, c0 + nc);
          if (lo >= hi) continue;
          const PlanLeaf& P = leaves[ls[i]];
          TcSeg sg{};
          sg.base = P.off + (uint64_t)P.n1 * k + (uint64_t)(lo - coloff[i]) * P.n2 + j0;
          sg.ld = P.n2;
          sg.ncols = hi - lo;
          sg.start = lo - c0;
          L.segs.push_back(sg);
        }
        T.nseg = (uint32_t)L.segs.size() - T.seg0;
        L.vtasks.push_back(T);
        L.vunits.push_back(u);
        vcost.push_back((uint64_t)u.bytes + (uint64_t)kp * s_t);
        L.vbytes += u.bytes;
        L.payload_bytes += (uint64_t)jn * nc * es;
      }
      G.u1 = L.vunits.size();
      vgroups.push_back(G);
    }
  }
  balance_ranges(vcost, nparts, L.vranges);
  {
    std::vector<uint32_t> owner(L.vunits.size());
    for (uint32_t w = 0; w < nparts; ++w)
      for (uint32_t u = L.vranges[w]; u < L.vranges[w + 1]; ++u) owner[u] = w;
    for (const VGroup& G : vgroups) {
      std::vector<std::pair<size_t, size_t>> pieces;
      size_t a = G.u0;
      for (size_t u = G.u0 + 1; u <= G.u1; ++u)
        if (u == G.u1 || owner[u] != owner[u - 1]) {
          pieces.push_back({a, u});
          a = u;
        }
      uint32_t extra = 0;
      if (pieces.size() > 1) {
        extra = L.t_rows;
        L.t_rows += (uint32_t)(pieces.size() - 1) * G.ncols;
        L.treduce.push_back(TcTReduce{G.trow, extra, G.ncols, (uint32_t)(pieces.size() - 1)});
      }
      for (size_t pi = 0; pi < pieces.size(); ++pi) {
        for (size_t u = pieces[pi].first; u < pieces[pi].second; ++u)
          L.vunits[u].trow = pi == 0 ? G.trow : extra + (uint32_t)(pi - 1) * G.ncols;
        L.vunits[pieces[pi].first].flags |= 1u;
        L.vunits[pieces[pi].second - 1].flags |= 2u;
      }
    }
  }

  // ---- rows stream: block rows (row clusters), 64-row tiles, group 0 = low
  // rank (U columns, A = T rows), group 1 = dense (A = X rows)
  std::map<std::pair<uint32_t, uint32_t>, std::vector<size_t>> rowsets;
  for (size_t q = 0; q < leaves.size(); ++q)
    if (leaves[q].rank != 0) rowsets[{leaves[q].b1, leaves[q].n1}].push_back(q);
  std::vector<uint64_t> rcost;
  for (auto& kv : rowsets) {
    const uint32_t row_b1 = kv.first.first, n1 = kv.first.second;
    std::vector<size_t> e0l, e1l;  // leaves of group 0 / 1
    std::vector<uint32_t> st0, st1;
    uint32_t K0 = 0, K1 = 0;
    for (size_t q : kv.second) {
      if (leaves[q].rank > 0) {
        e0l.push_back(q);
        st0.push_back(K0);
        K0 += (uint32_t)leaves[q].rank;
      } else {
        e1l.push_back(q);
        st1.push_back(K1);
        K1 += leaves[q].n2;
      }
    }
    for (uint32_t r0 = 0; r0 < n1; r0 += 64) {
      const uint32_t nr = std::min(64u, n1 - r0), nt = (nr + 7) / 8;
      const uint32_t cb0 = nt * 8 * es + s_t, cb1 = nt * 8 * 4 + s_x;  // bytes per padded column
      uint32_t a0 = 0, c0g1 = 0;  // next column of each group
      while (a0 < K0 || c0g1 < K1) {
        // grow one unit block by block
        uint32_t a1 = a0, c1g1 = c0g1;
        auto entries = [&](uint32_t x0, uint32_t x1, const std::vector<uint32_t>& st) -> uint32_t {
          return x1 > x0 ? (uint32_t)(entry_of(st, x1 - 1) - entry_of(st, x0) + 1) : 0u;
        };
        for (;;) {
          uint32_t na1 = a1, nc1g1 = c1g1;
          if (a1 < K0) na1 = std::min(K0, a1 + kblk0);
          else if (c1g1 < K1) nc1g1 = std::min(K1, c1g1 + 8);
          else break;
          const uint32_t nbytes = round8(na1 - a0) * cb0 + round8(nc1g1 - c0g1) * cb1;
          const uint32_t ne = entries(a0, na1, st0) + entries(c0g1, nc1g1, st1);
          if ((a1 > a0 || c1g1 > c0g1) && (nbytes > cap || ne > 32)) break;
          a1 = na1;
          c1g1 = nc1g1;
        }
        const uint32_t kv0 = a1 - a0, kv1 = c1g1 - c0g1;
        const uint32_t kp0 = round8(kv0), kp1 = round8(kv1);
        TcRowUnit u{};
        u.src = L.rbytes;
        u.bytes = kp0 * nt * 8 * es + kp1 * nt * 8 * 4;
        u.row0 = row_b1 + r0;
        u.e0 = (uint32_t)L.sides.size();
        u.nr = (uint16_t)nr;
        u.kp0 = (uint16_t)kp0;
        u.kp1 = (uint16_t)kp1;
        // group 0: T rows of the low-rank leaves, U columns
        if (kv0) {
          TcFragTask T{};
          T.dst = L.rbytes;
          T.dtype = lr_bf16 ? 1u : 0u;
          T.kp = kp0;
          T.nt = nt;
          T.kvalid = kv0;
          T.nvalid = nr;
          T.seg0 = (uint32_t)L.segs.size();
          for (size_t ei = entry_of(st0, a0); ei < e0l.size() && st0[ei] < a1; ++ei) {
            const PlanLeaf& P = leaves[e0l[ei]];
            const uint32_t lo = std::max(st0[ei], a0), hi = std::min(st0[ei] + (uint32_t)P.rank, a1);
            TcSide sd{trow[e0l[ei]] + (lo - st0[ei]), hi - lo, lo - a0, 0u};
            L.sides.push_back(sd);
            TcSeg sg{};
            sg.base = P.off + (uint64_t)(lo - st0[ei]) * P.n1 + r0;
            sg.ld = P.n1;
            sg.ncols = hi - lo;
            sg.start = lo - a0;
            L.segs.push_back(sg);
          }
          L.sides.back().nrows += kp0 - kv0;
          T.nseg = (uint32_t)L.segs.size() - T.seg0;
          L.rtasks.push_back(T);
        }
        // group 1: X rows of the dense leaves, D columns
        if (kv1) {
          TcFragTask T{};
          T.dst = L.rbytes + (uint64_t)kp0 * nt * 8 * es;
          T.dtype = lr_bf16 ? 2u : 0u;  // one TF32 pass beside BF16 factors: round once here
          T.kp = kp1;
          T.nt = nt;
          T.kvalid = kv1;
          T.nvalid = nr;
          T.seg0 = (uint32_t)L.segs.size();
          for (size_t ei = entry_of(st1, c0g1); ei < e1l.size() && st1[ei] < c1g1; ++ei) {
            const PlanLeaf& P = leaves[e1l[ei]];
            const uint32_t lo = std::max(st1[ei], c0g1), hi = std::min(st1[ei] + P.n2, c1g1);
            TcSide sd{P.b2 + (lo - st1[ei]), hi - lo, lo - c0g1, 1u};
            L.sides.push_back(sd);
            TcSeg sg{};
            sg.base = P.off + (uint64_t)(lo - st1[ei]) * P.n1 + r0;
            sg.ld = P.n1;
            sg.ncols = hi - lo;
            sg.start = lo - c0g1;
            L.segs.push_back(sg);
          }
          L.sides.back().nrows += kp1 - kv1;
          T.nseg = (uint32_t)L.segs.size() - T.seg0;
          L.rtasks.push_back(T);
        }
        u.ne = (uint16_t)(L.sides.size() - u.e0);
        L.runits.push_back(u);
        rcost.push_back((uint64_t)u.bytes + (uint64_t)kp0 * s_t + (uint64_t)kp1 * s_x);
        L.rbytes += u.bytes;
        L.payload_bytes += (uint64_t)nr * (kv0 * es + kv1 * 4);
        a0 = a1;
        c0g1 = c1g1;
      }
    }
  }
  balance_ranges(rcost, nparts, L.rranges);
  for (uint32_t w = 0; w < nparts; ++w) {
    const uint32_t u0 = L.rranges[w], u1 = L.rranges[w + 1];
    for (uint32_t u = u0; u < u1; ++u) {
      const bool first = u == u0 || L.runits[u].row0 != L.runits[u - 1].row0 || L.runits[u].nr != L.runits[u - 1].nr;
      const bool last = u + 1 == u1 || L.runits[u].row0 != L.runits[u + 1].row0 || L.runits[u].nr != L.runits[u + 1].nr;
      L.runits[u].flags = (first ? 1u : 0u) | (last ? 2u : 0u);
    }
  }
}

cudaError_t launch_tc_build(const TcFragTask* tasks, uint32_t ntasks, const TcSeg* segs, const double* arena64,
                            unsigned char* dst, cudaStream_t s) {
  if (ntasks == 0) return cudaSuccess;
  tc_build_kernel<<<ntasks, 256, 0, s>>>(tasks, segs, arena64, dst);
  return cudaGetLastError();
}

cudaError_t launch_matvec_tc(int prec, const TcPlan& pl, double d, uint32_t p, const double* X, uint64_t ldX,
                             double* Y, uint64_t ldY, cudaStream_t s) {
  if (p == 0 || pl.n == 0) return cudaSuccess;
  switch (prec) {
    case kFP32: return run_tc<false>(pl, d, p, X, ldX, Y, ldY, s);
    case kBF16FP32: return run_tc<true>(pl, d, p, X, ldX, Y, ldY, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace ahx
