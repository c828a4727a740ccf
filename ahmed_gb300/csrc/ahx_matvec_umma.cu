// H-matrix product on the fifth-generation tensor cores (tcgen05.mma with
// tensor-memory accumulators, kind::f16) over leaf streams of FP16 pairs; the
// layout, the sweeps and the precision scheme are described in ahx_umma.cuh.
//
// One persistent CTA per SM, 20 warps with fixed roles:
//   warp 0      producer: walks the CTA's contiguous range of tiles (ranges
//               balanced by bytes; descriptors fetched 32 at a time) and
//               bulk-copies (cp.async.bulk) each chunk image into one of
//               kSlots ring slots
//   warp 1      MMA issuer (one thread) and owner of the tensor memory: per
//               chunk, kc / 16 tcgen05.mma of N = 2 n16 (the first FP16
//               part of B in rows 0 .. n8 - 1, the second in rows n16 ..
//               128 + n8 - 1: one wide MMA per K step instead of two narrow
//               ones, whose fixed issue cost dominates) into one of two
//               256-column accumulators, A read MN-major from the slot, then
//               tcgen05.commit to the ring slot and to the accumulator
//   warps 2-3   Z rows: each gathers half of a chunk's Z rows (indices
//               kLidx chunks ahead in a small queue, one bulk copy each) with
//               16-byte cp.async straight into the slot's A operand: MN-major
//               with the 128-byte swizzle (the row of K position p is the Z
//               row itself, its first 64 FP16 values in one atom column, its
//               second 64 in the next), so no transposition sits between the
//               copies and the MMAs
//   warps 4-19  epilogue, four warps per tensor-memory lane quadrant (output
//               rows 0-31, 32-63, 64-95, 96-127): each thread adds its accumulator row
//               (the two parts of B summed), times the chunk's scale, to
//               registers (round-to-nearest FP32) per chunk; at the end of a
//               tile the rows of the two parts of A are
//               summed through shared memory into Y (FP64, in place) or into
//               T rows (split into FP16 pairs; FP32 atomics for split tiles)
// Every wait is bounded: on timeout the kernel raises the error word and all
// roles return after the copies and MMAs they started have completed.
#include <algorithm>
#include <cstdlib>
#include <map>
#include <mutex>
#include <vector>

#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_fp16.h>

#include "ahx_ptx.cuh"
#include "ahx_umma.cuh"

namespace ahx {
namespace {

using namespace ptx;

// ---- shared-memory plan (offsets from the dynamic base, which is 1024-byte aligned)
constexpr uint32_t kSlots = 4;                            // ring slots (chunk image + its A operand)
constexpr uint32_t kLidx = 6;                             // Z-row indices are fetched this many chunks ahead
constexpr uint32_t kQ = 7;                                // index queue entries (> kLidx)
constexpr uint32_t kZWarps = 2;                           // Z-row warps, each gathers kZPos positions of a chunk
constexpr uint32_t kZPos = kUmKc / kZWarps;
constexpr uint32_t kARegion = 128 * kUmKc * 2;            // A operand of a chunk: 128 x 64 FP16
constexpr uint32_t kAHalf = kARegion / 2;                 // first parts (M 0-63) | second parts (M 64-127)
constexpr uint32_t kAKStep = 16 * 128;                    // bytes of 16 K positions (two swizzle atoms)
constexpr uint32_t kImgHead = 0;                          // image-slot offset of the chunk head
constexpr uint32_t kImgB = kImgHead + 32;                 // image-slot offset of the b1 image
constexpr uint32_t kImgMax = kUmN * kUmKc * 4;            // b1 + b2 images of the largest chunk
constexpr uint32_t kImgSlot = kImgB + kImgMax;
constexpr uint32_t kZRowPitch = kUmZPitch;
constexpr uint32_t kOffImg = kSlots * kARegion;           // the A operands first (1024-byte aligned)
constexpr uint32_t kAcc = 2;                              // tensor-memory accumulators (256 columns each)
constexpr uint32_t kAccCols = 2 * kUmN;
constexpr uint32_t kSRow = 32;                            // staging row (floats), columns XOR-swizzled by the row
constexpr uint32_t kOffStaging = kOffImg + kSlots * kImgSlot;
constexpr uint32_t kStagingBytes = 64 * kSRow * 4;        // per quarter of the output rows
constexpr uint32_t kOffYs = kOffStaging + 4 * kStagingBytes;   // 64 doubles: Y factor per right-hand side
constexpr uint32_t kOffAccHdr = kOffYs + 64 * 8;
constexpr uint32_t kOffMeta = kOffAccHdr + kAcc * sizeof(UmHead);
constexpr uint32_t kOffIssue = kOffMeta + kSlots * 16;    // per slot: clock of the copies' issue (diagnostics)
constexpr uint32_t kOffIdxQ = (kOffIssue + kSlots * 8 + 15) / 16 * 16;  // index queues: per Z warp kQ x kZPos words
constexpr uint32_t kOffBar = kOffIdxQ + kZWarps * kQ * kZPos * 4;
constexpr uint32_t kNumBars = 3 * kSlots + kZWarps * kQ + 2 * kAcc + 4;
constexpr uint32_t kOffTmem = kOffBar + kNumBars * 8;
constexpr uint32_t kSmemBytes = kOffTmem + 16;
constexpr uint32_t kThreads = 640;
constexpr uint32_t kEpiWarp0 = 2 + kZWarps;               // first epilogue warp
constexpr uint32_t kEpiWarps = 16;                        // epilogue warps: each arrives on accempty
static_assert(kThreads == 32 * (kEpiWarp0 + kEpiWarps), "roles");
constexpr uint32_t kTmemCols = kAcc * kAccCols;           // all 512 columns
static_assert(kTmemCols == 512, "tensor memory");
static_assert(kImgSlot % 16 == 0 && kOffIdxQ % 16 == 0 && (kZPos * 4) % 16 == 0, "bulk-copy destinations");
static_assert(kARegion % 1024 == 0, "swizzle atoms");
static_assert(kSmemBytes <= 232448, "shared memory per CTA");
static_assert(kQ > kLidx, "the queue entry of a chunk is read before a later prefetch reuses it");

// per-slot record written by the producer
struct SlotMeta {
  uint32_t hdr;       // bytes before the image pair in the stream (32); 0: stop marker
  uint32_t pad[3];
};

struct KArgs {
  CUtensorMap zmap;        // Z rows as a 2D tensor (128 FP16 x rows), boxes of 64 x kZPos, 128-byte swizzle
  const UmTile* tiles;
  const uint32_t* ranges;  // per CTA: first tile (gridDim.x + 1 entries), balanced by bytes
  const uint32_t* cranges; // per CTA: first chunk (gridDim.x + 1 entries)
  const uint32_t* zidx;    // Z-row indices, 32 per chunk
  const unsigned char* stream;
  uint16_t* z;          // Z rows (FP16 pairs), X rows then T rows
  float* tacc;          // FP32 accumulation rows of split V tiles
  const uint32_t* xmax; // max |X_j| of the pass (FP32 bits)
  double* y;            // rows sweep: Y (column-major, ldY), first column of this pass
  uint64_t ldy;
  uint64_t n;           // rows of X: Z row of T row t is n + t
  double d;
  uint32_t pg;          // right-hand sides of this pass (<= 64)
  uint32_t mode;        // 0: V sweep (T out), 1: rows sweep (Y out)
  uint32_t prof;        // 1: per-role cycle counters into g_um_prof
  int* err;
};

// Per-role cycle counters of the sweeps (diagnostics, off by default): summed
// over CTAs, lane 0 of warps 0 (producer), 1 (MMA), 2 (Z rows) and the first epilogue warp.
enum UmProf : uint32_t {
  kPfProdTotal, kPfProdSlot, kPfProdSpare, kPfChunks,
  kPfMmaImg, kPfMmaAccempty, kPfMmaFz, kPfMmaIssue,
  kPfEpiAccfull, kPfEpiDrain, kPfEpiTile, kPfZLatency,
  kPfZIdx, kPfZSlot, kPfZIssue, kPfZSpare,
  kPfCount = 16
};
__device__ unsigned long long g_um_prof[kPfCount];

struct ProfClock {
  bool on;
  unsigned long long acc[4] = {0, 0, 0, 0};
  __device__ explicit ProfClock(bool o) : on(o) {}
  __device__ __forceinline__ long long now() const { return on ? clock64() : 0; }
  __device__ __forceinline__ void add(int i, long long t0) {
    if (on) acc[i] += (unsigned long long)(clock64() - t0);
  }
  __device__ void flush(uint32_t base) const {
    if (!on) return;
    for (int i = 0; i < 4; ++i) atomicAdd(&g_um_prof[base + i], acc[i]);
  }
};

struct Smem {
  unsigned char* base;
  __device__ unsigned char* areg(uint32_t i) const { return base + i * kARegion; }
  __device__ unsigned char* img(uint32_t i) const { return base + kOffImg + i * kImgSlot; }
  __device__ const UmHead* head(uint32_t i) const { return reinterpret_cast<const UmHead*>(img(i) + kImgHead); }
  __device__ uint32_t* idxq(uint32_t w, uint32_t i) const {
    return reinterpret_cast<uint32_t*>(base + kOffIdxQ) + (w * kQ + i) * kZPos;
  }
  __device__ volatile long long* issued(uint32_t i) const {
    return reinterpret_cast<volatile long long*>(base + kOffIssue) + i;
  }
  __device__ float* staging(uint32_t quarter) const {
    return reinterpret_cast<float*>(base + kOffStaging + quarter * kStagingBytes);
  }
  __device__ double* ys() const { return reinterpret_cast<double*>(base + kOffYs); }
  __device__ UmHead* acchdr(uint32_t a) const { return reinterpret_cast<UmHead*>(base + kOffAccHdr) + a; }
  __device__ SlotMeta* meta(uint32_t i) const { return reinterpret_cast<SlotMeta*>(base + kOffMeta) + i; }
  __device__ uint32_t bar(uint32_t i) const { return smem_u32(base + kOffBar + 8 * i); }
  __device__ uint32_t fimg(uint32_t i) const { return bar(i); }
  __device__ uint32_t fz(uint32_t i) const { return bar(kSlots + i); }
  __device__ uint32_t empty(uint32_t i) const { return bar(2 * kSlots + i); }
  __device__ uint32_t idxbar(uint32_t w, uint32_t i) const { return bar(3 * kSlots + w * kQ + i); }
  __device__ uint32_t accfull(uint32_t i) const { return bar(3 * kSlots + kZWarps * kQ + i); }
  __device__ uint32_t accempty(uint32_t i) const { return bar(3 * kSlots + kZWarps * kQ + kAcc + i); }
  __device__ uint32_t quarter(uint32_t i) const { return bar(3 * kSlots + kZWarps * kQ + 2 * kAcc + i); }
  __device__ uint32_t* tmem_slot() const { return reinterpret_cast<uint32_t*>(base + kOffTmem); }
};

// staging element (right-hand side j, column c): 32 floats per j, the columns
// XOR-swizzled by j so that a warp's accesses along j or along c hit 32 banks
__device__ __forceinline__ uint32_t stg(uint32_t j, uint32_t c) { return j * kSRow + (c ^ (j & 31u)); }

// Bounded wait; it also gives up as soon as another role has raised the error
// word, so that one failed wait ends the whole CTA quickly.
__device__ __forceinline__ bool wait_bar(uint32_t bar, uint32_t parity, int* err) {
  for (uint32_t it = 0; it < kWaitLimit; ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((it & 1023u) == 1023u && *reinterpret_cast<volatile int*>(err)) return false;
  }
  atomicExch(err, 1);
  return false;
}

// Power of two s with |v| / s in [2^13, 2^14) for the largest |v| = m (1 for m = 0).
__host__ __device__ __forceinline__ int scale_exp(double m) {
  if (!(m > 0.0)) return 0;
  int ex;
  frexp(m, &ex);  // m = f 2^ex, f in [0.5, 1)
  return ex - 14;
}

// the two FP16 parts of v (v already scaled into the FP16 range)
__device__ __forceinline__ void split_h16(float v, __half& h1, __half& h2) {
  h1 = __float2half_rn(v);
  h2 = __float2half_rn(v - __half2float(h1));
}

// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads, 1) um_sweep_kernel(const __grid_constant__ KArgs a) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  const Smem S{smem_raw};
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // the swizzle atoms of the A operands need a 1024-byte aligned base (the
  // dynamic shared memory of a kernel without static shared memory starts there)
  if (smem_u32(smem_raw) & 1023u) {
    if (threadIdx.x == 0) atomicExch(a.err, 1);
    return;
  }

  if (threadIdx.x == 0) {
    for (uint32_t i = 0; i < kSlots; ++i) {
      mbar_init(S.fimg(i), 1);
      // per Z warp: one cp.async arrive per lane and one arrive (with the
      // tensor copies' bytes, or none) by lane 0
      mbar_init(S.fz(i), 33 * kZWarps);
      mbar_init(S.empty(i), 1);
    }
    for (uint32_t i = 0; i < kZWarps * kQ; ++i) mbar_init(S.bar(3 * kSlots + i), 1);
    for (uint32_t i = 0; i < 4; ++i) mbar_init(S.quarter(i), 4);
    for (uint32_t i = 0; i < kAcc; ++i) {
      mbar_init(S.accfull(i), 2);
      mbar_init(S.accempty(i), kEpiWarps);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // A rows past a chunk's K meet zero B values: they must hold finite
  // numbers, so every slot's A operand starts at zero (later chunks leave
  // only Z values behind)
  for (uint32_t i = threadIdx.x; i < kSlots * kARegion / 16; i += kThreads)
    reinterpret_cast<uint4*>(S.areg(0))[i] = make_uint4(0u, 0u, 0u, 0u);
  fence_proxy_async();
  if (threadIdx.x < 64) {
    // Y factor of right-hand side j: 1 / (the scale of X_j)
    const float m = __uint_as_float(a.xmax[threadIdx.x]);
    S.ys()[threadIdx.x] = ldexp(1.0, scale_exp((double)m));
  }
  if (warp == 1) {
    tmem_alloc(smem_u32(S.tmem_slot()), kTmemCols);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *S.tmem_slot();

  const bool pf = a.prof != 0 && lane == 0;
  if (warp == 0) {
    // ---------------- producer
    ProfClock P(pf);
    const long long tk0 = P.now();
    // L2: chunk images are read once (evict first)
    const uint64_t pol_img = policy_evict_first();
    uint32_t c = 0;  // chunks issued
    bool ok = true;
    // lane 0: the slot of chunk cc is free (its previous chunk has been consumed)
    auto slot_free = [&](uint32_t cc) -> bool {
      return cc < kSlots || wait_bar(S.empty(cc % kSlots), ((cc / kSlots) - 1) & 1, a.err);
    };
    const uint32_t t0 = a.ranges[blockIdx.x], t1 = a.ranges[blockIdx.x + 1];
    auto fetch = [&](uint32_t tb, uint4& w0, uint4& w1) {
      const uint32_t t = tb + lane;
      if (t < t1) {
        const uint4* d = reinterpret_cast<const uint4*>(a.tiles + t);
        w0 = __ldg(d);
        w1 = __ldg(d + 1);
      } else {
        w0 = w1 = make_uint4(0u, 0u, 0u, 0u);
      }
    };
    uint4 c0, c1, n0, n1;
    fetch(t0, c0, c1);
    fetch(t0 + 32, n0, n1);
    for (uint32_t t = t0; ok && t < t1; ++t) {
      const uint32_t r = (t - t0) & 31;
      if (r == 0 && t != t0) {
        c0 = n0;
        c1 = n1;
        fetch(t + 32, n0, n1);
      }
      // UmTile words: src (c0.x, c0.y), nchunks c0.z, n8 | hdr << 16 c0.w;
      // klast | kvlast << 16 c1.x
      const uint32_t w_sl = __shfl_sync(0xffffffffu, c0.x, r), w_sh = __shfl_sync(0xffffffffu, c0.y, r);
      const uint32_t nch = __shfl_sync(0xffffffffu, c0.z, r), w3 = __shfl_sync(0xffffffffu, c0.w, r);
      const uint32_t w4 = __shfl_sync(0xffffffffu, c1.x, r);
      const uint64_t tsrc = (uint64_t)w_sl | ((uint64_t)w_sh << 32);
      const uint32_t n8 = w3 & 0xffffu, hdr = w3 >> 16;
      const uint32_t klast = w4 & 0xffffu;  // (the valid positions, w4 >> 16, matter to no copy)
      const uint64_t cstride = (uint64_t)hdr + (uint64_t)n8 * kUmKc * 4;
      for (uint32_t ch = 0; ch < nch; ++ch) {
        const bool lastc = ch + 1 == nch;
        const uint32_t kc = lastc ? klast : kUmKc;
        const uint32_t bytes = hdr + n8 * kc * 4;
        const uint32_t sl = c % kSlots;
        bool okl = true;
        long long tp = P.now();
        if (lane == 0) okl = slot_free(c);
        P.add(1, tp);
        ok = __shfl_sync(0xffffffffu, okl ? 1u : 0u, 0) != 0;
        if (!ok) break;
        if (lane == 0) {
          if (pf) *S.issued(sl) = clock64();
          S.meta(sl)->hdr = hdr;
          mbar_expect_tx(S.fimg(sl), bytes);
          // head and b1 image, then the b2 image n16 rows after the b1 image's start
          const unsigned char* src = a.stream + tsrc + (uint64_t)ch * cstride;
          const uint32_t half_bytes = n8 * kc * 2, n16 = (n8 + 15u) & ~15u;
          bulk_g2s_hint(smem_u32(S.img(sl) + kImgB - hdr), src, hdr + half_bytes, S.fimg(sl), pol_img);
          bulk_g2s_hint(smem_u32(S.img(sl) + kImgB + n16 * kc * 2), src + hdr + half_bytes, half_bytes,
                        S.fimg(sl), pol_img);
        }
        ++c;
      }
    }
    if (lane == 0) {
      bool stopped = false;
      if (ok && slot_free(c)) {
        // stop marker: a slot record without an image (the MMA thread reads
        // it after the image barrier and waits for no Z rows; the Z warps
        // stop after the CTA's last chunk)
        const uint32_t sl = c % kSlots;
        S.meta(sl)->hdr = 0u;
        mbar_arrive(S.fimg(sl));
        stopped = true;
      }
      // every bulk copy issued has landed before the CTA may exit (bounded, but
      // not cut short by another role's error: a copy in flight must not land
      // after the CTA has exited).  Older chunks were consumed, hence landed;
      // so was chunk c - kSlots once the stop marker took its slot (its
      // image barrier has moved on by a phase since).
      const uint32_t keep = stopped ? kSlots - 1 : kSlots;
      const uint32_t lo = c > keep ? c - keep : 0u;
      for (uint32_t i = lo; i < c; ++i) mbar_wait_sleep(S.fimg(i % kSlots), (i / kSlots) & 1, a.err);
      P.add(0, tk0);
      P.acc[3] = c;
      P.flush(kPfProdTotal);
    }
    __syncwarp();
  } else if (warp == 1) {
    // ---------------- MMA issuer
    if (lane == 0) {
      ProfClock P(pf);
      unsigned long long zlat = 0;
      uint32_t c = 0;
      bool issued = false;
      while (true) {
        const uint32_t sl = c % kSlots, q = c % kAcc;
        long long tp = P.now();
        if (!wait_bar(S.fimg(sl), (c / kSlots) & 1, a.err)) break;
        P.add(0, tp);
        tp = P.now();
        if (c >= kAcc && !wait_bar(S.accempty(q), ((c / kAcc) - 1) & 1, a.err)) break;
        P.add(1, tp);
        if (S.meta(sl)->hdr == 0u) {
          // forward the stop to the epilogue (both arrivals of the phase)
          volatile uint32_t* f = &S.acchdr(q)->flags;
          *f = kUmStop;
          mbar_arrive(S.accfull(q));
          mbar_arrive(S.accfull(q));
          break;
        }
        tp = P.now();
        if (!wait_bar(S.fz(sl), (c / kSlots) & 1, a.err)) break;
        P.add(2, tp);
        if (P.on) zlat += (unsigned long long)(clock64() - *S.issued(sl));  // issue -> Z rows landed
        tp = P.now();
        const UmHead h = *S.head(sl);
        // the Z rows came through cp.async (generic proxy), the tensor core
        // reads them through the async proxy
        fence_proxy_async();
        tc_fence_after();
        // B rows 0 .. n8-1: first parts; rows n16 .. n16 + n8 - 1: second parts
        // (rows in between and past them are stale: their D columns are not read);
        // a narrow tile takes a narrow MMA
        const uint32_t n16 = ((uint32_t)h.n8 + 15u) & ~15u;
        const uint32_t idesc = umma_idesc_f16(128, 2 * n16) | kUmmaAMnMajor;
        const uint32_t sbo = (uint32_t)h.kc * 16u;  // 8 rows x kc FP16 per core-matrix row group
        const uint32_t sa = smem_u32(S.areg(sl));
        const uint32_t sb = smem_u32(S.img(sl) + kImgB);
        const uint32_t d = tmem + q * kAccCols;
        // A: M atoms (first / second parts) kAHalf apart, 8-position K atoms 1024 bytes apart
        for (uint32_t s = 0; s < (uint32_t)h.kc / 16u; ++s)
          umma_f16(d, umma_desc_sw128(sa + s * kAKStep, kAHalf, 1024u), umma_desc(sb + s * 256u, 128u, sbo), idesc,
                   s > 0 ? 1u : 0u);
        umma_commit(S.empty(sl));
        *S.acchdr(q) = h;
        umma_commit(S.accfull(q));
        mbar_arrive(S.accfull(q));  // publishes the head (release)
        P.add(3, tp);
        issued = true;
        ++c;
      }
      P.flush(kPfMmaImg);
      if (P.on) atomicAdd(&g_um_prof[kPfZLatency], zlat);
      // the MMAs issued last have completed before the tensor memory is freed
      // (bounded, not cut short by another role's error)
      if (issued) mbar_wait_sleep(S.empty((c - 1) % kSlots), ((c - 1) / kSlots) & 1, a.err);
    }
    __syncwarp();
  } else if (warp < kEpiWarp0) {
    // ---------------- Z rows: positions kZPos h .. kZPos h + kZPos - 1 of every chunk
    const uint32_t h = warp - 2;
    ProfClock P(pf && h == 0);
    const uint32_t cb0 = a.cranges[blockIdx.x], ncb = a.cranges[blockIdx.x + 1] - cb0;
    // L2: indices are read once (evict first); Z rows are read by many chunks (evict last)
    const uint64_t pol_idx = policy_evict_first(), pol_z = policy_evict_last();
    // lane 0: this warp's Z-row indices of chunk cc into its queue entry cc % kQ (nothing past the end)
    auto prefetch = [&](uint32_t cc) {
      if (lane == 0 && cc < ncb) {
        const uint32_t e = cc % kQ;
        mbar_expect_tx(S.idxbar(h, e), kZPos * 4);
        bulk_g2s_hint(smem_u32(S.idxq(h, e)), a.zidx + (uint64_t)(cb0 + cc) * kUmKc + kZPos * h, kZPos * 4,
                      S.idxbar(h, e), pol_idx);
      }
    };
    for (uint32_t i = 0; i < kLidx; ++i) prefetch(i);
    // Consecutive rows (a contiguous tile: X rows of a V tile or of a dense
    // leaf): two tensor copies, lane 0, of kZPos rows x 64 FP16 (first / second
    // parts); the copy engine writes them with the 128-byte swizzle.  Other
    // rows: lanes 0-15 move the 16 pieces of 16 bytes of position 2 r, lanes
    // 16-31 those of position 2 r + 1 (positions past a chunk's K copy Z row
    // 0, a finite row that meets zero B values).  Piece i = lane % 16 (FP16
    // values 8 i .. 8 i + 7 of the row) goes to the first-part (i < 8) or
    // second-part half of the A operand, 16-byte column (i % 8) ^ (p % 8) of
    // row p: the same 128-byte swizzle.
    const uint32_t zpiece = lane & 15u, odd = lane >> 4;
    const unsigned char* zsrc = reinterpret_cast<const unsigned char*>(a.z) + 16u * zpiece;
    uint32_t c = 0, tma_recent = 0;  // bit i: chunk c - 1 - i came by tensor copies
    for (; c < ncb; ++c) {
      const uint32_t sl = c % kSlots, e = c % kQ;
      long long tp = P.now();
      if (!__all_sync(0xffffffffu, wait_bar(S.idxbar(h, e), (c / kQ) & 1, a.err))) break;
      P.add(0, tp);
      tp = P.now();
      if (c >= kSlots && !__all_sync(0xffffffffu, wait_bar(S.empty(sl), ((c / kSlots) - 1) & 1, a.err))) break;
      P.add(1, tp);
      tp = P.now();
      // index of position 2 r + odd (of this warp's positions) in zi[r]
      uint32_t zi[kZPos / 2];
      const uint4* q4 = reinterpret_cast<const uint4*>(S.idxq(h, e));
      const uint32_t z0 = q4[0].x;
      bool seq = true;
#pragma unroll
      for (uint32_t v = 0; v < kZPos / 4; ++v) {
        const uint4 w = q4[v];
        zi[2 * v] = odd ? w.y : w.x;
        zi[2 * v + 1] = odd ? w.w : w.z;
        seq &= zi[2 * v] == z0 + 4 * v + odd && zi[2 * v + 1] == z0 + 4 * v + 2 + odd;
      }
      seq = __all_sync(0xffffffffu, seq);
      const uint32_t dst0 = smem_u32(S.areg(sl)) + kZPos * h * 128u;
      if (seq) {
        if (lane == 0) {
          mbar_expect_tx(S.fz(sl), kZPos * kUmZRowBytes);
          tma_load_2d_hint(dst0, &a.zmap, 0, (int32_t)z0, S.fz(sl), pol_z);
          tma_load_2d_hint(dst0 + kAHalf, &a.zmap, 64, (int32_t)z0, S.fz(sl), pol_z);
        }
      } else {
        if (lane == 0) mbar_arrive(S.fz(sl));
        const uint32_t dz = dst0 + (zpiece >> 3) * kAHalf;
#pragma unroll
        for (uint32_t r = 0; r < kZPos / 2; ++r) {
          const uint32_t p = 2 * r + odd;  // (kZPos h + p) % 8 = p % 8
          cp_async16_hint(dz + p * 128u + (((zpiece & 7u) ^ (p & 7u)) << 4), zsrc + (uint64_t)zi[r] * kZRowPitch,
                          pol_z);
        }
      }
      cp_async_mbar_arrive(S.fz(sl));
      tma_recent = (tma_recent << 1) | (seq ? 1u : 0u);
      P.add(2, tp);
      // the queue entry of chunk c + kLidx last held chunk c + kLidx - kQ < c,
      // whose indices every lane of this warp has read
      __syncwarp();
      prefetch(c + kLidx);
    }
    cp_async_commit();
    cp_async_wait<0>();  // this lane's Z copies have landed
    if (lane == 0) {
      // tensor copies of the last kSlots chunks have landed (older chunks were
      // consumed, hence landed; the wait gives up after its limit if the other
      // Z warp never arrived, long after the copy itself)
      for (uint32_t i = 0; i < kSlots && i < c; ++i)
        if ((tma_recent >> i) & 1u) mbar_wait_sleep(S.fz((c - 1 - i) % kSlots), ((c - 1 - i) / kSlots) & 1, a.err);
      // index copies issued for chunks that were not taken (an early stop)
      const uint32_t ie = min(ncb, c + kLidx);
      for (uint32_t i = c; i < ie; ++i) mbar_wait_sleep(S.idxbar(h, i % kQ), (i / kQ) & 1, a.err);
      P.flush(kPfZIdx);
    }
    __syncwarp();
  } else {
    // ---------------- epilogue
    const uint32_t q = warp & 3;                  // tensor-memory lane quadrant of this warp
    const uint32_t qr = (warp - kEpiWarp0) >> 2;  // output rows 32 qr .. 32 qr + 31 of the tile
    const uint32_t et = (threadIdx.x - 32 * kEpiWarp0) & 127;  // 0 .. 127 within the quarter's warps
    const uint32_t j = 32 * (q & 1) + lane;       // right-hand side of this lane's row
    const bool active = j < a.pg;                 // per lane: guards only the staging writes
    const bool qactive = 32 * (q & 1) < a.pg;     // warp-uniform: the quadrant holds rows
    const bool second = q >= 2;                   // rows 64 .. 127: the second parts
    float acc[32];
#pragma unroll
    for (int c = 0; c < 32; ++c) acc[c] = 0.f;
    float* Sg = S.staging(qr);
    // the quarter's four warps meet on an mbarrier with bounded waits (no
    // warp can be left waiting after another gave up on a failed wait)
    uint32_t quses = 0;
    auto qsync = [&]() -> bool {
      __syncwarp();
      if (lane == 0) mbar_arrive(S.quarter(qr));
      const bool ok = __all_sync(0xffffffffu, wait_bar(S.quarter(qr), quses & 1, a.err));
      ++quses;
      return ok;
    };
    ProfClock P(pf && warp == kEpiWarp0);
    uint32_t ai = 0;
    while (true) {
      const uint32_t qa = ai % kAcc, ka = ai / kAcc;
      long long tp = P.now();
      if (!wait_bar(S.accfull(qa), ka & 1, a.err)) break;
      P.add(0, tp);
      tp = P.now();
      const UmHead h = *S.acchdr(qa);
      if (h.flags & kUmStop) break;
      tc_fence_after();
      const bool first = h.flags & kUmFirst;
      const float sc = h.scale;
      // tcgen05.ld / wait::ld are warp-collective: warp-uniform conditions only.
      // Output row r of the tile: D column r (first parts of B) + column n16 + r
      // (second parts).  Rows r >= n8 read other columns (or columns past the
      // MMA's N); they are never written out.
      if (qactive && 32 * qr < h.n8) {
        const uint32_t t0 = tmem + ((32 * q) << 16) + qa * kAccCols + 32 * qr;
        const uint32_t n16 = ((uint32_t)h.n8 + 15u) & ~15u;
        float v[32];
        tmem_ld32(t0, v);
        tmem_wait_ld();
#pragma unroll
        for (int i = 0; i < 32; ++i) acc[i] = first ? v[i] * sc : fmaf(v[i], sc, acc[i]);
        tmem_ld32(t0 + n16, v);
        tmem_wait_ld();
#pragma unroll
        for (int i = 0; i < 32; ++i) acc[i] = fmaf(v[i], sc, acc[i]);
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(S.accempty(qa));
      ++ai;
      P.add(1, tp);
      if (!(h.flags & kUmLast) || 32 * qr >= h.nout) continue;
      tp = P.now();
      // ---- end of the tile: first-part rows, then second-part rows added, through the staging tile
      if (!qsync()) break;  // the staging tile is free
      if (active && !second) {
#pragma unroll
        for (int c = 0; c < 32; ++c) Sg[stg(j, c)] = acc[c];
      }
      if (!qsync()) break;
      if (active && second) {
#pragma unroll
        for (int c = 0; c < 32; ++c) Sg[stg(j, c)] += acc[c];
      }
      if (!qsync()) break;
      const uint32_t nh = min(32u, (uint32_t)h.nout - 32 * qr);
      const uint32_t row0 = h.out + 32 * qr;
      if (a.mode == 1) {
        // every Y element gets exactly one add (its row belongs to this tile
        // only): a fire-and-forget reduction keeps the warp from waiting on
        // the read of Y and gives the same rounding as y + v
        for (uint32_t e = et; e < a.pg * 32; e += 128) {
          const uint32_t jj = e >> 5, c = e & 31;
          if (c < nh)
            red_add_f64(a.y + (uint64_t)(row0 + c) + (uint64_t)jj * a.ldy,
                        a.d * S.ys()[jj] * (double)Sg[stg(jj, c)]);
        }
      } else if (h.flags & kUmRed) {
        for (uint32_t e = et; e < a.pg * 32; e += 128) {
          const uint32_t jj = e % a.pg, c = e / a.pg;
          if (c < nh) atomicAdd(a.tacc + (uint64_t)(h.tacc + 32 * qr + c) * 64 + jj, Sg[stg(jj, c)]);
        }
      } else {
        for (uint32_t e = et; e < a.pg * 32; e += 128) {
          const uint32_t jj = e % a.pg, c = e / a.pg;
          if (c < nh) {
            __half h1, h2;
            split_h16(Sg[stg(jj, c)], h1, h2);
            __half* zp = reinterpret_cast<__half*>(a.z) + (a.n + row0 + c) * (kUmZPitch / 2);
            zp[jj] = h1;
            zp[64 + jj] = h2;
          }
        }
      }
      P.add(2, tp);
    }
    P.flush(kPfEpiAccfull);
  }

  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem, kTmemCols);
  }
}

// max |X_j| over the rows, j < pg (FP32 bits, atomicMax; the words start at 0)
__global__ void __launch_bounds__(256) um_xmax_kernel(const double* __restrict__ X, uint64_t ldX, uint64_t n,
                                                      uint32_t pg, uint32_t* __restrict__ xmax) {
  __shared__ float wm[8][64];
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint32_t j = 0; j < pg; ++j) {
    float m = 0.f;
    for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += stride)
      m = fmaxf(m, (float)fabs(X[r + (uint64_t)j * ldX]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (lane == 0) wm[warp][j] = m;
  }
  __syncthreads();
  if (threadIdx.x < pg) {
    float m = 0.f;
    for (uint32_t w = 0; w < 8; ++w) m = fmaxf(m, wm[w][threadIdx.x]);
    atomicMax(xmax + threadIdx.x, __float_as_uint(m));
  }
}

// X (FP64, column-major, ld ldX), columns 0 .. pg-1 -> Z rows 0 .. n-1: X_j
// scaled by a power of two (its largest |value| into [2^13, 2^14)) and split
// into two FP16 parts; slots >= pg are zero.
__global__ void __launch_bounds__(256) um_prep_kernel(const double* __restrict__ X, uint64_t ldX, uint64_t n,
                                                      uint32_t pg, const uint32_t* __restrict__ xmax,
                                                      uint16_t* __restrict__ z) {
  __shared__ double tile[64][33];
  __shared__ double sx[64];
  if (threadIdx.x < 64) {
    const float m = __uint_as_float(xmax[threadIdx.x]);
    sx[threadIdx.x] = ldexp(1.0, -scale_exp((double)m));
  }
  __syncthreads();
  const uint64_t nblk = (n + 31) / 32;
  for (uint64_t b = blockIdx.x; b < nblk; b += gridDim.x) {
    const uint64_t r0 = b * 32;
    for (uint32_t e = threadIdx.x; e < 32u * 64u; e += blockDim.x) {
      const uint32_t row = e & 31, col = e >> 5;
      double v = 0.0;
      if (col < pg && r0 + row < n) v = X[(r0 + row) + (uint64_t)col * ldX] * sx[col];
      tile[col][row] = v;
    }
    __syncthreads();
    for (uint32_t e = threadIdx.x; e < 32u * 64u; e += blockDim.x) {
      const uint32_t col = e & 63, row = e >> 6;
      if (r0 + row < n) {
        const double v = tile[col][row];
        const __half h1 = __double2half(v);
        const __half h2 = __double2half(v - (double)__half2float(h1));
        __half* zp = reinterpret_cast<__half*>(z) + (r0 + row) * (kUmZPitch / 2);
        zp[col] = h1;
        zp[64 + col] = h2;
      }
    }
    __syncthreads();
  }
}

// split V tiles: FP32 accumulation rows -> Z rows (FP16 pairs); the rows are zeroed again
__global__ void __launch_bounds__(256) um_tconv_kernel(const UmRange* __restrict__ ranges, uint32_t nranges,
                                                       float* __restrict__ tacc, uint16_t* __restrict__ z,
                                                       uint64_t n) {
  for (uint32_t r = blockIdx.x; r < nranges; r += gridDim.x) {
    const UmRange R = ranges[r];
    for (uint32_t e = threadIdx.x; e < R.count * 64u; e += blockDim.x) {
      const uint32_t c = e >> 6, jj = e & 63;
      float* tp = tacc + (uint64_t)(R.off + c) * 64 + jj;
      const float v = *tp;
      *tp = 0.f;
      __half h1, h2;
      split_h16(v, h1, h2);
      __half* zp = reinterpret_cast<__half*>(z) + (n + R.row + c) * (kUmZPitch / 2);
      zp[jj] = h1;
      zp[64 + jj] = h2;
    }
  }
}

// T-row scales: one warp per low-rank leaf; s_t = 2^-e with ||V_t||_1 = f 2^e, f in [0.5, 1)
__global__ void __launch_bounds__(256) um_tscale_kernel(const UmTJob* __restrict__ jobs, uint32_t njobs,
                                                        const double* __restrict__ a64,
                                                        float* __restrict__ tscale) {
  const uint32_t lane = threadIdx.x & 31;
  const uint64_t w0 = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t jb = w0; jb < njobs; jb += nw) {
    const UmTJob J = jobs[jb];
    for (uint32_t col = 0; col < J.rank; ++col) {
      const double* v = a64 + J.vbase + (uint64_t)col * J.n2;
      double s = 0.0;
      for (uint32_t i = lane; i < J.n2; i += 32) s += fabs(v[i]);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (lane == 0) {
        int ex = 0;
        if (s > 0.0) frexp(s, &ex);
        ex = max(-100, min(100, ex));
        tscale[J.trow + col] = ldexpf(1.f, -ex);
      }
    }
  }
}

// One CTA per tile: chunk heads, Z-row indices and the FP16 image pairs from
// the FP64 arena (V values times the T-row scale, U values divided by it).
__global__ void __launch_bounds__(256) um_build_kernel(const UmBuild* __restrict__ tiles,
                                                       const UmEntry* __restrict__ entries,
                                                       const double* __restrict__ a64,
                                                       const float* __restrict__ tscale, uint64_t n,
                                                       unsigned char* __restrict__ stream,
                                                       uint32_t* __restrict__ zidx) {
  const UmBuild T = tiles[blockIdx.x];
  __shared__ int32_t ent[kUmN];
  __shared__ double red[8];
  static_assert(kUmKc <= kUmN, "per-position entry table");
  const bool byN = T.flags & kUmByN, contig = T.flags & kUmContig;
  const uint32_t tid = threadIdx.x;
  if (byN) {
    for (uint32_t i = tid; i < kUmN; i += blockDim.x) ent[i] = -1;
    __syncthreads();
    for (uint32_t e = 0; e < T.ne; ++e) {
      const UmEntry E = entries[T.e0 + e];
      for (uint32_t i = tid; i < E.nn; i += blockDim.x) ent[E.n0 + i] = (int32_t)e;
    }
    __syncthreads();
  }
  uint64_t off = T.src;
  for (uint32_t c = 0; c < T.nchunks; ++c) {
    const uint32_t kb = c * kUmKc, kval = min(kUmKc, T.K - kb), kc = (kval + 15u) & ~15u;
    unsigned char* img = stream + off;
    unsigned char* B = img + T.hdr;
    if (!byN) {
      __syncthreads();
      if (tid < kUmKc) {
        int32_t found = -1;
        if (tid < kval) {
          const uint32_t K = kb + tid;
          uint32_t lo = 0, hi = T.ne;  // last entry with k0 <= K
          while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) / 2;
            if (entries[T.e0 + mid].k0 <= K) lo = mid;
            else hi = mid;
          }
          const UmEntry E = entries[T.e0 + lo];
          if (K >= E.k0 && K < E.k0 + E.kn) found = (int32_t)lo;
        }
        ent[tid] = found;
      }
      __syncthreads();
    }
    // values of the chunk (recomputed in the second pass) and their largest magnitude
    const uint32_t cnt = (uint32_t)T.n8 * kc;
    auto value = [&](uint32_t e, uint32_t& nn, uint32_t& kk) -> double {
      if (byN) {
        kk = e % kc;
        nn = e / kc;
      } else {
        nn = e % T.n8;
        kk = e / T.n8;
      }
      double v = 0.0;
      if (nn < T.nout && kk < kval) {
        const int32_t ei = byN ? ent[nn] : ent[kk];
        if (ei >= 0) {
          const UmEntry E = entries[T.e0 + ei];
          const uint32_t K = kb + kk;
          if (K >= E.k0 && K < E.k0 + E.kn && nn >= E.n0 && nn < E.n0 + E.nn) {
            v = a64[E.base + (uint64_t)(K - E.k0) * E.sk + (uint64_t)(nn - E.n0) * E.sn];
            if (byN) v *= (double)tscale[T.out + nn];                               // V column of T row out + nn
            else if (E.zrow0 >= n) v /= (double)tscale[E.zrow0 - n + (K - E.k0)];  // U column of a T row
          }
        }
      }
      return v;
    };
    double m = 0.0;
    for (uint32_t e = tid; e < cnt; e += blockDim.x) {
      uint32_t nn, kk;
      m = fmax(m, fabs(value(e, nn, kk)));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((tid & 31) == 0) red[tid >> 5] = m;
    __syncthreads();
    double mx = 0.0;
    for (uint32_t w = 0; w < blockDim.x / 32; ++w) mx = fmax(mx, red[w]);
    const int se = max(-120, min(120, scale_exp(mx)));
    const double inv = ldexp(1.0, -se);
    if (tid == 0) {
      UmHead h{};
      h.zsrc = contig ? T.zrow0 + kb : 0u;
      h.kc = (uint16_t)kc;
      h.kvalid = (uint16_t)kval;
      h.n8 = T.n8;
      h.nout = (uint16_t)T.nout;
      h.out = T.out;
      h.flags = (c == 0 ? kUmFirst : 0u) | (c + 1 == T.nchunks ? kUmLast : 0u) | (T.flags & (kUmContig | kUmRed));
      h.scale = ldexpf(1.f, se);
      h.tacc = T.tacc;
      h.tile = blockIdx.x;
      *reinterpret_cast<UmHead*>(B - 32) = h;
    }
    if (tid < kUmKc) {
      // Z rows of the chunk's K positions.  Past kval the rows meet zero B
      // values: row 0 in indexed tiles; in contiguous tiles the run goes on, so
      // that every chunk's rows stay one run for the sweeps' tensor copies
      // (which read rows past the end of Z as zeros)
      uint32_t zr = 0;
      if (contig) {
        zr = T.zrow0 + kb + tid;
      } else if (tid < kval) {
        if (ent[tid] >= 0) {
          const UmEntry E = entries[T.e0 + ent[tid]];
          zr = E.zrow0 + (kb + tid - E.k0);
        }
      }
      zidx[(uint64_t)(T.cbase + c) * kUmKc + tid] = zr;
    }
    __half* B1 = reinterpret_cast<__half*>(B);
    __half* B2 = B1 + (size_t)T.n8 * kc;
    for (uint32_t e = tid; e < cnt; e += blockDim.x) {
      uint32_t nn, kk;
      const double v = value(e, nn, kk) * inv;
      const __half h1 = __double2half(v);
      const __half h2 = __double2half(v - (double)__half2float(h1));
      const uint32_t o = (nn >> 3) * (kc * 8u) + (kk >> 3) * 64u + (nn & 7u) * 8u + (kk & 7u);  // in FP16 units
      B1[o] = h1;
      B2[o] = h2;
    }
    __syncthreads();
    off += T.hdr + (uint64_t)T.n8 * kc * 4;
  }
}

// ---- optional event timing of the sweeps
struct TimingRec {
  int kind;
  cudaEvent_t e0, e1;
};
std::mutex g_tmu;
bool g_timing = false;
bool g_prof = false;
std::vector<TimingRec> g_trecs;

cudaError_t launch_sweep(const KArgs& a, int kind, uint32_t grid, cudaStream_t s) {
  TimingRec r{kind, nullptr, nullptr};
  bool timed = false;
  {
    std::lock_guard<std::mutex> lk(g_tmu);
    timed = g_timing;
  }
  if (timed) {
    cudaEventCreate(&r.e0);
    cudaEventCreate(&r.e1);
    cudaEventRecord(r.e0, s);
  }
  um_sweep_kernel<<<grid, kThreads, kSmemBytes, s>>>(a);
  cudaError_t e = cudaGetLastError();
  if (timed) {
    cudaEventRecord(r.e1, s);
    std::lock_guard<std::mutex> lk(g_tmu);
    g_trecs.push_back(r);
  }
  return e;
}

// Z rows (n + t_rows + 1 rows of 128 FP16, kUmZPitch bytes apart) as a 2D
// tensor for the sweeps' tensor copies: boxes of 64 values x kZPos rows, 128-byte swizzle
cudaError_t encode_zmap(CUtensorMap* m, const uint16_t* z, uint64_t zrows) {
  static const PFN_cuTensorMapEncodeTiled_v12000 encode = []() -> PFN_cuTensorMapEncodeTiled_v12000 {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      return nullptr;
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
  }();
  if (!encode) return cudaErrorNotSupported;
  const cuuint64_t dims[2] = {kUmZRowBytes / 2, zrows};
  const cuuint64_t strides[1] = {kUmZPitch};
  const cuuint32_t box[2] = {64, kZPos};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = encode(m, CU_TENSOR_MAP_DATA_TYPE_UINT16, 2, const_cast<uint16_t*>(z), dims, strides, box, estr,
                            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

cudaError_t run_um(const UmPlan& pl, double d, uint32_t r0, uint32_t pg, const double* X, uint64_t ldX, double* Y,
                   uint64_t ldY, cudaStream_t s) {
  const uint64_t nblk = (pl.n + 31) / 32;
  const unsigned grid = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(nblk, (uint64_t)pl.grid * 8));
  cudaError_t e = cudaMemsetAsync(pl.xmax, 0, 64 * sizeof(uint32_t), s);
  if (e != cudaSuccess) return e;
  const double* Xp = X + (uint64_t)r0 * ldX;
  const unsigned gx = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((pl.n + 255) / 256, (uint64_t)pl.grid * 4));
  um_xmax_kernel<<<gx, 256, 0, s>>>(Xp, ldX, pl.n, pg, pl.xmax);
  um_prep_kernel<<<grid, 256, 0, s>>>(Xp, ldX, pl.n, pg, pl.xmax, pl.z);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  uint64_t launches = 2;
  KArgs a{};
  if ((e = encode_zmap(&a.zmap, pl.z, pl.n + pl.t_rows + 1)) != cudaSuccess) return e;
  a.z = pl.z;
  a.tacc = pl.tacc;
  a.xmax = pl.xmax;
  a.err = pl.err;
  a.pg = pg;
  a.n = pl.n;
  {
    std::lock_guard<std::mutex> lk(g_tmu);
    a.prof = g_prof ? 1u : 0u;
  }
  if (pl.nvtiles) {
    a.tiles = pl.vtiles;
    a.ranges = pl.vranges;
    a.cranges = pl.vcranges;
    a.zidx = pl.vzidx;
    a.stream = pl.vstream;
    a.mode = 0;
    if ((e = launch_sweep(a, 0, pl.grid, s)) != cudaSuccess) return e;
    ++launches;
  }
  if (pl.nzero) {
    um_tconv_kernel<<<std::min<uint32_t>(pl.nzero, pl.grid * 4), 256, 0, s>>>(pl.zero, pl.nzero, pl.tacc, pl.z,
                                                                              pl.n);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    ++launches;
  }
  if (pl.nrtiles) {
    a.tiles = pl.rtiles;
    a.ranges = pl.rranges;
    a.cranges = pl.rcranges;
    a.zidx = pl.rzidx;
    a.stream = pl.rstream;
    a.y = Y + (uint64_t)r0 * ldY;
    a.ldy = ldY;
    a.d = d;
    a.mode = 1;
    if ((e = launch_sweep(a, 1, pl.grid, s)) != cudaSuccess) return e;
    ++launches;
  }
  count_product_launches(launches);
  return cudaSuccess;
}

uint32_t round8(uint32_t x) { return (x + 7u) & ~7u; }
uint32_t round16(uint32_t x) { return (x + 15u) & ~15u; }

}  // namespace

cudaError_t um_init_attributes() {
  return cudaFuncSetAttribute(um_sweep_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemBytes);
}

cudaError_t launch_um_tscale(const UmTJob* jobs, uint32_t njobs, const double* arena64, float* tscale,
                             cudaStream_t s) {
  if (njobs == 0) return cudaSuccess;
  const uint32_t blocks = std::min<uint32_t>((njobs + 7) / 8, 65535u);
  um_tscale_kernel<<<blocks, 256, 0, s>>>(jobs, njobs, arena64, tscale);
  count_product_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_um_build(const UmBuild* tiles, uint32_t ntiles, const UmEntry* entries, const double* arena64,
                            const float* tscale, uint64_t n, unsigned char* stream, uint32_t* zidx,
                            cudaStream_t s) {
  if (ntiles == 0) return cudaSuccess;
  um_build_kernel<<<ntiles, 256, 0, s>>>(tiles, entries, arena64, tscale, n, stream, zidx);
  count_product_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_matvec_um(const UmPlan& pl, double d, uint32_t p, const double* X, uint64_t ldX, double* Y,
                             uint64_t ldY, cudaStream_t s) {
  for (uint32_t r0 = 0; r0 < p; r0 += kUmSlots) {
    const uint32_t pg = std::min(kUmSlots, p - r0);
    const cudaError_t e = run_um(pl, d, r0, pg, X, ldX, Y, ldY, s);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

void um_timing_enable(bool on) {
  std::lock_guard<std::mutex> lk(g_tmu);
  g_timing = on;
}

void um_timing_read(double* ms2, uint64_t* count2, bool reset) {
  std::lock_guard<std::mutex> lk(g_tmu);
  ms2[0] = ms2[1] = 0.0;
  count2[0] = count2[1] = 0;
  for (const TimingRec& r : g_trecs) {
    float ms = 0.f;
    if (cudaEventSynchronize(r.e1) == cudaSuccess && cudaEventElapsedTime(&ms, r.e0, r.e1) == cudaSuccess) {
      ms2[r.kind] += ms;
      count2[r.kind] += 1;
    }
  }
  if (reset) {
    for (const TimingRec& r : g_trecs) {
      cudaEventDestroy(r.e0);
      cudaEventDestroy(r.e1);
    }
    g_trecs.clear();
  }
}

// ---------------------------------------------------------------------------
// Host layout
void build_um_layout(const std::vector<PlanLeaf>& leaves, uint64_t n, uint32_t grid, UmLayout& L, uint32_t kpiece) {
  L = UmLayout();
  kpiece = std::max<uint32_t>(kUmKc, kpiece / kUmKc * kUmKc);
  std::vector<uint32_t> trow(leaves.size(), 0);

  // ---- V sweep: low-rank leaves by column cluster (b2 ascending, larger clusters first)
  struct ColKey {
    uint32_t b2, n2;
    bool operator<(const ColKey& o) const { return b2 != o.b2 ? b2 < o.b2 : n2 > o.n2; }
  };
  std::map<ColKey, std::vector<size_t>> cols;
  for (size_t l = 0; l < leaves.size(); ++l)
    if (leaves[l].rank > 0) cols[{leaves[l].b2, leaves[l].n2}].push_back(l);
  uint32_t t_rows = 0;
  for (const auto& kv : cols) {
    const uint32_t b2 = kv.first.b2, n2 = kv.first.n2;
    const std::vector<size_t>& ls = kv.second;
    std::vector<uint32_t> coloff(ls.size());
    uint32_t nc = 0;
    for (size_t i = 0; i < ls.size(); ++i) {
      coloff[i] = nc;
      trow[ls[i]] = t_rows + nc;
      nc += (uint32_t)leaves[ls[i]].rank;
    }
    const uint32_t tc = t_rows;
    t_rows += nc;
    const uint32_t npieces = (n2 + kpiece - 1) / kpiece;
    for (uint32_t g0 = 0; g0 < nc; g0 += kUmN) {
      const uint32_t ng = std::min(kUmN, nc - g0);
      const bool red = npieces > 1;
      if (red) {
        L.zero.push_back({tc + g0, ng, L.tacc_rows, 0u});
        L.tacc_rows += ng;
      }
      for (uint32_t pc = 0; pc < npieces; ++pc) {
        const uint32_t k0 = pc * kpiece, K = std::min(kpiece, n2 - k0);
        UmBuild B{};
        B.e0 = (uint32_t)L.entries.size();
        B.K = K;
        B.nout = ng;
        B.out = tc + g0;
        B.zrow0 = b2 + k0;
        B.flags = kUmContig | kUmByN | (red ? kUmRed : 0u);
        B.n8 = (uint16_t)round8(ng);
        B.hdr = 32;
        B.tacc = red ? L.zero.back().off : 0u;
        B.nchunks = (K + kUmKc - 1) / kUmKc;
        for (size_t i = 0; i < ls.size(); ++i) {
          const PlanLeaf& q = leaves[ls[i]];
          const uint32_t lo = std::max(coloff[i], g0), hi = std::min(coloff[i] + (uint32_t)q.rank, g0 + ng);
          if (lo >= hi) continue;
          UmEntry e{};
          e.base = q.off + (uint64_t)q.rank * q.n1 + (uint64_t)(lo - coloff[i]) * q.n2 + k0;
          e.k0 = 0;
          e.kn = K;
          e.n0 = lo - g0;
          e.nn = hi - lo;
          e.sk = 1;
          e.sn = q.n2;
          L.entries.push_back(e);
        }
        B.ne = (uint32_t)L.entries.size() - B.e0;
        L.vbuild.push_back(B);
      }
    }
  }
  L.t_rows = t_rows;
  for (size_t l = 0; l < leaves.size(); ++l)
    if (leaves[l].rank > 0) {
      const PlanLeaf& q = leaves[l];
      L.tjobs.push_back({q.off + (uint64_t)q.rank * q.n1, q.n2, (uint32_t)q.rank, trow[l], 0u});
    }

  // ---- rows sweep: finest row blocks (<= kUmN rows) of the row clusters
  std::vector<uint32_t> bd{0u, (uint32_t)n};
  for (const PlanLeaf& q : leaves)
    if (q.rank != 0) {
      bd.push_back(q.b1);
      bd.push_back(q.b1 + q.n1);
    }
  std::sort(bd.begin(), bd.end());
  bd.erase(std::unique(bd.begin(), bd.end()), bd.end());
  std::vector<uint32_t> bs;  // block starts, then n
  for (size_t i = 0; i + 1 < bd.size(); ++i) {
    const uint32_t a0 = bd[i], len = bd[i + 1] - bd[i];
    const uint32_t np = (len + kUmN - 1) / kUmN;
    for (uint32_t p = 0; p < np; ++p) bs.push_back(a0 + (uint32_t)((uint64_t)len * p / np));
  }
  bs.push_back((uint32_t)n);
  const size_t nb = bs.size() - 1;
  std::vector<std::vector<UmEntry>> be(nb);
  for (size_t l = 0; l < leaves.size(); ++l) {
    const PlanLeaf& q = leaves[l];
    if (q.rank == 0) continue;
    size_t i = (size_t)(std::lower_bound(bs.begin(), bs.end(), q.b1) - bs.begin());
    for (; i < nb && bs[i] < q.b1 + q.n1; ++i) {
      const uint32_t r0 = bs[i], nr = bs[i + 1] - bs[i];
      UmEntry e{};
      e.base = q.off + (r0 - q.b1);
      e.kn = q.rank > 0 ? (uint32_t)q.rank : q.n2;
      e.n0 = 0;
      e.nn = nr;
      e.sk = q.n1;
      e.sn = 1;
      e.zrow0 = q.rank > 0 ? (uint32_t)n + trow[l] : q.b2;
      be[i].push_back(e);
    }
  }
  for (size_t i = 0; i < nb; ++i) {
    std::vector<UmEntry>& es = be[i];
    std::sort(es.begin(), es.end(), [](const UmEntry& x, const UmEntry& y) { return x.zrow0 < y.zrow0; });
    UmBuild B{};
    B.e0 = (uint32_t)L.entries.size();
    uint32_t K = 0;
    for (UmEntry& e : es) {
      e.k0 = K;
      K += e.kn;
      L.entries.push_back(e);
    }
    B.ne = (uint32_t)es.size();
    B.K = K;
    B.nout = bs[i + 1] - bs[i];
    B.out = bs[i];
    B.flags = 0;
    B.n8 = (uint16_t)round8(B.nout);
    B.hdr = 32;
    B.nchunks = (K + kUmKc - 1) / kUmKc;
    if (K > 0) L.rbuild.push_back(B);
    std::vector<UmEntry>().swap(es);
  }

  // ---- stream offsets and the kernel's tiles
  auto chunk_bytes = [](const UmBuild& B) {
    const uint32_t klast = round16(B.K - (B.nchunks - 1) * kUmKc);
    return (uint64_t)(B.nchunks - 1) * (B.hdr + (uint64_t)B.n8 * kUmKc * 4) + B.hdr + (uint64_t)B.n8 * klast * 4;
  };
  auto place = [&](std::vector<UmBuild>& bl, std::vector<UmTile>& tl, uint64_t& bytes, uint64_t& chunks) {
    bytes = 0;
    chunks = 0;
    tl.clear();
    for (UmBuild& B : bl) {
      B.src = bytes;
      B.cbase = (uint32_t)chunks;
      chunks += B.nchunks;
      bytes += chunk_bytes(B);
      UmTile T{};
      T.src = B.src;
      T.nchunks = B.nchunks;
      T.n8 = B.n8;
      T.hdr = B.hdr;
      T.klast = (uint16_t)round16(B.K - (B.nchunks - 1) * kUmKc);
      T.kvlast = (uint16_t)(B.K - (B.nchunks - 1) * kUmKc);
      T.zrow0 = B.zrow0;
      T.flags = B.flags & kUmContig;
      tl.push_back(T);
    }
  };
  place(L.vbuild, L.vtiles, L.vbytes, L.vchunks);
  place(L.rbuild, L.rtiles, L.rbytes, L.rchunks);
  // contiguous tile ranges per CTA, balanced by stream bytes
  auto ranges = [&](const std::vector<UmBuild>& bl, std::vector<uint32_t>& first) {
    std::vector<uint64_t> bytes(bl.size());
    // stream bytes plus the chunks' Z rows (mostly L2 hits: weighted by half)
    for (size_t t = 0; t < bl.size(); ++t) bytes[t] = chunk_bytes(bl[t]) + (uint64_t)bl[t].nchunks * kUmKc * kUmZRowBytes / 2;
    balance_ranges(bytes, std::max<uint32_t>(grid, 1), first);
  };
  ranges(L.vbuild, L.vranges);
  ranges(L.rbuild, L.rranges);
  // the first chunk of every CTA's range
  auto cranges = [&](const std::vector<UmBuild>& bl, const std::vector<uint32_t>& first, uint64_t chunks,
                     std::vector<uint32_t>& out) {
    out.resize(first.size());
    for (size_t i = 0; i < first.size(); ++i) out[i] = first[i] < bl.size() ? bl[first[i]].cbase : (uint32_t)chunks;
  };
  cranges(L.vbuild, L.vranges, L.vchunks, L.vcranges);
  cranges(L.rbuild, L.rranges, L.rchunks, L.rcranges);
  L.stream_bytes = L.vbytes + L.rbytes;
  for (const PlanLeaf& q : leaves)
    L.payload_bytes += 4ull * (q.rank >= 0 ? (uint64_t)q.rank * (q.n1 + q.n2) : (uint64_t)q.n1 * q.n2);
}

// Host evaluation of a layout's decomposition (test hook): Y += A X, X and Y
// column-major n x p, from the tiles' entries and Z rows exactly as the sweeps
// use them (T rows from the V tiles, then Y rows from the rows tiles), in FP64.
void um_host_product(const UmLayout& L, const double* arena, uint64_t n, uint32_t p, const double* X, double* Y) {
  std::vector<double> T((size_t)L.t_rows * p, 0.0);
  auto zval = [&](uint32_t zr, uint32_t j) {
    return zr < n ? X[zr + (uint64_t)j * n] : T[(size_t)(zr - n) * p + j];
  };
  for (const UmBuild& B : L.vbuild)
    for (uint32_t e = 0; e < B.ne; ++e) {
      const UmEntry& E = L.entries[B.e0 + e];
      for (uint32_t nn = E.n0; nn < E.n0 + E.nn; ++nn)
        for (uint32_t k = E.k0; k < E.k0 + E.kn && k < B.K; ++k) {
          const double v = arena[E.base + (uint64_t)(k - E.k0) * E.sk + (uint64_t)(nn - E.n0) * E.sn];
          for (uint32_t j = 0; j < p; ++j) T[(size_t)(B.out + nn) * p + j] += v * zval(B.zrow0 + k, j);
        }
    }
  for (const UmBuild& B : L.rbuild)
    for (uint32_t e = 0; e < B.ne; ++e) {
      const UmEntry& E = L.entries[B.e0 + e];
      for (uint32_t k = E.k0; k < E.k0 + E.kn; ++k) {
        const uint32_t zr = E.zrow0 + (k - E.k0);
        for (uint32_t nn = E.n0; nn < E.n0 + E.nn && nn < B.nout; ++nn) {
          const double v = arena[E.base + (uint64_t)(k - E.k0) * E.sk + (uint64_t)(nn - E.n0) * E.sn];
          for (uint32_t j = 0; j < p; ++j) Y[(B.out + nn) + (uint64_t)j * n] += v * zval(zr, j);
        }
      }
    }
}

}  // namespace ahx

// Test hook (not part of the drop-in interface): the product of a leaf set
// through the tcgen05 layout's decomposition, evaluated on the host.  leaves:
// 5 words per leaf (b1, n1, b2, n2, rank as int32, -1 dense), offs: element
// offset of each leaf in arena (FP64, mblock layout).  Also reports the layout's
// tile counts and stream bytes in info[4] = {V tiles, rows tiles, T rows,
// stream bytes / 16}.
extern "C" int ahx_um_host_product(uint64_t n, uint32_t nleaves, const uint32_t* leaves, const uint64_t* offs,
                                   const double* arena, uint32_t p, const double* X, double* Y, uint64_t* info,
                                   uint32_t kpiece) {
  if (!leaves || !offs || !arena || !X || !Y) return 2;
  std::vector<ahx::PlanLeaf> pls(nleaves);
  for (uint32_t l = 0; l < nleaves; ++l) {
    const uint32_t* w = leaves + 5 * (size_t)l;
    pls[l] = ahx::PlanLeaf{w[0], w[1], w[2], w[3], (int32_t)w[4], offs[l]};
  }
  ahx::UmLayout L;
  ahx::build_um_layout(pls, n, 152, L, kpiece ? kpiece : 4096);
  ahx::um_host_product(L, arena, n, p, X, Y);
  if (info) {
    info[0] = L.vtiles.size();
    info[1] = L.rtiles.size();
    info[2] = L.t_rows;
    info[3] = L.stream_bytes / 16;
  }
  return 0;
}

// Diagnostics hooks (not part of the drop-in interface): per-role cycle
// counters of the tcgen05 sweeps, summed over CTAs and launches since the last
// reset (16 words: producer total / slot waits / index waits / chunks; A-stage
// warp fz waits / stage waits / work; MMA A waits / accumulator waits / image
// waits / issue; epilogue accumulator waits / drains / tile ends).
extern "C" int ahx_um_counters_enable(int enable) {
  std::lock_guard<std::mutex> lk(ahx::g_tmu);
  ahx::g_prof = enable != 0;
  return 0;
}

extern "C" int ahx_um_counters(uint64_t* out16, int reset) {
  if (cudaDeviceSynchronize() != cudaSuccess) return 2;
  unsigned long long v[ahx::kPfCount];
  if (cudaMemcpyFromSymbol(v, ahx::g_um_prof, sizeof(v)) != cudaSuccess) return 2;
  for (int i = 0; i < (int)ahx::kPfCount; ++i) out16[i] = v[i];
  if (reset) {
    const unsigned long long z[ahx::kPfCount] = {};
    if (cudaMemcpyToSymbol(ahx::g_um_prof, z, sizeof(z)) != cudaSuccess) return 2;
  }
  return 0;
}
