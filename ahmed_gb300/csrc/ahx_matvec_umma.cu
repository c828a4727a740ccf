// H-matrix product on the fifth-generation tensor cores (tcgen05.mma with
// tensor-memory accumulators) over FP32 leaf streams; the layout, the sweeps
// and the precision scheme are described in ahx_umma.cuh.
//
// One persistent CTA per SM, 14 warps with fixed roles:
//   warp 0      producer: walks the CTA's contiguous range of tiles (ranges
//               balanced by bytes; descriptors fetched 32 at a time) and
//               bulk-copies (cp.async.bulk) each chunk image (indices, head, B)
//               into a byte ring of kRing bytes, as far ahead as the ring and
//               its kSlots slot records allow
//   warp 1      MMA issuer (one thread) and owner of the tensor memory: per
//               chunk, 2 * kc / 8 tcgen05.mma (B as copied, which the tensor
//               core reads truncated to TF32, and its remainder image) into one
//               of four 128-column accumulators, then tcgen05.commit to the
//               ring slot, the stage and the accumulator
//   warps 2-5   stage filling: 16-byte loads of the chunk's Z values one chunk
//               ahead, split into TF32 hi/lo parts and stored as A in one of
//               kA stages (128-byte-swizzled K-major), and the remainder image
//               B - trunc(B) beside it; then the stage is released to the MMA
//               issuer
//   warps 6-13  epilogue, two warps per tensor-memory lane quadrant (columns
//               0-63 and 64-127): each thread adds its accumulator row to
//               registers (round-to-nearest FP32) per chunk; at the end of a
//               tile the hi and lo rows are summed through shared memory into
//               Y (FP64, in place) or T
// Every wait is bounded: on timeout the kernel raises the error word and all
// roles return after the copies and MMAs they started have completed.
#include <algorithm>
#include <cstdlib>
#include <map>
#include <mutex>
#include <vector>

#include "ahx_ptx.cuh"
#include "ahx_umma.cuh"

namespace ahx {
namespace {

using namespace ptx;

constexpr uint32_t kPiece = kUmN * kUmKc * 4;           // 16 KB: largest B image / A piece
constexpr uint32_t kRing = 120u << 10;                  // ring of chunk images (head + B)
constexpr uint32_t kSlots = 16;                         // chunk records of the ring
constexpr uint32_t kA = 2;                              // stages (A + the B remainder image)
constexpr uint32_t kAcc = 4;                            // tensor-memory accumulators (128 columns each)
constexpr uint32_t kSRow = 65;                          // staging row stride (floats): conflict-free
constexpr uint32_t kOffA = kRing;                       // stage i: A at kOffA + 2 i kPiece, B lo after it
constexpr uint32_t kOffStaging = kOffA + 2 * kA * kPiece;
constexpr uint32_t kStagingBytes = 64 * kSRow * 4;      // per column half
constexpr uint32_t kOffAccHdr = kOffStaging + 2 * kStagingBytes;
constexpr uint32_t kOffSlotOff = kOffAccHdr + kAcc * sizeof(UmHead);
constexpr uint32_t kOffEnd = kOffSlotOff + kSlots * 4;   // producer's end positions (u64)
constexpr uint32_t kOffBar = kOffEnd + kSlots * 8;
constexpr uint32_t kNumBars = 2 * kSlots + 2 * kA + 2 * kAcc;
constexpr uint32_t kOffTmem = kOffBar + kNumBars * 8;
constexpr uint32_t kSmemBytes = kOffTmem + 16 + 1024;   // + alignment slack of the dynamic base
constexpr uint32_t kThreads = 448;
constexpr uint32_t kEpiWarps = 8;                       // epilogue warps: each arrives on accempty
constexpr uint32_t kTmemCols = kAcc * kUmN;             // all 512 columns
constexpr uint32_t kStop = 0xffffffffu;                 // slot record of the stop marker
constexpr uint32_t kMaxEntry = kUmIdxBytes + 32 + kPiece;
static_assert(kSmemBytes <= 232448, "shared memory per CTA");
// the gather keeps one chunk unconverted: two entries (and the wrap gap) fit the ring
static_assert(3 * kMaxEntry <= kRing, "ring size");

struct KArgs {
  const UmTile* tiles;
  const uint32_t* ranges;  // per CTA: first tile (gridDim.x + 1 entries), balanced by bytes
  const unsigned char* stream;
  const float* z;       // Z rows (P floats each)
  float* tout;          // V sweep: T rows (P floats each)
  double* y;            // rows sweep: Y (column-major, ldY), first column of this pass
  uint64_t ldy;
  double d;
  uint32_t pg;          // right-hand sides of this pass
  uint32_t mode;        // 0: V sweep (T out), 1: rows sweep (Y out)
  uint32_t drain;       // chunks accumulated in tensor memory per drain (>= 1)
  int* err;
};

struct Smem {
  unsigned char* base;
  __device__ unsigned char* ring() const { return base; }
  __device__ unsigned char* astage(uint32_t i) const { return base + kOffA + 2 * i * kPiece; }
  __device__ unsigned char* lostage(uint32_t i) const { return base + kOffA + (2 * i + 1) * kPiece; }
  __device__ float* staging(uint32_t half) const {
    return reinterpret_cast<float*>(base + kOffStaging + half * kStagingBytes);
  }
  __device__ UmHead* acchdr(uint32_t a) const { return reinterpret_cast<UmHead*>(base + kOffAccHdr) + a; }
  __device__ uint32_t* slot_off() const { return reinterpret_cast<uint32_t*>(base + kOffSlotOff); }
  __device__ uint64_t* endpos() const { return reinterpret_cast<uint64_t*>(base + kOffEnd); }
  __device__ uint32_t bar(uint32_t i) const { return smem_u32(base + kOffBar + 8 * i); }
  __device__ uint32_t bfull(uint32_t i) const { return bar(i); }
  __device__ uint32_t bempty(uint32_t i) const { return bar(kSlots + i); }
  __device__ uint32_t aready(uint32_t i) const { return bar(2 * kSlots + i); }
  __device__ uint32_t aempty(uint32_t i) const { return bar(2 * kSlots + kA + i); }
  __device__ uint32_t accfull(uint32_t i) const { return bar(2 * kSlots + 2 * kA + i); }
  __device__ uint32_t accempty(uint32_t i) const { return bar(2 * kSlots + 2 * kA + kAcc + i); }
  __device__ uint32_t* tmem_slot() const { return reinterpret_cast<uint32_t*>(base + kOffTmem); }
};

// a chunk image in the ring: [indices (hdr - 32 bytes)] [UmHead] [B]
struct Entry {
  const unsigned char* img;
  uint32_t hdr;
  __device__ const UmHead* head() const { return reinterpret_cast<const UmHead*>(img + hdr - 32); }
  __device__ const uint32_t* idx() const { return reinterpret_cast<const uint32_t*>(img); }
  __device__ unsigned char* b() const { return const_cast<unsigned char*>(img) + hdr; }
};

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

// (hi, lo) TF32 parts of x: hi = x rounded to 10 fraction bits (to nearest,
// ties away from zero: add half a TF32 unit to the magnitude bits, clear the 13
// low bits), lo = x - hi (exact).  lo keeps up to 13 significant bits, of which
// the tensor core uses 11: the pair carries x to 2^-22 relative.
__device__ __forceinline__ void split_tf32(float x, float& hi, float& lo) {
  hi = __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xffffe000u);
  lo = x - hi;
}

// The remainder of x beyond its TF32 truncation, x - trunc(x) (exact): the
// tensor core reads an FP32 operand as its truncation to TF32 (10 fraction
// bits), so the copied B and this image carry x to 2^-21 relative.
__device__ __forceinline__ float tf32_rest(float x) {
  return x - __uint_as_float(__float_as_uint(x) & 0xffffe000u);
}

// ---------------------------------------------------------------------------
template <int P>
__global__ void __launch_bounds__(kThreads, 1) um_sweep_kernel(KArgs a) {
  extern __shared__ unsigned char smem_raw[];
  // 1024-byte alignment of the shared-window offset (swizzle atoms, core matrices)
  const Smem S{smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u)};
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (uint32_t i = 0; i < kSlots; ++i) {
      mbar_init(S.bfull(i), 1);
      mbar_init(S.bempty(i), 1);
    }
    for (uint32_t i = 0; i < kA; ++i) {
      mbar_init(S.aready(i), 4);
      mbar_init(S.aempty(i), 1);
    }
    for (uint32_t i = 0; i < kAcc; ++i) {
      mbar_init(S.accfull(i), 2);
      mbar_init(S.accempty(i), kEpiWarps);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // A rows of absent right-hand sides are never gathered: zero the stages once
  // (those rows only feed D rows that are never read)
  for (uint32_t i = threadIdx.x; i < 2 * kA * (kPiece / 16); i += kThreads)
    reinterpret_cast<uint4*>(S.astage(0))[i] = make_uint4(0u, 0u, 0u, 0u);
  fence_proxy_async();
  if (warp == 1) {
    tmem_alloc(smem_u32(S.tmem_slot()), kTmemCols);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *S.tmem_slot();

  if (warp == 0) {
    // ---------------- producer (lane 0 issues; the warp fetches descriptors)
    uint32_t it = 0, oldest = 0;
    uint64_t pos = 0, done = 0;
    bool ok = true;
    // Frees ring slots (and their bytes, in order) until chunk `it` may take
    // `sz` bytes at position p0; lane 0 only.
    auto reserve = [&](uint64_t p0, uint32_t sz) -> bool {
      while (oldest < it && (it - oldest >= kSlots || p0 + sz > done + kRing)) {
        if (!wait_bar(S.bempty(oldest % kSlots), (oldest / kSlots) & 1, a.err)) return false;
        done = S.endpos()[oldest % kSlots];
        ++oldest;
      }
      return true;
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
      // UmTile words: src (x, y), nchunks z, n8 | hdr << 16 w; klast (c1.x & 0xffff)
      const uint32_t w_sl = __shfl_sync(0xffffffffu, c0.x, r), w_sh = __shfl_sync(0xffffffffu, c0.y, r);
      const uint32_t nch = __shfl_sync(0xffffffffu, c0.z, r), w3 = __shfl_sync(0xffffffffu, c0.w, r);
      const uint32_t klast = __shfl_sync(0xffffffffu, c1.x, r) & 0xffffu;
      if (lane == 0) {
        const uint64_t tsrc = (uint64_t)w_sl | ((uint64_t)w_sh << 32);
        const uint32_t n8 = w3 & 0xffffu, hdr = w3 >> 16;
        const uint64_t cstride = (uint64_t)hdr + (uint64_t)n8 * kUmKc * 4;
        for (uint32_t c = 0; c < nch; ++c) {
          const uint32_t kc = c + 1 == nch ? klast : kUmKc;
          const uint32_t bbytes = n8 * kc * 4, sz = hdr + bbytes;
          uint64_t p0 = pos;
          if ((p0 % kRing) + sz > kRing) p0 += kRing - p0 % kRing;  // no entry wraps
          if (!reserve(p0, sz)) {
            ok = false;
            break;
          }
          const uint32_t sl = it % kSlots, off = (uint32_t)(p0 % kRing);
          S.endpos()[sl] = p0 + sz;
          S.slot_off()[sl] = off | (hdr << 24);
          mbar_expect_tx(S.bfull(sl), hdr + bbytes);
          bulk_g2s(smem_u32(S.ring() + off), a.stream + tsrc + (uint64_t)c * cstride, hdr + bbytes, S.bfull(sl));
          pos = p0 + sz;
          ++it;
        }
      }
      ok = __shfl_sync(0xffffffffu, ok ? 1u : 0u, 0) != 0;
      it = __shfl_sync(0xffffffffu, it, 0);
    }
    if (lane == 0) {
      if (ok && reserve(pos, 0)) {
        // stop marker: a slot record without an image
        const uint32_t sl = it % kSlots;
        S.slot_off()[sl] = kStop;
        mbar_arrive(S.bfull(sl));
      }
      // every bulk copy issued has landed before the CTA may exit: the chunks
      // not yet consumed (the older ones were consumed, hence landed)
      // (bounded, but not cut short by another role's error: a copy in flight
      // must not land after the CTA has exited)
      for (uint32_t i = oldest; i < it; ++i) mbar_wait_sleep(S.bfull(i % kSlots), (i / kSlots) & 1, a.err);
    }
    __syncwarp();
  } else if (warp == 1) {
    // ---------------- MMA issuer
    if (lane == 0) {
      // Chunks accumulate in one tensor-memory accumulator for a drain group
      // (a.drain chunks of one tile, or the rest of the tile); the group's
      // last chunk commits the accumulator to the epilogue.
      uint32_t c = 0, gi = 0, gpos = 0;
      bool gfirst = false;
      bool issued = false;
      while (true) {
        const uint32_t sl = c % kSlots, as = c % kA, q = gi % kAcc;
        if (!wait_bar(S.aready(as), (c / kA) & 1, a.err)) break;
        const uint32_t so = S.slot_off()[sl];
        if (gpos == 0 && gi >= kAcc && !wait_bar(S.accempty(q), (gi / kAcc - 1) & 1, a.err)) break;
        if (so == kStop) {
          // forward the stop to the epilogue (both arrivals of the phase)
          volatile uint32_t* f = &S.acchdr(q)->flags;
          *f = kUmStop;
          mbar_arrive(S.accfull(q));
          mbar_arrive(S.accfull(q));
          break;
        }
        const Entry E{S.ring() + (so & 0xffffffu), so >> 24};
        UmHead h = *E.head();
        if (gpos == 0) gfirst = h.flags & kUmFirst;
        tc_fence_after();
        const uint32_t n16 = ((uint32_t)h.n8 + 15u) & ~15u;
        const uint32_t idesc = umma_idesc_tf32(128, n16);
        const uint32_t sbo = (uint32_t)h.kc * 32u;  // (kc / 4) core matrices of 128 bytes per 8-row group
        const uint32_t sa = smem_u32(S.astage(as));
        const uint32_t sb = smem_u32(E.b());
        const uint32_t sl2 = smem_u32(S.lostage(as));  // B remainder image
        const uint32_t d = tmem + q * kUmN;
        for (uint32_t kk = 0; kk < (uint32_t)h.kc / 8u; ++kk) {
          const uint64_t da = umma_desc_sw128(sa + kk * 32u, 1024u);
          umma_tf32(d, da, umma_desc(sb + kk * 256u, 128u, sbo), idesc, (kk > 0 || gpos > 0) ? 1u : 0u);
          umma_tf32(d, da, umma_desc(sl2 + kk * 256u, 128u, sbo), idesc, 1u);
        }
        umma_commit(S.bempty(sl));
        umma_commit(S.aempty(as));
        issued = true;
        ++c;
        if (++gpos == a.drain || (h.flags & kUmLast)) {
          h.flags = (h.flags & ~kUmFirst) | (gfirst ? kUmFirst : 0u);
          *S.acchdr(q) = h;
          umma_commit(S.accfull(q));
          mbar_arrive(S.accfull(q));  // publishes the head (release)
          gpos = 0;
          ++gi;
        }
      }
      // the MMAs issued last have completed before the tensor memory is freed
      // (bounded, not cut short by another role's error)
      if (issued) mbar_wait_sleep(S.aempty((c - 1) % kA), ((c - 1) / kA) & 1, a.err);
    }
    __syncwarp();
  } else if (warp < 6) {
    // ---------------- stage filling (A + the B remainder image)
    // A (128 x kc, TF32) in the 128-byte-swizzled K-major layout, rows m < 64
    // the hi parts of right-hand sides j = m, rows 64 + j their lo parts; atom
    // g = rows 8 g .. 8 g + 7 (1024 bytes), 16-byte chunk kb (k = 4 kb .. 4 kb
    // + 3) of row r at chunk kb ^ r.  Lane (kb = lane % 8, t = 4 q + lane / 8)
    // loads Z rows 4 kb .. 4 kb + 3 of right-hand sides 4 t .. 4 t + 3 (four
    // 16-byte loads), splits them and stores eight 16-byte row chunks (hi rows
    // 4 t + i, lo rows 64 + 4 t + i).  Loads run one chunk ahead of the stores.
    // All four warps then write the B remainder image.
    const uint32_t q = warp - 2;
    const uint32_t tid = threadIdx.x - 64;        // 0 .. 127
    const uint32_t kb = lane & 7, t4 = 4 * q + (lane >> 3);
    const bool gather = 4 * t4 < (uint32_t)P;     // this lane's right-hand sides exist
    float4 vn[4], vc[4];
#pragma unroll
    for (uint32_t i = 0; i < 4; ++i) vn[i] = vc[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    auto load = [&](const UmHead& h, const uint32_t* ix, float4 (&v)[4]) {
#pragma unroll
      for (uint32_t i = 0; i < 4; ++i) {
        const uint32_t kp = 4 * kb + i;
        v[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (gather && kp < h.kvalid) {
          const uint32_t zr = (h.flags & kUmContig) ? h.zsrc + kp : ix[kp];
          v[i] = __ldg(reinterpret_cast<const float4*>(a.z + (uint64_t)zr * P + 4 * t4));
        }
      }
    };
    auto finalize = [&](uint32_t c, const float4 (&vf)[4]) {
      const uint32_t so = S.slot_off()[c % kSlots], as = c % kA;
      const Entry E{S.ring() + (so & 0xffffffu), so >> 24};
      const UmHead h = *E.head();
      if (gather && 4 * kb < h.kc) {
        unsigned char* Ast = S.astage(as);
        const float x[4][4] = {{vf[0].x, vf[0].y, vf[0].z, vf[0].w}, {vf[1].x, vf[1].y, vf[1].z, vf[1].w},
                               {vf[2].x, vf[2].y, vf[2].z, vf[2].w}, {vf[3].x, vf[3].y, vf[3].z, vf[3].w}};
#pragma unroll
        for (uint32_t i = 0; i < 4; ++i) {
          float hi[4], lo[4];
#pragma unroll
          for (uint32_t k = 0; k < 4; ++k) split_tf32(x[k][i], hi[k], lo[k]);
          const uint32_t mh = 4 * t4 + i, ml = 64 + mh, r = mh & 7;  // ml & 7 == r
          *reinterpret_cast<float4*>(Ast + (mh >> 3) * 1024u + r * 128u + ((kb ^ r) << 4)) =
              make_float4(hi[0], hi[1], hi[2], hi[3]);
          *reinterpret_cast<float4*>(Ast + (ml >> 3) * 1024u + r * 128u + ((kb ^ r) << 4)) =
              make_float4(lo[0], lo[1], lo[2], lo[3]);
        }
      }
      const float4* B = reinterpret_cast<const float4*>(E.b());
      float4* L = reinterpret_cast<float4*>(S.lostage(as));
      const uint32_t nv = (uint32_t)h.n8 * h.kc / 4;
      for (uint32_t e = tid; e < nv; e += 128) {
        const float4 b = B[e];
        L[e] = make_float4(tf32_rest(b.x), tf32_rest(b.y), tf32_rest(b.z), tf32_rest(b.w));
      }
      fence_proxy_async();  // generic writes -> the tensor core's (async proxy) reads
      __syncwarp();
      if (lane == 0) mbar_arrive(S.aready(as));
    };
    // One step per chunk c: the loads of chunk c go into one register set while
    // chunk c - 1 is finalised from the other (ping-pong: the loads have a whole
    // step to land).  Returns false when the role is done.
    bool have_prev = false;
    auto step = [&](uint32_t c, float4 (&vload)[4], float4 (&vfin)[4]) -> bool {
      const uint32_t sl = c % kSlots;
      if (!wait_bar(S.bfull(sl), (c / kSlots) & 1, a.err)) return false;
      const uint32_t so = S.slot_off()[sl];
      const bool stop = so == kStop;
      if (!stop) {
        const Entry E{S.ring() + (so & 0xffffffu), so >> 24};
        const UmHead h = *E.head();
        load(h, E.idx(), vload);
      }
      if (have_prev) {
        // the A stage of chunk c - 1 is free once the MMAs of chunk c - 1 - kA are done
        const uint32_t cp = c - 1;
        if (cp >= kA && !wait_bar(S.aempty(cp % kA), (cp / kA - 1) & 1, a.err)) return false;
        finalize(cp, vfin);
      }
      have_prev = !stop;
      if (stop) {
        // pass the stop on to the MMA issuer through this chunk's A stage
        if (c >= kA && !wait_bar(S.aempty(c % kA), (c / kA - 1) & 1, a.err)) return false;
        __syncwarp();
        if (lane == 0) mbar_arrive(S.aready(c % kA));
        return false;
      }
      return true;
    };
    for (uint32_t c = 0;; c += 2) {
      if (!step(c, vn, vc)) break;
      if (!step(c + 1, vc, vn)) break;
    }
  } else {
    // ---------------- epilogue
    const uint32_t q = warp & 3;                  // tensor-memory lane quadrant of this warp
    const uint32_t half = (warp - 6) >> 2;        // columns 64 half .. 64 half + 63
    const uint32_t et = (threadIdx.x - 192) & 127;  // 0 .. 127 within the column half's warps
    const uint32_t j = 32 * (q & 1) + lane;       // right-hand side of this lane's row
    const bool active = j < (uint32_t)P;          // per lane: guards only the staging writes
    const bool qactive = 32 * (q & 1) < (uint32_t)P;  // warp-uniform: the quadrant holds rows
    const bool lo_row = q >= 2;                   // rows 64 .. 127: lo parts
    float acc[64];
#pragma unroll
    for (int c = 0; c < 64; ++c) acc[c] = 0.f;
    float* Sg = S.staging(half);
    uint32_t ai = 0;
    while (true) {
      const uint32_t qa = ai % kAcc, ka = ai / kAcc;
      if (!wait_bar(S.accfull(qa), ka & 1, a.err)) break;
      const UmHead h = *S.acchdr(qa);
      if (h.flags & kUmStop) break;
      tc_fence_after();
      const uint32_t n16 = ((uint32_t)h.n8 + 15u) & ~15u;
      const bool first = h.flags & kUmFirst;
      // tcgen05.ld / wait::ld are warp-collective: warp-uniform condition only
      if (qactive && 64 * half < n16) {
#pragma unroll
        for (uint32_t gg = 0; gg < 2; ++gg) {
          if (64 * half + 32 * gg < n16) {
            float v[32];
            tmem_ld32(tmem + ((32 * q) << 16) + qa * kUmN + 64 * half + 32 * gg, v);
            tmem_wait_ld();
#pragma unroll
            for (int i = 0; i < 32; ++i) acc[32 * gg + i] = first ? v[i] : acc[32 * gg + i] + v[i];
          }
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(S.accempty(qa));
      ++ai;
      if (!(h.flags & kUmLast) || 64 * half >= h.nout) continue;
      // ---- end of the tile: hi rows, then lo rows added, through the staging tile
      const uint32_t bid = 1 + half;
      named_bar(bid, 128);  // the staging tile is free
      if (active && !lo_row) {
#pragma unroll
        for (int c = 0; c < 64; ++c) Sg[j * kSRow + c] = acc[c];
      }
      named_bar(bid, 128);
      if (active && lo_row) {
#pragma unroll
        for (int c = 0; c < 64; ++c) Sg[j * kSRow + c] += acc[c];
      }
      named_bar(bid, 128);
      const uint32_t nh = min(64u, (uint32_t)h.nout - 64 * half);
      const uint32_t row0 = h.out + 64 * half;
      if (a.mode == 1) {
        for (uint32_t e = et; e < a.pg * 64; e += 128) {
          const uint32_t jj = e >> 6, c = e & 63;
          if (c < nh) {
            double* yp = a.y + (uint64_t)(row0 + c) + (uint64_t)jj * a.ldy;
            *yp += a.d * (double)Sg[jj * kSRow + c];
          }
        }
      } else {
        const bool red = h.flags & kUmRed;
        for (uint32_t e = et; e < (uint32_t)P * 64; e += 128) {
          const uint32_t jj = e % P, c = e / P;
          if (c < nh) {
            float* tp = a.tout + (uint64_t)(row0 + c) * P + jj;
            const float v = Sg[jj * kSRow + c];
            if (red) atomicAdd(tp, v);
            else *tp = v;
          }
        }
      }
    }
  }

  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem, kTmemCols);
  }
}

// X (FP64, column-major, ld ldX), columns 0 .. pg-1 -> Z rows 0 .. n-1 (P FP32
// each, zero beyond pg); T rows of split V tiles zeroed.
template <int P>
__global__ void um_prep_kernel(const double* __restrict__ X, uint64_t ldX, uint64_t n, uint32_t pg,
                               float* __restrict__ z, const UmRange* __restrict__ zero, uint32_t nzero) {
  __shared__ float tile[32][P + 1];
  const uint64_t nblk = (n + 31) / 32;
  for (uint64_t b = blockIdx.x; b < nblk; b += gridDim.x) {
    const uint64_t r0 = b * 32;
    for (uint32_t e = threadIdx.x; e < 32u * P; e += blockDim.x) {
      const uint32_t row = e & 31, col = e >> 5;
      float v = 0.f;
      if (col < pg && r0 + row < n) v = (float)X[(r0 + row) + (uint64_t)col * ldX];
      tile[row][col] = v;
    }
    __syncthreads();
    for (uint32_t e = threadIdx.x; e < 32u * P; e += blockDim.x) {
      const uint32_t col = e % P, row = e / P;
      if (r0 + row < n) z[(r0 + row) * P + col] = tile[row][col];
    }
    __syncthreads();
  }
  float* t = z + n * P;
  for (uint32_t r = blockIdx.x; r < nzero; r += gridDim.x) {
    const UmRange R = zero[r];
    for (uint32_t e = threadIdx.x; e < R.count * (uint32_t)P; e += blockDim.x) t[(uint64_t)R.row * P + e] = 0.f;
  }
}

// One CTA per tile: chunk heads, Z-row indices and B images from the FP64 arena.
__global__ void __launch_bounds__(256) um_build_kernel(const UmBuild* __restrict__ tiles,
                                                       const UmEntry* __restrict__ entries,
                                                       const double* __restrict__ a64,
                                                       unsigned char* __restrict__ stream) {
  const UmBuild T = tiles[blockIdx.x];
  __shared__ int32_t ent[kUmN];
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
    const uint32_t kb = c * kUmKc, kval = min(kUmKc, T.K - kb), kc = (kval + 7u) & ~7u;
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
    if (tid == 0) {
      UmHead h{};
      h.zsrc = contig ? T.zrow0 + kb : 0u;
      h.kc = (uint16_t)kc;
      h.kvalid = (uint16_t)kval;
      h.n8 = T.n8;
      h.nout = (uint16_t)T.nout;
      h.out = T.out;
      h.flags = (c == 0 ? kUmFirst : 0u) | (c + 1 == T.nchunks ? kUmLast : 0u) | (T.flags & (kUmContig | kUmRed));
      h.tile = blockIdx.x;
      *reinterpret_cast<UmHead*>(B - 32) = h;
    }
    if (!contig && tid < kUmKc) {
      uint32_t zr = 0;
      if (tid < kval && ent[tid] >= 0) {
        const UmEntry E = entries[T.e0 + ent[tid]];
        zr = E.zrow0 + (kb + tid - E.k0);
      }
      reinterpret_cast<uint32_t*>(img)[tid] = zr;
    }
    const uint32_t cnt = (uint32_t)T.n8 * kc;
    for (uint32_t e = tid; e < cnt; e += blockDim.x) {
      uint32_t nn, kk;
      if (byN) {
        kk = e % kc;
        nn = e / kc;
      } else {
        nn = e % T.n8;
        kk = e / T.n8;
      }
      float v = 0.f;
      if (nn < T.nout && kk < kval) {
        const int32_t ei = byN ? ent[nn] : ent[kk];
        if (ei >= 0) {
          const UmEntry E = entries[T.e0 + ei];
          const uint32_t K = kb + kk;
          if (K >= E.k0 && K < E.k0 + E.kn && nn >= E.n0 && nn < E.n0 + E.nn)
            v = (float)a64[E.base + (uint64_t)(K - E.k0) * E.sk + (uint64_t)(nn - E.n0) * E.sn];
        }
      }
      *reinterpret_cast<float*>(B + (nn >> 3) * (kc * 32u) + (kk >> 2) * 128u + (nn & 7u) * 16u + (kk & 3u) * 4u) = v;
    }
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
std::vector<TimingRec> g_trecs;

template <int P>
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
  um_sweep_kernel<P><<<grid, kThreads, kSmemBytes, s>>>(a);
  cudaError_t e = cudaGetLastError();
  if (timed) {
    cudaEventRecord(r.e1, s);
    std::lock_guard<std::mutex> lk(g_tmu);
    g_trecs.push_back(r);
  }
  return e;
}

template <int P>
cudaError_t run_um(const UmPlan& pl, double d, uint32_t r0, uint32_t pg, const double* X, uint64_t ldX, double* Y,
                   uint64_t ldY, cudaStream_t s) {
  const uint64_t nblk = (pl.n + 31) / 32;
  const unsigned grid = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(nblk, (uint64_t)pl.grid * 8));
  um_prep_kernel<P><<<grid, 256, 0, s>>>(X + (uint64_t)r0 * ldX, ldX, pl.n, pg, pl.z, pl.zero, pl.nzero);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  uint64_t launches = 1;
  KArgs a{};
  a.z = pl.z;
  a.err = pl.err;
  a.pg = pg;
  a.drain = std::max<uint32_t>(1u, pl.drain);
  if (pl.nvtiles) {
    a.tiles = pl.vtiles;
    a.ranges = pl.vranges;
    a.stream = pl.vstream;
    a.tout = pl.z + pl.n * P;
    a.mode = 0;
    if ((e = launch_sweep<P>(a, 0, pl.grid, s)) != cudaSuccess) return e;
    ++launches;
  }
  if (pl.nrtiles) {
    a.tiles = pl.rtiles;
    a.ranges = pl.rranges;
    a.stream = pl.rstream;
    a.tout = nullptr;
    a.y = Y + (uint64_t)r0 * ldY;
    a.ldy = ldY;
    a.d = d;
    a.mode = 1;
    if ((e = launch_sweep<P>(a, 1, pl.grid, s)) != cudaSuccess) return e;
    ++launches;
  }
  count_product_launches(launches);
  return cudaSuccess;
}

uint32_t round8(uint32_t x) { return (x + 7u) & ~7u; }

}  // namespace

cudaError_t um_init_attributes() {
  cudaError_t e;
  if ((e = cudaFuncSetAttribute(um_sweep_kernel<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemBytes)))
    return e;
  if ((e = cudaFuncSetAttribute(um_sweep_kernel<32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemBytes)))
    return e;
  return cudaFuncSetAttribute(um_sweep_kernel<64>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemBytes);
}

cudaError_t launch_um_build(const UmBuild* tiles, uint32_t ntiles, const UmEntry* entries, const double* arena64,
                            unsigned char* stream, cudaStream_t s) {
  if (ntiles == 0) return cudaSuccess;
  um_build_kernel<<<ntiles, 256, 0, s>>>(tiles, entries, arena64, stream);
  count_product_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_matvec_um(const UmPlan& pl, double d, uint32_t p, const double* X, uint64_t ldX, double* Y,
                             uint64_t ldY, cudaStream_t s) {
  for (uint32_t r0 = 0; r0 < p; r0 += 64) {
    const uint32_t pg = std::min(64u, p - r0);
    cudaError_t e;
    if (pg <= 16) e = run_um<16>(pl, d, r0, pg, X, ldX, Y, ldY, s);
    else if (pg <= 32) e = run_um<32>(pl, d, r0, pg, X, ldX, Y, ldY, s);
    else e = run_um<64>(pl, d, r0, pg, X, ldX, Y, ldY, s);
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
      if (red) L.zero.push_back({tc + g0, ng});
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
    B.hdr = (uint16_t)(32 + kUmIdxBytes);
    B.nchunks = (K + kUmKc - 1) / kUmKc;
    if (K > 0) L.rbuild.push_back(B);
    std::vector<UmEntry>().swap(es);
  }

  // ---- stream offsets and the kernel's tiles
  auto chunk_bytes = [](const UmBuild& B) {
    const uint32_t klast = round8(B.K - (B.nchunks - 1) * kUmKc);
    return (uint64_t)(B.nchunks - 1) * (B.hdr + (uint64_t)B.n8 * kUmKc * 4) + B.hdr + (uint64_t)B.n8 * klast * 4;
  };
  auto place = [&](std::vector<UmBuild>& bl, std::vector<UmTile>& tl, uint64_t& bytes) {
    bytes = 0;
    tl.clear();
    for (UmBuild& B : bl) {
      B.src = bytes;
      bytes += chunk_bytes(B);
      UmTile T{};
      T.src = B.src;
      T.nchunks = B.nchunks;
      T.n8 = B.n8;
      T.hdr = B.hdr;
      T.klast = (uint16_t)round8(B.K - (B.nchunks - 1) * kUmKc);
      tl.push_back(T);
    }
  };
  place(L.vbuild, L.vtiles, L.vbytes);
  place(L.rbuild, L.rtiles, L.rbytes);
  // contiguous tile ranges per CTA, balanced by stream bytes
  auto ranges = [&](const std::vector<UmBuild>& bl, std::vector<uint32_t>& first) {
    std::vector<uint64_t> bytes(bl.size());
    for (size_t t = 0; t < bl.size(); ++t) bytes[t] = chunk_bytes(bl[t]);
    balance_ranges(bytes, std::max<uint32_t>(grid, 1), first);
  };
  ranges(L.vbuild, L.vranges);
  ranges(L.rbuild, L.rranges);
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
