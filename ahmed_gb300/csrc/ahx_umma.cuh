// H-matrix product Y += d A X on the fifth-generation tensor cores
// (tcgen05.mma, accumulators in tensor memory), for leaves stored in FP32.
//
// Semantics: mltaGeHGeM (H/mltaGeHVec.cpp:38-59) with the leaf products of
// mltaLrMGeM_ / mltaGeMGeM (H/mblock.cpp:141-154, Include/mblock.h:105-109):
// every low-rank leaf adds d U (V^T X), every dense leaf d D X.
//
// Two sweeps of one kernel over "tiles", each a small GEMM
//     D[m][n] = sum_k A[m][k] B[k][n],    M = 128, N <= 128, K any
// with the right-hand sides on M and the stored leaf data on N:
//   V sweep:    B[k][n] = V[k][col n] of the low-rank leaves of one column
//               cluster (their V columns side by side), A = the cluster's X
//               rows -> T rows (T = V^T X per leaf, FP32, stored beside X)
//   rows sweep: one tile per finest row block (<= 128 rows of the cluster
//               tree's leaf clusters): B[k][n] = row n of every leaf whose row
//               cluster contains the block (U columns of low-rank leaves, the
//               columns of dense ones), A = the matching T rows / X rows.
//               Every Y row belongs to exactly one tile, so the tile's
//               epilogue updates Y in place (FP64) with no atomics.
// Precision (FP32-class products on the TF32 tensor path): A's 128 rows are
// the hi and lo TF32 parts of up to 64 right-hand sides (row 2 j + s, s = 0
// hi, 1 lo), and each K step runs twice, on B's hi and lo TF32 parts, so that
// hi*hi + hi*lo + lo*hi + lo*lo is formed.  Each chunk of 32 K positions
// accumulates into a fresh tensor-memory accumulator that the epilogue adds
// to registers with round-to-nearest FP32 adds.
//
// Layout of the stream: per tile, chunks of <= 32 K positions; each chunk image
// is [Z-row indices (128 B, indexed tiles only)] [UmHead (32 B)] [B image],
// the B image in the tensor core's K-major, no-swizzle canonical layout:
// core matrices of 8 rows x 16 bytes (4 K positions), byte offset of B[k][n]
//     (n / 8) * (kc / 4) * 128 + (k / 4) * 128 + (n % 8) * 16 + (k % 4) * 4
// (leading-dimension byte offset 128, stride byte offset kc * 32).  One bulk
// copy moves a chunk into the kernel's shared-memory ring.
#pragma once
#include <cstdint>
#include <vector>

#include <cuda_runtime.h>

#include "ahx_matvec.cuh"

namespace ahx {

constexpr uint32_t kUmKc = 32;    // K positions per chunk
constexpr uint32_t kUmN = 128;    // rows (N) per tile
constexpr uint32_t kUmIdxBytes = kUmKc * 4;

enum UmFlags : uint32_t {
  kUmFirst = 1u,    // first chunk of its tile
  kUmLast = 2u,     // last chunk of its tile
  kUmContig = 4u,   // A rows are Z rows zsrc + k (else the indices before the head)
  kUmRed = 8u,      // output rows are summed atomically (a tile split along K)
  kUmStop = 16u,    // no more work
  kUmByN = 32u,     // builder: the tile's entries partition N (V sweep), else K
};

struct UmHead {
  uint32_t zsrc;      // contiguous tiles: Z row of the chunk's k = 0
  uint16_t kc;        // K of the chunk (multiple of 8, <= 32)
  uint16_t kvalid;    // positions >= kvalid are zero
  uint16_t n8;        // rows of the B image (multiple of 8, <= 128)
  uint16_t nout;      // output rows of the tile (<= 128)
  uint32_t out;       // output row of n = 0 (Y row, or T row)
  uint32_t flags;     // UmFlags
  uint32_t tile;
  uint32_t pad[2];
};
static_assert(sizeof(UmHead) == 32, "chunk head");

// the kernel's view of a tile
struct UmTile {
  uint64_t src;       // byte offset of the first chunk image in the stream
  uint32_t nchunks;
  uint16_t n8;        // rows of the B images
  uint16_t hdr;       // bytes before each B image: 32, or 32 + kUmIdxBytes (indexed)
  uint16_t klast;     // K of the last chunk
  uint16_t pad0;
  uint32_t pad1, pad2, pad3;
};
static_assert(sizeof(UmTile) == 32, "tile");

// a 2D block of one leaf inside a tile, for the stream builder:
// B[K][N] = arena[base + (K - k0) sk + (N - n0) sn] for K in [k0, k0 + kn), N in [n0, n0 + nn)
struct UmEntry {
  uint64_t base;
  uint32_t k0, kn, n0, nn;
  uint32_t sk, sn;
  uint32_t zrow0;     // indexed tiles: Z row of K position k0 (the next positions follow)
  uint32_t pad;
};
static_assert(sizeof(UmEntry) == 40, "entry");

struct UmBuild {
  uint64_t src;
  uint32_t e0, ne;     // entries
  uint32_t K;          // K positions (the last chunk's are padded to 8)
  uint32_t nout;       // rows (N)
  uint32_t out;        // output row of n = 0
  uint32_t zrow0;      // contiguous tiles: Z row of K position 0
  uint32_t flags;      // kUmContig | kUmRed | kUmByN
  uint32_t nchunks;
  uint16_t n8, hdr;
  uint32_t pad;
};
static_assert(sizeof(UmBuild) == 48, "build");

struct UmRange {  // T rows to zero before the V sweep (tiles split along K add into them)
  uint32_t row, count;
};

struct UmLayout {
  std::vector<UmTile> vtiles, rtiles;
  std::vector<UmBuild> vbuild, rbuild;
  std::vector<UmEntry> entries;
  std::vector<UmRange> zero;
  std::vector<uint32_t> vranges, rranges;  // per CTA of a sweep launch: first tile (grid + 1 entries)
  uint64_t vbytes = 0, rbytes = 0;
  uint32_t t_rows = 0;
  uint64_t payload_bytes = 0;   // stored leaf bytes (FP32) without padding
  uint64_t stream_bytes = 0;    // both streams, headers and padding included
};

// grid: CTAs of a sweep launch (one per SM); kpiece: V-sweep tiles longer than
// this many K positions are split (their pieces add into zeroed T rows)
void build_um_layout(const std::vector<PlanLeaf>& leaves, uint64_t n, uint32_t grid, UmLayout& L,
                     uint32_t kpiece = 4096);

struct UmPlan {
  const UmTile* vtiles = nullptr;
  const UmTile* rtiles = nullptr;
  const uint32_t* vranges = nullptr;  // per CTA: first tile (grid + 1 entries)
  const uint32_t* rranges = nullptr;
  uint32_t grid = 0;
  uint32_t nvtiles = 0, nrtiles = 0;
  const unsigned char* vstream = nullptr;
  const unsigned char* rstream = nullptr;
  const UmRange* zero = nullptr;
  uint32_t nzero = 0;
  uint64_t n = 0;          // rows of X / Y
  uint32_t t_rows = 0;
  float* z = nullptr;      // Z rows: X rows (n) then T rows (t_rows), 64 floats each (P used)
  int* err = nullptr;
  uint32_t drain = 1;      // chunks accumulated in tensor memory per drain into registers
};

cudaError_t um_init_attributes();
// stream images of a layout from the FP64 arena
cudaError_t launch_um_build(const UmBuild* tiles, uint32_t ntiles, const UmEntry* entries, const double* arena64,
                            unsigned char* stream, cudaStream_t s);
// Y += d A X for p right-hand sides (passes of <= 64)
cudaError_t launch_matvec_um(const UmPlan& plan, double d, uint32_t p, const double* X, uint64_t ldX, double* Y,
                             uint64_t ldY, cudaStream_t s);

// Optional CUDA-event timing of the sweep launches (bench instrumentation):
// kind 0 = V sweep, 1 = rows sweep.
void um_timing_enable(bool on);
// total milliseconds and launch count per kind since the last reset (synchronises)
void um_timing_read(double* ms2, uint64_t* count2, bool reset);

}  // namespace ahx
