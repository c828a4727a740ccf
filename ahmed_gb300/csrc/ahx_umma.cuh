// H-matrix product Y += d A X on the fifth-generation tensor cores
// (tcgen05.mma, accumulators in tensor memory), for leaves stored in FP32-class
// precision as two FP16 parts.
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
//               rows -> T rows (T = V^T X per leaf, stored after X in Z)
//   rows sweep: one tile per finest row block (<= 128 rows of the cluster
//               tree's leaf clusters): B[k][n] = row n of every leaf whose row
//               cluster contains the block (U columns of low-rank leaves, the
//               columns of dense ones), A = the matching T rows / X rows.
//               Every Y row belongs to exactly one tile, so the tile's
//               epilogue updates Y in place (FP64) with no atomics.
//
// Precision (the FP32 storage of this library, about 22 significant bits):
// every stored value v is kept as two FP16 numbers, b1 = fp16(v / s) and
// b2 = fp16(v / s - b1), with s a power of two per chunk of 64 K positions
// (the chunk's largest |v| / s lies in [2^13, 2^14)).  Z rows (X rows and T
// rows) hold each of 64 right-hand-side slots the same way: 64 first parts,
// then 64 second parts (256 bytes per row, rows kUmZPitch bytes apart); A's row
// m < 64 is the first part of
// right-hand side m, row 64 + m its second part.  The tensor core forms the
// four exact FP16 products (x1 + x2)(b1 + b2) with FP32 accumulation; each
// chunk accumulates into a fresh tensor-memory accumulator that the epilogue
// scales by s and adds to registers with round-to-nearest FP32 adds.
// Magnitudes: X is scaled per right-hand side so that max |X_j| lies in
// [2^13, 2^14); the V column of T row t is scaled by a power of two s_t with
// ||V_t||_1 s_t <= 1 and the matching U column by 1 / s_t, so that every T
// row stays below 2^14 and no FP16 value overflows.
//
// Stream of each sweep: per tile, chunks of <= 64 K positions; each chunk
// image is [UmHead (32 B)] [b1 image] [b2 image], the images in the tensor
// core's K-major, no-swizzle
// canonical layout of 16-bit elements: core matrices of 8 rows x 16 bytes
// (8 K positions), byte offset of B[k][n]
//     (n / 8) * (kc * 16) + (k / 8) * 128 + (n % 8) * 16 + (k % 8) * 2
// (leading-dimension byte offset 128, stride byte offset kc * 16; kc a
// multiple of 16).  One bulk copy moves a chunk image into the kernel's ring.
// The Z rows of every chunk (64 row indices per chunk, in chunk order; past
// the chunk's K they meet zero B values: row 0, or in contiguous tiles the run
// continued) are a separate array, so that the kernel can fetch them well
// ahead of the images.
#pragma once
#include <cstdint>
#include <vector>

#include <cuda_runtime.h>

#include "ahx_matvec.cuh"

namespace ahx {

constexpr uint32_t kUmKc = 64;    // K positions per chunk
constexpr uint32_t kUmN = 128;    // rows (N) per tile
constexpr uint32_t kUmIdxBytes = kUmKc * 4;
constexpr uint32_t kUmSlots = 64;           // right-hand-side slots of a Z row
constexpr uint32_t kUmZRowBytes = 256;      // 64 first parts, 64 second parts (FP16)
constexpr uint32_t kUmZPitch = 272;         // bytes between Z rows (a multiple of 16: the row stride of the tensor copies)

enum UmFlags : uint32_t {
  kUmFirst = 1u,    // first chunk of its tile
  kUmLast = 2u,     // last chunk of its tile
  kUmContig = 4u,   // A rows are Z rows zsrc + k
  kUmRed = 8u,      // a V tile split along K: its pieces add into FP32 accumulation rows
  kUmStop = 16u,    // no more work
  kUmByN = 32u,     // builder: the tile's entries partition N (V sweep), else K
};

struct UmHead {
  uint32_t zsrc;      // contiguous tiles: Z row of the chunk's k = 0
  uint16_t kc;        // K of the chunk images (multiple of 16, <= 64)
  uint16_t kvalid;    // positions >= kvalid are zero
  uint16_t n8;        // rows of the images (multiple of 8, <= 128)
  uint16_t nout;      // output rows of the tile (<= 128)
  uint32_t out;       // output row of n = 0 (Y row, or T row)
  uint32_t flags;     // UmFlags
  float scale;        // the images hold the values divided by this power of two
  uint32_t tacc;      // kUmRed tiles: accumulation row of n = 0
  uint32_t tile;
};
static_assert(sizeof(UmHead) == 32, "chunk head");

// the kernel's view of a tile
struct UmTile {
  uint64_t src;       // byte offset of the first chunk image in the stream
  uint32_t nchunks;
  uint16_t n8;        // rows of the images
  uint16_t hdr;       // bytes before each image pair (the head, 32)
  uint16_t klast;     // K of the last chunk's images
  uint16_t kvlast;    // valid K positions of the last chunk
  uint32_t zrow0;     // contiguous tiles: Z row of K position 0
  uint32_t flags;     // kUmContig
  uint32_t pad;
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
  uint32_t K;          // K positions (the last chunk's are padded to 16)
  uint32_t nout;       // rows (N)
  uint32_t out;        // output row of n = 0
  uint32_t zrow0;      // contiguous tiles: Z row of K position 0
  uint32_t flags;      // kUmContig | kUmRed | kUmByN
  uint32_t nchunks;
  uint16_t n8, hdr;
  uint32_t tacc;       // kUmRed: accumulation row of n = 0
  uint32_t cbase;      // sweep-wide index of the tile's first chunk (Z-row index array)
  uint32_t pad;
};
static_assert(sizeof(UmBuild) == 56, "build");

// rows of V tiles split along K: T rows [row, row + count) accumulate in FP32
// rows [off, off + count) before they are split into Z rows
struct UmRange {
  uint32_t row, count, off, pad;
};

// T scale job: the V factor of one low-rank leaf (column-major n2 x rank at
// element offset vbase of the FP64 arena), its T rows trow .. trow + rank - 1
struct UmTJob {
  uint64_t vbase;
  uint32_t n2, rank, trow, pad;
};

struct UmLayout {
  std::vector<UmTile> vtiles, rtiles;
  std::vector<UmBuild> vbuild, rbuild;
  std::vector<UmEntry> entries;
  std::vector<UmRange> zero;
  std::vector<UmTJob> tjobs;
  std::vector<uint32_t> vranges, rranges;  // per CTA of a sweep launch: first tile (grid + 1 entries)
  std::vector<uint32_t> vcranges, rcranges;  // per CTA: first chunk (grid + 1 entries)
  uint64_t vchunks = 0, rchunks = 0;
  uint64_t vbytes = 0, rbytes = 0;
  uint32_t t_rows = 0;
  uint32_t tacc_rows = 0;
  uint64_t payload_bytes = 0;   // stored leaf bytes (4 per value) without padding
  uint64_t stream_bytes = 0;    // both streams, headers and padding included
};

// grid: CTAs of a sweep launch (one per SM); kpiece: V-sweep tiles longer than
// this many K positions are split (their pieces add into FP32 accumulation rows)
void build_um_layout(const std::vector<PlanLeaf>& leaves, uint64_t n, uint32_t grid, UmLayout& L,
                     uint32_t kpiece = 4096);

struct UmPlan {
  const UmTile* vtiles = nullptr;
  const UmTile* rtiles = nullptr;
  const uint32_t* vranges = nullptr;  // per CTA: first tile (grid + 1 entries)
  const uint32_t* rranges = nullptr;
  const uint32_t* vcranges = nullptr;  // per CTA: first chunk (grid + 1 entries)
  const uint32_t* rcranges = nullptr;
  const uint32_t* vzidx = nullptr;     // Z-row indices, kUmKc per chunk
  const uint32_t* rzidx = nullptr;
  uint32_t grid = 0;
  uint32_t nvtiles = 0, nrtiles = 0;
  const unsigned char* vstream = nullptr;
  const unsigned char* rstream = nullptr;
  const UmRange* zero = nullptr;
  uint32_t nzero = 0;
  uint64_t n = 0;          // rows of X / Y
  uint32_t t_rows = 0;
  uint16_t* z = nullptr;   // Z rows: X rows (n), T rows (t_rows), one spare row; kUmZPitch bytes apart
  float* tacc = nullptr;   // FP32 accumulation rows of split V tiles (64 floats each), zero between products
  uint32_t* xmax = nullptr;  // 64 words: max |X_j| of the pass (FP32 bits)
  int* err = nullptr;
};

cudaError_t um_init_attributes();
// T-row scales (powers of two) from the V factors of the FP64 arena
cudaError_t launch_um_tscale(const UmTJob* jobs, uint32_t njobs, const double* arena64, float* tscale,
                             cudaStream_t s);
// stream images of a layout from the FP64 arena (n: rows of X; Z rows >= n are T rows)
cudaError_t launch_um_build(const UmBuild* tiles, uint32_t ntiles, const UmEntry* entries, const double* arena64,
                            const float* tscale, uint64_t n, unsigned char* stream, uint32_t* zidx,
                            cudaStream_t s);
// Y += d A X for p right-hand sides (passes of <= 64)
cudaError_t launch_matvec_um(const UmPlan& plan, double d, uint32_t p, const double* X, uint64_t ldX, double* Y,
                             uint64_t ldY, cudaStream_t s);

// Optional CUDA-event timing of the sweep launches (bench instrumentation):
// kind 0 = V sweep, 1 = rows sweep.
void um_timing_enable(bool on);
// total milliseconds and launch count per kind since the last reset (synchronises)
void um_timing_read(double* ms2, uint64_t* count2, bool reset);

}  // namespace ahx
