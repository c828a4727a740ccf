// Batched H-matrix product Y += d A X over all leaves (dense and low-rank),
// for any number of right-hand sides and any number of H-matrix instances.
#pragma once
#include <cstdint>
#include <vector>

#include <cuda_runtime.h>

namespace ahx {

// Storage precisions of the leaf arena used by the product.
enum Precision : int {
  kFP64 = 0,      // plain form: every leaf in FP64
  kFP32 = 1,      // all leaves in FP32, FP32 accumulation
  kBF16FP32 = 2,  // low-rank factors in BF16, dense leaves in FP32, FP32 accumulation
};

// One leaf of the product, with absolute row/column offsets into the
// (possibly concatenated) vectors and an element offset into its arena.
struct MvLeaf {
  uint32_t b1, n1, b2, n2;
  int32_t rank;  // -1: dense (n1 x n2); >= 0: U (n1 x rank) then V (n2 x rank)
  uint32_t dense_in_lr_arena;  // 1 when the leaf lives in the low-rank arena (FP64/FP32)
  uint64_t off;
};

struct MvArgs {
  const MvLeaf* leaves;
  const uint32_t* order;  // launch order (descending cost)
  uint32_t nleaves;
  const void* arena_lr;   // low-rank factors (and dense leaves unless split)
  const void* arena_dn;   // dense leaves for kBF16FP32
  double d;
  uint32_t p;
  const double* X;
  uint64_t ldX;
  double* Y;
  uint64_t ldY;
};

cudaError_t launch_matvec(int prec, const MvArgs& a, cudaStream_t s);

// ---------------------------------------------------------------------------
// Mixed-precision product (FP32 or BF16 low-rank factors, FP32 dense leaves,
// FP32 accumulation) as two linear sweeps over a re-laid-out arena.
//
// The product copy stores the leaves in processing order:
//   V stream:    chunks of <= 256 rows x <= kVRank columns of the V factors
//   rows stream: for every 64-row tile of every row cluster, the tile's rows of
//                every leaf of that block row (dense columns or U columns)
// so every work unit is one contiguous, 16-byte aligned byte range.  A producer
// warp per CTA moves units into a shared-memory ring with cp.async.bulk
// (mbarrier completion); consumer warps compute from shared memory.
//   1. X (FP64, column-major) -> Xr (FP32, row-major n x P),  Yr = 0
//   2. V sweep:    T = V^T Xr per chunk (partial T rows, no atomics)
//   3. rows sweep: per unit, one warp accumulates the tile rows in registers
//                  and adds them to Yr once (vector reductions)
//   4. Y += d * Yr  (FP64)
// for groups of P <= 16 right-hand sides.

constexpr uint32_t kTileRows = 64;
constexpr uint32_t kVRank = 16;           // columns of V per V unit
constexpr uint32_t kSlotBytes = 12288;    // leaf bytes of one unit (at most)
constexpr uint32_t kSideBytes = 6144;     // X / T rows staged with a unit (at most, P = 16)
constexpr uint32_t kSideRows = kSideBytes / 64;

struct StreamVUnit {
  uint64_t src;    // byte offset in the V stream
  uint32_t bytes;  // multiple of 16, <= kSlotBytes
  uint32_t jn;     // rows (ld of the chunk)
  uint32_t kn;     // columns
  uint32_t xrow;   // first X row
  uint32_t t_row;  // T row of the chunk's first column
  uint32_t pad;
};

struct StreamEnt {
  uint32_t boff;   // byte offset of the chunk inside its unit
  uint32_t kind;   // 0 dense (FP32 columns), 1 low rank (U columns, plan's low-rank type)
  uint32_t ncols;  // columns in this chunk
  uint32_t xrow;   // dense: X row of column 0; low rank: T row of column 0 (summed T)
};

// Low-rank leaves whose V spans several V units: their partial T are summed
// into the first chunk's rows between the two sweeps.
struct TReduce {
  uint32_t t_row, k, nchunk, pad;
};

struct StreamUnit {
  uint64_t src;    // byte offset in the rows stream
  uint32_t bytes;  // multiple of 16, <= kSlotBytes
  uint32_t row0;   // first Y row
  uint32_t nrows;  // <= kTileRows (ld of every chunk of the unit)
  uint32_t e0, ne; // entries
  uint32_t pad;
};

// Host description of one leaf for plan building: its data in the FP64 arena.
struct PlanLeaf {
  uint32_t b1, n1, b2, n2;
  int32_t rank;
  uint64_t off;  // element offset in the FP64 arena (mblock layout)
};

// Gather-and-convert task building the streams from the FP64 arena.
struct StreamCopy {
  uint64_t src;      // FP64 element offset of the sub-block's (0,0)
  uint64_t dst;      // byte offset in the destination stream
  uint32_t src_ld;   // column stride in the FP64 arena
  uint32_t nrows, ncols;
  uint32_t dtype;    // 0 FP32, 1 BF16
};

struct StreamLayout {
  std::vector<StreamVUnit> vunits;
  std::vector<StreamUnit> units;
  std::vector<StreamEnt> ents;
  std::vector<StreamCopy> vcopies, rcopies;
  std::vector<TReduce> treduce;
  uint64_t vbytes = 0, rbytes = 0;
  uint32_t t_rows = 0;
  uint64_t payload_bytes = 0;  // stored leaf bytes (without alignment padding)
};

// lr_dtype: 0 FP32 low-rank factors, 1 BF16
void build_stream_layout(const std::vector<PlanLeaf>& leaves, int lr_dtype, StreamLayout& L);

struct MvPlan {
  const StreamVUnit* vunits = nullptr;
  uint32_t nvunits = 0;
  const StreamUnit* units = nullptr;
  uint32_t nunits = 0;
  const StreamEnt* ents = nullptr;
  const uint32_t* vranges = nullptr;  // per CTA: first V unit (grid + 1 entries)
  const uint32_t* rranges = nullptr;  // per CTA: first rows unit (grid + 1 entries)
  const TReduce* treduce = nullptr;
  uint32_t ntreduce = 0;
  uint32_t grid = 0;
  const unsigned char* vstream = nullptr;
  const unsigned char* rstream = nullptr;
  uint64_t n = 0;
  float* xr = nullptr;  // n * 16
  float* yr = nullptr;  // n * 16
  float* t = nullptr;   // t_rows * 16
  int* err = nullptr;   // set when a bounded wait gives up
};

cudaError_t launch_stream_copies(const StreamCopy* copies, uint32_t n, const double* arena64,
                                 unsigned char* dst, cudaStream_t s);
cudaError_t launch_matvec_mixed(int prec, const MvPlan& plan, double d, uint32_t p,
                                const double* X, uint64_t ldX, double* Y, uint64_t ldY,
                                cudaStream_t s);
// Per-CTA unit ranges balancing bytes over `grid` CTAs.
void balance_ranges(const std::vector<uint64_t>& bytes, uint32_t grid, std::vector<uint32_t>& first);

}  // namespace ahx
