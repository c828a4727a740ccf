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
  kDF64 = 3,      // FP64 leaves as float pairs, double-float arithmetic (FP64-class)
};
constexpr int kNumPrecisions = 4;

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
  uint32_t transposed = 0;  // 1: Y += d A^T X (H/mltaGeHVec.cpp:62-150)
};

cudaError_t launch_matvec(int prec, const MvArgs& a, cudaStream_t s);

// Double-float product Y += A X (ahx_matvec_df.cu): arena = the FP64 arena's
// elements as (hi, lo) float pairs at the same offsets; X = d X split the same
// way, column-major with leading dimension ldX.
struct DfArgs {
  const MvLeaf* leaves;
  const uint32_t* order;
  uint32_t nleaves;
  const float2* arena;
  const float2* X;
  uint64_t ldX;
  uint32_t p;
  double* Y;
  uint64_t ldY;
};
cudaError_t launch_matvec_df(const DfArgs& a, cudaStream_t s);
// dst[r + c rows] = (hi, lo) of scale * src[r + c ld], r < rows, c < cols
cudaError_t launch_split_df(const double* src, uint64_t ld, uint64_t rows, uint32_t cols, double scale,
                            void* dst, cudaStream_t s);

// Complex product Y += d op(A) X (ahx_matvec_z.cu) over complex leaves in the
// mblock<dcomp> layout; MvLeaf offsets count complex elements.  arena: complex128
// (single = 0) or complex64 (single = 1, FP32 accumulation); X, Y: complex128,
// column-major, leading dimensions in complex elements.
enum ZOp : int { kZOpN = 0, kZOpH = 1, kZOpT = 2 };  // A, A^H, A^T
struct ZArgs {
  const MvLeaf* leaves;
  const uint32_t* order;
  uint32_t nleaves;
  const void* arena;
  int single;
  double dre, dim;
  uint32_t p;
  const double2* X;
  uint64_t ldX;
  double2* Y;
  uint64_t ldY;
  int op;
};
cudaError_t launch_matvec_z(const ZArgs& a, cudaStream_t s);
// dst[i] = (float) src[i], complex128 -> complex64
cudaError_t launch_z_to_c64(const double2* src, uint64_t n, float2* dst, cudaStream_t s);

// Host description of one leaf for plan building: its data in the FP64 arena.
struct PlanLeaf {
  uint32_t b1, n1, b2, n2;
  int32_t rank;
  uint64_t off;  // element offset in the FP64 arena (mblock layout)
};

// ---------------------------------------------------------------------------
// Tensor-core product (warp-level mma.sync) over fragment-ordered streams.
//
// Both sweeps are small GEMMs C[p][n] += sum_k A[p][k] B[k][n] with the
// right-hand sides p as the M dimension (16 per m-tile) and the stored leaf
// data as B:
//   V sweep:    B[k][n] = V[j0 + k][l] of the low-rank leaves of one column
//               cluster (columns n = the leaves' V columns, <= 64 per unit),
//               A[p][k] = X[b2 + j0 + k][p]           -> C = T^T (T = V^T X)
//   rows sweep: B[k][n] = U[r0 + n][l] (group 0, low rank) or D[r0 + n][j]
//               (group 1, dense), rows n of one 64-row tile of a row cluster,
//               A[p][k] = T[leaf row + l][p] or X[b2 + j][p] -> C = (A_tile X)^T
// B is stored in the exact register order of the mma B fragments (one 8-byte
// load per lane per fragment, k-block major, then n-tile), so every unit is
// one contiguous, 16-byte aligned byte range moved by one bulk copy; A comes
// from rows of X / T (stride P + 8 elements: conflict-free fragment loads)
// staged beside it.
//   FP32 storage:       TF32 mma with the 3-pass split (hi*hi + hi*lo + lo*hi),
//                       FP32-level products
//   BF16/FP32 storage:  low rank BF16 mma (T and X rows in BF16); dense leaves
//                       in 4-byte words holding their TF32 rounding, one TF32
//                       pass (the product is the one of FP32 words rounded at
//                       load)
#ifndef AHX_TC_SLOT
#define AHX_TC_SLOT 11264
#endif
#ifndef AHX_TC_GROUPS
#define AHX_TC_GROUPS 5
#endif
#ifndef AHX_TC_RING
#define AHX_TC_RING 4
#endif
constexpr uint32_t kTcSlot = AHX_TC_SLOT;     // bytes of one ring slot
constexpr uint32_t kTcHead = 32;              // the unit's descriptor, copied to the head of its slot
constexpr uint32_t kTcSlotData = kTcSlot - kTcHead;  // B fragments + A rows of one unit
constexpr uint32_t kTcGroups = AHX_TC_GROUPS;  // consumer groups per CTA (one ring each)
constexpr uint32_t kTcRing = AHX_TC_RING;      // slots per group (split evenly between its unit sequences)

struct TcRowUnit {
  uint64_t src;       // byte offset in the rows stream
  uint32_t bytes;     // fragment bytes (group 0, then group 1)
  uint32_t row0;      // first Y row of the tile
  uint32_t e0;        // first A-row entry
  uint16_t ne, nr;    // entries (<= 32), rows of the tile (<= 64)
  uint16_t kp0, kp1;  // K of group 0 / group 1, multiples of 8
  uint32_t flags;     // bit 0: first unit of a tile run, bit 1: last unit
};

struct TcSide {
  uint32_t src_row;  // first row in T (group 0) or in the X rows (group 1)
  uint32_t nrows;
  uint32_t dst_k;    // first k of the group
  uint32_t group;
};

struct TcVUnit {
  uint64_t src;     // byte offset in the V stream
  uint32_t bytes;
  uint32_t xrow;    // X row of k = 0
  uint16_t kp;      // K (rows of V), multiple of 8
  uint16_t ncols;   // columns n (<= 64)
  uint32_t trow;    // T row of column 0 (final rows or a partial block)
  uint32_t flags;   // bit 0: first unit of a piece, bit 1: last unit
  uint32_t pad;
};

// T[dst + c] += sum_{q < nsrc} T[src + q * ncols + c], c < ncols
struct TcTReduce {
  uint32_t dst, src, ncols, nsrc;
};

// Fragment-ordering copy of one group of one unit from the FP64 arena:
// segments s = seg0 .. seg0 + nseg - 1 each give `ncols` consecutive columns
// starting at column `start`; mode 0: B[k][n] = a64[base + (k - start) * ld + n]
// (k = start ..), mode 1: B[k][n] = a64[base + (n - start) * ld + k].
struct TcFragTask {
  uint64_t dst;
  uint32_t dtype;  // 0 FP32, 1 BF16, 2 FP32 rounded to TF32 (dense leaves beside BF16 factors)
  uint32_t kp, nt;
  uint32_t kvalid, nvalid;
  uint32_t seg0, nseg;
  uint32_t mode;
};

struct TcSeg {
  uint64_t base;
  uint32_t ld, ncols, start, pad;
};

struct TcLayout {
  std::vector<TcVUnit> vunits;
  std::vector<TcRowUnit> runits;
  std::vector<TcSide> sides;
  std::vector<TcTReduce> treduce;
  std::vector<TcFragTask> vtasks, rtasks;
  std::vector<TcSeg> segs;
  std::vector<uint32_t> vranges, rranges;  // per consumer group: first unit (nparts + 1 entries)
  uint64_t vbytes = 0, rbytes = 0;
  uint32_t t_rows = 0;        // rows of T (final + partial blocks)
  uint64_t payload_bytes = 0;  // stored leaf bytes without padding
};

// lr_bf16: low-rank factors in BF16 (else FP32); pmax: right-hand sides the
// units are sized for; nparts: consumer groups of one sweep launch
// (grid * kTcGroups), each given a contiguous unit range; unit_bytes: cap of
// one unit's fragments + A rows (<= kTcSlotData)
void build_tc_layout(const std::vector<PlanLeaf>& leaves, bool lr_bf16, uint32_t pmax, uint32_t nparts,
                     TcLayout& L, uint32_t unit_bytes = kTcSlotData);

struct TcPlan {
  const TcVUnit* vunits = nullptr;
  const TcRowUnit* runits = nullptr;
  const TcSide* sides = nullptr;
  const TcTReduce* treduce = nullptr;
  const uint32_t* vranges = nullptr;
  const uint32_t* rranges = nullptr;
  uint32_t nvunits = 0, nrunits = 0, ntreduce = 0, grid = 0;
  const unsigned char* vstream = nullptr;
  const unsigned char* rstream = nullptr;
  uint64_t n = 0;
  void* xb = nullptr;   // X rows, BF16 (BF16 storage only)
  float* xf = nullptr;  // X rows, FP32
  void* t = nullptr;    // T rows (BF16 or FP32)
  float* yr = nullptr;  // Y rows, FP32, n x P
  int* err = nullptr;
  uint32_t pmax = 16;
};

cudaError_t tc_init_attributes();

// kernels launched by the products of this process (FP64 and mixed)
uint64_t product_launches();
void count_product_launches(uint64_t n);

cudaError_t launch_tc_build(const TcFragTask* tasks, uint32_t ntasks, const TcSeg* segs,
                            const double* arena64, unsigned char* dst, cudaStream_t s);
cudaError_t launch_matvec_tc(int prec, const TcPlan& plan, double d, uint32_t p, const double* X,
                             uint64_t ldX, double* Y, uint64_t ldY, cudaStream_t s);

// Contiguous unit ranges balancing bytes over `grid` parts (grid + 1 boundaries).
void balance_ranges(const std::vector<uint64_t>& bytes, uint32_t grid, std::vector<uint32_t>& first);

}  // namespace ahx
