// Batched H-matrix product Y += d A X over all leaves (dense and low-rank),
// for any number of right-hand sides and any number of H-matrix instances.
#pragma once
#include <cstdint>
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

}  // namespace ahx
