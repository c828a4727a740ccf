// Batched ACA assembly of admissible leaves with SVD recompression, and the
// dense fill of inadmissible leaves (FP64 throughout).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "ahx_device.cuh"

namespace ahx {

// One admissible leaf to approximate.  Workspace layout at `ws` (doubles):
//   U[n1*kcap] V[n2*kcap] Un[n1*kcap] Vn[n2*kcap] R[kcap*kcap] Vs[kcap*kcap] sig[kcap]
//   tau[2*kcap]
// and at `zs` (ints): Z[n1] S[n2]  (ACA.h:38-42 row/column success counters).
struct AcaTask {
  uint32_t b1, n1, b2, n2;
  uint32_t i0, kmax, kcap, leaf;
  uint64_t ws;
  uint64_t zs;
};

enum AcaStatus : int32_t { kAcaFail = 0, kAcaOk = 1, kAcaOverflow = 2 };

// ACA of the general assembly (Include/ACA.h:217-350) or ACAr of the symmetric one
// (Include/ACA.h:657-720, Include/apprx.h:86-132)
enum AcaVariant : int32_t { kAcaVariantGeneral = 0, kAcaVariantSym = 1 };

struct AcaResult {
  int32_t status;
  uint32_t k_aca;  // rank returned by ACA (before recompression)
  uint32_t kt;     // rank after recompression
  uint32_t pad;
};

// 64-bit throughout: n1 + n2 and kcap * kcap overflow 32 bits for large blocks
inline uint64_t aca_ws_doubles(uint32_t n1, uint32_t n2, uint32_t kcap) {
  const uint64_t n = (uint64_t)n1 + n2, k = kcap;
  return 2ull * n * k + 2ull * k * k + 3ull * k;
}

struct AcaParams {
  PointsSoA pts;
  double diag;  // 1/(4 pi h)
  double eps;
  const AcaTask* tasks;
  uint32_t ntasks;
  double* ws;
  int* zs;
  AcaResult* res;
  int32_t variant = kAcaVariantGeneral;
};

// Launchers (ahx_aca.cu)
cudaError_t launch_aca_small(const AcaParams& p, cudaStream_t s);  // one warp per leaf
cudaError_t launch_aca_large(const AcaParams& p, cudaStream_t s);  // one CTA per leaf

// Dense leaves: fill n1 x n2 column-major blocks of the generator.
struct DenseTask {
  uint32_t b1, n1, b2, n2;
  uint64_t off;  // element offset in the arena
};
cudaError_t launch_dense_fill(const PointsSoA& pts, double diag, const DenseTask* tasks,
                              uint32_t ntasks, double* arena, cudaStream_t s);

// Mirror image of an upper block of a symmetric H-matrix into the same arena:
// rank > 0: U (n1 x rank), V (n2 x rank) at src -> V, U at dst (the leaf V U^T);
// rank < 0: the n1 x n2 block at src -> its transpose (n2 x n1) at dst.
struct MirrorTask {
  uint64_t src, dst;
  uint32_t n1, n2;
  int32_t rank;
  uint32_t pad;
};
cudaError_t launch_mirror(const MirrorTask* tasks, uint32_t ntasks, double* arena, cudaStream_t s);

// Agglomeration: recompression of merged sibling blocks.  Workspace at `ws`
// (doubles, aca_ws_doubles(m, n, k) + merge_qrcp_doubles(k)): U (m x k) and V
// (n x k) hold the gathered factors; Un, Vn receive the result; `zs` (ints):
// m + n + 1 scratch.
inline uint64_t merge_qrcp_doubles(uint32_t k) { return (uint64_t)k * k + 3ull * k; }
struct MergeTask {
  uint32_t m, n, k, pad;
  uint64_t ws, zs;
};
struct MergeParams {
  const MergeTask* tasks;
  uint32_t ntasks;
  double* ws;
  int* zs;
  double eps;
  AcaResult* res;  // k_aca = k, kt = recompressed rank
};
// large: one CTA per task (m or n above 4096), else one warp
cudaError_t launch_merge(const MergeParams& p, bool large, cudaStream_t s);
// Complex unions (ahx_aca_helm.cu): the same tasks and workspace layout in complex
// elements (MergeParams::ws holds them as interleaved doubles), one warp per union.
cudaError_t launch_zmerge(const MergeParams& p, cudaStream_t s);
// dst[s.dst + c * ld_dst + r] = src[s.src + c * nrows + r], r < nrows, c < ncols;
// src == kSegIdentity: ones on the diagonal (r == c) of the zeroed destination,
// at dst[s.dst + c * ld_dst + c * (1 + cplx)] (cplx = 1: the real parts of a
// complex identity stored as interleaved doubles)
constexpr uint64_t kSegIdentity = ~0ull;
struct Seg2D {
  uint64_t src, dst;
  uint32_t nrows, ncols, ld_dst, cplx;
};
cudaError_t launch_copy2d(const Seg2D* segs, uint32_t nsegs, const double* src, double* dst, cudaStream_t s);

// Copy recompressed factors (Un, Vn, kt columns) from the workspace into the arena.
struct CopyTask {
  uint64_t src_u, src_v;  // workspace offsets (doubles)
  uint64_t dst;           // arena offset
  uint32_t n1, n2, kt, pad;
};
cudaError_t launch_copy_factors(const CopyTask* tasks, uint32_t ntasks, const double* ws,
                                double* arena, cudaStream_t s);

}  // namespace ahx
