// Internal state of an H-matrix handle (shared by the C-ABI translation units).
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <string>
#include <vector>

#include "../../include/ahx.h"
#include "ahx_matvec.cuh"
#include "ahx_tree.hpp"

namespace ahx {

void set_error(const std::string& msg);
int cuda_fail(cudaError_t e, const char* where);

#define AHX_CUDA(call)                                    \
  do {                                                    \
    cudaError_t e_ = (call);                              \
    if (e_ != cudaSuccess) return ::ahx::cuda_fail(e_, #call); \
  } while (0)

// Device buffer owned by a handle.
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  int reserve(size_t b);  // grow-only
  void release();
  template <class T>
  T* as() const { return static_cast<T*>(p); }
};

// A temporary device buffer released when the scope ends (error paths included).
struct ScopedBuf : DevBuf {
  ScopedBuf() = default;
  ScopedBuf(const ScopedBuf&) = delete;
  ScopedBuf& operator=(const ScopedBuf&) = delete;
  ~ScopedBuf() { release(); }
};

// The product's view of one storage precision.
struct ProdCopy {
  bool valid = false;
  DevBuf lr, dn;           // FP64 product: arena (lr) when it is not the handle's own
  DevBuf leaves, order;    // FP64 product: MvLeaf[nleaves], uint32 launch order
  uint32_t nleaves = 0;
  DevBuf tleaves, torder;  // symmetric tree, FP64: the off-diagonal leaves applied transposed
  uint32_t ntleaves = 0;
  uint64_t bytes = 0;      // stored leaf bytes of this precision
  // mixed-precision fragment streams (FP32 / BF16 products, tensor cores)
  DevBuf vstream, rstream, vunits, runits, sides, vranges, rranges, treduce, xb, xf, yr, t, err;
  uint32_t nvunits = 0, nrunits = 0, grid = 0, t_rows = 0, ntreduce = 0, pmax = 16;
  uint32_t unit_bytes = 0;  // unit cap the streams were built with
  // FP32 leaves on the tcgen05 path (ahx_umma.cuh), products of >= 2 right-hand sides
  bool um_valid = false;
  DevBuf um_vstream, um_rstream, um_vtiles, um_rtiles, um_zero, um_z, um_vranges, um_rranges, um_tacc, um_xmax;
  DevBuf um_vcranges, um_rcranges, um_vzidx, um_rzidx;
  uint32_t um_nv = 0, um_nr = 0, um_nzero = 0, um_trows = 0, um_grid = 0;
  uint64_t um_payload = 0, um_stream_bytes = 0;
  void release_um() {
    for (DevBuf* b : {&um_vstream, &um_rstream, &um_vtiles, &um_rtiles, &um_zero, &um_z, &um_vranges, &um_rranges,
                      &um_tacc, &um_xmax, &um_vcranges, &um_rcranges, &um_vzidx, &um_rzidx})
      b->release();
    um_valid = false;
    um_nv = um_nr = um_nzero = um_trows = um_grid = 0;
    um_payload = um_stream_bytes = 0;
  }
  void release_all() {
    for (DevBuf* b : {&lr, &dn, &leaves, &order, &tleaves, &torder, &vstream, &rstream, &vunits, &runits, &sides,
                      &vranges, &rranges, &treduce, &xb, &xf, &yr, &t, &err})
      b->release();
    valid = false;
    bytes = 0;
    nleaves = ntleaves = nvunits = nrunits = grid = t_rows = ntreduce = 0;
    release_um();
  }
};

// Complex (Helmholtz) leaves of a handle's block tree in the mblock<dcomp>
// layout (low rank: U (n1 x k) then V (n2 x k), the block U V^H; dense: n1 x n2
// column-major), complex elements interleaved (re, im).
struct ZState {
  bool assembled = false;
  double k = 0.0, h = 0.0, eps = 0.0;
  std::vector<int32_t> rank, aca_rank;  // per leaf, -1 dense
  std::vector<uint64_t> off;            // complex element offset of each leaf
  DevBuf arena;                         // complex128 elements
  uint64_t elems = 0;
  DevBuf arena32;                       // complex64 copy (AHX_FP32 storage)
  bool valid32 = false;
  DevBuf leaves, order;                 // product leaf table, launch order
  uint32_t nleaves = 0;
  DevBuf tleaves, torder;               // symmetric tree: the off-diagonal leaves, applied transposed
  uint32_t ntleaves = 0;
  bool table = false;
  DevBuf gm;                            // GMRES workspace
  DevBuf xc;                            // conjugated right-hand sides (adjoint of a symmetric matrix)
  void release_all() {
    for (DevBuf* b : {&arena, &arena32, &leaves, &order, &tleaves, &torder, &gm, &xc}) b->release();
    assembled = valid32 = table = false;
    elems = 0;
    nleaves = ntleaves = 0;
  }
};

// Workspace budget of one ACA batch (bytes); AHX_ACA_WS_BYTES overrides.
inline size_t aca_ws_budget() {
  const char* e = std::getenv("AHX_ACA_WS_BYTES");
  if (e && *e) return (size_t)std::strtoull(e, nullptr, 10);
  return (size_t)4 << 30;
}

// first capacity of the ACA rank workspace per leaf; AHX_ACA_KCAP overrides
inline uint32_t aca_kcap_default() {
  const char* e = std::getenv("AHX_ACA_KCAP");
  if (e && *e) return std::max<uint32_t>(1u, (uint32_t)std::strtoul(e, nullptr, 10));
  return 48u;
}

// ACA rank bound of a leaf: unsigned arithmetic as in Include/apprx.h:143-144
inline uint32_t maxk_of(uint32_t n1, uint32_t n2, uint32_t rankmax) {
  uint32_t maxk = (uint32_t)(n1 * n2) / (n1 + n2) + 4u;
  return maxk > rankmax ? rankmax : maxk;
}

// Largest useful ACA column capacity of a leaf with rank bound kmax.  The
// reference allocates kmax + 1 columns (Include/ACA.h:231-232) because its
// column loop takes one more cross when the row loop stops at k == kmax
// (Include/ACA.h:311-334); that cross decides between success (no pivot left)
// and failure.  A capacity of kmax + 1 therefore never overflows, and the
// retry loops of the assembly end.
inline uint32_t kcap_limit(uint32_t kmax) { return kmax + 1u; }

template <class T>
int upload(DevBuf& b, const std::vector<T>& v, cudaStream_t s) {
  if (v.empty()) return AHX_OK;
  int rc = b.reserve(v.size() * sizeof(T));
  if (rc) return rc;
  AHX_CUDA(cudaMemcpyAsync(b.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s));
  return AHX_OK;
}

// Builds the streams of a mixed precision from FP64 leaves (offsets into arena64).
// pmax / unit_bytes 0: the defaults (64 for BF16 factors, 16 for FP32; kTcSlotData)
int build_mixed_streams(ProdCopy& pc, int prec, const std::vector<PlanLeaf>& leaves,
                        const double* arena64, uint64_t n, int device, cudaStream_t s, uint32_t pmax = 0,
                        uint32_t unit_bytes = 0);
TcPlan mixed_plan(const ProdCopy& pc, uint64_t n);
// Reports (and clears) a timeout raised by a streaming kernel.
int check_stream_error(ProdCopy& pc, cudaStream_t s);

}  // namespace ahx

struct ahx_hmat {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  ahx::Tree tree;
  ahx::DevBuf pts;  // permuted SoA: x[n] y[n] z[n]
  // assembly
  bool assembled = false;
  double h = 0.0, eps = 0.0;
  std::vector<int32_t> rank, aca_rank;
  std::vector<uint64_t> off;  // element offset of each leaf in arena64
  ahx::DevBuf arena64;
  uint64_t arena64_elems = 0;
  ahx::ProdCopy prod[ahx::kNumPrecisions];
  ahx::ZState z;  // Helmholtz (complex) leaves, when assembled
  // staging buffers for host vectors
  ahx::DevBuf stage_x, stage_y;
  ahx::DevBuf scratch;  // solver scratch
  // statistics of the last assembly
  uint64_t stat_ws_bytes = 0;   // largest ACA workspace batch (bytes)
  uint64_t stat_retries = 0;    // leaves re-run with a larger rank capacity
  uint64_t stat_batches = 0;    // workspace batches
};

namespace ahx {
int prepare_product(ahx_hmat* H, int prec);
// FP32 leaves as tcgen05 streams (ahx_umma.cuh); AHX_UMMA=0 keeps every FP32 product on the mma.sync sweeps
int prepare_um(ahx_hmat* H);
bool um_enabled();
// kDF64 product scratch for p right-hand sides (the split X), ahead of graph capture
int prepare_df_x(ahx::ProdCopy& pc, uint64_t n, uint32_t p);
// Y += d A X in double-float over a leaf table and pc.lr (the split FP64 arena)
int run_df(const ahx::MvLeaf* leaves, const uint32_t* order, uint32_t nleaves, ahx::ProdCopy& pc, uint64_t n,
           double d, uint32_t p, const double* X, uint64_t ldX, double* Y, uint64_t ldY, cudaStream_t s);
int ensure_device(ahx_hmat* H);
// Reserves count doubles at the end of the FP64 leaf arena (grows it, stream-ordered).
int arena_append(ahx_hmat* H, uint64_t count, uint64_t& off);
// Drops every precision's product copy (after the leaves change).
void invalidate_products(ahx_hmat* H);
// Y += d A X on device pointers
// Y += d A X (transposed: Y += d A^T X, plain FP64 leaves only)
int product_device(ahx_hmat* H, int prec, double d, uint32_t p, const double* X, uint64_t ldX,
                   double* Y, uint64_t ldY, bool transposed = false);
bool is_device_ptr(const void* p);
// Reserves count complex elements at the end of the Helmholtz leaf arena (ahx_aca_helm.cu).
int zarena_append(ahx_hmat* H, uint64_t count, uint64_t& off);
// Leaf table of a product in descending cost order (ahx_capi.cu)
int upload_leaf_table(ahx_hmat* H, const std::vector<PlanLeaf>& pls, DevBuf& leaves, DevBuf& order, uint32_t& n);
// Helmholtz leaves: Y += d op(A) X on device pointers (prec kFP64: complex128
// leaves; kFP32: complex64 leaves, FP32 accumulation)
int zproduct_device(ahx_hmat* H, int prec, int op, double dre, double dim, uint32_t p, const double2* X,
                    uint64_t ldX, double2* Y, uint64_t ldY);
}  // namespace ahx
