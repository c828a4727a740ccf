// C ABI of libahx: handle management, trees, assembly driver, product.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <new>
#include <numeric>

#include <cuda_bf16.h>

#include "ahx_aca.cuh"
#include "ahx_hmat.hpp"
#include "ahx_umma.cuh"

namespace ahx {

namespace {
thread_local std::string g_err;

// leaves with more rows or columns than this use the CTA-per-leaf kernel; the
// rest run one warp per leaf (warp reductions; the FP64 pipe is the limit)
constexpr uint32_t kLargeLeaf = 4096;

// Runs ACA + recompression for `tasks` in workspace-bounded batches, appends the
// factors to the arena; failed leaves go to `dense`, capacity overflows to `retry`.
int run_aca(ahx_hmat* H, std::vector<AcaTask>& tasks, double diag, double eps,
            std::vector<uint32_t>& dense, std::vector<AcaTask>& retry) {
  const size_t budget = aca_ws_budget();
  std::sort(tasks.begin(), tasks.end(), [](const AcaTask& a, const AcaTask& b) {
    return (uint64_t)(a.n1 + a.n2) * a.kcap > (uint64_t)(b.n1 + b.n2) * b.kcap;
  });
  DevBuf ws, zs, dtasks, dres, dcopy;
  size_t i = 0;
  while (i < tasks.size()) {
    // gather one batch
    std::vector<AcaTask> small, large;
    uint64_t wsd = 0, zsi = 0;
    size_t j = i;
    while (j < tasks.size()) {
      AcaTask t = tasks[j];
      const uint64_t w = aca_ws_doubles(t.n1, t.n2, t.kcap);
      if (j > i && (wsd + w) * 8 + (zsi + t.n1 + t.n2) * 4 > budget) break;
      t.ws = wsd;
      t.zs = zsi;
      wsd += w;
      zsi += t.n1 + t.n2;
      (std::max(t.n1, t.n2) > kLargeLeaf ? large : small).push_back(t);
      ++j;
    }
    i = j;
    H->stat_ws_bytes = std::max<uint64_t>(H->stat_ws_bytes, wsd * sizeof(double) + zsi * sizeof(int));
    H->stat_batches++;
    int rc = ws.reserve(std::max<uint64_t>(wsd, 1) * sizeof(double));
    if (rc) return rc;
    rc = zs.reserve(std::max<uint64_t>(zsi, 1) * sizeof(int));
    if (rc) return rc;
    std::vector<AcaTask> all(large);
    all.insert(all.end(), small.begin(), small.end());
    if ((rc = upload(dtasks, all, H->stream))) return rc;
    rc = dres.reserve(all.size() * sizeof(AcaResult));
    if (rc) return rc;
    AcaParams p;
    const double* pts = H->pts.as<double>();
    p.pts = PointsSoA{pts, pts + H->tree.n, pts + 2 * (size_t)H->tree.n};
    p.diag = diag;
    p.eps = eps;
    p.variant = H->tree.sym ? kAcaVariantSym : kAcaVariantGeneral;
    p.ws = ws.as<double>();
    p.zs = zs.as<int>();
    p.tasks = dtasks.as<AcaTask>();
    p.res = dres.as<AcaResult>();
    p.ntasks = (uint32_t)large.size();
    AHX_CUDA(launch_aca_large(p, H->stream));
    p.tasks = dtasks.as<AcaTask>() + large.size();
    p.res = dres.as<AcaResult>() + large.size();
    p.ntasks = (uint32_t)small.size();
    AHX_CUDA(launch_aca_small(p, H->stream));
    std::vector<AcaResult> res(all.size());
    AHX_CUDA(cudaMemcpyAsync(res.data(), dres.p, res.size() * sizeof(AcaResult),
                             cudaMemcpyDeviceToHost, H->stream));
    AHX_CUDA(cudaStreamSynchronize(H->stream));
    std::vector<CopyTask> copies;
    for (size_t q = 0; q < all.size(); ++q) {
      const AcaTask& t = all[q];
      const AcaResult& r = res[q];
      // an overflow at the full capacity cannot happen (kcap_limit); were it
      // to, the leaf is treated as an ACA failure so that the loop ends
      if (r.status == kAcaOverflow && t.kcap < kcap_limit(t.kmax)) {
        AcaTask u = t;
        u.kcap = std::min(kcap_limit(t.kmax), std::max(t.kcap * 4, 16u));
        retry.push_back(u);
        H->stat_retries++;
        continue;
      }
      if (r.status != kAcaOk) {
        dense.push_back(t.leaf);
        continue;
      }
      H->aca_rank[t.leaf] = (int32_t)r.k_aca;
      H->rank[t.leaf] = (int32_t)r.kt;
      if (r.kt == 0) continue;
      uint64_t off = 0;
      if ((rc = arena_append(H, (uint64_t)r.kt * (t.n1 + t.n2), off))) return rc;
      H->off[t.leaf] = off;
      const uint64_t un = t.ws + (uint64_t)(t.n1 + t.n2) * t.kcap;  // Un follows U and V
      CopyTask c;
      c.src_u = un;
      c.src_v = un + (uint64_t)t.n1 * t.kcap;
      c.dst = off;
      c.n1 = t.n1;
      c.n2 = t.n2;
      c.kt = r.kt;
      c.pad = 0;
      copies.push_back(c);
    }
    if (!copies.empty()) {
      if ((rc = upload(dcopy, copies, H->stream))) return rc;
      AHX_CUDA(launch_copy_factors(dcopy.as<CopyTask>(), (uint32_t)copies.size(), ws.as<double>(),
                                   H->arena64.as<double>(), H->stream));
    }
    AHX_CUDA(cudaStreamSynchronize(H->stream));
  }
  ws.release();
  zs.release();
  dtasks.release();
  dres.release();
  dcopy.release();
  return AHX_OK;
}

}  // namespace

// Append-only growable FP64 arena.
int arena_append(ahx_hmat* H, uint64_t count, uint64_t& off) {
  const uint64_t need = (H->arena64_elems + count) * sizeof(double);
  if (need > H->arena64.bytes) {
    size_t nb = std::max<size_t>(need, H->arena64.bytes * 2);
    void* np = nullptr;
    cudaError_t e = cudaMalloc(&np, nb);
    if (e != cudaSuccess) {
      cudaGetLastError();
      nb = need;
      e = cudaMalloc(&np, nb);
      if (e != cudaSuccess) {
        cudaGetLastError();
        set_error("device allocation of the leaf arena failed");
        return AHX_ERR_NOMEM;
      }
    }
    if (H->arena64_elems)
      AHX_CUDA(cudaMemcpyAsync(np, H->arena64.p, H->arena64_elems * sizeof(double),
                               cudaMemcpyDeviceToDevice, H->stream));
    AHX_CUDA(cudaStreamSynchronize(H->stream));
    if (H->arena64.p) cudaFree(H->arena64.p);
    H->arena64.p = np;
    H->arena64.bytes = nb;
  }
  off = H->arena64_elems;
  H->arena64_elems += count;
  return AHX_OK;
}

void invalidate_products(ahx_hmat* H) {
  for (auto& pc : H->prod) pc.release_all();
}

void set_error(const std::string& msg) { g_err = msg; }

int prepare_df_x(ProdCopy& pc, uint64_t n, uint32_t p) {
  return pc.xb.reserve(std::max<uint64_t>(n * p, 1) * 8);
}

int run_df(const MvLeaf* leaves, const uint32_t* order, uint32_t nleaves, ProdCopy& pc, uint64_t n, double d,
           uint32_t p, const double* X, uint64_t ldX, double* Y, uint64_t ldY, cudaStream_t s) {
  int rc = prepare_df_x(pc, n, p);
  if (rc) return rc;
  AHX_CUDA(launch_split_df(X, ldX, n, p, d, pc.xb.p, s));
  DfArgs a;
  a.leaves = leaves;
  a.order = order;
  a.nleaves = nleaves;
  a.arena = pc.lr.as<float2>();
  a.X = pc.xb.as<float2>();
  a.ldX = n;
  a.p = p;
  a.Y = Y;
  a.ldY = ldY;
  AHX_CUDA(launch_matvec_df(a, s));
  return AHX_OK;
}

int cuda_fail(cudaError_t e, const char* where) {
  g_err = std::string(where) + ": " + cudaGetErrorString(e);
  cudaGetLastError();
  return e == cudaErrorMemoryAllocation ? AHX_ERR_NOMEM : AHX_ERR_CUDA;
}

int DevBuf::reserve(size_t b) {
  if (b <= bytes) return AHX_OK;
  release();
  cudaError_t e = cudaMalloc(&p, b);
  if (e != cudaSuccess) {
    p = nullptr;
    return cuda_fail(e, "cudaMalloc");
  }
  bytes = b;
  return AHX_OK;
}

void DevBuf::release() {
  if (p) cudaFree(p);
  p = nullptr;
  bytes = 0;
}

bool is_device_ptr(const void* ptr) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// The leaves a product reads as a general H-matrix.  A symmetric tree stores the
// diagonal and upper blocks only; its blocks below the diagonal are the mirror
// images (V U^T, D^T) of the upper ones, written into `tmp` after a copy of the
// leaf arena.  `arena` is the arena the returned offsets refer to.
int full_leaves(ahx_hmat* H, std::vector<PlanLeaf>& pls, DevBuf& tmp, const double*& arena) {
  const auto& Ls = H->tree.leaves;
  const uint32_t nl = (uint32_t)Ls.size();
  pls.clear();
  for (uint32_t l = 0; l < nl; ++l)
    if (H->rank[l] != 0) pls.push_back(PlanLeaf{Ls[l].b1, Ls[l].n1, Ls[l].b2, Ls[l].n2, H->rank[l], H->off[l]});
  arena = H->arena64.as<double>();
  if (!H->tree.sym) return AHX_OK;
  std::vector<MirrorTask> mt;
  uint64_t end = H->arena64_elems;
  for (uint32_t l = 0; l < nl; ++l) {
    const Leaf& L = Ls[l];
    const int32_t r = H->rank[l];
    if (r == 0 || L.b1 == L.b2) continue;
    const uint64_t cnt = r < 0 ? (uint64_t)L.n1 * L.n2 : (uint64_t)r * (L.n1 + L.n2);
    mt.push_back(MirrorTask{H->off[l], end, L.n1, L.n2, r, 0u});
    pls.push_back(PlanLeaf{L.b2, L.n2, L.b1, L.n1, r, end});
    end += cnt;
  }
  int rc = tmp.reserve(std::max<uint64_t>(end, 1) * sizeof(double));
  if (rc) return rc;
  if (H->arena64_elems)
    AHX_CUDA(cudaMemcpyAsync(tmp.p, H->arena64.p, H->arena64_elems * sizeof(double), cudaMemcpyDeviceToDevice,
                             H->stream));
  ScopedBuf dmt;
  if ((rc = upload(dmt, mt, H->stream))) return rc;
  AHX_CUDA(launch_mirror(dmt.as<MirrorTask>(), (uint32_t)mt.size(), tmp.as<double>(), H->stream));
  AHX_CUDA(cudaStreamSynchronize(H->stream));
  dmt.release();
  arena = tmp.as<double>();
  return AHX_OK;
}

// Leaf table of the FP64-class products (descending cost order).  transposed:
// the off-diagonal blocks of a symmetric tree, applied as their transposes.
int upload_leaf_table(ahx_hmat* H, const std::vector<PlanLeaf>& pls, DevBuf& leaves, DevBuf& order, uint32_t& n) {
  std::vector<MvLeaf> mv;
  std::vector<uint64_t> cost;
  mv.reserve(pls.size());
  for (const PlanLeaf& q : pls) {
    MvLeaf m;
    m.b1 = q.b1;
    m.n1 = q.n1;
    m.b2 = q.b2;
    m.n2 = q.n2;
    m.rank = q.rank;
    m.dense_in_lr_arena = 1;
    m.off = q.off;
    mv.push_back(m);
    cost.push_back(q.rank < 0 ? (uint64_t)q.n1 * q.n2 : (uint64_t)q.rank * (q.n1 + q.n2));
  }
  std::vector<uint32_t> ord(mv.size());
  std::iota(ord.begin(), ord.end(), 0u);
  std::stable_sort(ord.begin(), ord.end(), [&](uint32_t a, uint32_t b) { return cost[a] > cost[b]; });
  int rc;
  if ((rc = upload(leaves, mv, H->stream))) return rc;
  if ((rc = upload(order, ord, H->stream))) return rc;
  n = (uint32_t)mv.size();
  return AHX_OK;
}

int prepare_product(ahx_hmat* H, int prec) {
  if (prec < 0 || prec >= kNumPrecisions) {
    set_error("unknown precision");
    return AHX_ERR_ARG;
  }
  ProdCopy& pc = H->prod[prec];
  if (pc.valid) return AHX_OK;
  const auto& Ls = H->tree.leaves;
  const uint32_t nl = (uint32_t)Ls.size();
  int rc;
  if (prec == kDF64) {
    // the FP64 leaves split into (hi, lo) float pairs; a symmetric tree's mirror
    // images are materialised, with their own leaf table
    if ((rc = prepare_product(H, kFP64))) return rc;
    std::vector<PlanLeaf> pls;
    ScopedBuf tmp;
    const double* src = nullptr;
    if ((rc = full_leaves(H, pls, tmp, src))) return rc;
    uint64_t elems = H->arena64_elems;
    for (const PlanLeaf& q : pls)
      elems = std::max<uint64_t>(elems, q.off + (q.rank < 0 ? (uint64_t)q.n1 * q.n2 : (uint64_t)q.rank * (q.n1 + q.n2)));
    if ((rc = pc.lr.reserve(std::max<uint64_t>(elems, 1) * 8))) return rc;
    AHX_CUDA(launch_split_df(src, elems, elems, 1, 1.0, pc.lr.p, H->stream));
    if (H->tree.sym && (rc = upload_leaf_table(H, pls, pc.leaves, pc.order, pc.nleaves))) return rc;
    AHX_CUDA(cudaStreamSynchronize(H->stream));
    tmp.release();
    pc.bytes = elems * 8;
    pc.valid = true;
    return AHX_OK;
  }
  if (prec != kFP64) {
    std::vector<PlanLeaf> pls;
    ScopedBuf tmp;
    const double* src = nullptr;
    if ((rc = full_leaves(H, pls, tmp, src))) return rc;
    rc = build_mixed_streams(pc, prec, pls, src, H->tree.n, H->device, H->stream);
    tmp.release();
    if (rc) return rc;
    pc.valid = true;
    return AHX_OK;
  }
  // every stored leaf; for a symmetric tree the off-diagonal ones again, applied
  // transposed (H/mltaGeHVec.cpp:421-446)
  std::vector<PlanLeaf> all, upper;
  for (uint32_t l = 0; l < nl; ++l) {
    const Leaf& L = Ls[l];
    if (H->rank[l] == 0) continue;
    const PlanLeaf q{L.b1, L.n1, L.b2, L.n2, H->rank[l], H->off[l]};
    all.push_back(q);
    if (H->tree.sym && L.b1 != L.b2) upper.push_back(q);
  }
  if ((rc = upload_leaf_table(H, all, pc.leaves, pc.order, pc.nleaves))) return rc;
  pc.ntleaves = 0;
  if (!upper.empty() && (rc = upload_leaf_table(H, upper, pc.tleaves, pc.torder, pc.ntleaves))) return rc;
  pc.bytes = H->arena64_elems * sizeof(double);
  AHX_CUDA(cudaStreamSynchronize(H->stream));
  pc.valid = true;
  return AHX_OK;
}

int build_mixed_streams(ProdCopy& pc, int prec, const std::vector<PlanLeaf>& leaves,
                        const double* arena64, uint64_t n, int device, cudaStream_t s, uint32_t pmax,
                        uint32_t unit_bytes) {
  const bool bf = prec == kBF16FP32;
  if (!bf || pmax == 0) pmax = bf ? 64u : 16u;  // FP32 storage: 16 per pass
  if (unit_bytes == 0 || unit_bytes > kTcSlotData) unit_bytes = kTcSlotData;
  int sms = 0;
  AHX_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  const uint32_t grid = (uint32_t)std::max(sms, 1);
  TcLayout L;
  build_tc_layout(leaves, bf, pmax, grid * kTcGroups, L, unit_bytes);
  {
    // every unit (fragments + its A rows) must fit one ring slot
    const uint64_t s_t = (uint64_t)(pmax + 8) * (bf ? 2 : 4), s_x = (uint64_t)(pmax + 8) * 4;
    for (const TcVUnit& u : L.vunits)
      if (u.bytes + u.kp * s_t > kTcSlotData) {
        set_error("mixed product layout: a V unit exceeds the ring slot");
        return AHX_ERR_ARG;
      }
    for (const TcRowUnit& u : L.runits)
      if (u.bytes + u.kp0 * s_t + u.kp1 * s_x > kTcSlotData) {
        set_error("mixed product layout: a rows unit exceeds the ring slot");
        return AHX_ERR_ARG;
      }
  }
  AHX_CUDA(tc_init_attributes());
  int rc;
  if ((rc = pc.vstream.reserve(std::max<uint64_t>(L.vbytes, 16)))) return rc;
  if ((rc = pc.rstream.reserve(std::max<uint64_t>(L.rbytes, 16)))) return rc;
  if ((rc = upload(pc.vunits, L.vunits, s))) return rc;
  if ((rc = upload(pc.runits, L.runits, s))) return rc;
  if ((rc = upload(pc.sides, L.sides, s))) return rc;
  if ((rc = upload(pc.vranges, L.vranges, s))) return rc;
  if ((rc = upload(pc.rranges, L.rranges, s))) return rc;
  if ((rc = upload(pc.treduce, L.treduce, s))) return rc;
  pc.ntreduce = (uint32_t)L.treduce.size();
  // X / T rows carry 16 zero rows past the end (read as K padding)
  const uint64_t xrows = std::max<uint64_t>(n, 1) + 16, trows = (uint64_t)L.t_rows + 16;
  const uint64_t es = bf ? 2 : 4;
  if ((rc = pc.xf.reserve(xrows * (pmax + 8) * 4))) return rc;
  if (bf && (rc = pc.xb.reserve(xrows * (pmax + 8) * 2))) return rc;
  if ((rc = pc.yr.reserve(std::max<uint64_t>(n, 1) * pmax * 4))) return rc;
  if ((rc = pc.t.reserve(trows * (pmax + 8) * es))) return rc;
  if ((rc = pc.err.reserve(sizeof(int)))) return rc;
  AHX_CUDA(cudaMemsetAsync(pc.xf.p, 0, xrows * (pmax + 8) * 4, s));
  if (bf) AHX_CUDA(cudaMemsetAsync(pc.xb.p, 0, xrows * (pmax + 8) * 2, s));
  AHX_CUDA(cudaMemsetAsync(pc.t.p, 0, trows * (pmax + 8) * es, s));
  AHX_CUDA(cudaMemsetAsync(pc.err.p, 0, sizeof(int), s));
  // fragment-ordered streams (padding stays zero)
  AHX_CUDA(cudaMemsetAsync(pc.vstream.p, 0, std::max<uint64_t>(L.vbytes, 16), s));
  AHX_CUDA(cudaMemsetAsync(pc.rstream.p, 0, std::max<uint64_t>(L.rbytes, 16), s));
  DevBuf dt, dseg;
  if ((rc = upload(dseg, L.segs, s))) return rc;
  if (!L.vtasks.empty()) {
    if ((rc = upload(dt, L.vtasks, s))) return rc;
    AHX_CUDA(launch_tc_build(dt.as<TcFragTask>(), (uint32_t)L.vtasks.size(), dseg.as<TcSeg>(), arena64,
                             pc.vstream.as<unsigned char>(), s));
    AHX_CUDA(cudaStreamSynchronize(s));
  }
  if (!L.rtasks.empty()) {
    if ((rc = upload(dt, L.rtasks, s))) return rc;
    AHX_CUDA(launch_tc_build(dt.as<TcFragTask>(), (uint32_t)L.rtasks.size(), dseg.as<TcSeg>(), arena64,
                             pc.rstream.as<unsigned char>(), s));
  }
  AHX_CUDA(cudaStreamSynchronize(s));
  dt.release();
  dseg.release();
  pc.nvunits = (uint32_t)L.vunits.size();
  pc.nrunits = (uint32_t)L.runits.size();
  pc.grid = grid;
  pc.t_rows = L.t_rows;
  pc.pmax = pmax;
  pc.unit_bytes = unit_bytes;
  pc.bytes = L.payload_bytes;
  return AHX_OK;
}

bool um_enabled() {
  static const bool on = [] {
    const char* e = std::getenv("AHX_UMMA");
    return !(e && e[0] == '0');
  }();
  return on;
}

int prepare_um(ahx_hmat* H) {
  ProdCopy& pc = H->prod[kFP32];
  if (pc.um_valid) return AHX_OK;
  std::vector<PlanLeaf> pls;
  ScopedBuf tmp;
  const double* src = nullptr;
  int rc;
  if ((rc = full_leaves(H, pls, tmp, src))) return rc;
  UmLayout L;
  int sms = 0;
  AHX_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, H->device));
  const uint32_t grid = (uint32_t)std::max(sms, 1);
  // AHX_UM_KPIECE: V-sweep tiles longer than this are split along K (default 4096)
  const char* kp = std::getenv("AHX_UM_KPIECE");
  build_um_layout(pls, H->tree.n, grid, L, (kp && *kp) ? (uint32_t)std::strtoul(kp, nullptr, 10) : 4096u);
  AHX_CUDA(um_init_attributes());
  pc.release_um();
  if ((rc = pc.um_vstream.reserve(std::max<uint64_t>(L.vbytes, 16)))) return rc;
  if ((rc = pc.um_rstream.reserve(std::max<uint64_t>(L.rbytes, 16)))) return rc;
  if ((rc = upload(pc.um_vtiles, L.vtiles, H->stream))) return rc;
  if ((rc = upload(pc.um_rtiles, L.rtiles, H->stream))) return rc;
  if ((rc = upload(pc.um_zero, L.zero, H->stream))) return rc;
  if ((rc = upload(pc.um_vranges, L.vranges, H->stream))) return rc;
  if ((rc = upload(pc.um_rranges, L.rranges, H->stream))) return rc;
  if ((rc = upload(pc.um_vcranges, L.vcranges, H->stream))) return rc;
  if ((rc = upload(pc.um_rcranges, L.rcranges, H->stream))) return rc;
  if ((rc = pc.um_vzidx.reserve(std::max<uint64_t>(L.vchunks * kUmIdxBytes, 16)))) return rc;
  if ((rc = pc.um_rzidx.reserve(std::max<uint64_t>(L.rchunks * kUmIdxBytes, 16)))) return rc;
  // Z rows: X rows, T rows, one 256-byte row of FP16 pairs each (64 right-hand-side slots)
  const uint64_t zrows = H->tree.n + (uint64_t)L.t_rows + 1;
  if ((rc = pc.um_z.reserve(zrows * kUmZPitch))) return rc;
  AHX_CUDA(cudaMemsetAsync(pc.um_z.p, 0, zrows * kUmZPitch, H->stream));
  // FP32 accumulation rows of split V tiles (zero between products)
  if ((rc = pc.um_tacc.reserve(std::max<uint64_t>((uint64_t)L.tacc_rows * 64 * sizeof(float), 16)))) return rc;
  AHX_CUDA(cudaMemsetAsync(pc.um_tacc.p, 0, std::max<uint64_t>((uint64_t)L.tacc_rows * 64 * sizeof(float), 16),
                           H->stream));
  if ((rc = pc.um_xmax.reserve(64 * sizeof(uint32_t)))) return rc;
  if ((rc = pc.err.reserve(sizeof(int)))) return rc;
  AHX_CUDA(cudaMemsetAsync(pc.err.p, 0, sizeof(int), H->stream));
  {
    ScopedBuf de, db, dj, dts;
    if ((rc = dts.reserve(std::max<uint64_t>((uint64_t)L.t_rows * sizeof(float), 16)))) return rc;
    if ((rc = upload(dj, L.tjobs, H->stream))) return rc;
    cudaError_t ce = launch_um_tscale(dj.as<UmTJob>(), (uint32_t)L.tjobs.size(), src, dts.as<float>(), H->stream);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(H->stream);
    dj.release();
    if (ce == cudaSuccess) {
      if ((rc = upload(de, L.entries, H->stream))) return rc;
      if ((rc = upload(db, L.vbuild, H->stream))) {
        de.release();
        return rc;
      }
      ce = launch_um_build(db.as<UmBuild>(), (uint32_t)L.vbuild.size(), de.as<UmEntry>(), src, dts.as<float>(),
                           H->tree.n, pc.um_vstream.as<unsigned char>(), pc.um_vzidx.as<uint32_t>(), H->stream);
      if (ce == cudaSuccess) ce = cudaStreamSynchronize(H->stream);
      db.release();
      if (ce == cudaSuccess && (rc = upload(db, L.rbuild, H->stream)) == AHX_OK) {
        ce = launch_um_build(db.as<UmBuild>(), (uint32_t)L.rbuild.size(), de.as<UmEntry>(), src, dts.as<float>(),
                             H->tree.n, pc.um_rstream.as<unsigned char>(), pc.um_rzidx.as<uint32_t>(), H->stream);
        if (ce == cudaSuccess) ce = cudaStreamSynchronize(H->stream);
      }
    }
    db.release();
    de.release();
    dts.release();
    if (rc) return rc;
    AHX_CUDA(ce);
  }
  tmp.release();
  pc.um_nv = (uint32_t)L.vtiles.size();
  pc.um_nr = (uint32_t)L.rtiles.size();
  pc.um_nzero = (uint32_t)L.zero.size();
  pc.um_trows = L.t_rows;
  pc.um_grid = grid;
  pc.um_payload = L.payload_bytes;
  pc.um_stream_bytes = L.stream_bytes;
  pc.um_valid = true;
  return AHX_OK;
}

UmPlan um_plan(ProdCopy& pc, uint64_t n) {
  UmPlan pl;
  pl.vtiles = pc.um_vtiles.as<UmTile>();
  pl.rtiles = pc.um_rtiles.as<UmTile>();
  pl.vranges = pc.um_vranges.as<uint32_t>();
  pl.rranges = pc.um_rranges.as<uint32_t>();
  pl.vcranges = pc.um_vcranges.as<uint32_t>();
  pl.rcranges = pc.um_rcranges.as<uint32_t>();
  pl.vzidx = pc.um_vzidx.as<uint32_t>();
  pl.rzidx = pc.um_rzidx.as<uint32_t>();
  pl.grid = pc.um_grid;
  pl.nvtiles = pc.um_nv;
  pl.nrtiles = pc.um_nr;
  pl.vstream = pc.um_vstream.as<unsigned char>();
  pl.rstream = pc.um_rstream.as<unsigned char>();
  pl.zero = pc.um_zero.as<UmRange>();
  pl.nzero = pc.um_nzero;
  pl.n = n;
  pl.t_rows = pc.um_trows;
  pl.z = pc.um_z.as<uint16_t>();
  pl.tacc = pc.um_tacc.as<float>();
  pl.xmax = pc.um_xmax.as<uint32_t>();
  pl.err = pc.err.as<int>();
  return pl;
}

TcPlan mixed_plan(const ProdCopy& pc, uint64_t n) {
  TcPlan pl;
  pl.vunits = pc.vunits.as<TcVUnit>();
  pl.runits = pc.runits.as<TcRowUnit>();
  pl.sides = pc.sides.as<TcSide>();
  pl.treduce = pc.treduce.as<TcTReduce>();
  pl.vranges = pc.vranges.as<uint32_t>();
  pl.rranges = pc.rranges.as<uint32_t>();
  pl.nvunits = pc.nvunits;
  pl.nrunits = pc.nrunits;
  pl.ntreduce = pc.ntreduce;
  pl.grid = pc.grid;
  pl.vstream = pc.vstream.as<unsigned char>();
  pl.rstream = pc.rstream.as<unsigned char>();
  pl.n = n;
  pl.xb = pc.xb.p;
  pl.xf = pc.xf.as<float>();
  pl.t = pc.t.p;
  pl.yr = pc.yr.as<float>();
  pl.err = pc.err.as<int>();
  pl.pmax = pc.pmax;
  return pl;
}

int check_stream_error(ProdCopy& pc, cudaStream_t s) {
  if (!pc.err.p) return AHX_OK;
  int e = 0;
  AHX_CUDA(cudaMemcpyAsync(&e, pc.err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  AHX_CUDA(cudaStreamSynchronize(s));
  if (e) {
    AHX_CUDA(cudaMemsetAsync(pc.err.p, 0, sizeof(int), s));
    set_error("a streaming product kernel timed out waiting for its shared-memory pipeline");
    return AHX_ERR_CUDA;
  }
  return AHX_OK;
}

int product_device(ahx_hmat* H, int prec, double d, uint32_t p, const double* X, uint64_t ldX,
                   double* Y, uint64_t ldY, bool transposed) {
  if (transposed && H->tree.sym) transposed = false;  // A^T = A
  if (transposed && prec != kFP64) {
    set_error("transposed products use the FP64 leaves");
    return AHX_ERR_ARG;
  }
  int rc;
  if (prec == kFP32 && p >= 2 && um_enabled()) {
    // FP32 leaves, several right-hand sides: the tcgen05 sweeps
    if ((rc = prepare_um(H))) return rc;
    const UmPlan pl = um_plan(H->prod[kFP32], H->tree.n);
    AHX_CUDA(launch_matvec_um(pl, d, p, X, ldX, Y, ldY, H->stream));
    return AHX_OK;
  }
  rc = prepare_product(H, prec);
  if (rc) return rc;
  ProdCopy& pc = H->prod[prec];
  if (prec == kDF64) {
    if ((rc = prepare_df_x(pc, H->tree.n, p))) return rc;
    const ProdCopy& f = H->tree.sym ? pc : H->prod[kFP64];
    return run_df(f.leaves.as<MvLeaf>(), f.order.as<uint32_t>(), f.nleaves, pc, H->tree.n, d, p, X, ldX, Y,
                  ldY, H->stream);
  }
  if (prec != kFP64) {
    const TcPlan pl = mixed_plan(pc, H->tree.n);
    AHX_CUDA(launch_matvec_tc(prec, pl, d, p, X, ldX, Y, ldY, H->stream));
    return AHX_OK;
  }
  MvArgs a;
  a.leaves = pc.leaves.as<MvLeaf>();
  a.order = pc.order.as<uint32_t>();
  a.nleaves = pc.nleaves;
  a.arena_lr = prec == kFP64 ? H->arena64.p : pc.lr.p;
  a.arena_dn = pc.dn.p;
  a.d = d;
  a.p = p;
  a.X = X;
  a.ldX = ldX;
  a.Y = Y;
  a.ldY = ldY;
  a.transposed = transposed ? 1u : 0u;
  AHX_CUDA(launch_matvec(prec, a, H->stream));
  if (pc.ntleaves) {
    // symmetric tree: the blocks below the diagonal are the upper ones transposed
    a.leaves = pc.tleaves.as<MvLeaf>();
    a.order = pc.torder.as<uint32_t>();
    a.nleaves = pc.ntleaves;
    a.transposed = 1u;
    AHX_CUDA(launch_matvec(prec, a, H->stream));
  }
  return AHX_OK;
}

int ensure_device(ahx_hmat* H) {
  AHX_CUDA(cudaSetDevice(H->device));
  if (!H->stream) {
    AHX_CUDA(cudaStreamCreateWithFlags(&H->stream, cudaStreamNonBlocking));
    H->own_stream = true;
  }
  if (!H->pts.p) {
    const uint32_t n = H->tree.n;
    std::vector<double> soa(3 * (size_t)n);
    for (uint32_t i = 0; i < n; ++i) {
      const uint32_t o = H->tree.op_perm[i];
      for (int j = 0; j < 3; ++j) soa[(size_t)j * n + i] = H->tree.pts[3 * (size_t)o + j];
    }
    int rc = upload(H->pts, soa, H->stream);
    if (rc) return rc;
    AHX_CUDA(cudaStreamSynchronize(H->stream));
  }
  return AHX_OK;
}

}  // namespace ahx

using namespace ahx;

extern "C" {

const char* ahx_last_error(void) { return g_err.c_str(); }

int ahx_version(void) { return 10000; }

double ahx_mean_nn(const double* pts, uint32_t n) {
  if (!pts) return 0.0;
  return mean_nn(pts, n);
}

uint64_t ahx_kernel_launches(void) { return product_launches(); }

double ahx_min_nn(const double* pts, uint32_t n) {
  if (!pts) return 0.0;
  double mn = 0.0;
  mean_nn(pts, n, &mn);
  return mn;
}

static int create_impl(const double* pts, uint32_t n, int tree_kind, uint32_t bmin, double eta2, int device,
                       void* stream, ahx_hmat** out, bool sym) {
  if (!out || !pts || n == 0 || bmin == 0 || (tree_kind != AHX_TREE_BBX && tree_kind != AHX_TREE_PCA) ||
      !(eta2 >= 0.0) || device < 0) {
    set_error("ahx_hmat_create: invalid argument");
    return AHX_ERR_ARG;
  }
  *out = nullptr;
  ahx_hmat* H = new (std::nothrow) ahx_hmat;
  if (!H) {
    set_error("host allocation failed");
    return AHX_ERR_NOMEM;
  }
  H->device = device;
  H->stream = (cudaStream_t)stream;
  // trees are host work; the device is touched on the first device call
  build_tree(H->tree, pts, n, tree_kind, bmin, eta2, sym);
  *out = H;
  return AHX_OK;
}

int ahx_hmat_create(const double* pts, uint32_t n, int tree_kind, uint32_t bmin, double eta2,
                    int device, void* stream, ahx_hmat** out) {
  return create_impl(pts, n, tree_kind, bmin, eta2, device, stream, out, false);
}

int ahx_hmat_create_sym(const double* pts, uint32_t n, int tree_kind, uint32_t bmin, double eta2,
                        int device, void* stream, ahx_hmat** out) {
  return create_impl(pts, n, tree_kind, bmin, eta2, device, stream, out, true);
}

int ahx_hmat_symmetric(const ahx_hmat* H) { return H && H->tree.sym ? 1 : 0; }

int ahx_hmat_destroy(ahx_hmat* H) {
  if (!H) return AHX_OK;
  const bool touched = H->stream || H->pts.p;
  if (touched) cudaSetDevice(H->device);
  // only a stream this handle created is synchronized; work queued on a
  // caller's stream is ordered before the frees by cudaFree's device sync
  if (H->own_stream && H->stream) cudaStreamSynchronize(H->stream);
  invalidate_products(H);
  H->pts.release();
  H->arena64.release();
  H->stage_x.release();
  H->stage_y.release();
  H->scratch.release();
  H->z.release_all();
  if (H->own_stream && H->stream) cudaStreamDestroy(H->stream);
  delete H;
  return AHX_OK;
}

int ahx_hmat_set_stream(ahx_hmat* H, void* stream) {
  if (!H) return AHX_ERR_ARG;
  if (H->stream) {
    AHX_CUDA(cudaSetDevice(H->device));
    AHX_CUDA(cudaStreamSynchronize(H->stream));
    if (H->own_stream) cudaStreamDestroy(H->stream);
  }
  H->own_stream = false;
  H->stream = (cudaStream_t)stream;  // NULL: a private stream is created on next use
  return AHX_OK;
}

void* ahx_hmat_stream(const ahx_hmat* H) { return H ? (void*)H->stream : nullptr; }
uint32_t ahx_hmat_n(const ahx_hmat* H) { return H ? H->tree.n : 0; }
uint32_t ahx_hmat_nleaves(const ahx_hmat* H) { return H ? (uint32_t)H->tree.leaves.size() : 0; }

int ahx_hmat_perm(const ahx_hmat* H, uint32_t* op_perm, uint32_t* po_perm) {
  if (!H) return AHX_ERR_ARG;
  if (op_perm) std::memcpy(op_perm, H->tree.op_perm.data(), H->tree.n * sizeof(uint32_t));
  if (po_perm) std::memcpy(po_perm, H->tree.po_perm.data(), H->tree.n * sizeof(uint32_t));
  return AHX_OK;
}

int ahx_hmat_leaves(const ahx_hmat* H, uint32_t* out) {
  if (!H || !out) return AHX_ERR_ARG;
  for (size_t l = 0; l < H->tree.leaves.size(); ++l) {
    const Leaf& L = H->tree.leaves[l];
    uint32_t* o = out + 7 * l;
    o[0] = L.b1;
    o[1] = L.n1;
    o[2] = L.b2;
    o[3] = L.n2;
    o[4] = L.adm;
    o[5] = L.idx;
    o[6] = L.i0;
  }
  return AHX_OK;
}

int ahx_assemble(ahx_hmat* H, double h, double eps, uint32_t rankmax) {
  return ahx_assemble_hinted(H, h, eps, rankmax, nullptr);
}

int ahx_assemble_hinted(ahx_hmat* H, double h, double eps, uint32_t rankmax,
                        const float* rank_hint) {
  if (!H || !(h > 0.0) || !(eps > 0.0)) {
    set_error("ahx_assemble: invalid argument");
    return AHX_ERR_ARG;
  }
  int rc = ensure_device(H);
  if (rc) return rc;
  invalidate_products(H);
  H->assembled = false;
  H->h = h;
  H->eps = eps;
  const auto& Ls = H->tree.leaves;
  const uint32_t nl = (uint32_t)Ls.size();
  H->rank.assign(nl, -1);
  H->aca_rank.assign(nl, -1);
  H->off.assign(nl, 0);
  H->arena64_elems = 0;
  H->stat_ws_bytes = H->stat_retries = H->stat_batches = 0;
  const double diag = 1.0 / (kFourPi * h);
  std::vector<AcaTask> tasks;
  std::vector<uint32_t> dense;
  const uint32_t kcap0 = aca_kcap_default();
  for (uint32_t l = 0; l < nl; ++l) {
    const Leaf& L = Ls[l];
    const uint32_t maxk = maxk_of(L.n1, L.n2, rankmax);
    if (L.adm && maxk) {
      AcaTask t{};
      t.b1 = L.b1;
      t.n1 = L.n1;
      t.b2 = L.b2;
      t.n2 = L.n2;
      t.i0 = L.i0;
      t.kmax = maxk;
      t.kcap = std::min(kcap_limit(maxk), kcap0);
      if (rank_hint && rank_hint[l] >= 0.f) {
        // predicted rank plus a margin; an under-prediction only costs a retry
        const float want = rank_hint[l] * 1.25f + 4.f;
        t.kcap = std::min(kcap_limit(maxk), std::max(8u, (uint32_t)std::ceil(want)));
      }
      t.leaf = l;
      tasks.push_back(t);
    } else {
      dense.push_back(l);
    }
  }
  // estimated arena capacity: dense leaves plus about 16 columns per low-rank leaf
  uint64_t est = 0;
  for (uint32_t l : dense) est += (uint64_t)Ls[l].n1 * Ls[l].n2;
  for (const AcaTask& t : tasks) est += (uint64_t)(t.n1 + t.n2) * std::min(t.kmax, 16u);
  if (H->arena64.bytes < est * sizeof(double)) {
    H->arena64.release();
    rc = H->arena64.reserve(std::max<uint64_t>(est, 1) * sizeof(double));
    if (rc) return rc;
  }
  while (!tasks.empty()) {
    std::vector<AcaTask> retry;
    if ((rc = run_aca(H, tasks, diag, eps, dense, retry))) return rc;
    tasks.swap(retry);
  }
  // dense leaves (inadmissible and failed ACA), filled in leaf order
  std::sort(dense.begin(), dense.end());
  std::vector<DenseTask> dt;
  for (uint32_t l : dense) {
    const Leaf& L = Ls[l];
    uint64_t off = 0;
    if ((rc = arena_append(H, (uint64_t)L.n1 * L.n2, off))) return rc;
    H->off[l] = off;
    H->rank[l] = -1;
    H->aca_rank[l] = -1;
    dt.push_back(DenseTask{L.b1, L.n1, L.b2, L.n2, off});
  }
  if (!dt.empty()) {
    DevBuf ddt;
    if ((rc = upload(ddt, dt, H->stream))) return rc;
    const double* pts = H->pts.as<double>();
    PointsSoA P{pts, pts + H->tree.n, pts + 2 * (size_t)H->tree.n};
    AHX_CUDA(launch_dense_fill(P, diag, ddt.as<DenseTask>(), (uint32_t)dt.size(),
                               H->arena64.as<double>(), H->stream));
    AHX_CUDA(cudaStreamSynchronize(H->stream));
  }
  AHX_CUDA(cudaStreamSynchronize(H->stream));
  H->assembled = true;
  return AHX_OK;
}

int ahx_hmat_assembly_stats(const ahx_hmat* H, uint64_t* out) {
  if (!H || !out) return AHX_ERR_ARG;
  out[0] = H->stat_ws_bytes;
  out[1] = H->stat_retries;
  out[2] = H->stat_batches;
  return AHX_OK;
}

// Autotuner for the mixed-precision streams: for each candidate bucketing (the
// right-hand-side width the units are sized for: 64 / 32 / 16 with BF16
// factors, 16 with FP32 storage; the unit byte cap: 11, 8.25 or 5.5 KB) it
// builds the streams, times 3 products with p right-hand sides after one
// warm-up (CUDA events on the handle's stream) and keeps the fastest.
// out4 = {chosen width, chosen unit cap, best time in ns, candidates timed}.
int ahx_hmat_autotune(ahx_hmat* H, int precision, uint32_t p, uint32_t* out4) {
  if (!H || p == 0 || (precision != AHX_FP32 && precision != AHX_BF16_FP32)) {
    set_error("ahx_hmat_autotune: invalid argument (mixed precisions only)");
    return AHX_ERR_ARG;
  }
  if (!H->assembled) {
    set_error("not assembled");
    return AHX_ERR_STATE;
  }
  int rc = ensure_device(H);
  if (rc) return rc;
  const int prec = precision == AHX_FP32 ? kFP32 : kBF16FP32;
  std::vector<PlanLeaf> pls;
  ScopedBuf full;
  const double* src = nullptr;
  if ((rc = full_leaves(H, pls, full, src))) return rc;
  const uint64_t n = H->tree.n;
  DevBuf X, Y;
  if ((rc = X.reserve(n * p * sizeof(double))) || (rc = Y.reserve(n * p * sizeof(double)))) return rc;
  AHX_CUDA(cudaMemsetAsync(X.p, 0, n * p * sizeof(double), H->stream));
  AHX_CUDA(cudaMemsetAsync(Y.p, 0, n * p * sizeof(double), H->stream));
  std::vector<uint32_t> widths = prec == kBF16FP32 ? std::vector<uint32_t>{64u, 32u, 16u} : std::vector<uint32_t>{16u};
  const uint32_t units[3] = {kTcSlotData, (kTcSlotData * 3 / 4) & ~15u, (kTcSlotData / 2) & ~15u};
  cudaEvent_t e0, e1;
  AHX_CUDA(cudaEventCreate(&e0));
  AHX_CUDA(cudaEventCreate(&e1));
  float best = INFINITY;
  uint32_t bw = widths[0], bu = units[0], count = 0;
  for (uint32_t w : widths) {
    for (uint32_t u : units) {
      ProdCopy cand;
      if ((rc = build_mixed_streams(cand, prec, pls, src, n, H->device, H->stream, w, u))) {
        cand.release_all();
        break;
      }
      const TcPlan pl = mixed_plan(cand, n);
      cudaError_t ce = launch_matvec_tc(prec, pl, 1.0, p, X.as<double>(), n, Y.as<double>(), n, H->stream);
      if (ce == cudaSuccess) ce = cudaEventRecord(e0, H->stream);
      for (int r = 0; r < 3 && ce == cudaSuccess; ++r)
        ce = launch_matvec_tc(prec, pl, 1.0, p, X.as<double>(), n, Y.as<double>(), n, H->stream);
      if (ce == cudaSuccess) ce = cudaEventRecord(e1, H->stream);
      if (ce == cudaSuccess) ce = cudaEventSynchronize(e1);
      float ms = 0.f;
      if (ce == cudaSuccess) ce = cudaEventElapsedTime(&ms, e0, e1);
      const int se = check_stream_error(cand, H->stream);
      cand.release_all();
      if (ce != cudaSuccess) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        return cuda_fail(ce, "autotune");
      }
      if (se) {
        rc = se;
        break;
      }
      ++count;
      if (ms < best) {
        best = ms;
        bw = w;
        bu = u;
      }
    }
    if (rc) break;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  X.release();
  Y.release();
  if (rc) {
    full.release();
    return rc;
  }
  ProdCopy& pc = H->prod[prec];
  pc.release_all();
  rc = build_mixed_streams(pc, prec, pls, src, n, H->device, H->stream, bw, bu);
  full.release();
  if (rc) return rc;
  pc.valid = true;
  if (out4) {
    out4[0] = bw;
    out4[1] = bu;
    out4[2] = (uint32_t)std::min(best / 3.f * 1e6f, 4e9f);
    out4[3] = count;
  }
  return AHX_OK;
}

int ahx_hmat_features(const ahx_hmat* H, double wavenumber, double eps, float* out) {
  if (!H || !out) return AHX_ERR_ARG;
  for (size_t l = 0; l < H->tree.leaves.size(); ++l)
    leaf_features(H->tree, H->tree.leaves[l], wavenumber, eps, out + 8 * l);
  return AHX_OK;
}

int ahx_hmat_ranks(const ahx_hmat* H, int32_t* ranks) {
  if (!H || !ranks) return AHX_ERR_ARG;
  if (!H->assembled) {
    set_error("not assembled");
    return AHX_ERR_STATE;
  }
  std::memcpy(ranks, H->rank.data(), H->rank.size() * sizeof(int32_t));
  return AHX_OK;
}

int ahx_hmat_aca_ranks(const ahx_hmat* H, int32_t* ranks) {
  if (!H || !ranks) return AHX_ERR_ARG;
  if (!H->assembled) {
    set_error("not assembled");
    return AHX_ERR_STATE;
  }
  std::memcpy(ranks, H->aca_rank.data(), H->aca_rank.size() * sizeof(int32_t));
  return AHX_OK;
}

// a dense diagonal leaf of a symmetric tree is Hermitian (mblock::setHeM): its data
// is the packed upper triangle (Include/apprx.h:122-126)
static bool packed_leaf(const ahx_hmat* H, uint32_t l) {
  const Leaf& L = H->tree.leaves[l];
  return H->tree.sym && L.b1 == L.b2 && H->rank[l] < 0;
}

uint64_t ahx_hmat_leaf_size(const ahx_hmat* H, uint32_t l) {
  if (!H || !H->assembled || l >= H->tree.leaves.size()) return 0;
  const Leaf& L = H->tree.leaves[l];
  const int32_t r = H->rank[l];
  if (packed_leaf(H, l)) return (uint64_t)L.n1 * (L.n1 + 1) / 2;
  return r < 0 ? (uint64_t)L.n1 * L.n2 : (uint64_t)r * (L.n1 + L.n2);
}

int ahx_hmat_get_leaf(const ahx_hmat* H, uint32_t l, double* out) {
  if (!H || !out || l >= H->tree.leaves.size()) return AHX_ERR_ARG;
  if (!H->assembled) {
    set_error("not assembled");
    return AHX_ERR_STATE;
  }
  const uint64_t cnt = ahx_hmat_leaf_size(H, l);
  if (!cnt) return AHX_OK;
  AHX_CUDA(cudaSetDevice(H->device));
  if (packed_leaf(H, l)) {
    const uint32_t n1 = H->tree.leaves[l].n1;
    std::vector<double> full((uint64_t)n1 * n1);
    AHX_CUDA(cudaMemcpyAsync(full.data(), H->arena64.as<double>() + H->off[l], full.size() * sizeof(double),
                             cudaMemcpyDeviceToHost, H->stream));
    AHX_CUDA(cudaStreamSynchronize(H->stream));
    for (uint32_t j = 0; j < n1; ++j)
      for (uint32_t i = 0; i <= j; ++i) out[i + (uint64_t)j * (j + 1) / 2] = full[i + (uint64_t)j * n1];
    return AHX_OK;
  }
  AHX_CUDA(cudaMemcpyAsync(out, H->arena64.as<double>() + H->off[l], cnt * sizeof(double),
                           cudaMemcpyDeviceToHost, H->stream));
  AHX_CUDA(cudaStreamSynchronize(H->stream));
  return AHX_OK;
}

int ahx_hmat_set_leaves(ahx_hmat* H, const int32_t* ranks, const double* data,
                        const uint64_t* offsets) {
  if (!H || !ranks || !offsets) return AHX_ERR_ARG;
  const auto& Ls = H->tree.leaves;
  const uint32_t nl = (uint32_t)Ls.size();
  // dense diagonal leaves of a symmetric tree may come packed (mblock HeM data)
  std::vector<uint64_t> expand;
  for (uint32_t l = 0; l < nl; ++l) {
    const uint64_t want = ranks[l] < 0 ? (uint64_t)Ls[l].n1 * Ls[l].n2
                                       : (uint64_t)ranks[l] * (Ls[l].n1 + Ls[l].n2);
    const uint64_t got = offsets[l + 1] >= offsets[l] ? offsets[l + 1] - offsets[l] : ~0ull;
    const bool packed = H->tree.sym && ranks[l] < 0 && Ls[l].b1 == Ls[l].b2 && Ls[l].n1 > 1 &&
                        got == (uint64_t)Ls[l].n1 * (Ls[l].n1 + 1) / 2;
    if (packed) {
      expand.push_back(l);
    } else if (got != want) {
      set_error("ahx_hmat_set_leaves: offsets do not match the leaf sizes");
      return AHX_ERR_ARG;
    }
  }
  if (!expand.empty()) {
    std::vector<double> full;
    std::vector<uint64_t> offs(nl + 1, 0);
    for (uint32_t l = 0; l < nl; ++l) {
      const uint64_t want = ranks[l] < 0 ? (uint64_t)Ls[l].n1 * Ls[l].n2
                                         : (uint64_t)ranks[l] * (Ls[l].n1 + Ls[l].n2);
      offs[l + 1] = offs[l] + want;
    }
    full.resize(offs[nl]);
    size_t e = 0;
    for (uint32_t l = 0; l < nl; ++l) {
      const double* src = data + offsets[l];
      double* dst = full.data() + offs[l];
      if (e < expand.size() && expand[e] == l) {
        ++e;
        const uint32_t n1 = Ls[l].n1;
        for (uint32_t j = 0; j < n1; ++j)
          for (uint32_t i = 0; i <= j; ++i) {
            const double v = src[i + (uint64_t)j * (j + 1) / 2];
            dst[i + (uint64_t)j * n1] = v;
            dst[j + (uint64_t)i * n1] = v;
          }
      } else {
        std::copy(src, src + (offs[l + 1] - offs[l]), dst);
      }
    }
    return ahx_hmat_set_leaves(H, ranks, full.data(), offs.data());
  }
  int rc = ensure_device(H);
  if (rc) return rc;
  invalidate_products(H);
  const uint64_t total = offsets[nl];
  H->arena64.release();
  rc = H->arena64.reserve(std::max<uint64_t>(total, 1) * sizeof(double));
  if (rc) return rc;
  if (total) {
    if (!data) return AHX_ERR_ARG;
    AHX_CUDA(cudaMemcpyAsync(H->arena64.p, data, total * sizeof(double), cudaMemcpyHostToDevice,
                             H->stream));
  }
  AHX_CUDA(cudaStreamSynchronize(H->stream));
  H->arena64_elems = total;
  H->rank.assign(ranks, ranks + nl);
  H->aca_rank.assign(ranks, ranks + nl);
  H->off.assign(offsets, offsets + nl);
  H->assembled = true;
  return AHX_OK;
}

uint64_t ahx_hmat_storage_bytes(ahx_hmat* H, int precision) {
  if (!H || !H->assembled) return 0;
  if (ensure_device(H)) return 0;
  if (precision == kFP32 && um_enabled()) {
    if (prepare_um(H)) return 0;
    return H->prod[kFP32].um_payload;
  }
  if (prepare_product(H, precision)) return 0;
  return H->prod[precision].bytes;
}

int ahx_hmat_stream_bytes(ahx_hmat* H, int precision, uint64_t* out) {
  if (!H || !out || precision != kFP32) return AHX_ERR_ARG;
  if (!H->assembled) return AHX_ERR_STATE;
  int rc = ensure_device(H);
  if (rc) return rc;
  if ((rc = prepare_um(H))) return rc;
  *out = H->prod[kFP32].um_stream_bytes;
  return AHX_OK;
}

int ahx_timing(int enable) {
  um_timing_enable(enable != 0);
  return AHX_OK;
}

int ahx_timing_read(double* ms2, uint64_t* count2, int reset) {
  if (!ms2 || !count2) return AHX_ERR_ARG;
  um_timing_read(ms2, count2, reset != 0);
  return AHX_OK;
}

int ahx_hmat_prepare(ahx_hmat* H, int precision) {
  if (!H) return AHX_ERR_ARG;
  if (!H->assembled) {
    set_error("not assembled");
    return AHX_ERR_STATE;
  }
  int rc = ensure_device(H);
  if (rc) return rc;
  if (precision == kFP32 && um_enabled()) return prepare_um(H);
  return prepare_product(H, precision);
}

int ahx_hmat_release(ahx_hmat* H, int precision) {
  if (!H || precision < 0 || precision >= kNumPrecisions) return AHX_ERR_ARG;
  if (precision == kFP64) return AHX_OK;  // the handle's own leaves
  int rc = ensure_device(H);
  if (rc) return rc;
  AHX_CUDA(cudaStreamSynchronize(H->stream));
  H->prod[precision].release_all();
  return AHX_OK;
}

namespace {
int matvec_any(ahx_hmat* H, int precision, double d, uint32_t p, const double* X, uint64_t ldX, double* Y,
               uint64_t ldY, bool transposed) {
  if (!H || !X || !Y || ldX < H->tree.n || ldY < H->tree.n) {
    set_error("ahx_matvec: invalid argument");
    return AHX_ERR_ARG;
  }
  if (!H->assembled) {
    set_error("ahx_matvec: H-matrix not assembled");
    return AHX_ERR_STATE;
  }
  if (p == 0) return AHX_OK;
  int rc = ensure_device(H);
  if (rc) return rc;
  const uint64_t n = H->tree.n;
  const bool xd = is_device_ptr(X), yd = is_device_ptr(Y);
  const double* Xd = X;
  double* Yd = Y;
  uint64_t lx = ldX, ly = ldY;
  if (!xd) {
    if ((rc = H->stage_x.reserve(n * p * sizeof(double)))) return rc;
    AHX_CUDA(cudaMemcpy2DAsync(H->stage_x.p, n * sizeof(double), X, ldX * sizeof(double),
                               n * sizeof(double), p, cudaMemcpyHostToDevice, H->stream));
    Xd = H->stage_x.as<double>();
    lx = n;
  }
  if (!yd) {
    if ((rc = H->stage_y.reserve(n * p * sizeof(double)))) return rc;
    AHX_CUDA(cudaMemcpy2DAsync(H->stage_y.p, n * sizeof(double), Y, ldY * sizeof(double),
                               n * sizeof(double), p, cudaMemcpyHostToDevice, H->stream));
    Yd = H->stage_y.as<double>();
    ly = n;
  }
  if ((rc = product_device(H, precision, d, p, Xd, lx, Yd, ly, transposed))) return rc;
  if (!yd) {
    AHX_CUDA(cudaMemcpy2DAsync(Y, ldY * sizeof(double), Yd, n * sizeof(double), n * sizeof(double),
                               p, cudaMemcpyDeviceToHost, H->stream));
  }
  if (!xd || !yd) {
    AHX_CUDA(cudaStreamSynchronize(H->stream));
    if (precision != kFP64) return check_stream_error(H->prod[precision], H->stream);
  }
  return AHX_OK;
}
}  // namespace

int ahx_matvec(ahx_hmat* H, int precision, double d, uint32_t p, const double* X, uint64_t ldX, double* Y,
               uint64_t ldY) {
  return matvec_any(H, precision, d, p, X, ldX, Y, ldY, false);
}

int ahx_matvec_transposed(ahx_hmat* H, double d, uint32_t p, const double* X, uint64_t ldX, double* Y,
                          uint64_t ldY) {
  return matvec_any(H, AHX_FP64, d, p, X, ldX, Y, ldY, true);
}

}  // extern "C"
