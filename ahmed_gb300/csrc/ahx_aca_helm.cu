// Complex ACA ranks of the Helmholtz single-layer matrix exp(i k r) / (4 pi r)
// (diagonal exp(i k h) / (4 pi h)): the reference's ACA with T = dcomp
// (Include/ACA.h:46-350; complex arithmetic of Include/cmplx.h:80-245: own
// complex type, |z| = sqrt(re^2 + im^2), a / z = a / |z|^2 * conj(z), scpr =
// sum conj(x) y), one warp per admissible leaf, every leaf with the
// reference's stopping rule and counters.  The factors are not kept: the
// entry point reports the rank per leaf (training data and verification of
// the rank predictor on oscillatory kernels).
#include <algorithm>
#include <cmath>
#include <vector>

#include "ahx_aca.cuh"
#include "ahx_hmat.hpp"

namespace ahx {
namespace {

constexpr int kWarps = 4;  // leaves per CTA

struct Cx {
  double re, im;
};

__device__ __forceinline__ double cabs2(Cx a) { return __dadd_rn(__dmul_rn(a.re, a.re), __dmul_rn(a.im, a.im)); }
__device__ __forceinline__ double cabs(Cx a) { return __dsqrt_rn(cabs2(a)); }
__device__ __forceinline__ Cx cconj(Cx a) { return Cx{a.re, -a.im}; }
__device__ __forceinline__ Cx nconj(Cx a) { return Cx{-a.re, a.im}; }
// y += a x (zaxpy)
__device__ __forceinline__ void caxpy(Cx a, Cx x, Cx& y) {
  y.re += a.re * x.re - a.im * x.im;
  y.im += a.re * x.im + a.im * x.re;
}
// a *= b (Include/cmplx.h:187-194)
__device__ __forceinline__ void cmul_eq(Cx& a, Cx b) {
  const double t = __dsub_rn(__dmul_rn(a.re, b.re), __dmul_rn(a.im, b.im));
  a.im = __dmul_rn(a.im, b.re);
  a.im = __dadd_rn(a.im, __dmul_rn(a.re, b.im));
  a.re = t;
}
// real / complex (Include/cmplx.h:235-241)
__device__ __forceinline__ Cx rdiv(double a, Cx b) {
  const double d = __ddiv_rn(a, cabs2(b));
  return Cx{__dmul_rn(b.re, d), __dmul_rn(b.im, -d)};
}

struct HBlk {
  PointsSoA P;
  double k, h;
  uint32_t b1, n1, b2, n2;
  Cx* U;
  Cx* V;
  int* Z;
  int* S;
};

__device__ __forceinline__ Cx helm_entry(const HBlk& B, uint32_t i, uint32_t j) {
  double r = B.h;
  if (i != j) {
    const double dx = __dsub_rn(B.P.x[i], B.P.x[j]);
    const double dy = __dsub_rn(B.P.y[i], B.P.y[j]);
    const double dz = __dsub_rn(B.P.z[i], B.P.z[j]);
    r = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)));
  }
  const double s = __ddiv_rn(1.0, __dmul_rn(kFourPi, r));
  double sn, cs;
  sincos(__dmul_rn(B.k, r), &sn, &cs);
  return Cx{__dmul_rn(cs, s), __dmul_rn(sn, s)};
}

using G32 = Group<32>;

__device__ uint32_t nexti(const G32& g, const int* Z, uint32_t n, uint32_t j) {
  uint32_t d = 0xffffffffu;
  for (uint32_t i = g.rank; i < n; i += 32)
    if (Z[i] != -1) d = min(d, i >= j ? i - j : i + n - j);
  d = G32::umin(d);
  return d == 0xffffffffu ? j : (j + d) % n;
}

// ACA_row_step (ACA.h:46-130), T = dcomp: V holds conjugated rows
__device__ bool row_step(const G32& g, const HBlk& B, uint32_t& klast, uint32_t& i0, uint32_t k, uint32_t& no,
                         double& nrmlsk2, double scale) {
  const uint32_t n1 = B.n1, n2 = B.n2;
  Cx* const pu = B.U + (size_t)k * n1;
  Cx* const pv = B.V + (size_t)k * n2;
  ArgMax am;
  for (;;) {
    __syncwarp();
    am = ArgMax{0.0, 0xffffffffu, 0.0};
    for (uint32_t j = g.rank; j < n2; j += 32) {
      Cx v = cconj(helm_entry(B, B.b1 + i0, B.b2 + j));
      for (uint32_t l = 0; l < k; ++l) caxpy(nconj(B.U[(size_t)l * n1 + i0]), B.V[(size_t)l * n2 + j], v);
      pv[j] = v;
      if (B.S[j] >= 0) {
        const double a = cabs(v);
        if (gt_nonneg(a, am.v)) am = ArgMax{a, j, 0.0};
      }
    }
    am = G32::argmax(am);
    if (!(am.v < 1e-14 * scale)) break;
    if (i0 % 32 == g.rank) B.Z[i0] = -1;
    if (++no >= n1) return false;
    __syncwarp();
    i0 = nexti(g, B.Z, n1, i0);
  }
  __syncwarp();
  const uint32_t j0 = am.idx;
  const double sqrtpiv = sqrt(am.v);
  const Cx sca = rdiv(sqrtpiv, pv[j0]);
  const double thr = 1e-8 * scale * sqrtpiv;
  __syncwarp();
  double nrmv2 = 0.0;
  for (uint32_t j = g.rank; j < n2; j += 32) {
    if (B.S[j] >= 0) {
      Cx e = pv[j];
      cmul_eq(e, sca);
      pv[j] = e;
      nrmv2 += cabs2(e);
      if (gt_nonneg(cabs(e), thr)) ++B.S[j];
    }
  }
  for (uint32_t i = g.rank; i < n1; i += 32) {
    Cx u = helm_entry(B, B.b1 + i, B.b2 + j0);
    for (uint32_t l = 0; l < k; ++l) caxpy(nconj(B.V[(size_t)l * n2 + j0]), B.U[(size_t)l * n1 + i], u);
    pu[i] = u;
  }
  klast = (uint32_t)G32::imax(i0 % 32 == g.rank ? B.Z[i0] : INT_MIN);
  if (i0 % 32 == g.rank) B.Z[i0] = -1;
  if (j0 % 32 == g.rank) B.S[j0] = -1;
  ++no;
  const double dsca = 1.0 / sqrtpiv;
  double nrmu2 = 0.0;
  ArgMax nm{0.0, 0xffffffffu, 0.0};
  for (uint32_t i = g.rank; i < n1; i += 32) {
    Cx e = pu[i];
    e.re *= dsca;
    e.im *= dsca;
    pu[i] = e;
    const double ea = cabs(e);
    if (B.Z[i] >= 0 && gt_nonneg(ea, thr)) ++B.Z[i];
    nrmu2 += ea * ea;
    if (B.Z[i] >= 0 && gt_nonneg(ea, nm.v)) nm = ArgMax{ea, i, 0.0};
  }
  G32::sum2(nrmu2, nrmv2);
  nm = G32::argmax(nm);
  if (nm.v > 0.0) i0 = nm.idx;
  nrmlsk2 = nrmu2 * nrmv2;
  return true;
}

// ACA_col_step (ACA.h:134-213), T = dcomp
__device__ bool col_step(const G32& g, const HBlk& B, uint32_t& j0, uint32_t k, uint32_t& no, double& nrmlsk2,
                         double scale) {
  const uint32_t n1 = B.n1, n2 = B.n2;
  Cx* const pu = B.U + (size_t)k * n1;
  Cx* const pv = B.V + (size_t)k * n2;
  ArgMax am;
  for (;;) {
    __syncwarp();
    am = ArgMax{0.0, 0xffffffffu, 0.0};
    for (uint32_t i = g.rank; i < n1; i += 32) {
      Cx u = helm_entry(B, B.b1 + i, B.b2 + j0);
      for (uint32_t l = 0; l < k; ++l) caxpy(nconj(B.V[(size_t)l * n2 + j0]), B.U[(size_t)l * n1 + i], u);
      pu[i] = u;
      if (B.Z[i] >= 0) {
        const double a = cabs(u);
        if (gt_nonneg(a, am.v)) am = ArgMax{a, i, 0.0};
      }
    }
    am = G32::argmax(am);
    if (!(am.v < 1e-14 * scale)) break;
    if (j0 % 32 == g.rank) B.S[j0] = -1;
    if (++no >= n2) return false;
    __syncwarp();
    j0 = nexti(g, B.S, n2, j0);
  }
  __syncwarp();
  const uint32_t i0 = am.idx;
  const double sqrtpiv = sqrt(am.v);
  const Cx sca = rdiv(sqrtpiv, pu[i0]);
  const double thr = 1e-8 * scale * sqrtpiv;
  __syncwarp();
  double nrmu2 = 0.0;
  for (uint32_t i = g.rank; i < n1; i += 32) {
    if (B.Z[i] >= 0) {
      Cx e = pu[i];
      cmul_eq(e, sca);
      pu[i] = e;
      nrmu2 += cabs2(e);
      if (gt_nonneg(cabs(e), thr)) ++B.Z[i];
    }
  }
  for (uint32_t j = g.rank; j < n2; j += 32) {
    Cx v = cconj(helm_entry(B, B.b1 + i0, B.b2 + j));
    for (uint32_t l = 0; l < k; ++l) caxpy(nconj(B.U[(size_t)l * n1 + i0]), B.V[(size_t)l * n2 + j], v);
    pv[j] = v;
  }
  if (i0 % 32 == g.rank) B.Z[i0] = -1;
  if (j0 % 32 == g.rank) B.S[j0] = -1;
  ++no;
  const double dsca = 1.0 / sqrtpiv;
  double nrmv2 = 0.0;
  ArgMax nm{0.0, 0xffffffffu, 0.0};
  for (uint32_t j = g.rank; j < n2; j += 32) {
    Cx e = pv[j];
    e.re *= dsca;
    e.im *= dsca;
    pv[j] = e;
    const double ea = cabs(e);
    if (B.S[j] >= 0 && gt_nonneg(ea, thr)) ++B.S[j];
    nrmv2 += ea * ea;
    if (gt_nonneg(ea, nm.v)) nm = ArgMax{ea, j, 0.0};  // no S filter, as in the reference
  }
  G32::sum2(nrmu2, nrmv2);
  nm = G32::argmax(nm);
  if (nm.v > 0.0) j0 = nm.idx;
  nrmlsk2 = nrmu2 * nrmv2;
  return true;
}

// ACA driver (ACA.h:217-350), T = dcomp.  Returns the status, the rank in k.
__device__ int aca(const G32& g, const HBlk& B, uint32_t i0, uint32_t kmax, uint32_t kcap, double eps,
                   uint32_t& kout) {
  const uint32_t n1 = B.n1, n2 = B.n2;
  for (uint32_t i = g.rank; i < n1; i += 32) B.Z[i] = 0;
  for (uint32_t j = g.rank; j < n2; j += 32) B.S[j] = 0;
  double scale = cabs(helm_entry(B, B.b1, B.b2));
  uint32_t k = 0, no = 0, klast = 0, inext = i0, j0 = 0;
  int kmin = -2, keps = -1;
  double nrmlsk2 = 0.0, nrms2 = 0.0;
  int outcome = -1;
  do {
    if (k >= kcap) { outcome = kAcaOverflow; break; }
    inext = i0;
    if (!row_step(g, B, klast, inext, k, no, nrmlsk2, scale)) {
      nrmlsk2 = 0.0;
      outcome = kAcaOk;
      break;
    }
    __syncwarp();
    // sum_l scpr(U_l, U_k) * scpr(V_l, V_k), scpr = sum conj(x) y
    double sre = 0.0, sim = 0.0;
    const Cx* uk = B.U + (size_t)k * n1;
    const Cx* vk = B.V + (size_t)k * n2;
    for (uint32_t l = 0; l < k; ++l) {
      double ur = 0.0, ui = 0.0, vr = 0.0, vi = 0.0;
      for (uint32_t i = g.rank; i < n1; i += 32) {
        const Cx a = B.U[(size_t)l * n1 + i], b = uk[i];
        ur += a.re * b.re + a.im * b.im;
        ui += a.re * b.im - a.im * b.re;
      }
      for (uint32_t j = g.rank; j < n2; j += 32) {
        const Cx a = B.V[(size_t)l * n2 + j], b = vk[j];
        vr += a.re * b.re + a.im * b.im;
        vi += a.re * b.im - a.im * b.re;
      }
      G32::sum2(ur, ui);
      G32::sum2(vr, vi);
      sre += ur * vr - ui * vi;
      sim += ur * vi + ui * vr;
    }
    nrms2 += 2.0 * sre + nrmlsk2;
    const bool stpcrit = nrmlsk2 < eps * eps * nrms2;
    if (stpcrit && keps == -1) keps = (int)klast + 1;
    ++k;
    scale = sqrt(nrmlsk2 / (double)(uint32_t)(n1 * n2));
    if (keps > 0) {
      ArgMinI m{INT_MAX, 0xffffffffu};
      for (uint32_t i = g.rank; i < n1; i += 32)
        if (B.Z[i] >= 0 && B.Z[i] < m.v) m = ArgMinI{B.Z[i], i};
      m = G32::argmin(m);
      if (m.v == INT_MAX) {
        nrmlsk2 = 0.0;
        outcome = kAcaOk;
        break;
      }
      kmin = m.v;
      i0 = m.idx;
      if ((uint32_t)kmin == k) i0 = inext;
    } else {
      i0 = inext;
    }
  } while (no < n1 && k < kmax && kmin < keps);

  if (outcome < 0) {
    if ((no == n1 || k == kmax) && kmin < keps) {
      outcome = kAcaFail;
    } else {
      do {
        ArgMinI m{INT_MAX, 0xffffffffu};
        for (uint32_t j = g.rank; j < n2; j += 32)
          if (B.S[j] >= 0 && B.S[j] < m.v) m = ArgMinI{B.S[j], j};
        m = G32::argmin(m);
        if (m.v == INT_MAX) {
          nrmlsk2 = 0.0;
          outcome = kAcaOk;
          break;
        }
        kmin = m.v;
        j0 = m.idx;
        if (kmin >= keps) { outcome = kAcaOk; break; }
        if (k >= kcap) { outcome = kAcaOverflow; break; }
        if (!col_step(g, B, j0, k, no, nrmlsk2, scale)) {
          nrmlsk2 = 0.0;
          outcome = kAcaOk;
          break;
        }
        ++k;
      } while (no < n2 && k < kmax);
      if (outcome < 0) outcome = kAcaFail;
    }
  }
  if (outcome == kAcaOk) {
    const double epsa = sqrt(nrmlsk2 / nrms2);
    if (epsa >= eps) outcome = kAcaFail;
  }
  kout = k;
  __syncwarp();
  return outcome;
}

struct HTask {
  uint32_t b1, n1, b2, n2, kmax, kcap, leaf, pad;
  uint64_t ws;  // Cx offset of U (then V) in the batch workspace
  uint64_t zs;  // int offset of Z (then S)
};

__global__ void __launch_bounds__(32 * kWarps)
    helm_aca_kernel(PointsSoA P, double k, double h, double eps, const HTask* __restrict__ tasks, uint32_t n,
                    Cx* __restrict__ ws, int* __restrict__ zs, int2* __restrict__ res) {
  const uint32_t t = blockIdx.x * kWarps + (threadIdx.x >> 5);
  if (t >= n) return;
  const HTask T = tasks[t];
  G32 g(threadIdx.x & 31);
  HBlk B;
  B.P = P;
  B.k = k;
  B.h = h;
  B.b1 = T.b1;
  B.n1 = T.n1;
  B.b2 = T.b2;
  B.n2 = T.n2;
  B.U = ws + T.ws;
  B.V = B.U + (size_t)T.n1 * T.kcap;
  B.Z = zs + T.zs;
  B.S = B.Z + T.n1;
  uint32_t kk = 0;
  const int st = aca(g, B, 0u, T.kmax, T.kcap, eps, kk);
  if (g.rank == 0) res[t] = make_int2(st, (int)kk);
}

}  // namespace
}  // namespace ahx

using namespace ahx;

extern "C" int ahx_helm_aca_ranks(ahx_hmat* H, double wavenumber, double h, double eps, uint32_t rankmax,
                                  const float* rank_hint, int32_t* ranks) {
  if (!H || !ranks || !(h > 0.0) || !(eps > 0.0) || H->tree.kind != kTreeBbx) {
    set_error("ahx_helm_aca_ranks: invalid argument (bounding-box trees only)");
    return AHX_ERR_ARG;
  }
  int rc = ensure_device(H);
  if (rc) return rc;
  const auto& Ls = H->tree.leaves;
  const uint32_t nl = (uint32_t)Ls.size();
  std::vector<HTask> tasks;
  for (uint32_t l = 0; l < nl; ++l) {
    const Leaf& L = Ls[l];
    ranks[l] = -1;
    const uint32_t maxk = maxk_of(L.n1, L.n2, rankmax);
    if (!L.adm || !maxk) continue;
    HTask t{};
    t.b1 = L.b1;
    t.n1 = L.n1;
    t.b2 = L.b2;
    t.n2 = L.n2;
    t.kmax = maxk;
    t.kcap = std::min(maxk, aca_kcap_default());
    if (rank_hint && rank_hint[l] >= 0.f)
      t.kcap = std::min(maxk, std::max(8u, (uint32_t)std::ceil(rank_hint[l] * 1.25f + 4.f)));
    t.leaf = l;
    tasks.push_back(t);
  }
  H->stat_ws_bytes = H->stat_retries = H->stat_batches = 0;
  const size_t budget = aca_ws_budget();
  const double* pts = H->pts.as<double>();
  const PointsSoA P{pts, pts + H->tree.n, pts + 2 * (size_t)H->tree.n};
  DevBuf ws, zs, dtasks, dres;
  while (!tasks.empty()) {
    std::sort(tasks.begin(), tasks.end(), [](const HTask& a, const HTask& b) {
      return (uint64_t)(a.n1 + a.n2) * a.kcap > (uint64_t)(b.n1 + b.n2) * b.kcap;
    });
    std::vector<HTask> retry;
    size_t i = 0;
    while (i < tasks.size()) {
      uint64_t wsc = 0, zsi = 0;
      size_t j = i;
      for (; j < tasks.size(); ++j) {
        const uint64_t w = (uint64_t)(tasks[j].n1 + tasks[j].n2) * tasks[j].kcap;
        if (j > i && (wsc + w) * sizeof(Cx) + (zsi + tasks[j].n1 + tasks[j].n2) * 4 > budget) break;
        tasks[j].ws = wsc;
        tasks[j].zs = zsi;
        wsc += w;
        zsi += tasks[j].n1 + tasks[j].n2;
      }
      std::vector<HTask> batch(tasks.begin() + i, tasks.begin() + j);
      i = j;
      H->stat_ws_bytes = std::max<uint64_t>(H->stat_ws_bytes, wsc * sizeof(Cx) + zsi * 4);
      H->stat_batches++;
      if ((rc = ws.reserve(std::max<uint64_t>(wsc, 1) * sizeof(Cx)))) return rc;
      if ((rc = zs.reserve(std::max<uint64_t>(zsi, 1) * 4))) return rc;
      if ((rc = upload(dtasks, batch, H->stream))) return rc;
      if ((rc = dres.reserve(batch.size() * sizeof(int2)))) return rc;
      const uint32_t nb = (uint32_t)batch.size();
      helm_aca_kernel<<<(nb + kWarps - 1) / kWarps, 32 * kWarps, 0, H->stream>>>(
          P, wavenumber, h, eps, dtasks.as<HTask>(), nb, ws.as<Cx>(), zs.as<int>(), dres.as<int2>());
      AHX_CUDA(cudaGetLastError());
      std::vector<int2> res(nb);
      AHX_CUDA(cudaMemcpyAsync(res.data(), dres.p, nb * sizeof(int2), cudaMemcpyDeviceToHost, H->stream));
      AHX_CUDA(cudaStreamSynchronize(H->stream));
      for (uint32_t q = 0; q < nb; ++q) {
        const HTask& t = batch[q];
        if (res[q].x == kAcaOverflow) {
          HTask u = t;
          u.kcap = std::min(t.kmax, std::max(t.kcap * 4, 16u));
          retry.push_back(u);
          H->stat_retries++;
        } else {
          ranks[t.leaf] = res[q].x == kAcaOk ? res[q].y : -2;
        }
      }
    }
    tasks.swap(retry);
  }
  return AHX_OK;
}
