// Helmholtz single-layer matrix exp(i k r) / (4 pi r) (diagonal exp(i k h) /
// (4 pi h)) on the GPU: the reference's ACA with T = dcomp (Include/ACA.h:46-350;
// complex arithmetic of Include/cmplx.h:80-245: |z| = sqrt(re^2 + im^2), a / z
// = a / |z|^2 * conj(z), scpr = sum conj(x) y), one warp per admissible leaf,
// every leaf with the reference's stopping rule and counters.
//   ahx_helm_aca_ranks: the ACA rank per leaf only (training data and
//     verification of the rank predictor on oscillatory kernels);
//   ahx_helm_assemble: the complex H-matrix (apprx_unsym, Include/apprx.h:136-172,
//     with T = dcomp): ACA, recompression as mblock<dcomp>::addtrll
//     (H/mblock_Z.cpp:200-300), dense leaves where ACA fails or the block is
//     inadmissible; leaves in the mblock<dcomp> layout in a complex arena.
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

// ACAr_step (ACA.h:579-655) with T = dcomp, the cross of the symmetric assembly:
// rows are skipped only for a small pivot, the pivot column is searched over all
// columns, the next row is the largest unused entry of the new column.
__device__ bool acar_step(const G32& g, const HBlk& B, uint32_t& i0, uint32_t k, uint32_t& no, double& nrmlsk2,
                          double scale) {
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
      const double a = cabs(v);
      if (gt_nonneg(a, am.v)) am = ArgMax{a, j, 0.0};
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
  __syncwarp();
  double nrmv2 = 0.0;
  for (uint32_t j = g.rank; j < n2; j += 32) {
    Cx e = pv[j];
    cmul_eq(e, sca);
    pv[j] = e;
    nrmv2 += cabs2(e);
  }
  for (uint32_t i = g.rank; i < n1; i += 32) {
    Cx u = helm_entry(B, B.b1 + i, B.b2 + j0);
    for (uint32_t l = 0; l < k; ++l) caxpy(nconj(B.V[(size_t)l * n2 + j0]), B.U[(size_t)l * n1 + i], u);
    pu[i] = u;
  }
  if (i0 % 32 == g.rank) B.Z[i0] = -1;
  ++no;
  __syncwarp();
  const double dsca = 1.0 / sqrtpiv;
  double nrmu2 = 0.0;
  ArgMax nm{0.0, 0xffffffffu, 0.0};
  for (uint32_t i = g.rank; i < n1; i += 32) {
    Cx e = pu[i];
    e.re *= dsca;
    e.im *= dsca;
    pu[i] = e;
    const double ea = cabs(e);
    nrmu2 += ea * ea;
    if (B.Z[i] >= 0 && gt_nonneg(ea, nm.v)) nm = ArgMax{ea, i, 0.0};
  }
  G32::sum2(nrmu2, nrmv2);
  nm = G32::argmax(nm);
  if (nm.v > 0.0) i0 = nm.idx;
  nrmlsk2 = nrmu2 * nrmv2;
  return true;
}

// ACAr (ACA.h:657-720) with T = dcomp: crosses until the last one is below eps of
// the approximation's norm, no more than n2 rows used, or kmax crosses.
__device__ int acar(const G32& g, const HBlk& B, uint32_t i0, uint32_t kmax, uint32_t kcap, double eps,
                    uint32_t& kout) {
  const uint32_t n1 = B.n1, n2 = B.n2;
  for (uint32_t i = g.rank; i < n1; i += 32) B.Z[i] = 0;
  double scale = cabs(helm_entry(B, B.b1, B.b2));
  uint32_t k = 0, no = 0;
  double nrmlsk2 = 0.0, nrms2 = 0.0;
  int outcome = -1;
  do {
    if (k >= kcap) {
      outcome = kAcaOverflow;
      break;
    }
    if (!acar_step(g, B, i0, k, no, nrmlsk2, scale)) {
      nrmlsk2 = 0.0;
      break;
    }
    __syncwarp();
    // Re sum_l scpr(U_l, U_k) scpr(V_l, V_k)
    double sre = 0.0;
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
    }
    nrms2 += 2.0 * sre + nrmlsk2;
    ++k;
    scale = sqrt(nrmlsk2 / (double)(uint32_t)(n1 * n2));
  } while (no < n2 && k < kmax && nrmlsk2 >= eps * eps * nrms2);
  if (outcome < 0) {
    const double epsa = sqrt(nrmlsk2 / nrms2);
    outcome = epsa >= eps ? kAcaFail : kAcaOk;  // NaN (0/0) stays a success, as in the reference
  }
  kout = k;
  __syncwarp();
  return outcome;
}

// ---------------------------------------------------------------------------
// Recompression of a complex low-rank block U V^H (mblock<dcomp>::addtrll,
// H/mblock_Z.cpp:200-300: QR of U and V, SVD of R1 R2^H after dropping entries
// below delta |R|_F / sqrt(mmin nmin), truncation at delta sigma_0, Q applied),
// by one warp.  The row i of every column belongs to lane i % 32.

__device__ __forceinline__ Cx cmul(Cx a, Cx b) { return Cx{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
// conj(a) b
__device__ __forceinline__ Cx cmulc(Cx a, Cx b) { return Cx{a.re * b.re + a.im * b.im, a.re * b.im - a.im * b.re}; }
__device__ __forceinline__ Cx cinv(Cx a) {
  const double s = 1.0 / (a.re * a.re + a.im * a.im);
  return Cx{a.re * s, -a.im * s};
}

// Householder QR of A (m x k, column-major) in LAPACK's zgeqrf form:
// H_c = I - tau_c v_c v_c^H with v_c(c) = 1, a real diagonal beta in R.
__device__ void zqr(const G32& g, uint32_t m, uint32_t k, Cx* A, Cx* tau) {
  const uint32_t kk = min(m, k);
  for (uint32_t c = 0; c < kk; ++c) {
    Cx* a = A + (size_t)c * m;
    double xn2 = 0.0, ar = 0.0, ai = 0.0;
    for (uint32_t i = g.rank; i < m; i += 32) {
      const Cx v = a[i];
      if (i > c) xn2 += v.re * v.re + v.im * v.im;
      else if (i == c) {
        ar = v.re;
        ai = v.im;
      }
    }
    G32::sum3(xn2, ar, ai);
    if (xn2 == 0.0 && ai == 0.0) {
      if (g.rank == 0) tau[c] = Cx{0.0, 0.0};
      continue;
    }
    const double nrm = sqrt(ar * ar + ai * ai + xn2);
    const double beta = ar >= 0.0 ? -nrm : nrm;
    const Cx t{(beta - ar) / beta, -ai / beta};
    const Cx sc = cinv(Cx{ar - beta, ai});
    if (g.rank == 0) tau[c] = t;
    for (uint32_t i = g.rank; i < m; i += 32) {
      if (i > c) a[i] = cmul(a[i], sc);
      else if (i == c) a[i] = Cx{beta, 0.0};
    }
    // the remaining columns: b -= conj(tau) v (v^H b)
    const Cx tc = cconj(t);
    for (uint32_t q = c + 1; q < k; ++q) {
      Cx* b = A + (size_t)q * m;
      double sr = 0.0, si = 0.0;
      for (uint32_t i = g.rank; i < m; i += 32) {
        if (i > c) {
          const Cx z = cmulc(a[i], b[i]);
          sr += z.re;
          si += z.im;
        } else if (i == c) {
          sr += b[i].re;
          si += b[i].im;
        }
      }
      G32::sum2(sr, si);
      const Cx f = cmul(tc, Cx{sr, si});
      for (uint32_t i = g.rank; i < m; i += 32) {
        if (i > c) {
          const Cx z = cmul(f, a[i]);
          b[i].re -= z.re;
          b[i].im -= z.im;
        } else if (i == c) {
          b[i].re -= f.re;
          b[i].im -= f.im;
        }
      }
    }
  }
}

// C (m x nc, ld m) := Q C with Q = H_0 ... H_{kr-1} from zqr (tau read after a
// warp barrier).
__device__ void zapply_q(const G32& g, uint32_t m, uint32_t kr, const Cx* A, const Cx* tau, uint32_t nc, Cx* C) {
  for (int c = (int)kr - 1; c >= 0; --c) {
    const Cx t = tau[c];
    if (t.re == 0.0 && t.im == 0.0) continue;
    const Cx* a = A + (size_t)c * m;
    for (uint32_t q = 0; q < nc; ++q) {
      Cx* b = C + (size_t)q * m;
      double sr = 0.0, si = 0.0;
      for (uint32_t i = g.rank; i < m; i += 32) {
        if (i > (uint32_t)c) {
          const Cx z = cmulc(a[i], b[i]);
          sr += z.re;
          si += z.im;
        } else if (i == (uint32_t)c) {
          sr += b[i].re;
          si += b[i].im;
        }
      }
      G32::sum2(sr, si);
      const Cx f = cmul(t, Cx{sr, si});
      for (uint32_t i = g.rank; i < m; i += 32) {
        if (i > (uint32_t)c) {
          const Cx z = cmul(f, a[i]);
          b[i].re -= z.re;
          b[i].im -= z.im;
        } else if (i == (uint32_t)c) {
          b[i].re -= f.re;
          b[i].im -= f.im;
        }
      }
    }
  }
}

// Un (n1 x kt), Vn (n2 x kt) with Un Vn^H = the truncated U V^H (rank k); R, Vs:
// column-major with stride ld >= k; sig: k doubles; tau: 2k; perm: nmin + 1 ints.
__device__ uint32_t zrecompress(const G32& g, uint32_t n1, uint32_t n2, uint32_t k, Cx* U, Cx* V, Cx* Un, Cx* Vn,
                                double delta, Cx* R, Cx* Vs, uint32_t ld, double* sig, Cx* tau, int* perm) {
  const uint32_t mmin = min(n1, k), nmin = min(n2, k), amin = min(mmin, nmin);
  Cx* tau1 = tau;
  Cx* tau2 = tau + k;
  zqr(g, n1, k, U, tau1);
  zqr(g, n2, k, V, tau2);
  __syncwarp();
  // R = R1 R2^H (Include/blas.h utrmmh)
  double fro = 0.0;
  for (uint32_t i = g.rank; i < mmin; i += 32) {
    for (uint32_t j = 0; j < nmin; ++j) {
      double dr = 0.0, di = 0.0;
      for (uint32_t l = max(i, j); l < k; ++l) {
        const Cx u = U[i + (size_t)l * n1], v = V[j + (size_t)l * n2];
        dr += u.re * v.re + u.im * v.im;
        di += u.im * v.re - u.re * v.im;
      }
      R[i + (size_t)j * ld] = Cx{dr, di};
      fro += dr * dr + di * di;
    }
  }
  fro = G32::sum(fro);
  const double thresh = delta * sqrt(fro) / (double)sqrtf((float)mmin * (float)nmin);
  for (uint32_t i = g.rank; i < mmin; i += 32)
    for (uint32_t j = 0; j < nmin; ++j)
      if (cabs(R[i + (size_t)j * ld]) < thresh) R[i + (size_t)j * ld] = Cx{0.0, 0.0};
  for (uint32_t i = g.rank; i < nmin; i += 32)
    for (uint32_t j = 0; j < nmin; ++j) Vs[i + (size_t)j * ld] = Cx{i == j ? 1.0 : 0.0, 0.0};
  // one-sided Jacobi (Hestenes) on the columns of R with complex rotations
  // [x y] <- [c x - s e y, s x + c e y], e = conj(gamma) / |gamma|, gamma = x^H y
  for (int sweep = 0; sweep < 40; ++sweep) {
    bool rotated = false;
    for (uint32_t p = 0; p + 1 < nmin; ++p) {
      for (uint32_t q = p + 1; q < nmin; ++q) {
        double al = 0.0, be = 0.0, gr = 0.0, gi = 0.0;
        for (uint32_t i = g.rank; i < mmin; i += 32) {
          const Cx x = R[i + (size_t)p * ld], y = R[i + (size_t)q * ld];
          al += x.re * x.re + x.im * x.im;
          be += y.re * y.re + y.im * y.im;
          const Cx z = cmulc(x, y);
          gr += z.re;
          gi += z.im;
        }
        G32::sum2(al, be);
        G32::sum2(gr, gi);
        const double ga = sqrt(gr * gr + gi * gi);
        if (ga == 0.0 || ga <= 1e-15 * sqrt(al * be)) continue;
        rotated = true;
        const double zeta = (be - al) / (2.0 * ga);
        const double t = (zeta >= 0.0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
        const double c = 1.0 / sqrt(1.0 + t * t);
        const double s = c * t;
        const Cx e{gr / ga, -gi / ga};
        for (uint32_t i = g.rank; i < mmin; i += 32) {
          const Cx x = R[i + (size_t)p * ld], ey = cmul(e, R[i + (size_t)q * ld]);
          R[i + (size_t)p * ld] = Cx{c * x.re - s * ey.re, c * x.im - s * ey.im};
          R[i + (size_t)q * ld] = Cx{s * x.re + c * ey.re, s * x.im + c * ey.im};
        }
        for (uint32_t i = g.rank; i < nmin; i += 32) {
          const Cx x = Vs[i + (size_t)p * ld], ey = cmul(e, Vs[i + (size_t)q * ld]);
          Vs[i + (size_t)p * ld] = Cx{c * x.re - s * ey.re, c * x.im - s * ey.im};
          Vs[i + (size_t)q * ld] = Cx{s * x.re + c * ey.re, s * x.im + c * ey.im};
        }
      }
    }
    if (!rotated) break;
  }
  for (uint32_t j = 0; j < nmin; ++j) {
    double sj = 0.0;
    for (uint32_t i = g.rank; i < mmin; i += 32) sj += cabs2(R[i + (size_t)j * ld]);
    sj = G32::sum(sj);
    if (g.rank == 0) sig[j] = sqrt(sj);
  }
  __syncwarp();
  if (g.rank == 0) {
    for (uint32_t j = 0; j < nmin; ++j) perm[j] = (int)j;
    for (uint32_t j = 0; j < nmin; ++j) {
      uint32_t b = j;
      for (uint32_t q = j + 1; q < nmin; ++q)
        if (sig[perm[q]] > sig[perm[b]]) b = q;
      const int t = perm[j];
      perm[j] = perm[b];
      perm[b] = t;
    }
    uint32_t kt = min(amin, k);
    const double s0 = nmin ? sig[perm[0]] : 0.0;
    while (kt > 0 && (sig[perm[kt - 1]] <= delta * s0 || sig[perm[kt - 1]] < 1e-64)) --kt;
    perm[nmin] = (int)kt;
  }
  __syncwarp();
  const uint32_t kt = (uint32_t)perm[nmin];
  // Un = Q1 [R(:, perm[:kt]); 0] (R's columns are sigma_j u_j), Vn = Q2 [Vs(:, perm[:kt]); 0]
  for (uint32_t j = 0; j < kt; ++j) {
    const int pj = perm[j];
    for (uint32_t i = g.rank; i < n1; i += 32) Un[i + (size_t)j * n1] = i < mmin ? R[i + (size_t)pj * ld] : Cx{0.0, 0.0};
    for (uint32_t i = g.rank; i < n2; i += 32) Vn[i + (size_t)j * n2] = i < nmin ? Vs[i + (size_t)pj * ld] : Cx{0.0, 0.0};
  }
  zapply_q(g, n1, mmin, U, tau1, kt, Un);
  zapply_q(g, n2, nmin, V, tau2, kt, Vn);
  __syncwarp();
  return kt;
}

// Recompression of a union of complex low-rank blocks (agglomeration of mblock<dcomp>
// leaves, H/agglH.cpp:14-107 with T = dcomp) by one warp: QR of both factors,
// R = R1 R2^H, small entries dropped as in addtrll, then a column-pivoted
// Householder QR of R stopped once the trailing columns' Frobenius norm is at most
// 1e-2 delta max_j |R(:, j)|, one-sided Jacobi on Tt = T^H of the kept rows T
// (T^H Z = W S), and R = (Qr Z S) (P W)^H.  Workspaces as the real union's
// (complex elements): R (mmin x nmin, stride ld, then the reflectors), Tt
// (nmin x rr), Z (rr x rr); cn: nmin doubles; qtau: nmin; cperm: nmin ints;
// perm: rr + 1 ints.
__device__ uint32_t zrecompress_qrcp(const G32& g, uint32_t n1, uint32_t n2, uint32_t k, Cx* U, Cx* V, Cx* Un,
                                     Cx* Vn, double delta, Cx* R, Cx* Tt, Cx* Z, uint32_t ld, double* sig, Cx* tau,
                                     double* cn, Cx* qtau, int* cperm, int* perm) {
  if (k == 0) return 0;
  const uint32_t lane = g.rank;
  const uint32_t mmin = min(n1, k), nmin = min(n2, k), amin = min(mmin, nmin);
  Cx* tau1 = tau;
  Cx* tau2 = tau + k;
  zqr(g, n1, k, U, tau1);
  zqr(g, n2, k, V, tau2);
  __syncwarp();
  double fro = 0.0;
  for (uint32_t i = lane; i < mmin; i += 32) {
    for (uint32_t j = 0; j < nmin; ++j) {
      double dr = 0.0, di = 0.0;
      for (uint32_t l = max(i, j); l < k; ++l) {
        const Cx u = U[i + (size_t)l * n1], v = V[j + (size_t)l * n2];
        dr += u.re * v.re + u.im * v.im;
        di += u.im * v.re - u.re * v.im;
      }
      R[i + (size_t)j * ld] = Cx{dr, di};
      fro += dr * dr + di * di;
    }
  }
  fro = G32::sum(fro);
  const double thresh = delta * sqrt(fro) / (double)sqrtf((float)mmin * (float)nmin);
  for (uint32_t i = lane; i < mmin; i += 32)
    for (uint32_t j = 0; j < nmin; ++j)
      if (cabs(R[i + (size_t)j * ld]) < thresh) R[i + (size_t)j * ld] = Cx{0.0, 0.0};
  __syncwarp();
  ArgMax cm{0.0, 0xffffffffu, 0.0};
  for (uint32_t j = 0; j < nmin; ++j) {
    double sj = 0.0;
    for (uint32_t i = lane; i < mmin; i += 32) sj += cabs2(R[i + (size_t)j * ld]);
    sj = G32::sum(sj);
    if (lane == 0) {
      cn[j] = sj;
      cperm[j] = (int)j;
    }
    if (gt_nonneg(sj, cm.v)) cm = ArgMax{sj, j, 0.0};
  }
  __syncwarp();
  const double tol2 = (1e-2 * delta) * (1e-2 * delta) * cm.v;
  uint32_t rr = amin;
  for (uint32_t c = 0; c < amin; ++c) {
    double tot = 0.0;
    ArgMax am{0.0, 0xffffffffu, 0.0};
    for (uint32_t j = c + lane; j < nmin; j += 32) {
      const double v = cn[j];
      tot += v;
      if (gt_nonneg(v, am.v)) am = ArgMax{v, j, 0.0};
    }
    tot = G32::sum(tot);
    am = G32::argmax(am);
    if (tot <= tol2 || am.idx >= nmin) {
      rr = c;
      break;
    }
    const uint32_t p = am.idx;
    __syncwarp();
    if (p != c) {
      for (uint32_t i = lane; i < mmin; i += 32) {
        const Cx x = R[i + (size_t)c * ld];
        R[i + (size_t)c * ld] = R[i + (size_t)p * ld];
        R[i + (size_t)p * ld] = x;
      }
      if (lane == 0) {
        const double x = cn[c];
        cn[c] = cn[p];
        cn[p] = x;
        const int q = cperm[c];
        cperm[c] = cperm[p];
        cperm[p] = q;
      }
    }
    __syncwarp();
    Cx* a = R + (size_t)c * ld;
    double xn2 = 0.0, ar = 0.0, ai = 0.0;
    for (uint32_t i = lane; i < mmin; i += 32) {
      const Cx v = a[i];
      if (i > c) xn2 += v.re * v.re + v.im * v.im;
      else if (i == c) {
        ar = v.re;
        ai = v.im;
      }
    }
    G32::sum3(xn2, ar, ai);
    Cx t{0.0, 0.0};
    if (!(xn2 == 0.0 && ai == 0.0)) {
      const double nrm = sqrt(ar * ar + ai * ai + xn2);
      const double beta = ar >= 0.0 ? -nrm : nrm;
      t = Cx{(beta - ar) / beta, -ai / beta};
      const Cx sc = cinv(Cx{ar - beta, ai});
      for (uint32_t i = lane; i < mmin; i += 32) {
        if (i > c) a[i] = cmul(a[i], sc);
        else if (i == c) a[i] = Cx{beta, 0.0};
      }
    }
    if (lane == 0) qtau[c] = t;
    __syncwarp();
    // trailing columns: b -= conj(t) v (v^H b), then their norms below row c
    const Cx tc = cconj(t);
    for (uint32_t j = c + 1; j < nmin; ++j) {
      Cx* b = R + (size_t)j * ld;
      if (t.re != 0.0 || t.im != 0.0) {
        double sr = 0.0, si = 0.0;
        for (uint32_t i = c + lane; i < mmin; i += 32) {
          if (i > c) {
            const Cx z = cmulc(a[i], b[i]);
            sr += z.re;
            si += z.im;
          } else {
            sr += b[i].re;
            si += b[i].im;
          }
        }
        G32::sum2(sr, si);
        const Cx f = cmul(tc, Cx{sr, si});
        for (uint32_t i = c + lane; i < mmin; i += 32) {
          if (i > c) {
            const Cx z = cmul(f, a[i]);
            b[i].re -= z.re;
            b[i].im -= z.im;
          } else {
            b[i].re -= f.re;
            b[i].im -= f.im;
          }
        }
      }
      double s2 = 0.0;
      for (uint32_t i = c + lane; i < mmin; i += 32)
        if (i > c) s2 += cabs2(b[i]);
      s2 = G32::sum(s2);
      if (lane == 0) cn[j] = s2;
    }
    __syncwarp();
  }
  // Tt = T^H (nmin x rr), Z = I (rr x rr)
  for (uint32_t e = lane; e < nmin * rr; e += 32) {
    const uint32_t i = e / nmin, j = e - i * nmin;
    Tt[j + (size_t)i * ld] = j >= i ? cconj(R[i + (size_t)j * ld]) : Cx{0.0, 0.0};
  }
  for (uint32_t e = lane; e < rr * rr; e += 32) {
    const uint32_t i = e % rr, j = e / rr;
    Z[i + (size_t)j * ld] = Cx{i == j ? 1.0 : 0.0, 0.0};
  }
  __syncwarp();
  // one-sided Jacobi on the columns of Tt (the rotations of zrecompress)
  for (int sweep = 0; sweep < 40; ++sweep) {
    bool rotated = false;
    for (uint32_t p = 0; p + 1 < rr; ++p) {
      for (uint32_t q = p + 1; q < rr; ++q) {
        double al = 0.0, be = 0.0, gr = 0.0, gi = 0.0;
        for (uint32_t i = lane; i < nmin; i += 32) {
          const Cx x = Tt[i + (size_t)p * ld], y = Tt[i + (size_t)q * ld];
          al += x.re * x.re + x.im * x.im;
          be += y.re * y.re + y.im * y.im;
          const Cx z = cmulc(x, y);
          gr += z.re;
          gi += z.im;
        }
        G32::sum2(al, be);
        G32::sum2(gr, gi);
        const double ga = sqrt(gr * gr + gi * gi);
        if (ga == 0.0 || ga <= 1e-15 * sqrt(al * be)) continue;
        rotated = true;
        const double zeta = (be - al) / (2.0 * ga);
        const double tt = (zeta >= 0.0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
        const double cs = 1.0 / sqrt(1.0 + tt * tt);
        const double sn = cs * tt;
        const Cx e{gr / ga, -gi / ga};
        for (uint32_t i = lane; i < nmin; i += 32) {
          const Cx x = Tt[i + (size_t)p * ld], ey = cmul(e, Tt[i + (size_t)q * ld]);
          Tt[i + (size_t)p * ld] = Cx{cs * x.re - sn * ey.re, cs * x.im - sn * ey.im};
          Tt[i + (size_t)q * ld] = Cx{sn * x.re + cs * ey.re, sn * x.im + cs * ey.im};
        }
        for (uint32_t i = lane; i < rr; i += 32) {
          const Cx x = Z[i + (size_t)p * ld], ey = cmul(e, Z[i + (size_t)q * ld]);
          Z[i + (size_t)p * ld] = Cx{cs * x.re - sn * ey.re, cs * x.im - sn * ey.im};
          Z[i + (size_t)q * ld] = Cx{sn * x.re + cs * ey.re, sn * x.im + cs * ey.im};
        }
      }
    }
    if (!rotated) break;
  }
  for (uint32_t j = 0; j < rr; ++j) {
    double sj = 0.0;
    for (uint32_t i = lane; i < nmin; i += 32) sj += cabs2(Tt[i + (size_t)j * ld]);
    sj = G32::sum(sj);
    if (lane == 0) sig[j] = sqrt(sj);
  }
  __syncwarp();
  if (lane == 0) {
    for (uint32_t j = 0; j < rr; ++j) perm[j] = (int)j;
    for (uint32_t j = 0; j < rr; ++j) {
      uint32_t b = j;
      for (uint32_t q = j + 1; q < rr; ++q)
        if (sig[perm[q]] > sig[perm[b]]) b = q;
      const int t = perm[j];
      perm[j] = perm[b];
      perm[b] = t;
    }
    uint32_t kt = rr;
    const double s0 = rr ? sig[perm[0]] : 0.0;
    while (kt > 0 && (sig[perm[kt - 1]] <= delta * s0 || sig[perm[kt - 1]] < 1e-64)) --kt;
    perm[rr] = (int)kt;
  }
  __syncwarp();
  const uint32_t kt = (uint32_t)perm[rr];
  // Un = Q1 [Qr [Z(:, p) s_p; 0]; 0],  Vn = Q2 [P W(:, p); 0]
  for (uint32_t j = 0; j < kt; ++j) {
    const int pj = perm[j];
    const double sj = sig[pj];
    for (uint32_t i = lane; i < n1; i += 32) {
      const Cx z = i < rr ? Z[i + (size_t)pj * ld] : Cx{0.0, 0.0};
      Un[i + (size_t)j * n1] = Cx{z.re * sj, z.im * sj};
    }
    for (uint32_t i = lane; i < n2; i += 32) {
      if (i < nmin) {
        const Cx w = Tt[i + (size_t)pj * ld];
        Vn[(uint32_t)cperm[i] + (size_t)j * n2] = Cx{w.re / sj, w.im / sj};
      } else {
        Vn[i + (size_t)j * n2] = Cx{0.0, 0.0};
      }
    }
  }
  __syncwarp();
  for (int c = (int)rr - 1; c >= 0; --c) {
    const Cx t = qtau[c];
    if (t.re != 0.0 || t.im != 0.0) {
      const Cx* a = R + (size_t)c * ld;
      for (uint32_t j = 0; j < kt; ++j) {
        Cx* b = Un + (size_t)j * n1;
        double sr = 0.0, si = 0.0;
        for (uint32_t i = (uint32_t)c + lane; i < mmin; i += 32) {
          if (i > (uint32_t)c) {
            const Cx z = cmulc(a[i], b[i]);
            sr += z.re;
            si += z.im;
          } else {
            sr += b[i].re;
            si += b[i].im;
          }
        }
        G32::sum2(sr, si);
        const Cx f = cmul(t, Cx{sr, si});
        for (uint32_t i = (uint32_t)c + lane; i < mmin; i += 32) {
          if (i > (uint32_t)c) {
            const Cx z = cmul(f, a[i]);
            b[i].re -= z.re;
            b[i].im -= z.im;
          } else {
            b[i].re -= f.re;
            b[i].im -= f.im;
          }
        }
      }
    }
    __syncwarp();
  }
  zapply_q(g, n1, mmin, U, tau1, kt, Un);
  zapply_q(g, n2, nmin, V, tau2, kt, Vn);
  __syncwarp();
  return kt;
}

// one warp per union (CTA of one warp: consecutive unions on different SMs)
__global__ void __launch_bounds__(32) zmerge_kernel(MergeParams p) {
  const uint32_t ti = blockIdx.x;
  if (ti >= p.ntasks) return;
  G32 g(threadIdx.x & 31);
  const MergeTask t = p.tasks[ti];
  const uint32_t m = t.m, n = t.n, kc = t.k;
  Cx* U = reinterpret_cast<Cx*>(p.ws) + t.ws;
  Cx* V = U + (size_t)m * kc;
  Cx* Un = V + (size_t)n * kc;
  Cx* Vn = Un + (size_t)m * kc;
  Cx* R = Vn + (size_t)n * kc;
  Cx* Tt = R + (size_t)kc * kc;
  double* sig = reinterpret_cast<double*>(Tt + (size_t)kc * kc);
  Cx* tau = Tt + (size_t)kc * kc + kc;
  Cx* Z = tau + 2 * (size_t)kc;
  double* cn = reinterpret_cast<double*>(Z + (size_t)kc * kc);
  Cx* qtau = Z + (size_t)kc * kc + kc;
  int* cperm = reinterpret_cast<int*>(qtau + kc);
  uint32_t kt = 0;
  if (kc > 0) kt = zrecompress_qrcp(g, m, n, kc, U, V, Un, Vn, p.eps, R, Tt, Z, kc, sig, tau, cn, qtau, cperm,
                                    p.zs + t.zs);
  if (g.rank == 0) p.res[ti] = AcaResult{kAcaOk, kc, kt, 0u};
}

// One leaf of the Helmholtz assembly.  Workspace (complex, at ws):
//   U[n1 kcap] V[n2 kcap] Un[n1 kcap] Vn[n2 kcap] R[kcap^2] Vs[kcap^2] sig[kcap] tau[2 kcap]
// ints at zs: Z[n1] S[n2] (later the SVD permutation).
struct ZTask {
  uint32_t b1, n1, b2, n2, i0, kmax, kcap, leaf;
  uint64_t ws, zs;
};

__global__ void __launch_bounds__(32 * kWarps)
    helm_assemble_kernel(PointsSoA P, double k, double h, double eps, const ZTask* __restrict__ tasks, uint32_t n,
                         Cx* __restrict__ ws, int* __restrict__ zs, AcaResult* __restrict__ res, int sym) {
  const uint32_t t = blockIdx.x * kWarps + (threadIdx.x >> 5);
  if (t >= n) return;
  const ZTask T = tasks[t];
  G32 g(threadIdx.x & 31);
  HBlk B;
  B.P = P;
  B.k = k;
  B.h = h;
  B.b1 = T.b1;
  B.n1 = T.n1;
  B.b2 = T.b2;
  B.n2 = T.n2;
  const uint32_t kc = T.kcap;
  B.U = ws + T.ws;
  B.V = B.U + (size_t)T.n1 * kc;
  B.Z = zs + T.zs;
  B.S = B.Z + T.n1;
  uint32_t kk = 0, kt = 0;
  const int st = sym ? acar(g, B, T.i0, T.kmax, kc, eps, kk) : aca(g, B, T.i0, T.kmax, kc, eps, kk);
  if (st == kAcaOk && kk > 0) {
    Cx* Un = B.V + (size_t)T.n2 * kc;
    Cx* Vn = Un + (size_t)T.n1 * kc;
    Cx* R = Vn + (size_t)T.n2 * kc;
    Cx* Vs = R + (size_t)kc * kc;
    double* sig = reinterpret_cast<double*>(Vs + (size_t)kc * kc);
    Cx* tau = Vs + (size_t)kc * kc + kc;
    __syncwarp();
    kt = zrecompress(g, T.n1, T.n2, kk, B.U, B.V, Un, Vn, eps, R, Vs, kc, sig, tau, B.Z);
  }
  if (g.rank == 0) res[t] = AcaResult{st, kk, kt, 0u};
}

struct ZDense {
  uint32_t b1, n1, b2, n2;
  uint64_t off;
};

__global__ void helm_dense_kernel(PointsSoA P, double k, double h, const ZDense* __restrict__ tasks,
                                  Cx* __restrict__ arena) {
  const ZDense t = tasks[blockIdx.x];
  HBlk B;
  B.P = P;
  B.k = k;
  B.h = h;
  const uint64_t cnt = (uint64_t)t.n1 * t.n2;
  Cx* out = arena + t.off;
  for (uint64_t e = threadIdx.x; e < cnt; e += blockDim.x) {
    const uint32_t i = (uint32_t)(e % t.n1), j = (uint32_t)(e / t.n1);
    out[e] = helm_entry(B, t.b1 + i, t.b2 + j);
  }
}

struct ZCopy {
  uint64_t src_u, src_v, dst;
  uint32_t n1, n2, kt, pad;
};

__global__ void helm_copy_kernel(const ZCopy* __restrict__ tasks, const Cx* __restrict__ ws, Cx* __restrict__ arena) {
  const ZCopy t = tasks[blockIdx.x];
  const uint64_t nu = (uint64_t)t.n1 * t.kt, nv = (uint64_t)t.n2 * t.kt;
  Cx* dst = arena + t.dst;
  for (uint64_t e = threadIdx.x; e < nu; e += blockDim.x) dst[e] = ws[t.src_u + e];
  for (uint64_t e = threadIdx.x; e < nv; e += blockDim.x) dst[nu + e] = ws[t.src_v + e];
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
    t.kcap = std::min(kcap_limit(maxk), aca_kcap_default());
    if (rank_hint && rank_hint[l] >= 0.f)
      t.kcap = std::min(kcap_limit(maxk), std::max(8u, (uint32_t)std::ceil(rank_hint[l] * 1.25f + 4.f)));
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
        if (res[q].x == kAcaOverflow && t.kcap < kcap_limit(t.kmax)) {
          HTask u = t;
          u.kcap = std::min(kcap_limit(t.kmax), std::max(t.kcap * 4, 16u));
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

namespace ahx {

// Append-only growable complex arena of the Helmholtz leaves.
int zarena_append(ahx_hmat* H, uint64_t count, uint64_t& off) {
  ZState& Z = H->z;
  const uint64_t need = (Z.elems + count) * sizeof(Cx);
  if (need > Z.arena.bytes) {
    size_t nb = std::max<size_t>(need, Z.arena.bytes * 2);
    void* np = nullptr;
    cudaError_t e = cudaMalloc(&np, nb);
    if (e != cudaSuccess) {
      cudaGetLastError();
      nb = need;
      e = cudaMalloc(&np, nb);
      if (e != cudaSuccess) {
        cudaGetLastError();
        set_error("device allocation of the complex leaf arena failed");
        return AHX_ERR_NOMEM;
      }
    }
    if (Z.elems) {
      const cudaError_t ce = cudaMemcpyAsync(np, Z.arena.p, Z.elems * sizeof(Cx), cudaMemcpyDeviceToDevice, H->stream);
      if (ce != cudaSuccess) {
        cudaFree(np);
        return cuda_fail(ce, "cudaMemcpyAsync (complex arena)");
      }
    }
    AHX_CUDA(cudaStreamSynchronize(H->stream));
    if (Z.arena.p) cudaFree(Z.arena.p);
    Z.arena.p = np;
    Z.arena.bytes = nb;
  }
  off = Z.elems;
  Z.elems += count;
  return AHX_OK;
}

namespace {
uint64_t zws_elems(const ZTask& t) { return aca_ws_doubles(t.n1, t.n2, t.kcap); }

}  // namespace
}  // namespace ahx

extern "C" int ahx_helm_assemble(ahx_hmat* H, double wavenumber, double h, double eps, uint32_t rankmax) {
  if (!H || !(h > 0.0) || !(eps > 0.0) || !std::isfinite(wavenumber)) {
    set_error("ahx_helm_assemble: invalid argument");
    return AHX_ERR_ARG;
  }
  int rc = ensure_device(H);
  if (rc) return rc;
  ZState& Z = H->z;
  Z.assembled = Z.valid32 = Z.table = false;
  Z.elems = 0;
  Z.k = wavenumber;
  Z.h = h;
  Z.eps = eps;
  const auto& Ls = H->tree.leaves;
  const uint32_t nl = (uint32_t)Ls.size();
  Z.rank.assign(nl, -1);
  Z.aca_rank.assign(nl, -1);
  Z.off.assign(nl, 0);
  H->stat_ws_bytes = H->stat_retries = H->stat_batches = 0;
  std::vector<ZTask> tasks;
  std::vector<uint32_t> dense;
  const uint32_t kcap0 = aca_kcap_default();
  for (uint32_t l = 0; l < nl; ++l) {
    const Leaf& L = Ls[l];
    const uint32_t maxk = maxk_of(L.n1, L.n2, rankmax);
    if (L.adm && maxk) {
      ZTask t{};
      t.b1 = L.b1;
      t.n1 = L.n1;
      t.b2 = L.b2;
      t.n2 = L.n2;
      t.i0 = L.i0;
      t.kmax = maxk;
      t.kcap = std::min(kcap_limit(maxk), kcap0);
      t.leaf = l;
      tasks.push_back(t);
    } else {
      dense.push_back(l);
    }
  }
  uint64_t est = 0;
  for (uint32_t l : dense) est += (uint64_t)Ls[l].n1 * Ls[l].n2;
  for (const ZTask& t : tasks) est += (uint64_t)(t.n1 + t.n2) * std::min(t.kmax, 16u);
  if (Z.arena.bytes < est * sizeof(Cx)) {
    Z.arena.release();
    if ((rc = Z.arena.reserve(std::max<uint64_t>(est, 1) * sizeof(Cx)))) return rc;
  }
  const size_t budget = aca_ws_budget();
  const double* pts = H->pts.as<double>();
  const PointsSoA P{pts, pts + H->tree.n, pts + 2 * (size_t)H->tree.n};
  ScopedBuf ws, zs, dtasks, dres, dcopy;
  while (!tasks.empty()) {
    std::sort(tasks.begin(), tasks.end(), [](const ZTask& a, const ZTask& b) {
      return (uint64_t)(a.n1 + a.n2) * a.kcap > (uint64_t)(b.n1 + b.n2) * b.kcap;
    });
    std::vector<ZTask> retry;
    size_t i = 0;
    while (i < tasks.size()) {
      uint64_t wsc = 0, zsi = 0;
      size_t j = i;
      for (; j < tasks.size(); ++j) {
        const uint64_t w = zws_elems(tasks[j]);
        if (j > i && (wsc + w) * sizeof(Cx) + (zsi + tasks[j].n1 + tasks[j].n2) * 4 > budget) break;
        tasks[j].ws = wsc;
        tasks[j].zs = zsi;
        wsc += w;
        zsi += tasks[j].n1 + tasks[j].n2;
      }
      std::vector<ZTask> batch(tasks.begin() + i, tasks.begin() + j);
      i = j;
      H->stat_ws_bytes = std::max<uint64_t>(H->stat_ws_bytes, wsc * sizeof(Cx) + zsi * 4);
      H->stat_batches++;
      if ((rc = ws.reserve(std::max<uint64_t>(wsc, 1) * sizeof(Cx)))) return rc;
      if ((rc = zs.reserve(std::max<uint64_t>(zsi, 1) * 4))) return rc;
      if ((rc = upload(dtasks, batch, H->stream))) return rc;
      if ((rc = dres.reserve(batch.size() * sizeof(AcaResult)))) return rc;
      const uint32_t nb = (uint32_t)batch.size();
      helm_assemble_kernel<<<(nb + kWarps - 1) / kWarps, 32 * kWarps, 0, H->stream>>>(
          P, wavenumber, h, eps, dtasks.as<ZTask>(), nb, ws.as<Cx>(), zs.as<int>(), dres.as<AcaResult>(),
          H->tree.sym ? 1 : 0);
      AHX_CUDA(cudaGetLastError());
      std::vector<AcaResult> res(nb);
      AHX_CUDA(cudaMemcpyAsync(res.data(), dres.p, nb * sizeof(AcaResult), cudaMemcpyDeviceToHost, H->stream));
      AHX_CUDA(cudaStreamSynchronize(H->stream));
      std::vector<ZCopy> copies;
      for (uint32_t q = 0; q < nb; ++q) {
        const ZTask& t = batch[q];
        const AcaResult& r = res[q];
        if (r.status == kAcaOverflow && t.kcap < kcap_limit(t.kmax)) {
          ZTask u = t;
          u.kcap = std::min(kcap_limit(t.kmax), std::max(t.kcap * 4, 16u));
          retry.push_back(u);
          H->stat_retries++;
          continue;
        }
        if (r.status != kAcaOk) {
          dense.push_back(t.leaf);
          continue;
        }
        Z.aca_rank[t.leaf] = (int32_t)r.k_aca;
        Z.rank[t.leaf] = (int32_t)r.kt;
        if (r.kt == 0) continue;
        uint64_t off = 0;
        if ((rc = zarena_append(H, (uint64_t)r.kt * (t.n1 + t.n2), off))) return rc;
        Z.off[t.leaf] = off;
        const uint64_t un = t.ws + (uint64_t)(t.n1 + t.n2) * t.kcap;  // Un follows U and V
        copies.push_back(ZCopy{un, un + (uint64_t)t.n1 * t.kcap, off, t.n1, t.n2, r.kt, 0u});
      }
      if (!copies.empty()) {
        if ((rc = upload(dcopy, copies, H->stream))) return rc;
        helm_copy_kernel<<<(uint32_t)copies.size(), 128, 0, H->stream>>>(dcopy.as<ZCopy>(), ws.as<Cx>(),
                                                                          Z.arena.as<Cx>());
        AHX_CUDA(cudaGetLastError());
      }
      AHX_CUDA(cudaStreamSynchronize(H->stream));
    }
    tasks.swap(retry);
  }
  // dense leaves (inadmissible and failed ACA) in leaf order
  std::sort(dense.begin(), dense.end());
  std::vector<ZDense> dt;
  for (uint32_t l : dense) {
    const Leaf& L = Ls[l];
    uint64_t off = 0;
    if ((rc = zarena_append(H, (uint64_t)L.n1 * L.n2, off))) return rc;
    Z.off[l] = off;
    Z.rank[l] = -1;
    Z.aca_rank[l] = -1;
    dt.push_back(ZDense{L.b1, L.n1, L.b2, L.n2, off});
  }
  if (!dt.empty()) {
    ScopedBuf ddt;
    if ((rc = upload(ddt, dt, H->stream))) return rc;
    helm_dense_kernel<<<(uint32_t)dt.size(), 256, 0, H->stream>>>(P, wavenumber, h, ddt.as<ZDense>(), Z.arena.as<Cx>());
    AHX_CUDA(cudaGetLastError());
  }
  AHX_CUDA(cudaStreamSynchronize(H->stream));
  Z.assembled = true;
  return AHX_OK;
}

extern "C" int ahx_helm_ranks(const ahx_hmat* H, int32_t* ranks) {
  if (!H || !ranks) return AHX_ERR_ARG;
  if (!H->z.assembled) {
    set_error("ahx_helm_ranks: Helmholtz leaves not assembled");
    return AHX_ERR_STATE;
  }
  std::copy(H->z.rank.begin(), H->z.rank.end(), ranks);
  return AHX_OK;
}

namespace {
// dense diagonal block of a symmetric tree: stored full, given out packed (SyM)
bool packed_zleaf(const ahx_hmat* H, uint32_t l) {
  const Leaf& L = H->tree.leaves[l];
  return H->tree.sym && H->z.rank[l] < 0 && L.b1 == L.b2;
}
}  // namespace

extern "C" uint64_t ahx_helm_leaf_size(const ahx_hmat* H, uint32_t l) {
  if (!H || !H->z.assembled || l >= H->tree.leaves.size()) return 0;
  const Leaf& L = H->tree.leaves[l];
  const int32_t r = H->z.rank[l];
  if (packed_zleaf(H, l)) return (uint64_t)L.n1 * (L.n1 + 1) / 2;
  return r < 0 ? (uint64_t)L.n1 * L.n2 : (uint64_t)r * (L.n1 + L.n2);
}

extern "C" int ahx_helm_get_leaf(const ahx_hmat* H, uint32_t l, double* out) {
  if (!H || !out || l >= H->tree.leaves.size()) {
    set_error("ahx_helm_get_leaf: invalid argument");
    return AHX_ERR_ARG;
  }
  if (!H->z.assembled) {
    set_error("ahx_helm_get_leaf: Helmholtz leaves not assembled");
    return AHX_ERR_STATE;
  }
  const uint64_t cnt = ahx_helm_leaf_size(H, l);
  if (!cnt) return AHX_OK;
  AHX_CUDA(cudaSetDevice(H->device));
  if (packed_zleaf(H, l)) {
    // upper triangle column by column (data[i + j (j + 1) / 2] = A(i, j), i <= j)
    const uint32_t n1 = H->tree.leaves[l].n1;
    std::vector<Cx> full((size_t)n1 * n1);
    AHX_CUDA(cudaMemcpyAsync(full.data(), H->z.arena.as<Cx>() + H->z.off[l], full.size() * sizeof(Cx),
                             cudaMemcpyDeviceToHost, H->stream));
    AHX_CUDA(cudaStreamSynchronize(H->stream));
    Cx* o = reinterpret_cast<Cx*>(out);
    for (uint32_t j = 0; j < n1; ++j)
      for (uint32_t i = 0; i <= j; ++i) o[i + (size_t)j * (j + 1) / 2] = full[i + (size_t)j * n1];
    return AHX_OK;
  }
  AHX_CUDA(cudaMemcpyAsync(out, H->z.arena.as<Cx>() + H->z.off[l], cnt * sizeof(Cx), cudaMemcpyDeviceToHost,
                           H->stream));
  AHX_CUDA(cudaStreamSynchronize(H->stream));
  return AHX_OK;
}

namespace ahx {
cudaError_t launch_zmerge(const MergeParams& p, cudaStream_t s) {
  if (p.ntasks == 0) return cudaSuccess;
  zmerge_kernel<<<p.ntasks, 32, 0, s>>>(p);
  return cudaGetLastError();
}
}  // namespace ahx
