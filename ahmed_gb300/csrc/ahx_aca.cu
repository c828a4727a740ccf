// Batched adaptive cross approximation (ACA) with SVD recompression, FP64.
//
// One cooperative group per admissible leaf: a warp for leaves up to 256 rows
// and columns, a whole CTA for larger ones.  Every per-index array (rows of U,
// the row counters Z, columns of V, the column counters S) is owned by the
// thread with index % G == rank, so the only cross-thread traffic is through
// the group's all-reduces plus one barrier per cross.
//
// Algorithm (same control flow, same stopping rule and counters as the
// reference):
//   ACA row/column steps      Include/ACA.h:29-213
//   ACA driver                Include/ACA.h:217-350
//   leaf policy (maxk, i0)    Include/apprx.h:136-172
//   recompression addtrll     H/mblock_D.cpp:356-465 (Householder QR in place of
//                             dgeqrf/dormqr, one-sided Jacobi in place of dgesvd)
#include <climits>
#include <mutex>
#include <string>

#include "ahx_aca.cuh"
#include "ahx_hmat.hpp"

namespace ahx {
namespace {

constexpr int KSM = 32;        // ranks up to KSM keep the k x k SVD in shared memory
constexpr int LDS = KSM + 1;   // padded row stride of the shared k x k arrays
constexpr int kSmallWarps = 4; // warps (= leaves) per CTA of the small-leaf kernel

// per-group shared scratch (doubles)
constexpr int kSmemPerGroup = 2 * KSM * LDS + KSM + 2 * KSM + KSM;

struct Blk {
  PointsSoA P;
  double diag;
  uint32_t b1, n1, b2, n2;
  double* U;
  double* V;
  int* Z;
  int* S;
};

template <class Grp>
__device__ __forceinline__ bool owns(const Grp& g, uint32_t i, int G) {
  return (i % (uint32_t)G) == g.rank;
}

// next index >= j (cyclic) whose counter is not -1 (ACA.h:29-36)
template <int G, class Grp>
__device__ uint32_t nexti(const Grp& g, const int* Z, uint32_t n, uint32_t j) {
  uint32_t d = 0xffffffffu;
  for (uint32_t i = g.rank; i < n; i += G)
    if (Z[i] != -1) d = min(d, i >= j ? i - j : i + n - j);
  d = g.umin(d);
  return d == 0xffffffffu ? j : (j + d) % n;
}

// ACA_row_step (ACA.h:46-130)
template <int G, class Grp>
__device__ bool row_step(const Grp& g, const Blk& B, uint32_t& klast, uint32_t& i0, uint32_t k,
                         uint32_t& no, double& nrmlsk2, double scale) {
  const uint32_t n1 = B.n1, n2 = B.n2;
  double* const pu = B.U + (size_t)k * n1;
  double* const pv = B.V + (size_t)k * n2;
  ArgMax am;
  for (;;) {
    g.sync();
    const uint32_t gi = B.b1 + i0;
    const double xi = B.P.x[gi], yi = B.P.y[gi], zi = B.P.z[gi];
    am = ArgMax{0.0, 0xffffffffu, 0.0};
    for (uint32_t j = g.rank; j < n2; j += G) {
      double v = lap_entry_aca(B.P, gi, B.b2 + j, xi, yi, zi, B.diag);
      for (uint32_t l = 0; l < k; ++l) v = fma(-B.U[(size_t)l * n1 + i0], B.V[(size_t)l * n2 + j], v);
      pv[j] = v;
      if (B.S[j] >= 0) {
        const double a = fabs(v);
        if (gt_nonneg(a, am.v)) am = ArgMax{a, j, v};
      }
    }
    am = g.argmax(am);
    if (!(am.v < 1e-14 * scale)) break;
    if (owns(g, i0, G)) B.Z[i0] = -1;
    if (++no >= n1) return false;
    g.sync();
    i0 = nexti<G>(g, B.Z, n1, i0);
  }
  const uint32_t j0 = am.idx;
  const double sqrtpiv = sqrt(am.v);
  const double sca = sqrtpiv / am.sv;
  const double thr = 1e-8 * scale * sqrtpiv;
  double nrmv2 = 0.0;
  for (uint32_t j = g.rank; j < n2; j += G) {
    if (B.S[j] >= 0) {
      const double e = pv[j] * sca;
      pv[j] = e;
      nrmv2 += e * e;
      if (gt_nonneg(fabs(e), thr)) ++B.S[j];
    }
  }
  const uint32_t gj = B.b2 + j0;
  const double xj = B.P.x[gj], yj = B.P.y[gj], zj = B.P.z[gj];
  for (uint32_t i = g.rank; i < n1; i += G) {
    double u = lap_entry_aca(B.P, gj, B.b1 + i, xj, yj, zj, B.diag);
    for (uint32_t l = 0; l < k; ++l) u = fma(-B.V[(size_t)l * n2 + j0], B.U[(size_t)l * n1 + i], u);
    pu[i] = u;
  }
  klast = (uint32_t)g.imax(owns(g, i0, G) ? B.Z[i0] : INT_MIN);
  if (owns(g, i0, G)) B.Z[i0] = -1;
  if (owns(g, j0, G)) B.S[j0] = -1;
  ++no;
  const double dsca = 1.0 / sqrtpiv;
  double nrmu2 = 0.0;
  ArgMax nm{0.0, 0xffffffffu, 0.0};
  for (uint32_t i = g.rank; i < n1; i += G) {
    const double e = pu[i] * dsca;
    pu[i] = e;
    const double ea = fabs(e);
    if (B.Z[i] >= 0 && gt_nonneg(ea, thr)) ++B.Z[i];
    nrmu2 += ea * ea;
    if (B.Z[i] >= 0 && gt_nonneg(ea, nm.v)) nm = ArgMax{ea, i, e};
  }
  g.sum2(nrmu2, nrmv2);
  nm = g.argmax(nm);
  if (nm.v > 0.0) i0 = nm.idx;
  nrmlsk2 = nrmu2 * nrmv2;
  return true;
}

// ACA_col_step (ACA.h:134-213)
template <int G, class Grp>
__device__ bool col_step(const Grp& g, const Blk& B, uint32_t& j0, uint32_t k, uint32_t& no,
                         double& nrmlsk2, double scale) {
  const uint32_t n1 = B.n1, n2 = B.n2;
  double* const pu = B.U + (size_t)k * n1;
  double* const pv = B.V + (size_t)k * n2;
  ArgMax am;
  for (;;) {
    g.sync();
    const uint32_t gj = B.b2 + j0;
    const double xj = B.P.x[gj], yj = B.P.y[gj], zj = B.P.z[gj];
    am = ArgMax{0.0, 0xffffffffu, 0.0};
    for (uint32_t i = g.rank; i < n1; i += G) {
      double u = lap_entry_aca(B.P, gj, B.b1 + i, xj, yj, zj, B.diag);
      for (uint32_t l = 0; l < k; ++l) u = fma(-B.V[(size_t)l * n2 + j0], B.U[(size_t)l * n1 + i], u);
      pu[i] = u;
      if (B.Z[i] >= 0) {
        const double a = fabs(u);
        if (gt_nonneg(a, am.v)) am = ArgMax{a, i, u};
      }
    }
    am = g.argmax(am);
    if (!(am.v < 1e-14 * scale)) break;
    if (owns(g, j0, G)) B.S[j0] = -1;
    if (++no >= n2) return false;
    g.sync();
    j0 = nexti<G>(g, B.S, n2, j0);
  }
  const uint32_t i0 = am.idx;
  const double sqrtpiv = sqrt(am.v);
  const double sca = sqrtpiv / am.sv;
  const double thr = 1e-8 * scale * sqrtpiv;
  double nrmu2 = 0.0;
  for (uint32_t i = g.rank; i < n1; i += G) {
    if (B.Z[i] >= 0) {
      const double e = pu[i] * sca;
      pu[i] = e;
      nrmu2 += e * e;
      if (gt_nonneg(fabs(e), thr)) ++B.Z[i];
    }
  }
  const uint32_t gi = B.b1 + i0;
  const double xi = B.P.x[gi], yi = B.P.y[gi], zi = B.P.z[gi];
  for (uint32_t j = g.rank; j < n2; j += G) {
    double v = lap_entry_aca(B.P, gi, B.b2 + j, xi, yi, zi, B.diag);
    for (uint32_t l = 0; l < k; ++l) v = fma(-B.U[(size_t)l * n1 + i0], B.V[(size_t)l * n2 + j], v);
    pv[j] = v;
  }
  if (owns(g, i0, G)) B.Z[i0] = -1;
  if (owns(g, j0, G)) B.S[j0] = -1;
  ++no;
  const double dsca = 1.0 / sqrtpiv;
  double nrmv2 = 0.0;
  ArgMax nm{0.0, 0xffffffffu, 0.0};
  for (uint32_t j = g.rank; j < n2; j += G) {
    const double e = pv[j] * dsca;
    pv[j] = e;
    const double ea = fabs(e);
    if (B.S[j] >= 0 && gt_nonneg(ea, thr)) ++B.S[j];
    nrmv2 += ea * ea;
    if (gt_nonneg(ea, nm.v)) nm = ArgMax{ea, j, e};  // no S filter here, as in the reference
  }
  g.sum2(nrmu2, nrmv2);
  nm = g.argmax(nm);
  if (nm.v > 0.0) j0 = nm.idx;
  nrmlsk2 = nrmu2 * nrmv2;
  return true;
}

// ACA driver (ACA.h:217-350).  Returns the status, the rank in k.
template <int G, class Grp>
__device__ int aca(const Grp& g, const Blk& B, uint32_t i0, uint32_t kmax, uint32_t kcap,
                   double eps, uint32_t& kout) {
  const uint32_t n1 = B.n1, n2 = B.n2;
  for (uint32_t i = g.rank; i < n1; i += G) B.Z[i] = 0;
  for (uint32_t j = g.rank; j < n2; j += G) B.S[j] = 0;
  double scale;
  {
    const uint32_t a = B.b1, b = B.b2;
    scale = fabs(lap_entry(B.P, a, b, B.P.x[a], B.P.y[a], B.P.z[a], B.diag));
  }
  uint32_t k = 0, no = 0, klast = 0, inext = i0, j0 = 0;
  int kmin = -2, keps = -1;
  double nrmlsk2 = 0.0, nrms2 = 0.0;
  int outcome = -1;  // 0 NSUCC, 1 SUCC, 2 overflow
  do {
    if (k >= kcap) { outcome = kAcaOverflow; break; }
    inext = i0;
    if (!row_step<G>(g, B, klast, inext, k, no, nrmlsk2, scale)) {
      nrmlsk2 = 0.0;
      outcome = kAcaOk;
      break;
    }
    double sum = 0.0;
    const double* uk = B.U + (size_t)k * n1;
    const double* vk = B.V + (size_t)k * n2;
    for (uint32_t l = 0; l < k; ++l) {
      double du = 0.0, dv = 0.0;
      for (uint32_t i = g.rank; i < n1; i += G) du += B.U[(size_t)l * n1 + i] * uk[i];
      for (uint32_t j = g.rank; j < n2; j += G) dv += B.V[(size_t)l * n2 + j] * vk[j];
      g.sum2(du, dv);
      sum += du * dv;
    }
    nrms2 += 2.0 * sum + nrmlsk2;
    const bool stpcrit = nrmlsk2 < eps * eps * nrms2;
    if (stpcrit && keps == -1) keps = (int)klast + 1;
    ++k;
    scale = sqrt(nrmlsk2 / (double)(uint32_t)(n1 * n2));
    if (keps > 0) {
      ArgMinI m{INT_MAX, 0xffffffffu};
      for (uint32_t i = g.rank; i < n1; i += G)
        if (B.Z[i] >= 0 && B.Z[i] < m.v) m = ArgMinI{B.Z[i], i};
      m = g.argmin(m);
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
        for (uint32_t j = g.rank; j < n2; j += G)
          if (B.S[j] >= 0 && B.S[j] < m.v) m = ArgMinI{B.S[j], j};
        m = g.argmin(m);
        if (m.v == INT_MAX) {
          nrmlsk2 = 0.0;
          outcome = kAcaOk;
          break;
        }
        kmin = m.v;
        j0 = m.idx;
        if (kmin >= keps) { outcome = kAcaOk; break; }
        if (k >= kcap) { outcome = kAcaOverflow; break; }
        if (!col_step<G>(g, B, j0, k, no, nrmlsk2, scale)) {
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
    if (epsa >= eps) outcome = kAcaFail;  // NaN (0/0) stays a success, as in the reference
  }
  kout = k;
  g.sync();
  return outcome;
}

// ACAr_step (ACA.h:579-655), the simplified cross of the symmetric assembly:
// rows are skipped only for a small pivot, the pivot column is searched over
// all columns, and the next row is the largest unused entry of the new column.
template <int G, class Grp>
__device__ bool acar_step(const Grp& g, const Blk& B, uint32_t& i0, uint32_t k, uint32_t& no, double& nrmlsk2,
                          double scale) {
  const uint32_t n1 = B.n1, n2 = B.n2;
  double* const pu = B.U + (size_t)k * n1;
  double* const pv = B.V + (size_t)k * n2;
  ArgMax am;
  for (;;) {
    g.sync();
    const uint32_t gi = B.b1 + i0;
    const double xi = B.P.x[gi], yi = B.P.y[gi], zi = B.P.z[gi];
    am = ArgMax{0.0, 0xffffffffu, 0.0};
    for (uint32_t j = g.rank; j < n2; j += G) {
      double v = lap_entry_aca(B.P, gi, B.b2 + j, xi, yi, zi, B.diag);
      for (uint32_t l = 0; l < k; ++l) v = fma(-B.U[(size_t)l * n1 + i0], B.V[(size_t)l * n2 + j], v);
      pv[j] = v;
      const double a = fabs(v);
      if (gt_nonneg(a, am.v)) am = ArgMax{a, j, v};
    }
    am = g.argmax(am);
    if (!(am.v < 1e-14 * scale)) break;
    if (owns(g, i0, G)) B.Z[i0] = -1;
    if (++no >= n1) return false;
    g.sync();
    i0 = nexti<G>(g, B.Z, n1, i0);
  }
  const uint32_t j0 = am.idx;
  const double sqrtpiv = sqrt(am.v);
  const double sca = sqrtpiv / am.sv;
  double nrmv2 = 0.0;
  for (uint32_t j = g.rank; j < n2; j += G) {
    const double e = pv[j] * sca;
    pv[j] = e;
    nrmv2 += e * e;
  }
  const uint32_t gj = B.b2 + j0;
  const double xj = B.P.x[gj], yj = B.P.y[gj], zj = B.P.z[gj];
  for (uint32_t i = g.rank; i < n1; i += G) {
    double u = lap_entry_aca(B.P, gj, B.b1 + i, xj, yj, zj, B.diag);
    for (uint32_t l = 0; l < k; ++l) u = fma(-B.V[(size_t)l * n2 + j0], B.U[(size_t)l * n1 + i], u);
    pu[i] = u;
  }
  if (owns(g, i0, G)) B.Z[i0] = -1;
  ++no;
  const double dsca = 1.0 / sqrtpiv;
  double nrmu2 = 0.0;
  ArgMax nm{0.0, 0xffffffffu, 0.0};
  for (uint32_t i = g.rank; i < n1; i += G) {
    const double e = pu[i] * dsca;
    pu[i] = e;
    const double ea = fabs(e);
    nrmu2 += ea * ea;
    if (B.Z[i] >= 0 && gt_nonneg(ea, nm.v)) nm = ArgMax{ea, i, e};
  }
  g.sum2(nrmu2, nrmv2);
  nm = g.argmax(nm);
  if (nm.v > 0.0) i0 = nm.idx;
  nrmlsk2 = nrmu2 * nrmv2;
  return true;
}

// ACAr driver (ACA.h:657-720): crosses until the last one is below eps of the
// approximation's norm, no more than n2 rows used, or kmax crosses.
template <int G, class Grp>
__device__ int acar(const Grp& g, const Blk& B, uint32_t i0, uint32_t kmax, uint32_t kcap, double eps,
                    uint32_t& kout) {
  const uint32_t n1 = B.n1, n2 = B.n2;
  for (uint32_t i = g.rank; i < n1; i += G) B.Z[i] = 0;
  double scale;
  {
    const uint32_t a = B.b1, b = B.b2;
    scale = fabs(lap_entry(B.P, a, b, B.P.x[a], B.P.y[a], B.P.z[a], B.diag));
  }
  uint32_t k = 0, no = 0;
  double nrmlsk2 = 0.0, nrms2 = 0.0;
  int outcome = -1;
  do {
    if (k >= kcap) {
      outcome = kAcaOverflow;
      break;
    }
    if (!acar_step<G>(g, B, i0, k, no, nrmlsk2, scale)) {
      nrmlsk2 = 0.0;
      break;
    }
    double sum = 0.0;
    const double* uk = B.U + (size_t)k * n1;
    const double* vk = B.V + (size_t)k * n2;
    for (uint32_t l = 0; l < k; ++l) {
      double du = 0.0, dv = 0.0;
      for (uint32_t i = g.rank; i < n1; i += G) du += B.U[(size_t)l * n1 + i] * uk[i];
      for (uint32_t j = g.rank; j < n2; j += G) dv += B.V[(size_t)l * n2 + j] * vk[j];
      g.sum2(du, dv);
      sum += du * dv;
    }
    nrms2 += 2.0 * sum + nrmlsk2;
    ++k;
    scale = sqrt(nrmlsk2 / (double)(uint32_t)(n1 * n2));
  } while (no < n2 && k < kmax && nrmlsk2 >= eps * eps * nrms2);
  if (outcome < 0) {
    const double epsa = sqrt(nrmlsk2 / nrms2);
    outcome = epsa >= eps ? kAcaFail : kAcaOk;  // NaN (0/0) stays a success, as in the reference
  }
  kout = k;
  g.sync();
  return outcome;
}

// In-place Householder QR of A (m x k, column-major) by the group; tau[k].
template <int G, class Grp>
__device__ void group_qr(const Grp& g, uint32_t m, uint32_t k, double* A, double* tau) {
  const uint32_t kk = min(m, k);
  for (uint32_t c = 0; c < kk; ++c) {
    double* a = A + (size_t)c * m;
    double xn2 = 0.0, alpha = 0.0;
    for (uint32_t i = g.rank; i < m; i += G) {
      if (i > c) xn2 += a[i] * a[i];
      else if (i == c) alpha = a[i];
    }
    g.sum2(xn2, alpha);
    if (xn2 == 0.0) {
      if (g.rank == 0) tau[c] = 0.0;
      continue;
    }
    const double nrm = sqrt(alpha * alpha + xn2);
    const double beta = alpha >= 0.0 ? -nrm : nrm;
    const double t = (beta - alpha) / beta;
    const double sc = 1.0 / (alpha - beta);
    if (g.rank == 0) tau[c] = t;
    for (uint32_t i = g.rank; i < m; i += G) {
      if (i > c) a[i] *= sc;
      else if (i == c) a[i] = beta;
    }
    for (uint32_t q = c + 1; q < k; ++q) {
      double* b = A + (size_t)q * m;
      double s = 0.0;
      for (uint32_t i = g.rank; i < m; i += G) {
        if (i > c) s += a[i] * b[i];
        else if (i == c) s += b[i];
      }
      s = g.sum(s) * t;
      for (uint32_t i = g.rank; i < m; i += G) {
        if (i > c) b[i] -= s * a[i];
        else if (i == c) b[i] -= s;
      }
    }
  }
}

// C (m x nc, column-major, ldc m) := Q C, Q = H_0 ... H_{kr-1} stored in A/tau.
// Rows of C are owned like rows of A; tau is read from memory written by rank 0
// before a group barrier.
template <int G, class Grp>
__device__ void group_apply_q(const Grp& g, uint32_t m, uint32_t kr, const double* A,
                              const double* tau, uint32_t nc, double* C) {
  for (int c = (int)kr - 1; c >= 0; --c) {
    const double t = tau[c];
    if (t == 0.0) continue;
    const double* a = A + (size_t)c * m;
    for (uint32_t q = 0; q < nc; ++q) {
      double* b = C + (size_t)q * m;
      double s = 0.0;
      for (uint32_t i = g.rank; i < m; i += G) {
        if (i > (uint32_t)c) s += a[i] * b[i];
        else if (i == (uint32_t)c) s += b[i];
      }
      s = g.sum(s) * t;
      for (uint32_t i = g.rank; i < m; i += G) {
        if (i > (uint32_t)c) b[i] -= s * a[i];
        else if (i == (uint32_t)c) b[i] -= s;
      }
    }
  }
}

// One-sided Jacobi on the columns of R (m x n, m, n <= 16) by one warp, in
// tournament order (Brent-Luk round robin): every round rotates n/2 disjoint
// column pairs at once, one group of 4 lanes per pair, each lane holding rows
// sub, sub + 4, sub + 8, sub + 12.  Rotations are accumulated in Vs (n x n).
__device__ void jacobi_warp16(uint32_t m, uint32_t n, double* R, double* Vs, uint32_t ld) {
  const uint32_t lane = threadIdx.x & 31, grp = lane >> 2, sub = lane & 3;
  const uint32_t ne = n + (n & 1);  // a dummy column when n is odd
  for (int sweep = 0; sweep < 40; ++sweep) {
    bool rotated = false;
    for (uint32_t r = 0; r + 1 < ne; ++r) {
      __syncwarp();
      uint32_t a = 0, b = 0;
      bool live = grp < ne / 2;
      if (live) {
        const uint32_t pa = grp, pb = ne - 1 - grp;
        a = pa == 0 ? 0 : 1 + (pa - 1 + r) % (ne - 1);
        b = pb == 0 ? 0 : 1 + (pb - 1 + r) % (ne - 1);
        if (a > b) {
          const uint32_t t = a;
          a = b;
          b = t;
        }
        live = b < n;
      }
      double al = 0.0, be = 0.0, ga = 0.0;
      if (live) {
        for (uint32_t i = sub; i < m; i += 4) {
          const double x = R[i * ld + a], y = R[i * ld + b];
          al = fma(x, x, al);
          be = fma(y, y, be);
          ga = fma(x, y, ga);
        }
      }
#pragma unroll
      for (int o = 1; o < 4; o <<= 1) {
        al += __shfl_xor_sync(0xffffffffu, al, o);
        be += __shfl_xor_sync(0xffffffffu, be, o);
        ga += __shfl_xor_sync(0xffffffffu, ga, o);
      }
      // rotate unless |ga| <= 1e-15 sqrt(al be)  (tested without a square root)
      const bool rot = live && ga != 0.0 && ga * ga > 1e-30 * (al * be);
      if (rot) {
        const double zeta = (be - al) / (2.0 * ga);
        const double t = copysign(1.0, zeta) / (fabs(zeta) + sqrt(fma(zeta, zeta, 1.0)));
        const double c = rsqrt(fma(t, t, 1.0));
        const double s = c * t;
        for (uint32_t i = sub; i < m; i += 4) {
          const double x = R[i * ld + a], y = R[i * ld + b];
          R[i * ld + a] = c * x - s * y;
          R[i * ld + b] = s * x + c * y;
        }
        for (uint32_t i = sub; i < n; i += 4) {
          const double x = Vs[i * ld + a], y = Vs[i * ld + b];
          Vs[i * ld + a] = c * x - s * y;
          Vs[i * ld + b] = s * x + c * y;
        }
      }
      rotated |= rot;
    }
    if (!__any_sync(0xffffffffu, rotated)) break;
  }
  __syncwarp();
}

// One-sided Jacobi (Hestenes) on the columns of R (mmin x nmin, column-major with
// stride ld), rotations accumulated in Vs: the column pairs of a round-robin
// tournament (circle method) rotate in parallel, one warp per pair, so that a
// whole CTA works on one wide SVD.  Same rotation formulas and stopping rule as
// the serial sweeps; the pair order differs.
__device__ void jacobi_cta(uint32_t mmin, uint32_t nmin, double* R, double* Vs, uint32_t ld) {
  __shared__ int rotated;
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  const uint32_t np = (nmin + 1) & ~1u;  // players: a dummy one when nmin is odd
  for (int sweep = 0; sweep < 40; ++sweep) {
    __syncthreads();
    if (threadIdx.x == 0) rotated = 0;
    __syncthreads();
    for (uint32_t r = 0; r + 1 < np; ++r) {
      for (uint32_t k = warp; k < np / 2; k += nw) {
        const uint32_t pa = k, pb = np - 1 - k;
        const uint32_t a = pa == 0 ? 0 : (pa - 1 + r) % (np - 1) + 1;
        const uint32_t b = pb == 0 ? 0 : (pb - 1 + r) % (np - 1) + 1;
        const uint32_t p = min(a, b), q = max(a, b);
        if (q >= nmin) continue;  // the dummy's pair
        double* cp = R + (size_t)p * ld;
        double* cq = R + (size_t)q * ld;
        double al = 0.0, be = 0.0, ga = 0.0;
        for (uint32_t i = lane; i < mmin; i += 32) {
          const double x = cp[i], y = cq[i];
          al += x * x;
          be += y * y;
          ga += x * y;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          al += __shfl_xor_sync(0xffffffffu, al, o);
          be += __shfl_xor_sync(0xffffffffu, be, o);
          ga += __shfl_xor_sync(0xffffffffu, ga, o);
        }
        if (ga == 0.0 || fabs(ga) <= 1e-15 * sqrt(al * be)) continue;
        if (lane == 0) rotated = 1;
        const double zeta = (be - al) / (2.0 * ga);
        const double t = (zeta >= 0.0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
        const double c = 1.0 / sqrt(1.0 + t * t);
        const double s = c * t;
        for (uint32_t i = lane; i < mmin; i += 32) {
          const double x = cp[i], y = cq[i];
          cp[i] = c * x - s * y;
          cq[i] = s * x + c * y;
        }
        double* vp = Vs + (size_t)p * ld;
        double* vq = Vs + (size_t)q * ld;
        for (uint32_t i = lane; i < nmin; i += 32) {
          const double x = vp[i], y = vq[i];
          vp[i] = c * x - s * y;
          vq[i] = s * x + c * y;
        }
      }
      __syncthreads();
    }
    if (!rotated) break;
  }
  __syncthreads();
}

// addtrll (H/mblock_D.cpp:356-465) for a fresh low-rank block: recompress U V^T
// of rank k to kt <= k columns (relative threshold delta, absolute 1e-64).
// Results in Un (n1 x kt) and Vn (n2 x kt).
template <int G, class Grp>
__device__ uint32_t recompress(const Grp& g, uint32_t n1, uint32_t n2, uint32_t k, double* U,
                               double* V, double* Un, double* Vn, double delta, double* R,
                               double* Vs, uint32_t ld, double* sig, double* tau, int* perm, bool cm = false) {
  if (k == 0) return 0;
  // R and Vs: row-major with a padded stride in shared memory, column-major (the
  // Jacobi sweeps read columns) in the global workspace
  auto ix = [&](uint32_t i, uint32_t j) -> size_t { return cm ? (size_t)j * ld + i : (size_t)i * ld + j; };
  const uint32_t mmin = min(n1, k), nmin = min(n2, k), amin = min(mmin, nmin);
  double* tau1 = tau;
  double* tau2 = tau + k;
  group_qr<G>(g, n1, k, U, tau1);
  group_qr<G>(g, n2, k, V, tau2);
  g.sync();
  // R = R1 R2^T (Include/blas.h:2767-2781), rows owned by i % G
  double fro = 0.0;
  for (uint32_t i = g.rank; i < mmin; i += G) {
    for (uint32_t j = 0; j < nmin; ++j) {
      double d = 0.0;
      for (uint32_t l = max(i, j); l < k; ++l) d += U[i + (size_t)l * n1] * V[j + (size_t)l * n2];
      R[ix(i, j)] = d;
      fro += d * d;
    }
  }
  fro = g.sum(fro);
  const double thresh = delta * sqrt(fro) / (double)sqrtf((float)mmin * (float)nmin);
  for (uint32_t i = g.rank; i < mmin; i += G)
    for (uint32_t j = 0; j < nmin; ++j)
      if (fabs(R[ix(i, j)]) < thresh) R[ix(i, j)] = 0.0;
  for (uint32_t i = g.rank; i < nmin; i += G)
    for (uint32_t j = 0; j < nmin; ++j) Vs[ix(i, j)] = (i == j) ? 1.0 : 0.0;
  // one-sided Jacobi on the columns of R (Hestenes), rotations accumulated in Vs
  if (G == 32 && !cm && mmin <= 16 && nmin <= 16) {
    g.sync();
    jacobi_warp16(mmin, nmin, R, Vs, ld);
  } else if (G > 32 && cm) {
    g.sync();
    jacobi_cta(mmin, nmin, R, Vs, ld);
  } else
  for (int sweep = 0; sweep < 40; ++sweep) {
    bool rotated = false;
    for (uint32_t p = 0; p + 1 < nmin; ++p) {
      for (uint32_t q = p + 1; q < nmin; ++q) {
        double al = 0.0, be = 0.0, ga = 0.0;
        for (uint32_t i = g.rank; i < mmin; i += G) {
          const double x = R[ix(i, p)], y = R[ix(i, q)];
          al += x * x;
          be += y * y;
          ga += x * y;
        }
        g.sum3(al, be, ga);
        if (ga == 0.0 || fabs(ga) <= 1e-15 * sqrt(al * be)) continue;
        rotated = true;
        const double zeta = (be - al) / (2.0 * ga);
        const double t = (zeta >= 0.0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
        const double c = 1.0 / sqrt(1.0 + t * t);
        const double s = c * t;
        for (uint32_t i = g.rank; i < mmin; i += G) {
          const double x = R[ix(i, p)], y = R[ix(i, q)];
          R[ix(i, p)] = c * x - s * y;
          R[ix(i, q)] = s * x + c * y;
        }
        for (uint32_t i = g.rank; i < nmin; i += G) {
          const double x = Vs[ix(i, p)], y = Vs[ix(i, q)];
          Vs[ix(i, p)] = c * x - s * y;
          Vs[ix(i, q)] = s * x + c * y;
        }
      }
    }
    if (!rotated) break;
  }
  g.sync();
  for (uint32_t j = 0; j < nmin; ++j) {
    double s = 0.0;
    for (uint32_t i = g.rank; i < mmin; i += G) s += R[ix(i, j)] * R[ix(i, j)];
    s = g.sum(s);
    if (g.rank == 0) sig[j] = sqrt(s);
  }
  g.sync();
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
    const double s0 = sig[perm[0]];
    while (kt > 0 && (sig[perm[kt - 1]] <= delta * s0 || sig[perm[kt - 1]] < 1e-64)) --kt;
    perm[nmin] = (int)kt;  // the slot after the permutation holds kt
  }
  g.sync();
  const uint32_t kt = (uint32_t)perm[nmin];
  // Un = Q1 [R(:, perm[:kt]); 0],  Vn = Q2 [Vs(:, perm[:kt]); 0]
  for (uint32_t j = 0; j < kt; ++j) {
    const int pj = perm[j];
    for (uint32_t i = g.rank; i < n1; i += G) Un[i + (size_t)j * n1] = i < mmin ? R[ix(i, pj)] : 0.0;
    for (uint32_t i = g.rank; i < n2; i += G) Vn[i + (size_t)j * n2] = i < nmin ? Vs[ix(i, pj)] : 0.0;
  }
  group_apply_q<G>(g, n1, mmin, U, tau1, kt, Un);
  group_apply_q<G>(g, n2, nmin, V, tau2, kt, Vn);
  return kt;
}

// Recompression of a wide union (agglomeration) by a warp or a whole CTA.  The steps of
// recompress up to R = R1 R2^T (QR of both factors, small entries dropped), then
// a column-pivoted Householder QR of R that stops once the trailing columns'
// Frobenius norm is at most 1e-2 delta max_j |R(:, j)| (<= 1e-2 delta sigma_0,
// so no singular value moves by more than that), then one-sided Jacobi on the
// transpose of the kept rows: rr columns instead of nmin, and the pivoted
// triangle converges in fewer sweeps.  R = Qr T P^T, T^T Z = W S gives
// R = (Qr Z) S (P W)^T.  Workspaces (column-major, stride ld): R (mmin x nmin,
// later the reflectors), Tt (nmin x rr), Z (rr x rr); cn, qtau: nmin doubles;
// cperm: nmin ints; perm: rr + 1 ints.
template <int G, class Grp>
__device__ uint32_t recompress_qrcp(const Grp& g, uint32_t n1, uint32_t n2, uint32_t k, double* U, double* V,
                                    double* Un, double* Vn, double delta, double* R, double* Tt, double* Z,
                                    uint32_t ld, double* sig, double* tau, double* cn, double* qtau, int* cperm,
                                    int* perm) {
  if (k == 0) return 0;
  constexpr uint32_t NW = G / 32;
  const uint32_t warp = g.rank >> 5, lane = g.rank & 31;
  const uint32_t mmin = min(n1, k), nmin = min(n2, k), amin = min(mmin, nmin);
  double* tau1 = tau;
  double* tau2 = tau + k;
  group_qr<G>(g, n1, k, U, tau1);
  group_qr<G>(g, n2, k, V, tau2);
  g.sync();
  double fro = 0.0;
  for (uint32_t i = g.rank; i < mmin; i += G) {
    for (uint32_t j = 0; j < nmin; ++j) {
      double d = 0.0;
      for (uint32_t l = max(i, j); l < k; ++l) d += U[i + (size_t)l * n1] * V[j + (size_t)l * n2];
      R[i + (size_t)j * ld] = d;
      fro += d * d;
    }
  }
  fro = g.sum(fro);
  const double thresh = delta * sqrt(fro) / (double)sqrtf((float)mmin * (float)nmin);
  for (uint32_t i = g.rank; i < mmin; i += G)
    for (uint32_t j = 0; j < nmin; ++j)
      if (fabs(R[i + (size_t)j * ld]) < thresh) R[i + (size_t)j * ld] = 0.0;
  g.sync();
  // column norms
  for (uint32_t j = warp; j < nmin; j += NW) {
    double s = 0.0;
    for (uint32_t i = lane; i < mmin; i += 32) {
      const double x = R[i + (size_t)j * ld];
      s += x * x;
    }
    s = Group<32>::sum(s);
    if (lane == 0) {
      cn[j] = s;
      cperm[j] = (int)j;
    }
  }
  g.sync();
  ArgMax cm{0.0, 0xffffffffu, 0.0};
  for (uint32_t j = g.rank; j < nmin; j += G)
    if (gt_nonneg(cn[j], cm.v)) cm = ArgMax{cn[j], j, 0.0};
  cm = g.argmax(cm);
  const double tol2 = (1e-2 * delta) * (1e-2 * delta) * cm.v;
  // column-pivoted QR, stopped at the trailing norm tol
  uint32_t rr = amin;
  for (uint32_t c = 0; c < amin; ++c) {
    double tot = 0.0;
    ArgMax am{0.0, 0xffffffffu, 0.0};
    for (uint32_t j = c + g.rank; j < nmin; j += G) {
      const double v = cn[j];
      tot += v;
      if (gt_nonneg(v, am.v)) am = ArgMax{v, j, 0.0};
    }
    tot = g.sum(tot);
    am = g.argmax(am);
    if (tot <= tol2 || am.idx >= nmin) {
      rr = c;
      break;
    }
    const uint32_t p = am.idx;
    if (p != c) {
      for (uint32_t i = g.rank; i < mmin; i += G) {
        const double x = R[i + (size_t)c * ld];
        R[i + (size_t)c * ld] = R[i + (size_t)p * ld];
        R[i + (size_t)p * ld] = x;
      }
      if (g.rank == 0) {
        const double x = cn[c];
        cn[c] = cn[p];
        cn[p] = x;
        const int q = cperm[c];
        cperm[c] = cperm[p];
        cperm[p] = q;
      }
    }
    g.sync();
    double* a = R + (size_t)c * ld;
    double xn2 = 0.0, alpha = 0.0;
    for (uint32_t i = g.rank; i < mmin; i += G) {
      if (i > c) xn2 += a[i] * a[i];
      else if (i == c) alpha = a[i];
    }
    g.sum2(xn2, alpha);
    double t = 0.0;
    if (xn2 != 0.0) {
      const double nrm = sqrt(alpha * alpha + xn2);
      const double beta = alpha >= 0.0 ? -nrm : nrm;
      t = (beta - alpha) / beta;
      const double sc = 1.0 / (alpha - beta);
      for (uint32_t i = g.rank; i < mmin; i += G) {
        if (i > c) a[i] *= sc;
        else if (i == c) a[i] = beta;
      }
    }
    if (g.rank == 0) qtau[c] = t;
    g.sync();
    // the trailing columns: b -= t v (v^T b), then their norms below row c
    for (uint32_t j = c + 1 + warp; j < nmin; j += NW) {
      double* b = R + (size_t)j * ld;
      if (t != 0.0) {
        double s = 0.0;
        for (uint32_t i = c + lane; i < mmin; i += 32) s += (i == c ? 1.0 : a[i]) * b[i];
        s = Group<32>::sum(s) * t;
        for (uint32_t i = c + lane; i < mmin; i += 32) b[i] -= s * (i == c ? 1.0 : a[i]);
      }
      double s2 = 0.0;
      for (uint32_t i = c + lane; i < mmin; i += 32)
        if (i > c) s2 += b[i] * b[i];
      s2 = Group<32>::sum(s2);
      if (lane == 0) cn[j] = s2;
    }
    g.sync();
  }
  // Tt = T^T (T = the first rr rows of the triangle, pivoted column order), Z = I
  for (uint32_t e = g.rank; e < nmin * rr; e += G) {
    const uint32_t i = e / nmin, j = e - i * nmin;
    Tt[j + (size_t)i * ld] = j >= i ? R[i + (size_t)j * ld] : 0.0;
  }
  for (uint32_t e = g.rank; e < rr * rr; e += G) {
    const uint32_t i = e % rr, j = e / rr;
    Z[i + (size_t)j * ld] = i == j ? 1.0 : 0.0;
  }
  g.sync();
  if (rr > 1) jacobi_cta(nmin, rr, Tt, Z, ld);
  for (uint32_t j = warp; j < rr; j += NW) {
    double s = 0.0;
    for (uint32_t i = lane; i < nmin; i += 32) {
      const double x = Tt[i + (size_t)j * ld];
      s += x * x;
    }
    s = Group<32>::sum(s);
    if (lane == 0) sig[j] = sqrt(s);
  }
  g.sync();
  if (g.rank == 0) {
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
  g.sync();
  const uint32_t kt = (uint32_t)perm[rr];
  // Un = Q1 [Qr [Z(:, p) s_p; 0]; 0],  Vn = Q2 [P W(:, p); 0]
  for (uint32_t j = 0; j < kt; ++j) {
    const int pj = perm[j];
    const double sj = sig[pj];
    for (uint32_t i = g.rank; i < n1; i += G) Un[i + (size_t)j * n1] = i < rr ? Z[i + (size_t)pj * ld] * sj : 0.0;
    for (uint32_t i = g.rank; i < n2; i += G) {
      if (i < nmin) Vn[(uint32_t)cperm[i] + (size_t)j * n2] = Tt[i + (size_t)pj * ld] / sj;
      else Vn[i + (size_t)j * n2] = 0.0;
    }
  }
  g.sync();
  for (int c = (int)rr - 1; c >= 0; --c) {
    const double t = qtau[c];
    if (t != 0.0) {
      const double* a = R + (size_t)c * ld;
      for (uint32_t j = warp; j < kt; j += NW) {
        double* b = Un + (size_t)j * n1;
        double s = 0.0;
        for (uint32_t i = (uint32_t)c + lane; i < mmin; i += 32) s += (i == (uint32_t)c ? 1.0 : a[i]) * b[i];
        s = Group<32>::sum(s) * t;
        for (uint32_t i = (uint32_t)c + lane; i < mmin; i += 32) b[i] -= s * (i == (uint32_t)c ? 1.0 : a[i]);
      }
    }
    g.sync();
  }
  group_apply_q<G>(g, n1, mmin, U, tau1, kt, Un);
  group_apply_q<G>(g, n2, nmin, V, tau2, kt, Vn);
  return kt;
}

template <int G, class Grp>
__device__ void aca_task(const Grp& g, const AcaParams& p, uint32_t ti, double* smem) {
  const AcaTask t = p.tasks[ti];
  Blk B;
  B.P = p.pts;
  B.diag = p.diag;
  B.b1 = t.b1;
  B.n1 = t.n1;
  B.b2 = t.b2;
  B.n2 = t.n2;
  double* ws = p.ws + t.ws;
  const uint32_t kc = t.kcap;
  B.U = ws;
  B.V = B.U + (size_t)t.n1 * kc;
  double* Un = B.V + (size_t)t.n2 * kc;
  double* Vn = Un + (size_t)t.n1 * kc;
  double* Rg = Vn + (size_t)t.n2 * kc;
  double* Vsg = Rg + (size_t)kc * kc;
  double* sigg = Vsg + (size_t)kc * kc;
  double* taug = sigg + kc;
  B.Z = p.zs + t.zs;
  B.S = B.Z + t.n1;
  uint32_t k = 0;
  const int st = p.variant == kAcaVariantSym ? acar<G>(g, B, t.i0, t.kmax, t.kcap, p.eps, k)
                                             : aca<G>(g, B, t.i0, t.kmax, t.kcap, p.eps, k);
  uint32_t kt = 0;
  if (st == kAcaOk && k > 0) {
    // small ranks: k x k work arrays in shared memory; larger: in the workspace
    const bool sm = k <= (uint32_t)KSM;
    double* R = sm ? smem : Rg;
    double* Vs = sm ? smem + KSM * LDS : Vsg;
    double* sig = sm ? smem + 2 * KSM * LDS : sigg;
    double* tau = sm ? smem + 2 * KSM * LDS + KSM : taug;
    // perm needs nmin+1 ints: shared memory when small, else the dead Z/S counters
    // (n1 + n2 ints >= nmin + 1)
    int* perm = sm ? reinterpret_cast<int*>(smem + 2 * KSM * LDS + 3 * KSM) : B.Z;
    g.sync();
    kt = recompress<G>(g, t.n1, t.n2, k, B.U, B.V, Un, Vn, p.eps, R, Vs, sm ? LDS : kc, sig, tau,
                       perm, !sm);
  }
  if (g.rank == 0) p.res[ti] = AcaResult{st, k, kt, 0u};
}

// Agglomeration (H/agglH.cpp:14-107): the concatenated factors of sibling
// low-rank blocks (gathered into the task's workspace, zero elsewhere)
// recompressed to the parent's rank with the relative threshold of
// mblock::unify_cols / unify_rows (H/mblock_D.cpp:662-862).
template <int G, class Grp>
__device__ void merge_task(const Grp& g, const MergeParams& p, uint32_t ti, double* smem) {
  const MergeTask t = p.tasks[ti];
  const uint32_t m = t.m, n = t.n, kc = t.k;
  double* U = p.ws + t.ws;
  double* V = U + (size_t)m * kc;
  double* Un = V + (size_t)n * kc;
  double* Vn = Un + (size_t)m * kc;
  double* Rg = Vn + (size_t)n * kc;
  double* Vsg = Rg + (size_t)kc * kc;
  double* sigg = Vsg + (size_t)kc * kc;
  double* taug = sigg + kc;
  uint32_t kt = 0;
  if (kc > 0) {
    const bool sm = kc <= (uint32_t)KSM;
    double* R = sm ? smem : Rg;
    double* Vs = sm ? smem + KSM * LDS : Vsg;
    double* sig = sm ? smem + 2 * KSM * LDS : sigg;
    double* tau = sm ? smem + 2 * KSM * LDS + KSM : taug;
    int* perm = sm ? reinterpret_cast<int*>(smem + 2 * KSM * LDS + 3 * KSM) : p.zs + t.zs;
    g.sync();
    if (!sm) {
      // k x k beyond shared memory: pivoted QR first; Z, cn, qtau, cperm follow tau
      double* Z = taug + 2 * (size_t)kc;
      double* cn = Z + (size_t)kc * kc;
      double* qtau = cn + kc;
      int* cperm = reinterpret_cast<int*>(qtau + kc);
      kt = recompress_qrcp<G>(g, m, n, kc, U, V, Un, Vn, p.eps, R, Vs, Z, kc, sig, tau, cn, qtau, cperm, perm);
    } else {
      kt = recompress<G>(g, m, n, kc, U, V, Un, Vn, p.eps, R, Vs, sm ? LDS : kc, sig, tau, perm, !sm);
    }
  }
  if (g.rank == 0) p.res[ti] = AcaResult{kAcaOk, kc, kt, 0u};
}

// one warp per CTA: consecutive (similarly costly) unions go to different SMs
__global__ void __launch_bounds__(32) merge_small_kernel(MergeParams p) {
  extern __shared__ double smem_all[];
  const uint32_t task = blockIdx.x;
  if (task >= p.ntasks) return;
  Group<32> g(threadIdx.x & 31);
  merge_task<32>(g, p, task, smem_all);
}

__global__ void copy2d_kernel(const Seg2D* __restrict__ segs, const double* __restrict__ src,
                              double* __restrict__ dst) {
  const Seg2D s = segs[blockIdx.x];
  if (s.src == kSegIdentity) {
    for (uint32_t c = threadIdx.x; c < s.ncols; c += blockDim.x)
      dst[s.dst + (uint64_t)c * s.ld_dst + (uint64_t)c * (1 + s.cplx)] = 1.0;
    return;
  }
  const uint64_t cnt = (uint64_t)s.nrows * s.ncols;
  for (uint64_t e = threadIdx.x; e < cnt; e += blockDim.x) {
    const uint64_t c = e / s.nrows, r = e - c * s.nrows;
    dst[s.dst + c * s.ld_dst + r] = src[s.src + e];
  }
}

__global__ void __launch_bounds__(32 * kSmallWarps) aca_small_kernel(AcaParams p) {
  extern __shared__ double smem_all[];
  const uint32_t w = threadIdx.x >> 5;
  const uint32_t task = blockIdx.x * kSmallWarps + w;
  if (task >= p.ntasks) return;
  Group<32> g(threadIdx.x & 31);
  aca_task<32>(g, p, task, smem_all + (size_t)w * kSmemPerGroup);
}

constexpr int kLargeThreads = 256;

__global__ void __launch_bounds__(kLargeThreads) aca_large_kernel(AcaParams p) {
  extern __shared__ double smem_all[];
  const uint32_t task = blockIdx.x;
  if (task >= p.ntasks) return;
  Group<kLargeThreads> g(threadIdx.x, smem_all + kSmemPerGroup);
  aca_task<kLargeThreads>(g, p, task, smem_all);
}

__global__ void __launch_bounds__(kLargeThreads) merge_large_kernel(MergeParams p) {
  extern __shared__ double smem_all[];
  const uint32_t task = blockIdx.x;
  if (task >= p.ntasks) return;
  Group<kLargeThreads> g(threadIdx.x, smem_all + kSmemPerGroup);
  merge_task<kLargeThreads>(g, p, task, smem_all);
}

__global__ void dense_fill_kernel(PointsSoA P, double diag, const DenseTask* __restrict__ tasks,
                                  double* __restrict__ arena) {
  const DenseTask t = tasks[blockIdx.x];
  const uint64_t cnt = (uint64_t)t.n1 * t.n2;
  double* out = arena + t.off;
  for (uint64_t e = threadIdx.x; e < cnt; e += blockDim.x) {
    const uint32_t i = (uint32_t)(e % t.n1), j = (uint32_t)(e / t.n1);
    const uint32_t gj = t.b2 + j;
    out[e] = lap_entry(P, gj, t.b1 + i, P.x[gj], P.y[gj], P.z[gj], diag);
  }
}

// Mirror images of upper blocks: V U^T (the factors swapped) or D^T.
__global__ void mirror_kernel(const MirrorTask* __restrict__ tasks, double* __restrict__ arena) {
  const MirrorTask t = tasks[blockIdx.x];
  const double* src = arena + t.src;
  double* dst = arena + t.dst;
  if (t.rank > 0) {
    const uint64_t nu = (uint64_t)t.n1 * t.rank, nv = (uint64_t)t.n2 * t.rank;
    for (uint64_t e = threadIdx.x; e < nv; e += blockDim.x) dst[e] = src[nu + e];
    for (uint64_t e = threadIdx.x; e < nu; e += blockDim.x) dst[nv + e] = src[e];
  } else {
    const uint64_t cnt = (uint64_t)t.n1 * t.n2;
    for (uint64_t e = threadIdx.x; e < cnt; e += blockDim.x) {
      const uint32_t j = (uint32_t)(e % t.n2), i = (uint32_t)(e / t.n2);  // D^T(j, i) = D(i, j)
      dst[e] = src[i + (uint64_t)j * t.n1];
    }
  }
}

__global__ void copy_factors_kernel(const CopyTask* __restrict__ tasks, const double* __restrict__ ws,
                                    double* __restrict__ arena) {
  const CopyTask t = tasks[blockIdx.x];
  const uint64_t nu = (uint64_t)t.n1 * t.kt, nv = (uint64_t)t.n2 * t.kt;
  double* dst = arena + t.dst;
  for (uint64_t e = threadIdx.x; e < nu; e += blockDim.x) dst[e] = ws[t.src_u + e];
  for (uint64_t e = threadIdx.x; e < nv; e += blockDim.x) dst[nu + e] = ws[t.src_v + e];
}

}  // namespace

cudaError_t launch_aca_small(const AcaParams& p, cudaStream_t s) {
  if (p.ntasks == 0) return cudaSuccess;
  const size_t smem = sizeof(double) * kSmemPerGroup * kSmallWarps;
  cudaError_t e = cudaFuncSetAttribute(aca_small_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  const uint32_t grid = (p.ntasks + kSmallWarps - 1) / kSmallWarps;
  aca_small_kernel<<<grid, 32 * kSmallWarps, smem, s>>>(p);
  return cudaGetLastError();
}

cudaError_t launch_aca_large(const AcaParams& p, cudaStream_t s) {
  if (p.ntasks == 0) return cudaSuccess;
  const size_t smem = sizeof(double) * (kSmemPerGroup + 3 * (kLargeThreads / 32) + 8);
  cudaError_t e = cudaFuncSetAttribute(aca_large_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  aca_large_kernel<<<p.ntasks, kLargeThreads, smem, s>>>(p);
  return cudaGetLastError();
}

cudaError_t launch_dense_fill(const PointsSoA& pts, double diag, const DenseTask* tasks,
                              uint32_t ntasks, double* arena, cudaStream_t s) {
  if (ntasks == 0) return cudaSuccess;
  dense_fill_kernel<<<ntasks, 256, 0, s>>>(pts, diag, tasks, arena);
  return cudaGetLastError();
}

cudaError_t launch_merge(const MergeParams& p, bool large, cudaStream_t s) {
  if (p.ntasks == 0) return cudaSuccess;
  if (!large) {
    const size_t smem = sizeof(double) * kSmemPerGroup;
    cudaError_t e = cudaFuncSetAttribute(merge_small_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    merge_small_kernel<<<p.ntasks, 32, smem, s>>>(p);
  } else {
    const size_t smem = sizeof(double) * (kSmemPerGroup + 3 * (kLargeThreads / 32) + 8);
    cudaError_t e = cudaFuncSetAttribute(merge_large_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    merge_large_kernel<<<p.ntasks, kLargeThreads, smem, s>>>(p);
  }
  return cudaGetLastError();
}

cudaError_t launch_copy2d(const Seg2D* segs, uint32_t nsegs, const double* src, double* dst, cudaStream_t s) {
  if (nsegs == 0) return cudaSuccess;
  copy2d_kernel<<<nsegs, 256, 0, s>>>(segs, src, dst);
  return cudaGetLastError();
}

cudaError_t launch_mirror(const MirrorTask* tasks, uint32_t ntasks, double* arena, cudaStream_t s) {
  if (ntasks == 0) return cudaSuccess;
  mirror_kernel<<<ntasks, 256, 0, s>>>(tasks, arena);
  return cudaGetLastError();
}

cudaError_t launch_copy_factors(const CopyTask* tasks, uint32_t ntasks, const double* ws,
                                double* arena, cudaStream_t s) {
  if (ntasks == 0) return cudaSuccess;
  copy_factors_kernel<<<ntasks, 256, 0, s>>>(tasks, ws, arena);
  return cudaGetLastError();
}

}  // namespace ahx

// ---------------------------------------------------------------------------
// ACA of one block with no device allocation.
//
// Some callers cannot call cudaMalloc: code that runs while a framework's
// caching allocator has reserved the device memory, latency-critical paths
// where the implicit device synchronisation of cudaMalloc/cudaFree is not
// acceptable, or hosts that own every device allocation themselves and only
// hand out buffers.  For them, ahx_aca_block_noalloc approximates one
// admissible block with the same kernel code as ahx_assemble, taking its
// scratch (the ACA columns, the row/column counters and the recompression
// work arrays) from the file-scope array below instead of an allocation.
//
// The array is 8 MiB and lives on every GPU that loads the library until the
// process exits.  Every call shares it and it keeps the last call's contents;
// the kernel rewrites every word it reads (the counters are set to zero by the
// ACA itself), so nothing carries over between calls.  Calls whose kernels
// overlap on the GPU (on different streams) race on the array: serialise them.

namespace ahx {
namespace {

constexpr size_t kNoAllocScratchBytes = (size_t)8 << 20;
constexpr size_t kNoAllocHeader = 256;  // task slot + result slot

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Blocks beyond this many rows or columns, or rank bounds beyond kNoAllocMaxK,
// are refused before any size arithmetic (they could never fit the array).
constexpr uint32_t kNoAllocMaxDim = 1u << 20;
constexpr uint32_t kNoAllocMaxK = 1u << 16;

// bytes of scratch for a block; the ACA columns have the reference's kmax + 1
// capacity (Include/ACA.h:231-232).  64-bit arithmetic throughout.
uint64_t noalloc_bytes(uint32_t n1, uint32_t n2, uint32_t kmax) {
  const uint64_t ws = aca_ws_doubles(n1, n2, kcap_limit(kmax)) * sizeof(double);
  return kNoAllocHeader + ws + ((uint64_t)n1 + n2) * sizeof(int);
}

template <int G>
__global__ void __launch_bounds__(G < 64 ? 32 : G)
    aca_noalloc_kernel(AcaTask t, uint64_t ws_doubles, PointsSoA P, double diag, double eps,
                       unsigned char* scratch, double* __restrict__ Uout,
                       double* __restrict__ Vout, int32_t* info) {
  extern __shared__ double smem_na[];
  AcaTask* slot = reinterpret_cast<AcaTask*>(scratch);
  AcaResult* res = reinterpret_cast<AcaResult*>(scratch + 128);
  double* ws = reinterpret_cast<double*>(scratch + kNoAllocHeader);
  int* zs = reinterpret_cast<int*>(ws + ws_doubles);
  if (threadIdx.x == 0) {
    t.ws = 0;
    t.zs = 0;
    *slot = t;
    *res = AcaResult{kAcaFail, 0u, 0u, 0u};
  }
  __syncthreads();
  AcaParams p;
  p.pts = P;
  p.diag = diag;
  p.eps = eps;
  p.tasks = slot;
  p.ntasks = 1;
  p.ws = ws;
  p.zs = zs;
  p.res = res;
  if constexpr (G == 32) {
    Group<32> g(threadIdx.x);
    aca_task<32>(g, p, 0, smem_na);
  } else {
    Group<G> g(threadIdx.x, smem_na + kSmemPerGroup);
    aca_task<G>(g, p, 0, smem_na);
  }
  __syncthreads();
  const AcaResult r = *res;
  const uint64_t kc = t.kcap;
  const double* Un = ws + (uint64_t)(t.n1 + t.n2) * kc;
  const double* Vn = Un + (uint64_t)t.n1 * kc;
  if (r.status == kAcaOk) {
    for (uint64_t e = threadIdx.x; e < (uint64_t)t.n1 * r.kt; e += blockDim.x) Uout[e] = Un[e];
    for (uint64_t e = threadIdx.x; e < (uint64_t)t.n2 * r.kt; e += blockDim.x) Vout[e] = Vn[e];
  }
  if (threadIdx.x == 0) {
    info[0] = r.status;
    info[1] = (int32_t)r.k_aca;
    info[2] = (int32_t)r.kt;
  }
}

// Device address of the scratch array, looked up once per device and context:
// a context torn down and created again (cudaDeviceReset) loads the module
// again, so an address resolved in the old context is not reused.
std::mutex g_noalloc_mu;
void* g_noalloc_ptr[256] = {};
void* g_noalloc_ctx[256] = {};

// the calling thread's current driver context (cuCtxGetCurrent through the
// runtime's entry-point query, so that the library needs no -lcuda)
void* current_context() {
  using Fn = int (*)(void**);
  static Fn fn = [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPoint("cuCtxGetCurrent", &f, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      f = nullptr;
    return reinterpret_cast<Fn>(f);
  }();
  void* ctx = nullptr;
  if (fn && fn(&ctx) != 0) ctx = nullptr;
  return ctx;
}

}  // namespace
}  // namespace ahx

extern "C" int ahx_aca_block_noalloc(const double* px, const double* py, const double* pz,
                                     uint32_t b1, uint32_t n1, uint32_t b2, uint32_t n2,
                                     uint32_t i0, double h, double eps, uint32_t kmax, double* U,
                                     double* V, int32_t* info, void* stream) {
  using namespace ahx;
  if (!px || !py || !pz || !U || !V || !info || n1 == 0 || n2 == 0 || i0 >= n1 || kmax == 0 ||
      !(h > 0.0) || !(eps > 0.0)) {
    set_error("ahx_aca_block_noalloc: invalid argument");
    return AHX_ERR_ARG;
  }
  if (n1 > kNoAllocMaxDim || n2 > kNoAllocMaxDim || kmax > kNoAllocMaxK) {
    set_error("ahx_aca_block_noalloc: block " + std::to_string(n1) + " x " + std::to_string(n2) +
              " with kmax " + std::to_string(kmax) + " exceeds the fixed scratch array (" +
              std::to_string(kNoAllocScratchBytes) + " bytes)");
    return AHX_ERR_ARG;
  }
  const uint64_t need = noalloc_bytes(n1, n2, kmax);
  if (need > kNoAllocScratchBytes) {
    set_error("ahx_aca_block_noalloc: block " + std::to_string(n1) + " x " + std::to_string(n2) +
              " with kmax " + std::to_string(kmax) + " needs " + std::to_string(need) +
              " bytes of scratch; the fixed scratch array holds " +
              std::to_string(kNoAllocScratchBytes) + " bytes");
    return AHX_ERR_ARG;
  }
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (dev < 0 || dev >= 256) {
    set_error("ahx_aca_block_noalloc: device ordinal out of range");
    return AHX_ERR_ARG;
  }
  void* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    void* ctx = current_context();
    if (!g_noalloc_ptr[dev] || ctx != g_noalloc_ctx[dev]) {
      // first call on this device (or in a new context): resolve the array's
      // device address; the current device is the one the kernel will run on
      void* ptr = nullptr;
      e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
      if (e != cudaSuccess) {
        g_noalloc_ptr[dev] = nullptr;
        return cuda_fail(e, "cudaGetSymbolAddress(scratch)");
      }
      g_noalloc_ptr[dev] = ptr;
      g_noalloc_ctx[dev] = current_context();
    }
    scratch = g_noalloc_ptr[dev];
  }
  AcaTask t{};
  t.b1 = b1;
  t.n1 = n1;
  t.b2 = b2;
  t.n2 = n2;
  t.i0 = i0;
  t.kmax = kmax;
  t.kcap = kcap_limit(kmax);  // never overflows: status is 1 or 0
  t.leaf = 0;
  const PointsSoA P{px, py, pz};
  const double diag = 1.0 / (kFourPi * h);
  const uint64_t wsd = aca_ws_doubles(n1, n2, t.kcap);
  cudaStream_t s = (cudaStream_t)stream;
  if (std::max(n1, n2) > 256) {
    const size_t smem = sizeof(double) * (kSmemPerGroup + 3 * (kLargeThreads / 32) + 8);
    aca_noalloc_kernel<kLargeThreads><<<1, kLargeThreads, smem, s>>>(t, wsd, P, diag, eps,
                                                                     (unsigned char*)scratch, U, V, info);
  } else {
    const size_t smem = sizeof(double) * kSmemPerGroup;
    aca_noalloc_kernel<32><<<1, 32, smem, s>>>(t, wsd, P, diag, eps, (unsigned char*)scratch, U, V,
                                               info);
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "aca_noalloc_kernel launch");
  return AHX_OK;
}
