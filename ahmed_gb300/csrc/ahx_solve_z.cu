// Products and GMRES of the Helmholtz (complex) leaves.
//
// ahx_helm_matvec: Y += d op(A) X, op = A / A^H / A^T (mltaGeHVec, mltaGeHhVec,
// mltaGeHtVec and their GeM forms with T = dcomp, H/mltaGeHVec.cpp:770-805).
// ahx_helm_gmres: restarted GMRES(m) with T = dcomp (solvers/GMRES.cpp:246-366):
// the same Arnoldi steps, Givens rotations with a real cosine and a complex sine
// that annihilate the subdiagonal, the same convergence tests and step counts.
// Orthogonalisation is classical Gram-Schmidt applied twice (one reduction
// kernel per pass instead of one per basis vector); each step ends in one host
// round trip for the Hessenberg column.  After a full cycle the residual is
// recomputed from x: r = b - A x (the reference's complex GMRes forms it from its
// last Krylov work vector instead, solvers/GMRES.cpp:357, which only matters
// when a solve restarts).  With complex64 leaves (AHX_FP32) the solve runs FP64
// iterative refinement: residuals with the complex128 leaves, inner GMRES on the
// complex64 product.
#include <algorithm>
#include <cmath>
#include <complex>
#include <vector>

#include "ahx_hmat.hpp"

namespace ahx {
namespace {

using zc = std::complex<double>;

constexpr int kZRed = 256;
constexpr uint64_t kZChunk = 4096;  // elements per reduction block (at least)

uint32_t zblocks(uint64_t n) { return (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>((n + kZChunk - 1) / kZChunk, 1024)); }

unsigned zgrid(uint64_t n) { return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((n + 255) / 256, 152ull * 16)); }

// partial[b * nk + k] = sum over block b's elements e of conj(V_k[e]) W[e]
__global__ void __launch_bounds__(kZRed) zdots_kernel(const double2* __restrict__ V, uint64_t vstride, uint32_t nk,
                                                      const double2* __restrict__ W, uint64_t n, uint64_t per,
                                                      double2* __restrict__ partial) {
  __shared__ double red[2][kZRed / 32];
  const uint64_t e0 = blockIdx.x * per, e1 = min(n, e0 + per);
  for (uint32_t k = 0; k < nk; ++k) {
    const double2* v = V + k * vstride;
    double sr = 0.0, si = 0.0;
    for (uint64_t e = e0 + threadIdx.x; e < e1; e += kZRed) {
      const double2 a = v[e], w = W[e];
      sr = fma(a.x, w.x, fma(a.y, w.y, sr));
      si = fma(a.x, w.y, fma(-a.y, w.x, si));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      sr += __shfl_xor_sync(0xffffffffu, sr, o);
      si += __shfl_xor_sync(0xffffffffu, si, o);
    }
    if ((threadIdx.x & 31) == 0) {
      red[0][threadIdx.x >> 5] = sr;
      red[1][threadIdx.x >> 5] = si;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double tr = red[0][0], ti = red[1][0];
      for (int q = 1; q < kZRed / 32; ++q) {
        tr += red[0][q];
        ti += red[1][q];
      }
      partial[(uint64_t)blockIdx.x * nk + k] = make_double2(tr, ti);
    }
    __syncthreads();
  }
}

// out[k] = sum over the blocks (in order) of partial[b * nk + k]
__global__ void zreduce_kernel(const double2* __restrict__ partial, uint32_t nblk, uint32_t nk,
                               double2* __restrict__ out) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nk) return;
  double sr = 0.0, si = 0.0;
  for (uint32_t b = 0; b < nblk; ++b) {
    const double2 v = partial[(uint64_t)b * nk + k];
    sr += v.x;
    si += v.y;
  }
  out[k] = make_double2(sr, si);
}

// W += sign * sum_{k < nk} c[k] V_k
__global__ void zcomb_kernel(double2* __restrict__ W, const double2* __restrict__ V, uint64_t vstride, uint32_t nk,
                             const double2* __restrict__ c, double sign, uint64_t n) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    double2 w = W[i];
    for (uint32_t k = 0; k < nk; ++k) {
      const double2 a = c[k], v = V[k * vstride + i];
      w.x = fma(sign * a.x, v.x, fma(-sign * a.y, v.y, w.x));
      w.y = fma(sign * a.x, v.y, fma(sign * a.y, v.x, w.y));
    }
    W[i] = w;
  }
}

// Y = s X (real s)
__global__ void zscale_kernel(double2* Y, const double2* X, double s, uint64_t n) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const double2 v = X[i];
    Y[i] = make_double2(s * v.x, s * v.y);
  }
}

// Y += X
__global__ void zadd_kernel(double2* Y, const double2* X, uint64_t n) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const double2 v = X[i];
    Y[i].x += v.x;
    Y[i].y += v.y;
  }
}

// Y[:, c] = conj(X[:, c]) (in place when X == Y)
__global__ void zconj_kernel(const double2* X, uint64_t ldX, double2* Y, uint64_t ldY, uint64_t n, uint32_t p) {
  const uint64_t total = n * p;
  for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < total; e += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t c = e / n, i = e - c * n;
    const double2 v = X[c * ldX + i];
    Y[c * ldY + i] = make_double2(v.x, -v.y);
  }
}

// Leaf tables of the complex products; a symmetric tree (complex symmetric
// matrix, mltaSyHVec_ H/mltaGeHVec.cpp:490-515) adds its off-diagonal leaves a
// second time, applied transposed.
int build_ztable(ahx_hmat* H) {
  ZState& Z = H->z;
  if (Z.table) return AHX_OK;
  const auto& Ls = H->tree.leaves;
  std::vector<PlanLeaf> pls, tls;
  for (uint32_t l = 0; l < (uint32_t)Ls.size(); ++l) {
    if (Z.rank[l] == 0) continue;
    const PlanLeaf q{Ls[l].b1, Ls[l].n1, Ls[l].b2, Ls[l].n2, Z.rank[l], Z.off[l]};
    pls.push_back(q);
    if (H->tree.sym && Ls[l].b1 != Ls[l].b2) tls.push_back(q);
  }
  int rc = upload_leaf_table(H, pls, Z.leaves, Z.order, Z.nleaves);
  if (rc) return rc;
  Z.ntleaves = 0;
  if (!tls.empty() && (rc = upload_leaf_table(H, tls, Z.tleaves, Z.torder, Z.ntleaves))) return rc;
  Z.table = true;
  return AHX_OK;
}

int prepare_z(ahx_hmat* H, int prec) {
  ZState& Z = H->z;
  int rc = build_ztable(H);
  if (rc) return rc;
  if (prec == kFP32 && !Z.valid32) {
    if ((rc = Z.arena32.reserve(std::max<uint64_t>(Z.elems, 1) * sizeof(float2)))) return rc;
    AHX_CUDA(launch_z_to_c64(Z.arena.as<double2>(), Z.elems, Z.arena32.as<float2>(), H->stream));
    Z.valid32 = true;
  }
  return AHX_OK;
}

int check_z(const ahx_hmat* H, int prec, const char* who) {
  if (!H->z.assembled) {
    set_error(std::string(who) + ": Helmholtz leaves not assembled");
    return AHX_ERR_STATE;
  }
  if (prec != kFP64 && prec != kFP32) {
    set_error(std::string(who) + ": complex leaves are stored as complex128 (AHX_FP64) or complex64 (AHX_FP32)");
    return AHX_ERR_ARG;
  }
  return AHX_OK;
}

// Device scratch of the complex GMRES: basis V ((m + 1) n), r, b, x, and the
// refinement's residual e and correction d (n each), reduction partials and the
// small vectors (two Gram-Schmidt passes and |w|: 3 (m + 1); y: m).
struct ZGm {
  double2 *V, *r, *b, *x, *e, *d, *partial, *small;
  uint32_t nblk;
};

constexpr int kMaxRefine = 30;
constexpr double kInnerTolFloor = 1e-5;

// <V_k, W> for k < nk into small[off + k] (device) and host out[k]
struct ZDots {
  ahx_hmat* H;
  const ZGm& g;
  uint64_t n;
  int run(const double2* V, uint64_t vstride, uint32_t nk, const double2* W, uint32_t off) {
    const uint64_t per = (n + g.nblk - 1) / g.nblk;
    zdots_kernel<<<g.nblk, kZRed, 0, H->stream>>>(V, vstride, nk, W, n, per, g.partial);
    zreduce_kernel<<<(nk + 127) / 128, 128, 0, H->stream>>>(g.partial, g.nblk, nk, g.small + off);
    AHX_CUDA(cudaGetLastError());
    return AHX_OK;
  }
};

// Givens rotation (cs real, sn complex) with [cs sn; -conj(sn) cs] [a; b] = [*; 0]
// (solvers/GMRES.cpp:187-221)
void gen_rot(zc a, zc b, double& cs, zc& sn) {
  if (b == zc(0.0, 0.0)) {
    cs = 1.0;
    sn = zc(0.0, 0.0);
  } else if (a == zc(0.0, 0.0)) {
    cs = 0.0;
    sn = zc(1.0, 0.0);
  } else {
    const zc q = std::conj(b / a);  // sn / cs
    cs = 1.0 / std::sqrt(1.0 + std::norm(q));
    sn = cs * q;
  }
}

void appl_rot(zc& a, zc& b, double cs, zc sn) {
  const zc t = cs * a + sn * b;
  b = cs * b - std::conj(sn) * a;
  a = t;
}

// One right-hand side: GMRES(m) with the product at precision prec from the
// initial guess x (device, length n) for the right-hand side b (device); uses
// g.V, g.r, g.partial and g.small.
int zgmres_one(ahx_hmat* H, int prec, const ZGm& g, const double2* b, double2* x, double tol, uint32_t m,
               uint32_t maxit, uint32_t& iters, double& resid, bool& converged) {
  const uint64_t n = H->tree.n;
  cudaStream_t st = H->stream;
  ZDots dots{H, g, n};
  int rc;
  std::vector<double2> hs(3 * (size_t)(m + 1) + 2);
  auto fetch = [&](uint32_t cnt) -> int {
    AHX_CUDA(cudaMemcpyAsync(hs.data(), g.small, cnt * sizeof(double2), cudaMemcpyDeviceToHost, st));
    AHX_CUDA(cudaStreamSynchronize(st));
    return AHX_OK;
  };
  converged = false;
  iters = 0;
  // normb, |x|
  if ((rc = dots.run(b, 0, 1, b, 0))) return rc;
  if ((rc = dots.run(x, 0, 1, x, 1))) return rc;
  if ((rc = fetch(2))) return rc;
  const double normb = std::sqrt(hs[0].x);
  if (normb == 0.0) {
    AHX_CUDA(cudaMemsetAsync(x, 0, n * sizeof(double2), st));
    AHX_CUDA(cudaStreamSynchronize(st));
    resid = 0.0;
    converged = true;
    return AHX_OK;
  }
  const bool x_zero = hs[1].x == 0.0;
  auto residual = [&](double& beta) -> int {
    AHX_CUDA(cudaMemcpyAsync(g.r, b, n * sizeof(double2), cudaMemcpyDeviceToDevice, st));
    int e = AHX_OK;
    if ((e = zproduct_device(H, prec, kZOpN, -1.0, 0.0, 1, x, n, g.r, n))) return e;
    if ((e = dots.run(g.r, 0, 1, g.r, 0))) return e;
    if ((e = fetch(1))) return e;
    beta = std::sqrt(hs[0].x);
    return AHX_OK;
  };
  double beta = normb;
  if (x_zero) {
    AHX_CUDA(cudaMemcpyAsync(g.r, b, n * sizeof(double2), cudaMemcpyDeviceToDevice, st));
  } else if ((rc = residual(beta))) {
    return rc;
  }
  resid = beta / normb;
  if (resid <= tol) {
    converged = true;
    return AHX_OK;
  }
  const uint32_t K = m + 1;
  std::vector<zc> R((size_t)m * K), s(K), y(m), sn(K);
  std::vector<double> cs(K);
  uint32_t j = 1;
  while (j <= maxit) {
    zscale_kernel<<<zgrid(n), 256, 0, st>>>(g.V, g.r, 1.0 / beta, n);
    std::fill(s.begin(), s.end(), zc(0.0, 0.0));
    s[0] = beta;
    uint32_t i = 0;
    bool done = false;
    for (; i < m && j <= maxit; ++i, ++j) {
      const double2* vi = g.V + (size_t)i * n;
      double2* w = g.V + (size_t)(i + 1) * n;
      AHX_CUDA(cudaMemsetAsync(w, 0, n * sizeof(double2), st));
      if ((rc = zproduct_device(H, prec, kZOpN, 1.0, 0.0, 1, vi, n, w, n))) return rc;
      // two classical Gram-Schmidt passes, then |w|
      if ((rc = dots.run(g.V, n, i + 1, w, 0))) return rc;
      zcomb_kernel<<<zgrid(n), 256, 0, st>>>(w, g.V, n, i + 1, g.small, -1.0, n);
      if ((rc = dots.run(g.V, n, i + 1, w, K))) return rc;
      zcomb_kernel<<<zgrid(n), 256, 0, st>>>(w, g.V, n, i + 1, g.small + K, -1.0, n);
      if ((rc = dots.run(w, 0, 1, w, 2 * K))) return rc;
      if ((rc = fetch(2 * K + 1))) return rc;
      zc* col = R.data() + (size_t)i * K;
      for (uint32_t k = 0; k <= i; ++k) col[k] = zc(hs[k].x + hs[K + k].x, hs[k].y + hs[K + k].y);
      const double hn = std::sqrt(hs[2 * K].x);
      col[i + 1] = hn;
      if (hn > 0.0) zscale_kernel<<<zgrid(n), 256, 0, st>>>(w, w, 1.0 / hn, n);
      for (uint32_t k = 0; k < i; ++k) appl_rot(col[k], col[k + 1], cs[k], sn[k]);
      gen_rot(col[i], col[i + 1], cs[i], sn[i]);
      appl_rot(col[i], col[i + 1], cs[i], sn[i]);
      appl_rot(s[i], s[i + 1], cs[i], sn[i]);
      resid = std::abs(s[i + 1]) / normb;
      if (resid < tol) {
        iters = j;
        ++i;
        done = true;
        break;
      }
    }
    // x += V y, y = R^{-1} s over the i steps of this cycle (ztrtrs)
    if (i > 0) {
      for (uint32_t q = 0; q < i; ++q) y[q] = s[q];
      for (int q = (int)i - 1; q >= 0; --q) {
        y[q] /= R[(size_t)q * K + q];
        for (int t = 0; t < q; ++t) y[t] -= y[q] * R[(size_t)q * K + t];
      }
      std::vector<double2> yd(i);
      for (uint32_t q = 0; q < i; ++q) yd[q] = make_double2(y[q].real(), y[q].imag());
      AHX_CUDA(cudaMemcpyAsync(g.small + 3 * K, yd.data(), i * sizeof(double2), cudaMemcpyHostToDevice, st));
      zcomb_kernel<<<zgrid(n), 256, 0, st>>>(x, g.V, n, i, g.small + 3 * K, 1.0, n);
      AHX_CUDA(cudaGetLastError());
    }
    if (done) {
      AHX_CUDA(cudaStreamSynchronize(st));
      converged = true;
      return AHX_OK;
    }
    iters = j - 1;
    if (j > maxit) break;
    if ((rc = residual(beta))) return rc;
    resid = beta / normb;
    if (resid < tol) {
      iters = j;  // the count the reference reports after a cycle
      converged = true;
      return AHX_OK;
    }
  }
  AHX_CUDA(cudaStreamSynchronize(st));
  return AHX_OK;
}

}  // namespace

int zproduct_device(ahx_hmat* H, int prec, int op, double dre, double dim, uint32_t p, const double2* X,
                    uint64_t ldX, double2* Y, uint64_t ldY) {
  int rc = prepare_z(H, prec);
  if (rc) return rc;
  ZState& Z = H->z;
  if (H->tree.sym && op == kZOpH) {
    // complex symmetric A: A^H X = conj(A conj(X)) (mltaSyHhVec_, H/mltaGeHVec.cpp:546-555)
    const uint64_t n = H->tree.n;
    if ((rc = Z.xc.reserve(std::max<uint64_t>(n * p, 1) * sizeof(double2)))) return rc;
    double2* Xc = Z.xc.as<double2>();
    const unsigned grid = zgrid(n * p);
    zconj_kernel<<<grid, 256, 0, H->stream>>>(X, ldX, Xc, n, n, p);
    zconj_kernel<<<grid, 256, 0, H->stream>>>(Y, ldY, Y, ldY, n, p);
    AHX_CUDA(cudaGetLastError());
    if ((rc = zproduct_device(H, prec, kZOpN, dre, -dim, p, Xc, n, Y, ldY))) return rc;
    zconj_kernel<<<grid, 256, 0, H->stream>>>(Y, ldY, Y, ldY, n, p);
    AHX_CUDA(cudaGetLastError());
    return AHX_OK;
  }
  if (H->tree.sym) op = kZOpN;  // A^T = A
  ZArgs a;
  a.leaves = H->z.leaves.as<MvLeaf>();
  a.order = H->z.order.as<uint32_t>();
  a.nleaves = H->z.nleaves;
  a.single = prec == kFP32 ? 1 : 0;
  a.arena = a.single ? H->z.arena32.p : H->z.arena.p;
  a.dre = dre;
  a.dim = dim;
  a.p = p;
  a.X = X;
  a.ldX = ldX;
  a.Y = Y;
  a.ldY = ldY;
  a.op = op;
  AHX_CUDA(launch_matvec_z(a, H->stream));
  if (Z.ntleaves) {
    // the blocks below the diagonal: the upper ones transposed
    a.leaves = Z.tleaves.as<MvLeaf>();
    a.order = Z.torder.as<uint32_t>();
    a.nleaves = Z.ntleaves;
    a.op = kZOpT;
    AHX_CUDA(launch_matvec_z(a, H->stream));
  }
  return AHX_OK;
}

}  // namespace ahx

using namespace ahx;

extern "C" {

uint64_t ahx_helm_storage_bytes(const ahx_hmat* H, int precision) {
  if (!H || !H->z.assembled) return 0;
  if (precision == AHX_FP64) return H->z.elems * 16;
  if (precision == AHX_FP32) return H->z.elems * 8;
  return 0;
}

int ahx_helm_matvec(ahx_hmat* H, int precision, int op, double d_re, double d_im, uint32_t p, const double* X,
                    uint64_t ldX, double* Y, uint64_t ldY) {
  if (!H || !X || !Y || ldX < H->tree.n || ldY < H->tree.n || op < kZOpN || op > kZOpT) {
    set_error("ahx_helm_matvec: invalid argument");
    return AHX_ERR_ARG;
  }
  int rc = check_z(H, precision, "ahx_helm_matvec");
  if (rc) return rc;
  if (p == 0) return AHX_OK;
  if ((rc = ensure_device(H))) return rc;
  const uint64_t n = H->tree.n;
  const bool xd = is_device_ptr(X), yd = is_device_ptr(Y);
  const double2* Xd = reinterpret_cast<const double2*>(X);
  double2* Yd = reinterpret_cast<double2*>(Y);
  uint64_t lx = ldX, ly = ldY;
  const size_t row = n * sizeof(double2);
  if (!xd) {
    if ((rc = H->stage_x.reserve(row * p))) return rc;
    AHX_CUDA(cudaMemcpy2DAsync(H->stage_x.p, row, X, ldX * sizeof(double2), row, p, cudaMemcpyHostToDevice,
                               H->stream));
    Xd = H->stage_x.as<double2>();
    lx = n;
  }
  if (!yd) {
    if ((rc = H->stage_y.reserve(row * p))) return rc;
    AHX_CUDA(cudaMemcpy2DAsync(H->stage_y.p, row, Y, ldY * sizeof(double2), row, p, cudaMemcpyHostToDevice,
                               H->stream));
    Yd = H->stage_y.as<double2>();
    ly = n;
  }
  if ((rc = zproduct_device(H, precision, op, d_re, d_im, p, Xd, lx, Yd, ly))) return rc;
  if (!yd)
    AHX_CUDA(cudaMemcpy2DAsync(Y, ldY * sizeof(double2), Yd, row, row, p, cudaMemcpyDeviceToHost, H->stream));
  if (!xd || !yd) AHX_CUDA(cudaStreamSynchronize(H->stream));
  return AHX_OK;
}

int ahx_helm_gmres(ahx_hmat* H, int precision, uint32_t p, const double* B, uint64_t ldB, double* X, uint64_t ldX,
                   double tol, uint32_t m, uint32_t maxit, uint32_t* iters, double* resid) {
  if (!H || !B || !X || p == 0 || m == 0 || ldB < H->tree.n || ldX < H->tree.n || !(tol >= 0.0)) {
    set_error("ahx_helm_gmres: invalid argument");
    return AHX_ERR_ARG;
  }
  int rc = check_z(H, precision, "ahx_helm_gmres");
  if (rc) return rc;
  if ((rc = ensure_device(H))) return rc;
  if ((rc = prepare_z(H, precision))) return rc;
  const uint64_t n = H->tree.n;
  const uint32_t K = m + 1;
  ZGm g;
  g.nblk = zblocks(n);
  const uint64_t elems = (uint64_t)K * n + 5 * n + (uint64_t)g.nblk * K + 4 * (uint64_t)K + 2;
  if ((rc = H->z.gm.reserve(elems * sizeof(double2)))) return rc;
  double2* q = H->z.gm.as<double2>();
  g.V = q;
  q += (uint64_t)K * n;
  g.r = q;
  q += n;
  g.b = q;
  q += n;
  g.x = q;
  q += n;
  g.e = q;
  q += n;
  g.d = q;
  q += n;
  g.partial = q;
  q += (uint64_t)g.nblk * K;
  g.small = q;
  cudaStream_t st = H->stream;
  const size_t row = n * sizeof(double2);
  bool all = true;
  for (uint32_t c = 0; c < p; ++c) {
    AHX_CUDA(cudaMemcpyAsync(g.b, B + 2 * (uint64_t)c * ldB, row, cudaMemcpyDefault, st));
    AHX_CUDA(cudaMemcpyAsync(g.x, X + 2 * (uint64_t)c * ldX, row, cudaMemcpyDefault, st));
    uint32_t it = 0;
    double res = 0.0;
    bool conv = false;
    if (precision == kFP64) {
      if ((rc = zgmres_one(H, kFP64, g, g.b, g.x, tol, m, maxit, it, res, conv))) return rc;
    } else {
      // FP64 refinement: r = b - A x with the complex128 leaves, A e = r with the
      // complex64 ones (GMRES from e = 0), x += e
      ZDots dots{H, g, n};
      double2 hb;
      if ((rc = dots.run(g.b, 0, 1, g.b, 0))) return rc;
      AHX_CUDA(cudaMemcpyAsync(&hb, g.small, sizeof(double2), cudaMemcpyDeviceToHost, st));
      AHX_CUDA(cudaStreamSynchronize(st));
      const double normb = std::sqrt(hb.x);
      for (int outer = 0; outer < kMaxRefine; ++outer) {
        AHX_CUDA(cudaMemcpyAsync(g.e, g.b, row, cudaMemcpyDeviceToDevice, st));
        if ((rc = zproduct_device(H, kFP64, kZOpN, -1.0, 0.0, 1, g.x, n, g.e, n))) return rc;
        if ((rc = dots.run(g.e, 0, 1, g.e, 0))) return rc;
        AHX_CUDA(cudaMemcpyAsync(&hb, g.small, sizeof(double2), cudaMemcpyDeviceToHost, st));
        AHX_CUDA(cudaStreamSynchronize(st));
        const double rn = std::sqrt(hb.x);
        res = normb > 0.0 ? rn / normb : 0.0;
        if (res < tol || normb == 0.0) {
          conv = true;
          break;
        }
        if (it >= maxit) break;
        // the inner tolerance relative to |r|: what is left of tol, at most the
        // complex64 leaves' resolution
        const double inner = std::max(kInnerTolFloor, tol * normb / rn);
        AHX_CUDA(cudaMemsetAsync(g.d, 0, row, st));
        uint32_t iti = 0;
        double ri = 0.0;
        bool ci = false;
        if ((rc = zgmres_one(H, kFP32, g, g.e, g.d, inner, m, maxit - it, iti, ri, ci))) return rc;
        it += iti;
        zadd_kernel<<<zgrid(n), 256, 0, st>>>(g.x, g.d, n);
        AHX_CUDA(cudaGetLastError());
      }
    }
    if (iters) iters[c] = it;
    if (resid) resid[c] = res;
    all = all && conv;
    AHX_CUDA(cudaMemcpyAsync(X + 2 * (uint64_t)c * ldX, g.x, row, cudaMemcpyDefault, st));
  }
  AHX_CUDA(cudaStreamSynchronize(st));
  return all ? AHX_OK : AHX_NOT_CONVERGED;
}

}  // extern "C"
