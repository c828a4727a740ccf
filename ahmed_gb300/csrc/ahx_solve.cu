// Iterative solvers on the device product: restarted GMRES(m) and CG for many
// independent systems at once, and the multi-instance batch.
//
// A "system" is one right-hand side of one H-matrix instance.  Vectors hold
// p columns of length ntot (the concatenation of all instances); system
// q = c * nseg + s is the segment s of column c.  Every reduction is split
// into fixed chunks whose partial sums are combined in a fixed order, so the
// solvers are run-to-run deterministic.
//
// Reference algorithms:
//   GMRes   solvers/GMRES.cpp:32-181 (Givens rotations genPlRot/applPlRot,
//           restart residual r = b - A x, convergence |s[i+1]|/|b| < eps)
//   CG      solvers/CG.cpp:31-113
// Orthogonalisation is classical Gram-Schmidt applied twice (CGS2), which is
// as stable as the reference's modified Gram-Schmidt and maps to two blocked
// kernels per pass.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "ahx_hmat.hpp"

namespace ahx {
namespace {

constexpr uint32_t kChunk = 4096;  // elements per reduction item
constexpr int kRedThreads = 256;
constexpr int kPerThread = kChunk / kRedThreads;

struct Item {
  uint64_t base;  // element index in the (ntot x p) array
  uint32_t len;
  uint32_t q;     // system
};

// partial[it * ldp + k] = sum_e V_k[base+e] * W[base+e],  V_k = V + k * vstride
__global__ void __launch_bounds__(kRedThreads) dots_kernel(const Item* __restrict__ items,
                                                           const double* __restrict__ V,
                                                           uint64_t vstride, uint32_t nk,
                                                           const double* __restrict__ W,
                                                           double* __restrict__ partial,
                                                           uint32_t ldp) {
  __shared__ double red[kRedThreads / 32];
  const Item it = items[blockIdx.x];
  double w[kPerThread];
#pragma unroll
  for (int e = 0; e < kPerThread; ++e) {
    const uint32_t o = threadIdx.x + e * kRedThreads;
    w[e] = o < it.len ? W[it.base + o] : 0.0;
  }
  for (uint32_t k = 0; k < nk; ++k) {
    const double* v = V + k * vstride + it.base;
    double s = 0.0;
#pragma unroll
    for (int e = 0; e < kPerThread; ++e) {
      const uint32_t o = threadIdx.x + e * kRedThreads;
      if (o < it.len) s = fma(v[o], w[e], s);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = red[0];
      for (int q = 1; q < kRedThreads / 32; ++q) t += red[q];
      partial[(uint64_t)blockIdx.x * ldp + k] = t;
    }
    __syncthreads();
  }
}

// out[q * ldo + k] = sum over the items of q (in order) of partial[it * ldp + k]
__global__ void reduce_items_kernel(const double* __restrict__ partial, uint32_t ldp,
                                    const uint32_t* __restrict__ first, uint32_t nsys, uint32_t nk,
                                    double* __restrict__ out, uint32_t ldo) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nsys * nk) return;
  const uint32_t q = t / nk, k = t % nk;
  double s = 0.0;
  for (uint32_t it = first[q]; it < first[q + 1]; ++it) s += partial[(uint64_t)it * ldp + k];
  out[(uint64_t)q * ldo + k] = s;
}

__device__ __forceinline__ uint32_t sys_of(uint64_t idx, uint64_t ntot, const uint32_t* seg_id,
                                           uint32_t nseg) {
  const uint64_t c = idx / ntot;
  const uint32_t s = seg_id ? seg_id[idx - c * ntot] : 0u;
  return (uint32_t)c * nseg + s;
}

// W -= sum_{k < nk} coef[q * ldc + k] V_k   (per element's system q)
__global__ void sub_combination_kernel(double* __restrict__ W, const double* __restrict__ V,
                                       uint64_t vstride, uint32_t nk,
                                       const double* __restrict__ coef, uint32_t ldc,
                                       uint64_t total, uint64_t ntot,
                                       const uint32_t* __restrict__ seg_id, uint32_t nseg) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t q = sys_of(i, ntot, seg_id, nseg);
    const double* c = coef + (uint64_t)q * ldc;
    double w = W[i];
    for (uint32_t k = 0; k < nk; ++k) w = fma(-c[k], V[k * vstride + i], w);
    W[i] = w;
  }
}

// X += sum_{k < len[q]} y[q * ldy + k] V_k
__global__ void add_combination_kernel(double* __restrict__ X, const double* __restrict__ V,
                                       uint64_t vstride, const uint32_t* __restrict__ len,
                                       const double* __restrict__ y, uint32_t ldy, uint64_t total,
                                       uint64_t ntot, const uint32_t* __restrict__ seg_id,
                                       uint32_t nseg) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t q = sys_of(i, ntot, seg_id, nseg);
    const double* c = y + (uint64_t)q * ldy;
    double x = X[i];
    for (uint32_t k = 0; k < len[q]; ++k) x = fma(c[k], V[k * vstride + i], x);
    X[i] = x;
  }
}

// Y = a[q * lda] * X (per-system factor; mode 1: the factor is 1/sqrt(a) unless a == 0)
__global__ void scale_kernel(double* Y, const double* X, const double* __restrict__ a,
                             uint32_t lda, int mode, uint64_t total, uint64_t ntot,
                             const uint32_t* __restrict__ seg_id, uint32_t nseg) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t q = sys_of(i, ntot, seg_id, nseg);
    double f = a[(uint64_t)q * lda];
    if (mode == 1) f = f > 0.0 ? 1.0 / sqrt(f) : 0.0;
    Y[i] = f * X[i];
  }
}

// Y = X + a[q] * Z   (Y may alias X or Z)
__global__ void axpy_sys_kernel(double* Y, const double* X, const double* Z,
                                const double* __restrict__ a, uint64_t total, uint64_t ntot,
                                const uint32_t* __restrict__ seg_id, uint32_t nseg) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t q = sys_of(i, ntot, seg_id, nseg);
    Y[i] = fma(a[q], Z[i], X[i]);
  }
}

unsigned grid_for(uint64_t total) {
  return (unsigned)std::min<uint64_t>((total + 255) / 256, 152ull * 16);
}

// Givens rotations of solvers/GMRES.cpp:32-56, with explicitly rounded
// operations (no contraction into FMA).
__device__ __forceinline__ void gen_rot_d(double dx, double dy, double& cs, double& sn) {
  if (dy == 0.0) {
    cs = 1.0;
    sn = 0.0;
  } else if (fabs(dy) > fabs(dx)) {
    const double t = __ddiv_rn(dx, dy);
    sn = __ddiv_rn(1.0, __dsqrt_rn(__dadd_rn(1.0, __dmul_rn(t, t))));
    cs = __dmul_rn(t, sn);
  } else {
    const double t = __ddiv_rn(dy, dx);
    cs = __ddiv_rn(1.0, __dsqrt_rn(__dadd_rn(1.0, __dmul_rn(t, t))));
    sn = __dmul_rn(t, cs);
  }
}

__device__ __forceinline__ void appl_rot_d(double& dx, double& dy, double cs, double sn) {
  const double t = __dadd_rn(__dmul_rn(cs, dx), __dmul_rn(sn, dy));
  dy = __dsub_rn(__dmul_rn(cs, dy), __dmul_rn(sn, dx));
  dx = t;
}

// Device state of restarted GMRES(m) for nsys systems; K >= m + 1 entries per
// system; R holds the rotated Hessenberg columns, system q column i at
// R[(q * m + i) * K].
struct GmDev {
  double *R, *cs, *sn, *s, *y, *normb, *resid;
  uint32_t *flags;  // bit 0: running in this cycle, bit 1: converged
  uint32_t *ylen, *iters, *jbase, *nactive;
  const double* tol;      // in device memory so that captured graphs stay valid
  const uint32_t* maxit;  // across calls with other tolerances and step limits
};

// y = R^{-1} s over the first k columns (solvers/GMRES.cpp:62-78, dtrsv)
__device__ void tri_solve_d(const GmDev& g, uint32_t q, uint32_t k, uint32_t m, uint32_t K) {
  const double* Rq = g.R + (size_t)q * m * K;
  double* y = g.y + (size_t)q * K;
  for (uint32_t i = 0; i < k; ++i) y[i] = g.s[(size_t)q * K + i];
  for (int jj = (int)k - 1; jj >= 0; --jj) {
    y[jj] = __ddiv_rn(y[jj], Rq[(size_t)jj * K + jj]);
    for (int i = 0; i < jj; ++i) y[i] = __dsub_rn(y[i], __dmul_rn(y[jj], Rq[(size_t)jj * K + i]));
  }
  g.ylen[q] = k;
}

// One Arnoldi step i of every running system: Hessenberg column from the two
// Gram-Schmidt passes (h1 + h2) and |w|, the rotations, the residual estimate.
__global__ void arnoldi_kernel(GmDev g, uint32_t i, uint32_t m, uint32_t K, const double* __restrict__ h1,
                               const double* __restrict__ h2, const double* __restrict__ nrm, uint32_t nsys) {
  const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nsys) return;
  const uint32_t f = g.flags[q];
  if (!(f & 1u) || (f & 2u)) return;
  const uint32_t j = g.jbase[0] + i + 1;
  if (j > g.maxit[0]) return;
  double* col = g.R + ((size_t)q * m + i) * K;
  for (uint32_t k = 0; k <= i; ++k) col[k] = __dadd_rn(h1[(size_t)q * K + k], h2[(size_t)q * K + k]);
  col[i + 1] = __dsqrt_rn(nrm[(size_t)q * K]);
  double* csq = g.cs + (size_t)q * K;
  double* snq = g.sn + (size_t)q * K;
  double* sq = g.s + (size_t)q * K;
  for (uint32_t k = 0; k < i; ++k) appl_rot_d(col[k], col[k + 1], csq[k], snq[k]);
  gen_rot_d(col[i], col[i + 1], csq[i], snq[i]);
  appl_rot_d(col[i], col[i + 1], csq[i], snq[i]);
  appl_rot_d(sq[i], sq[i + 1], csq[i], snq[i]);
  const double r = fabs(__ddiv_rn(sq[i + 1], g.normb[q]));
  g.resid[q] = r;
  g.iters[q] = j;
  if (r < g.tol[0]) {
    tri_solve_d(g, q, i + 1, m, K);
    g.flags[q] = f | 2u;
  }
}

// running systems at the end of a cycle of `icount` steps: y from those steps
__global__ void cycle_end_kernel(GmDev g, uint32_t icount, uint32_t m, uint32_t K, uint32_t nsys) {
  const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nsys) return;
  const uint32_t f = g.flags[q];
  if ((f & 1u) && !(f & 2u) && icount > 0) tri_solve_d(g, q, icount, m, K);
}

__global__ void count_active_kernel(GmDev g, uint32_t nsys) {
  __shared__ uint32_t c;
  if (threadIdx.x == 0) c = 0;
  __syncthreads();
  uint32_t mine = 0;
  for (uint32_t q = threadIdx.x; q < nsys; q += blockDim.x) mine += ((g.flags[q] & 3u) == 1u) ? 1u : 0u;
  atomicAdd(&c, mine);
  __syncthreads();
  if (threadIdx.x == 0) g.nactive[0] = c;
}

}  // namespace

// Linear operator over ntot x p device vectors (ld = ntot).
struct Operator {
  uint64_t ntot = 0;
  uint32_t nseg = 1;
  std::vector<uint64_t> seg_off;  // nseg + 1
  DevBuf seg_id;                  // ntot uint32 (only when nseg > 1)
  cudaStream_t stream = nullptr;
  virtual ~Operator() { seg_id.release(); }
  // Y += d A X in storage precision prec
  virtual int apply(int prec, double d, uint32_t p, const double* X, double* Y) = 0;
  // leaf bytes one product at precision prec reads (0: unknown)
  virtual uint64_t product_bytes(int prec) const {
    (void)prec;
    return 0;
  }
  // everything apply(prec, ...) allocates, done ahead (graph capture allows no allocation)
  virtual int prepare(int prec, uint32_t p) {
    (void)prec;
    (void)p;
    return AHX_OK;
  }
  int init_segments() {
    if (nseg <= 1) return AHX_OK;
    std::vector<uint32_t> id(ntot);
    for (uint32_t s = 0; s < nseg; ++s)
      for (uint64_t i = seg_off[s]; i < seg_off[s + 1]; ++i) id[i] = s;
    int rc = seg_id.reserve(ntot * sizeof(uint32_t));
    if (rc) return rc;
    AHX_CUDA(cudaMemcpyAsync(seg_id.p, id.data(), ntot * 4, cudaMemcpyHostToDevice, stream));
    AHX_CUDA(cudaStreamSynchronize(stream));
    return AHX_OK;
  }
};

struct HmatOp : Operator {
  ahx_hmat* H;
  explicit HmatOp(ahx_hmat* h) : H(h) {
    ntot = h->tree.n;
    seg_off = {0, ntot};
    stream = h->stream;
  }
  int apply(int prec, double d, uint32_t p, const double* X, double* Y) override {
    return product_device(H, prec, d, p, X, ntot, Y, ntot);
  }
  uint64_t product_bytes(int prec) const override { return H->prod[prec].bytes; }
  int prepare(int prec, uint32_t p) override {
    int rc = prepare_product(H, prec);
    if (rc || prec != kDF64) return rc;
    return prepare_df_x(H->prod[kDF64], ntot, p);
  }
};

// Reduction plan + device scratch for a family of systems.
class Solver {
 public:
  Solver(Operator& op, uint32_t p) : op_(op), p_(p) {}
  ~Solver() {
    for (DevBuf* b : {&items_, &first_, &partial_, &small_, &small2_, &small3_, &len_, &gm_}) b->release();
  }

  int init(uint32_t maxk) {
    nsys_ = op_.nseg * p_;
    total_ = op_.ntot * p_;
    std::vector<Item> items;
    std::vector<uint32_t> first(nsys_ + 1, 0);
    for (uint32_t c = 0; c < p_; ++c)
      for (uint32_t s = 0; s < op_.nseg; ++s) {
        const uint32_t q = c * op_.nseg + s;
        first[q] = (uint32_t)items.size();
        const uint64_t b = op_.seg_off[s], e = op_.seg_off[s + 1];
        for (uint64_t o = b; o < e; o += kChunk)
          items.push_back(Item{(uint64_t)c * op_.ntot + o, (uint32_t)std::min<uint64_t>(kChunk, e - o), q});
      }
    // systems are numbered c * nseg + s, which is the order items were produced in
    first[nsys_] = (uint32_t)items.size();
    nitems_ = (uint32_t)items.size();
    maxk_ = maxk;
    int rc;
    if ((rc = items_.reserve(std::max<size_t>(items.size(), 1) * sizeof(Item)))) return rc;
    if ((rc = first_.reserve(first.size() * sizeof(uint32_t)))) return rc;
    if ((rc = partial_.reserve((size_t)std::max(nitems_, 1u) * maxk * sizeof(double)))) return rc;
    if ((rc = small_.reserve((size_t)nsys_ * maxk * sizeof(double)))) return rc;
    if ((rc = small2_.reserve((size_t)nsys_ * maxk * sizeof(double)))) return rc;
    if ((rc = small3_.reserve((size_t)nsys_ * maxk * sizeof(double)))) return rc;
    if ((rc = len_.reserve((size_t)nsys_ * sizeof(uint32_t)))) return rc;
    if (!items.empty())
      AHX_CUDA(cudaMemcpyAsync(items_.p, items.data(), items.size() * sizeof(Item),
                               cudaMemcpyHostToDevice, op_.stream));
    AHX_CUDA(cudaMemcpyAsync(first_.p, first.data(), first.size() * 4, cudaMemcpyHostToDevice,
                             op_.stream));
    return AHX_OK;
  }

  // out[q * maxk + k] = <V_k, W>_q  (device out)
  int dots(const double* V, uint64_t vstride, uint32_t nk, const double* W, double* out) {
    if (nitems_ == 0) return AHX_OK;
    dots_kernel<<<nitems_, kRedThreads, 0, op_.stream>>>(items_.as<Item>(), V, vstride, nk, W,
                                                         partial_.as<double>(), maxk_);
    const uint32_t nt = nsys_ * nk;
    reduce_items_kernel<<<(nt + 255) / 256, 256, 0, op_.stream>>>(
        partial_.as<double>(), maxk_, first_.as<uint32_t>(), nsys_, nk, out, maxk_);
    AHX_CUDA(cudaGetLastError());
    return AHX_OK;
  }

  const uint32_t* segid() const { return op_.nseg > 1 ? op_.seg_id.as<uint32_t>() : nullptr; }

  Operator& op_;
  uint32_t p_, nsys_ = 0, nitems_ = 0, maxk_ = 0;
  uint64_t total_ = 0;
  DevBuf items_, first_, partial_, small_, small2_, small3_, len_;
  DevBuf gm_;  // device GMRES state (GmDev arrays)
};

// CUDA graphs of GMRES steps: one executable graph per chunk of kGraphChunk
// consecutive steps of a cycle, valid while the operator precision, the basis
// buffer and m stay the same (tolerance and step limit are read from device
// memory, so they may change between calls).
// A chunk ends in a host check of the running systems, so a cycle may run up to
// chunk - 1 steps past the last system's convergence: steps whose product reads
// more leaf data than kLongStepBytes (a millisecond or more) run one per chunk.
constexpr uint32_t kGraphChunk = 5;
constexpr uint64_t kLongStepBytes = 256ull << 20;
struct GmresGraphs {
  int prec = -1;
  const void* vptr = nullptr;
  uint32_t m = 0;
  uint32_t chunk = 0;
  bool failed = false;  // capture is not possible on this stream: launch directly
  std::vector<cudaGraphExec_t> exec;
  ~GmresGraphs() { reset(); }
  void reset() {
    for (cudaGraphExec_t e : exec)
      if (e) cudaGraphExecDestroy(e);
    exec.clear();
    prec = -1;
    vptr = nullptr;
    m = 0;
    chunk = 0;
  }
};

namespace {

// Restarted GMRES(m) on `sv`'s systems with the operator at precision prec.
// B, X: device, ntot x p.  done[q] excludes systems.  Mirrors
// solvers/GMRES.cpp:80-181 per system; the Arnoldi steps (product, two
// classical Gram-Schmidt passes, rotations, residual estimate) run without
// host round trips and are replayed as CUDA graphs of kGraphChunk steps; the
// host checks progress once per chunk and restarts once per cycle.
int gmres_core(Solver& sv, int prec, const double* B, double* X, double tol, uint32_t m,
               uint32_t maxit, std::vector<uint32_t>& iters, std::vector<double>& resid,
               std::vector<char>& done, DevBuf& vbuf, DevBuf& rbuf, GmresGraphs* graphs) {
  Operator& op = sv.op_;
  cudaStream_t st = op.stream;
  const uint32_t nsys = sv.nsys_;
  const uint64_t total = sv.total_;
  const uint64_t vstride = total;
  const uint32_t* sid = sv.segid();
  int rc;
  if ((rc = op.prepare(prec, sv.p_))) return rc;
  if ((rc = vbuf.reserve((size_t)(m + 1) * total * sizeof(double)))) return rc;
  if ((rc = rbuf.reserve(total * sizeof(double)))) return rc;
  double* V = vbuf.as<double>();
  double* r = rbuf.as<double>();
  const uint32_t K = sv.maxk_;  // >= m + 1
  double* d1 = sv.small_.as<double>();
  double* d2 = sv.small2_.as<double>();
  double* d3 = sv.small3_.as<double>();
  // device state
  const size_t nd = (size_t)nsys * ((size_t)m * K + 4 * (size_t)K + 2) + 1;  // R, cs, sn, s, y, normb, resid, tol
  const size_t nu = (size_t)nsys * 3 + 3;                                    // flags, ylen, iters, jbase, nactive, maxit
  if ((rc = sv.gm_.reserve(nd * sizeof(double) + nu * sizeof(uint32_t)))) return rc;
  GmDev g;
  {
    double* p = sv.gm_.as<double>();
    g.R = p;
    p += (size_t)nsys * m * K;
    g.cs = p;
    p += (size_t)nsys * K;
    g.sn = p;
    p += (size_t)nsys * K;
    g.s = p;
    p += (size_t)nsys * K;
    g.y = p;
    p += (size_t)nsys * K;
    g.normb = p;
    p += nsys;
    g.resid = p;
    p += nsys;
    double* ptol = p;
    p += 1;
    uint32_t* u = reinterpret_cast<uint32_t*>(p);
    g.flags = u;
    g.ylen = u + nsys;
    g.iters = u + 2 * (size_t)nsys;
    g.jbase = u + 3 * (size_t)nsys;
    g.nactive = g.jbase + 1;
    uint32_t* pmaxit = g.jbase + 2;
    g.tol = ptol;
    g.maxit = pmaxit;
    AHX_CUDA(cudaMemcpyAsync(ptol, &tol, sizeof(double), cudaMemcpyHostToDevice, st));
    AHX_CUDA(cudaMemcpyAsync(pmaxit, &maxit, sizeof(uint32_t), cudaMemcpyHostToDevice, st));
  }
  std::vector<double> hbuf((size_t)nsys * K);
  auto fetch = [&](const double* dev) -> int {
    AHX_CUDA(cudaMemcpyAsync(hbuf.data(), dev, (size_t)nsys * K * sizeof(double), cudaMemcpyDeviceToHost, st));
    AHX_CUDA(cudaStreamSynchronize(st));
    return AHX_OK;
  };
  // normb
  if ((rc = sv.dots(B, 0, 1, B, d1))) return rc;
  if ((rc = fetch(d1))) return rc;
  std::vector<double> normb(nsys);
  for (uint32_t q = 0; q < nsys; ++q) normb[q] = std::sqrt(hbuf[(size_t)q * K]);
  AHX_CUDA(cudaMemcpyAsync(g.normb, normb.data(), nsys * sizeof(double), cudaMemcpyHostToDevice, st));
  // r = b - A x (no product for a zero initial guess: r = b)
  if ((rc = sv.dots(X, 0, 1, X, d1))) return rc;
  if ((rc = fetch(d1))) return rc;
  bool x_zero = true;
  for (uint32_t q = 0; q < nsys; ++q) x_zero = x_zero && hbuf[(size_t)q * K] == 0.0;
  AHX_CUDA(cudaMemcpyAsync(r, B, total * sizeof(double), cudaMemcpyDeviceToDevice, st));
  if (!x_zero && (rc = op.apply(prec, -1.0, sv.p_, X, r))) return rc;
  if ((rc = sv.dots(r, 0, 1, r, d1))) return rc;
  if ((rc = fetch(d1))) return rc;
  std::vector<double> beta(nsys);
  std::vector<double> zero_fix(nsys, 0.0);
  for (uint32_t q = 0; q < nsys; ++q) {
    beta[q] = std::sqrt(hbuf[(size_t)q * K]);
    if (done[q]) continue;
    if (normb[q] == 0.0) {
      // x = 0 (solvers/GMRES.cpp:96-103)
      done[q] = 1;
      resid[q] = 0.0;
      iters[q] = 0;
      zero_fix[q] = 1.0;
      continue;
    }
    resid[q] = beta[q] / normb[q];
    if (resid[q] <= tol) {
      done[q] = 1;
      iters[q] = 0;
    }
  }
  // zero x of systems with b == 0:  X -= 1 * X on those systems
  if (std::any_of(zero_fix.begin(), zero_fix.end(), [](double v) { return v != 0.0; })) {
    std::vector<double> f(nsys);
    for (uint32_t q = 0; q < nsys; ++q) f[q] = zero_fix[q] != 0.0 ? 0.0 : 1.0;
    AHX_CUDA(cudaMemcpyAsync(d2, f.data(), nsys * sizeof(double), cudaMemcpyHostToDevice, st));
    scale_kernel<<<grid_for(total), 256, 0, st>>>(X, X, d2, 1, 0, total, op.ntot, sid, op.nseg);
  }
  auto active_left = [&]() {
    for (uint32_t q = 0; q < nsys; ++q)
      if (!done[q]) return true;
    return false;
  };
  const unsigned sgrid = (nsys + 127) / 128;
  // steps i0 .. i1 - 1 of a cycle, then the count of systems still running
  auto steps = [&](uint32_t i0, uint32_t i1) -> int {
    for (uint32_t i = i0; i < i1; ++i) {
      double* vi = V + (size_t)i * vstride;
      double* w = V + (size_t)(i + 1) * vstride;
      AHX_CUDA(cudaMemsetAsync(w, 0, total * sizeof(double), st));
      int e = op.apply(prec, 1.0, sv.p_, vi, w);
      if (e) return e;
      // CGS2: h = V^T w; w -= V h; h2 = V^T w; w -= V h2
      if ((e = sv.dots(V, vstride, i + 1, w, d1))) return e;
      sub_combination_kernel<<<grid_for(total), 256, 0, st>>>(w, V, vstride, i + 1, d1, K, total, op.ntot, sid,
                                                              op.nseg);
      if ((e = sv.dots(V, vstride, i + 1, w, d2))) return e;
      sub_combination_kernel<<<grid_for(total), 256, 0, st>>>(w, V, vstride, i + 1, d2, K, total, op.ntot, sid,
                                                              op.nseg);
      if ((e = sv.dots(w, 0, 1, w, d3))) return e;
      arnoldi_kernel<<<sgrid, 128, 0, st>>>(g, i, m, K, d1, d2, d3, nsys);
      // w /= |w|
      scale_kernel<<<grid_for(total), 256, 0, st>>>(w, w, d3, K, 1, total, op.ntot, sid, op.nseg);
    }
    count_active_kernel<<<1, 256, 0, st>>>(g, nsys);
    AHX_CUDA(cudaGetLastError());
    return AHX_OK;
  };
  const uint32_t chunk = op.product_bytes(prec) > kLongStepBytes ? 1u : kGraphChunk;
  if (graphs && (graphs->prec != prec || graphs->vptr != V || graphs->m != m || graphs->chunk != chunk)) {
    graphs->reset();
    graphs->prec = prec;
    graphs->vptr = V;
    graphs->m = m;
    graphs->chunk = chunk;
  }
  auto run_chunk = [&](uint32_t c, uint32_t i0, uint32_t i1) -> int {
    if (!graphs || graphs->failed) return steps(i0, i1);
    if (graphs->exec.size() <= c) graphs->exec.resize(c + 1, nullptr);
    if (!graphs->exec[c]) {
      cudaGraph_t graph = nullptr;
      if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        cudaGetLastError();
        graphs->failed = true;
        return steps(i0, i1);
      }
      const int e = steps(i0, i1);
      const cudaError_t ce = cudaStreamEndCapture(st, &graph);
      cudaGraphExec_t ex = nullptr;
      if (e || ce != cudaSuccess || !graph || cudaGraphInstantiate(&ex, graph, 0) != cudaSuccess) {
        // nothing ran while capturing: launch the same steps directly from now on
        if (graph) cudaGraphDestroy(graph);
        cudaGetLastError();
        graphs->failed = true;
        return steps(i0, i1);
      }
      cudaGraphDestroy(graph);
      graphs->exec[c] = ex;
    }
    AHX_CUDA(cudaGraphLaunch(graphs->exec[c], st));
    return AHX_OK;
  };
  uint32_t j = 1;  // global number of the next step
  std::vector<uint32_t> flags(nsys), hiters(nsys);
  std::vector<double> hres(nsys);
  while (active_left() && j <= maxit) {
    // V_0 = r / beta; a cycle of at most m steps for the running systems
    for (uint32_t q = 0; q < nsys; ++q) hbuf[q] = done[q] ? 0.0 : beta[q] * beta[q];
    AHX_CUDA(cudaMemcpyAsync(d2, hbuf.data(), nsys * sizeof(double), cudaMemcpyHostToDevice, st));
    scale_kernel<<<grid_for(total), 256, 0, st>>>(V, r, d2, 1, 1, total, op.ntot, sid, op.nseg);
    std::fill(hbuf.begin(), hbuf.end(), 0.0);
    for (uint32_t q = 0; q < nsys; ++q) {
      hbuf[(size_t)q * K] = beta[q];
      flags[q] = done[q] ? 0u : 1u;
    }
    AHX_CUDA(cudaMemcpyAsync(g.s, hbuf.data(), (size_t)nsys * K * sizeof(double), cudaMemcpyHostToDevice, st));
    AHX_CUDA(cudaMemcpyAsync(g.flags, flags.data(), nsys * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
    AHX_CUDA(cudaMemsetAsync(g.ylen, 0, nsys * sizeof(uint32_t), st));
    const uint32_t jb = j - 1;
    AHX_CUDA(cudaMemcpyAsync(g.jbase, &jb, sizeof(uint32_t), cudaMemcpyHostToDevice, st));
    const uint32_t icap = std::min(m, maxit - jb);  // steps this cycle may count
    uint32_t ran = 0;
    for (uint32_t c = 0; c * chunk < icap; ++c) {
      const uint32_t i0 = c * chunk, i1 = std::min(m, i0 + chunk);
      if ((rc = run_chunk(c, i0, i1))) return rc;
      ran = std::min(i1, icap);
      uint32_t nact = 0;
      AHX_CUDA(cudaMemcpyAsync(&nact, g.nactive, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
      AHX_CUDA(cudaStreamSynchronize(st));
      if (nact == 0) break;
    }
    cycle_end_kernel<<<sgrid, 128, 0, st>>>(g, ran, m, K, nsys);
    add_combination_kernel<<<grid_for(total), 256, 0, st>>>(X, V, vstride, g.ylen, g.y, K, total, op.ntot, sid,
                                                            op.nseg);
    AHX_CUDA(cudaGetLastError());
    j = jb + ran + 1;
    AHX_CUDA(cudaMemcpyAsync(flags.data(), g.flags, nsys * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    AHX_CUDA(cudaMemcpyAsync(hiters.data(), g.iters, nsys * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    AHX_CUDA(cudaMemcpyAsync(hres.data(), g.resid, nsys * sizeof(double), cudaMemcpyDeviceToHost, st));
    AHX_CUDA(cudaStreamSynchronize(st));
    for (uint32_t q = 0; q < nsys; ++q) {
      if (!(flags[q] & 1u)) continue;
      iters[q] = hiters[q];
      resid[q] = hres[q];
      if (flags[q] & 2u) done[q] = 1;
    }
    if (!active_left() || j > maxit) break;
    // r = b - A x for the running systems
    AHX_CUDA(cudaMemcpyAsync(r, B, total * sizeof(double), cudaMemcpyDeviceToDevice, st));
    if ((rc = op.apply(prec, -1.0, sv.p_, X, r))) return rc;
    if ((rc = sv.dots(r, 0, 1, r, d1))) return rc;
    if ((rc = fetch(d1))) return rc;
    for (uint32_t q = 0; q < nsys; ++q) {
      if (done[q]) continue;
      beta[q] = std::sqrt(hbuf[(size_t)q * K]);
      resid[q] = beta[q] / normb[q];
      if (resid[q] < tol) {
        // the step count after the cycle, as solvers/GMRES.cpp:168-172 reports it
        done[q] = 1;
        iters[q] = j;
      }
    }
  }
  AHX_CUDA(cudaStreamSynchronize(st));
  return AHX_OK;
}

// GMRES with the storage precision `prec`: FP64 runs gmres_core directly; the
// mixed forms run FP64 iterative refinement around inner GMRES cycles.
// AHX_TRACE=1: per outer refinement step, the residual product and inner
// solve times (CUDA events on the solver stream) on stderr.
struct StepTrace {
  bool on = false;
  cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
  explicit StepTrace(cudaStream_t s) : st(s) {
    const char* e = std::getenv("AHX_TRACE");
    on = e && *e && *e != '0';
    if (on)
      for (auto& x : ev) on = on && cudaEventCreate(&x) == cudaSuccess;
  }
  ~StepTrace() {
    for (auto& x : ev)
      if (x) cudaEventDestroy(x);
  }
  void mark(int i) {
    if (on) cudaEventRecord(ev[i], st);
  }
  // after mark(2): residual = ev0..ev1, inner solve = ev1..ev2
  void report(int step, int rprec, int iprec, uint32_t its, double res) {
    if (!on) return;
    float a = 0.f, b = 0.f;
    cudaEventSynchronize(ev[2]);
    cudaEventElapsedTime(&a, ev[0], ev[1]);
    cudaEventElapsedTime(&b, ev[1], ev[2]);
    std::fprintf(stderr, "ahx gmres refine step %d: residual[prec %d] %.3f ms (max rel %.3e), inner[prec %d] %u its %.3f ms\n",
                 step, rprec, a, res, iprec, its, b);
  }
  cudaStream_t st;
};

// Precision of the refinement's outer residual: kDF64 (default) or kFP64.
// The outer residual's product: double-float from two right-hand sides per system
// on, FP64 for one (there the FP64 product is the faster one: 0.64 vs 0.71 ms on a
// 65,536-point sphere, while two RHS take 1.12 vs 0.85 ms).  AHX_REFINE_RESIDUAL=fp64
// or df64 forces one of them.
int refine_residual_precision(uint32_t p) {
  const char* e = std::getenv("AHX_REFINE_RESIDUAL");
  if (e && std::string(e) == "fp64") return kFP64;
  if (e && std::string(e) == "df64") return kDF64;
  return p == 1 ? kFP64 : kDF64;
}

int gmres_driver(Operator& op, int prec, uint32_t p, const double* B, double* X, double tol,
                 uint32_t m, uint32_t maxit, uint32_t* iters_out, double* resid_out, int& status) {
  if (m == 0) {
    set_error("gmres: m must be positive");
    return AHX_ERR_ARG;
  }
  Solver sv(op, p);
  int rc = sv.init(m + 2);
  if (rc) return rc;
  const uint32_t nsys = sv.nsys_;
  std::vector<uint32_t> iters(nsys, 0);
  std::vector<double> resid(nsys, 0.0);
  std::vector<char> done(nsys, 0);
  DevBuf vbuf, rbuf, rr, z;
  GmresGraphs graphs[kNumPrecisions];  // per operator precision
  if (prec == kFP64 || prec == kDF64) {
    rc = gmres_core(sv, kFP64, B, X, tol, m, maxit, iters, resid, done, vbuf, rbuf, &graphs[kFP64]);
  } else {
    // FP64 refinement: r = b - A64 x (FP64 leaves), solve A_prec z = r by one
    // GMRES(m) cycle to an inner tolerance, x += z.
    const uint64_t total = sv.total_;
    if ((rc = rr.reserve(total * sizeof(double)))) return rc;
    if ((rc = z.reserve(total * sizeof(double)))) return rc;
    cudaStream_t st = op.stream;
    // the outer residual in FP64-class arithmetic: double-float on the FP32
    // pipes unless AHX_REFINE_RESIDUAL=fp64 asks for the FP64 product
    const int resid_prec = refine_residual_precision(p);
    if ((rc = op.prepare(resid_prec, p))) return rc;
    // inner tolerance near the storage precision's product accuracy (FP32
    // ~3e-7, BF16 factors ~4e-4): fewer outer steps, i.e. fewer FP64 products
    const double inner_tol = prec == kFP32 ? 1e-6 : 1e-3;
    std::vector<double> normb(nsys), nb((size_t)nsys * sv.maxk_);
    if ((rc = sv.dots(B, 0, 1, B, sv.small_.as<double>()))) return rc;
    AHX_CUDA(cudaMemcpyAsync(nb.data(), sv.small_.p, nb.size() * 8, cudaMemcpyDeviceToHost, st));
    AHX_CUDA(cudaStreamSynchronize(st));
    for (uint32_t q = 0; q < nsys; ++q) normb[q] = std::sqrt(nb[(size_t)q * sv.maxk_]);
    uint32_t used = 0;
    // Safeguard: an outer step that raises a system's FP64 residual is undone
    // for that system, and the remaining inner solves run on the FP64 leaves
    // (the storage precision's error can exceed what refinement contracts
    // when the matrix is ill-conditioned).
    int inner_prec = prec;
    bool undone = false;  // the residual just recomputed follows an undo: accept it
    std::vector<double> prev(nsys, INFINITY), undo(nsys, 0.0);
    // a zero initial guess needs no product for the first residual
    if ((rc = sv.dots(X, 0, 1, X, sv.small_.as<double>()))) return rc;
    AHX_CUDA(cudaMemcpyAsync(nb.data(), sv.small_.p, nb.size() * 8, cudaMemcpyDeviceToHost, st));
    AHX_CUDA(cudaStreamSynchronize(st));
    bool x_zero = true;
    for (uint32_t q = 0; q < nsys; ++q) x_zero = x_zero && nb[(size_t)q * sv.maxk_] == 0.0;
    StepTrace trace(st);
    int outer = 0;
    for (;;) {
      trace.mark(0);
      AHX_CUDA(cudaMemcpyAsync(rr.p, B, total * 8, cudaMemcpyDeviceToDevice, st));
      if (!x_zero && (rc = op.apply(resid_prec, -1.0, p, X, rr.as<double>()))) return rc;
      x_zero = false;
      if ((rc = sv.dots(rr.as<double>(), 0, 1, rr.as<double>(), sv.small_.as<double>()))) return rc;
      trace.mark(1);
      AHX_CUDA(cudaMemcpyAsync(nb.data(), sv.small_.p, nb.size() * 8, cudaMemcpyDeviceToHost, st));
      AHX_CUDA(cudaStreamSynchronize(st));
      bool worse = false;
      for (uint32_t q = 0; q < nsys; ++q) {
        const double rq = normb[q] > 0.0 ? std::sqrt(nb[(size_t)q * sv.maxk_]) / normb[q] : 0.0;
        undo[q] = 0.0;
        if (!undone && !done[q] && rq > prev[q]) {
          undo[q] = -1.0;
          worse = true;
        }
      }
      undone = false;
      if (worse) {
        // x -= z on the systems whose residual grew, then recompute r
        AHX_CUDA(cudaMemcpyAsync(sv.small2_.p, undo.data(), nsys * 8, cudaMemcpyHostToDevice, st));
        axpy_sys_kernel<<<grid_for(total), 256, 0, st>>>(X, X, z.as<double>(), sv.small2_.as<double>(), total,
                                                         op.ntot, sv.segid(), op.nseg);
        inner_prec = resid_prec;
        undone = true;
        continue;
      }
      bool any = false;
      std::vector<char> idone(nsys, 0);
      std::vector<double> mask(nsys, 1.0);
      for (uint32_t q = 0; q < nsys; ++q) {
        resid[q] = normb[q] > 0.0 ? std::sqrt(nb[(size_t)q * sv.maxk_]) / normb[q] : 0.0;
        prev[q] = resid[q];
        if (resid[q] < tol || normb[q] == 0.0) {
          done[q] = 1;
          idone[q] = 1;
          mask[q] = 0.0;
        } else {
          any = true;
        }
      }
      if (!any || used >= maxit) break;
      // masked residual (converged systems contribute nothing), z = 0
      AHX_CUDA(cudaMemcpyAsync(sv.small2_.p, mask.data(), nsys * 8, cudaMemcpyHostToDevice, st));
      scale_kernel<<<grid_for(total), 256, 0, st>>>(rr.as<double>(), rr.as<double>(),
                                                    sv.small2_.as<double>(), 1, 0, total, op.ntot,
                                                    sv.segid(), op.nseg);
      AHX_CUDA(cudaMemsetAsync(z.p, 0, total * 8, st));
      std::vector<uint32_t> it2(nsys, 0);
      std::vector<double> res2(nsys, 0.0);
      const uint32_t budget = std::min(m, maxit - used);
      // the inner solve reduces r (relative to itself) only as far as the outer
      // tolerance still needs, with a margin (0.5), and not below what the
      // storage precision's product supports: a later outer step does not
      // solve to the floor again
      double rmax = 0.0;
      for (uint32_t q = 0; q < nsys; ++q)
        if (!done[q]) rmax = std::max(rmax, resid[q]);
      const double need = rmax > 0.0 ? 0.5 * tol / rmax : 1.0;
      const double itol = std::min(0.5, std::max(inner_prec == resid_prec ? 1e-12 : inner_tol, need));
      if ((rc = gmres_core(sv, inner_prec, rr.as<double>(), z.as<double>(), itol, m, budget, it2, res2, idone,
                           vbuf, rbuf, &graphs[inner_prec])))
        return rc;
      uint32_t step = 0;
      for (uint32_t q = 0; q < nsys; ++q)
        if (!done[q]) {
          iters[q] += it2[q];
          step = std::max(step, it2[q]);
        }
      used += std::max(step, 1u);
      trace.mark(2);
      {
        double rmax = 0.0;
        for (uint32_t q = 0; q < nsys; ++q) rmax = std::max(rmax, prev[q]);
        trace.report(++outer, resid_prec, inner_prec, step, rmax);
      }
      // x += z
      std::vector<double> ones(nsys, 1.0);
      AHX_CUDA(cudaMemcpyAsync(sv.small2_.p, ones.data(), nsys * 8, cudaMemcpyHostToDevice, st));
      axpy_sys_kernel<<<grid_for(total), 256, 0, st>>>(X, X, z.as<double>(), sv.small2_.as<double>(),
                                                       total, op.ntot, sv.segid(), op.nseg);
      AHX_CUDA(cudaGetLastError());
    }
  }
  vbuf.release();
  rbuf.release();
  rr.release();
  z.release();
  if (rc) return rc;
  status = AHX_OK;
  for (uint32_t q = 0; q < nsys; ++q) {
    if (!done[q]) status = AHX_NOT_CONVERGED;
    if (iters_out) iters_out[q] = iters[q];
    if (resid_out) resid_out[q] = resid[q];
  }
  return AHX_OK;
}

// CG (solvers/CG.cpp:31-113) for every system, FP64 product.
int cg_driver(Operator& op, uint32_t p, const double* B, double* X, double tol, uint32_t maxit,
              uint32_t* iters_out, double* resid_out, int& status) {
  Solver sv(op, p);
  int rc = sv.init(4);
  if (rc) return rc;
  const uint32_t nsys = sv.nsys_, K = sv.maxk_;
  const uint64_t total = sv.total_;
  cudaStream_t st = op.stream;
  const uint32_t* sid = sv.segid();
  DevBuf buf;
  if ((rc = buf.reserve(3 * total * sizeof(double)))) return rc;
  double* P = buf.as<double>();
  double* Q = P + total;
  double* R = Q + total;
  double* ds = sv.small_.as<double>();
  double* da = sv.small2_.as<double>();
  std::vector<double> hb((size_t)nsys * K), coef(nsys);
  auto dot1 = [&](const double* a, const double* b, std::vector<double>& out) -> int {
    int r2 = sv.dots(a, 0, 1, b, ds);
    if (r2) return r2;
    AHX_CUDA(cudaMemcpyAsync(hb.data(), ds, hb.size() * 8, cudaMemcpyDeviceToHost, st));
    AHX_CUDA(cudaStreamSynchronize(st));
    out.resize(nsys);
    for (uint32_t q = 0; q < nsys; ++q) out[q] = hb[(size_t)q * K];
    return AHX_OK;
  };
  auto axpy = [&](double* Y, const double* Xv, const double* Z, const std::vector<double>& a) -> int {
    AHX_CUDA(cudaMemcpyAsync(da, a.data(), nsys * 8, cudaMemcpyHostToDevice, st));
    axpy_sys_kernel<<<grid_for(total), 256, 0, st>>>(Y, Xv, Z, da, total, op.ntot, sid, op.nseg);
    AHX_CUDA(cudaGetLastError());
    return AHX_OK;
  };
  std::vector<double> nrmb, res2, rho(nsys), rho1(nsys, 0.0), pq;
  if ((rc = dot1(B, B, nrmb))) return rc;
  std::vector<char> done(nsys, 0);
  std::vector<uint32_t> iters(nsys, 0);
  std::vector<double> resid(nsys, 0.0);
  AHX_CUDA(cudaMemcpyAsync(R, B, total * 8, cudaMemcpyDeviceToDevice, st));
  if ((rc = op.apply(kFP64, -1.0, p, X, R))) return rc;
  if ((rc = dot1(R, R, res2))) return rc;
  for (uint32_t q = 0; q < nsys; ++q) {
    nrmb[q] = std::sqrt(nrmb[q]);
    const double rs = std::sqrt(res2[q]);
    if (nrmb[q] < 1e-16) {
      done[q] = 1;
      resid[q] = 0.0;
    } else if (rs <= tol * nrmb[q]) {
      done[q] = 1;
      resid[q] = rs / nrmb[q];
    }
  }
  for (uint32_t l = 1; l <= maxit; ++l) {
    bool any = false;
    for (uint32_t q = 0; q < nsys; ++q) any |= !done[q];
    if (!any) break;
    if ((rc = dot1(R, R, rho))) return rc;
    if (l > 1) {
      for (uint32_t q = 0; q < nsys; ++q) coef[q] = done[q] ? 0.0 : rho[q] / rho1[q];
      // p = r + beta p
      if ((rc = axpy(P, R, P, coef))) return rc;
    } else {
      AHX_CUDA(cudaMemcpyAsync(P, R, total * 8, cudaMemcpyDeviceToDevice, st));
    }
    AHX_CUDA(cudaMemsetAsync(Q, 0, total * 8, st));
    if ((rc = op.apply(kFP64, 1.0, p, P, Q))) return rc;
    if ((rc = dot1(P, Q, pq))) return rc;
    for (uint32_t q = 0; q < nsys; ++q) coef[q] = done[q] ? 0.0 : rho[q] / pq[q];
    if ((rc = axpy(X, X, P, coef))) return rc;
    for (uint32_t q = 0; q < nsys; ++q) coef[q] = -coef[q];
    if ((rc = axpy(R, R, Q, coef))) return rc;
    if ((rc = dot1(R, R, res2))) return rc;
    for (uint32_t q = 0; q < nsys; ++q) {
      if (done[q]) continue;
      const double rs = std::sqrt(res2[q]);
      resid[q] = rs / nrmb[q];
      iters[q] = l;
      if (rs <= tol * nrmb[q]) done[q] = 1;
    }
    rho1 = rho;
  }
  buf.release();
  status = AHX_OK;
  for (uint32_t q = 0; q < nsys; ++q) {
    if (!done[q]) status = AHX_NOT_CONVERGED;
    if (iters_out) iters_out[q] = iters[q];
    if (resid_out) resid_out[q] = resid[q];
  }
  return AHX_OK;
}

// Host/device staging of an ntot x p block with leading dimension ld.
int stage_in(const double* src, uint64_t ld, uint64_t n, uint32_t p, DevBuf& buf, const double*& dev,
             cudaStream_t st) {
  if (is_device_ptr(src) && ld == n) {
    dev = src;
    return AHX_OK;
  }
  int rc = buf.reserve(n * p * sizeof(double));
  if (rc) return rc;
  AHX_CUDA(cudaMemcpy2DAsync(buf.p, n * 8, src, ld * 8, n * 8, p, cudaMemcpyDefault, st));
  dev = buf.as<double>();
  return AHX_OK;
}

}  // namespace
}  // namespace ahx

// ---------------------------------------------------------------------------
// multi-instance batch

struct ahx_batch : ahx::Operator {
  std::vector<ahx_hmat*> mats;
  int prec = 0;
  int device = 0;
  bool own_stream = false;
  // concatenated product tables per precision (FP64 always, for refinement)
  struct Tab {
    ahx::DevBuf leaves, order, lr, dn;
    uint32_t nleaves = 0;
    uint64_t elems = 0;  // FP64 arena elements (kFP64 table)
    ahx::ProdCopy plan;  // mixed-precision plan over the concatenated leaves
  } tab[ahx::kNumPrecisions];
  ahx::DevBuf stx, sty;

  // FP64: concatenated leaf table and arena; mixed precisions: streams built
  // from the concatenated FP64 arena.
  int build_tab(int pr) {
    using namespace ahx;
    Tab& T = tab[pr];
    if (pr == kDF64) {
      // the concatenated FP64 arena split into (hi, lo) float pairs
      Tab& F = tab[kFP64];
      const uint64_t elems = F.elems;
      int rc = T.plan.lr.reserve(std::max<uint64_t>(elems, 1) * 8);
      if (rc) return rc;
      AHX_CUDA(launch_split_df(F.lr.as<double>(), elems, elems, 1, 1.0, T.plan.lr.p, stream));
      AHX_CUDA(cudaStreamSynchronize(stream));
      T.nleaves = F.nleaves;
      T.plan.bytes = elems * 8;
      T.plan.valid = true;
      return AHX_OK;
    }
    if (pr != kFP64) {
      Tab& F = tab[kFP64];
      std::vector<MvLeaf> lv(F.nleaves);
      AHX_CUDA(cudaMemcpy(lv.data(), F.leaves.p, lv.size() * sizeof(MvLeaf), cudaMemcpyDeviceToHost));
      std::vector<PlanLeaf> pls;
      pls.reserve(lv.size());
      for (const MvLeaf& m : lv) pls.push_back(PlanLeaf{m.b1, m.n1, m.b2, m.n2, m.rank, m.off});
      const int rc = build_mixed_streams(T.plan, pr, pls, F.lr.as<double>(), ntot, device, stream);
      if (rc == AHX_OK) T.plan.valid = true;
      return rc;
    }
    std::vector<MvLeaf> all;
    std::vector<uint64_t> cost;
    uint64_t elems = 0;
    std::vector<std::pair<const void*, uint64_t>> src;  // (ptr, bytes)
    for (size_t i = 0; i < mats.size(); ++i) {
      ahx_hmat* H = mats[i];
      int rc = prepare_product(H, kFP64);
      if (rc) return rc;
      ProdCopy& pc = H->prod[kFP64];
      std::vector<MvLeaf> lv(pc.nleaves);
      AHX_CUDA(cudaMemcpy(lv.data(), pc.leaves.p, lv.size() * sizeof(MvLeaf), cudaMemcpyDeviceToHost));
      for (MvLeaf& L : lv) {
        L.b1 += (uint32_t)seg_off[i];
        L.b2 += (uint32_t)seg_off[i];
        L.off += elems;
        all.push_back(L);
        cost.push_back(L.rank < 0 ? (uint64_t)L.n1 * L.n2 : (uint64_t)L.rank * (L.n1 + L.n2));
      }
      src.push_back({H->arena64.p, H->arena64_elems * sizeof(double)});
      elems += H->arena64_elems;
    }
    std::vector<uint32_t> order(all.size());
    for (uint32_t k = 0; k < order.size(); ++k) order[k] = k;
    std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return cost[a] > cost[b]; });
    int rc;
    if ((rc = T.leaves.reserve(std::max<size_t>(all.size(), 1) * sizeof(MvLeaf)))) return rc;
    if ((rc = T.order.reserve(std::max<size_t>(order.size(), 1) * 4))) return rc;
    if ((rc = T.lr.reserve(std::max<uint64_t>(elems, 1) * sizeof(double)))) return rc;
    if (!all.empty()) {
      AHX_CUDA(cudaMemcpyAsync(T.leaves.p, all.data(), all.size() * sizeof(MvLeaf), cudaMemcpyHostToDevice, stream));
      AHX_CUDA(cudaMemcpyAsync(T.order.p, order.data(), order.size() * 4, cudaMemcpyHostToDevice, stream));
    }
    uint64_t o = 0;
    for (auto& sp : src) {
      if (sp.second)
        AHX_CUDA(cudaMemcpyAsync((char*)T.lr.p + o, sp.first, sp.second, cudaMemcpyDeviceToDevice, stream));
      o += sp.second;
    }
    AHX_CUDA(cudaStreamSynchronize(stream));
    T.nleaves = (uint32_t)all.size();
    T.elems = elems;
    return AHX_OK;
  }

  int prepare(int pr, uint32_t p) override {
    if (pr != ahx::kDF64) return AHX_OK;
    int rc;
    if (!tab[pr].plan.valid && (rc = build_tab(pr))) return rc;
    return ahx::prepare_df_x(tab[pr].plan, ntot, p);
  }

  uint64_t product_bytes(int pr) const override {
    return pr == ahx::kFP64 ? tab[pr].elems * sizeof(double) : tab[pr].plan.bytes;
  }

  int apply(int pr, double d, uint32_t p, const double* X, double* Y) override {
    using namespace ahx;
    Tab& T = tab[pr];
    if (pr == kDF64) {
      const Tab& F = tab[kFP64];
      return run_df(F.leaves.as<MvLeaf>(), F.order.as<uint32_t>(), F.nleaves, T.plan, ntot, d, p, X, ntot, Y,
                    ntot, stream);
    }
    if (pr != kFP64) {
      const TcPlan pl = mixed_plan(T.plan, ntot);
      AHX_CUDA(launch_matvec_tc(pr, pl, d, p, X, ntot, Y, ntot, stream));
      return AHX_OK;
    }
    MvArgs a;
    a.leaves = T.leaves.as<MvLeaf>();
    a.order = T.order.as<uint32_t>();
    a.nleaves = T.nleaves;
    a.arena_lr = T.lr.p;
    a.arena_dn = T.dn.p;
    a.d = d;
    a.p = p;
    a.X = X;
    a.ldX = ntot;
    a.Y = Y;
    a.ldY = ntot;
    AHX_CUDA(launch_matvec(pr, a, stream));
    return AHX_OK;
  }
};

using namespace ahx;

extern "C" {

int ahx_gmres(ahx_hmat* H, int precision, uint32_t p, const double* B, uint64_t ldB, double* X,
              uint64_t ldX, double tol, uint32_t m, uint32_t maxit, uint32_t* iters,
              double* resid) {
  if (!H || !B || !X || p == 0 || ldB < H->tree.n || ldX < H->tree.n || precision < 0 ||
      precision >= kNumPrecisions) {
    set_error("ahx_gmres: invalid argument");
    return AHX_ERR_ARG;
  }
  if (!H->assembled) {
    set_error("ahx_gmres: H-matrix not assembled");
    return AHX_ERR_STATE;
  }
  int rc = ensure_device(H);
  if (rc) return rc;
  HmatOp op(H);
  const uint64_t n = H->tree.n;
  DevBuf bb, xb;
  const double* Bd = nullptr;
  if ((rc = stage_in(B, ldB, n, p, bb, Bd, H->stream))) return rc;
  const double* Xc = nullptr;
  if ((rc = stage_in(X, ldX, n, p, xb, Xc, H->stream))) return rc;
  double* Xd = const_cast<double*>(Xc);
  int status = AHX_OK;
  rc = gmres_driver(op, precision, p, Bd, Xd, tol, m, maxit, iters, resid, status);
  if (rc) return rc;
  if (Xd != X) {
    AHX_CUDA(cudaMemcpy2DAsync(X, ldX * 8, Xd, n * 8, n * 8, p, cudaMemcpyDefault, H->stream));
  }
  AHX_CUDA(cudaStreamSynchronize(H->stream));
  bb.release();
  xb.release();
  return status;
}

// spctrlnrm (Include/matrix.h:50-75): it_num power steps on A^T A from x = 1
// (FP64 products; A^T by the transposed product), the square root of the last norm.
int ahx_spctrlnrm(ahx_hmat* H, uint32_t it_num, double* out) {
  if (!H || !out) return AHX_ERR_ARG;
  if (!H->assembled) {
    set_error("ahx_spctrlnrm: H-matrix not assembled");
    return AHX_ERR_STATE;
  }
  int rc = ensure_device(H);
  if (rc) return rc;
  HmatOp op(H);
  Solver sv(op, 1);
  if ((rc = sv.init(2))) return rc;
  const uint64_t n = H->tree.n;
  ScopedBuf xb, yb;
  if ((rc = xb.reserve(n * 8)) || (rc = yb.reserve(n * 8))) return rc;
  double* x = xb.as<double>();
  double* y = yb.as<double>();
  cudaStream_t st = H->stream;
  const std::vector<double> ones(n, 1.0);
  AHX_CUDA(cudaMemcpyAsync(x, ones.data(), n * 8, cudaMemcpyHostToDevice, st));
  double* d2 = sv.small_.as<double>();
  double dd = 0.0;
  for (uint32_t it = 0; it < it_num; ++it) {
    AHX_CUDA(cudaMemsetAsync(y, 0, n * 8, st));
    if ((rc = product_device(H, kFP64, 1.0, 1, x, n, y, n, false))) return rc;
    AHX_CUDA(cudaMemsetAsync(x, 0, n * 8, st));
    if ((rc = product_device(H, kFP64, 1.0, 1, y, n, x, n, true))) return rc;
    if ((rc = sv.dots(x, 0, 1, x, d2))) return rc;
    scale_kernel<<<grid_for(n), 256, 0, st>>>(x, x, d2, sv.maxk_, 1, n, n, nullptr, 1);  // x /= |x|
    AHX_CUDA(cudaGetLastError());
  }
  if (it_num) AHX_CUDA(cudaMemcpyAsync(&dd, d2, 8, cudaMemcpyDeviceToHost, st));
  AHX_CUDA(cudaStreamSynchronize(st));
  xb.release();
  yb.release();
  *out = std::sqrt(std::sqrt(dd));
  return AHX_OK;
}

int ahx_cg(ahx_hmat* H, uint32_t p, const double* B, uint64_t ldB, double* X, uint64_t ldX,
           double tol, uint32_t maxit, uint32_t* iters, double* resid) {
  if (!H || !B || !X || p == 0 || ldB < H->tree.n || ldX < H->tree.n) {
    set_error("ahx_cg: invalid argument");
    return AHX_ERR_ARG;
  }
  if (!H->assembled) {
    set_error("ahx_cg: H-matrix not assembled");
    return AHX_ERR_STATE;
  }
  int rc = ensure_device(H);
  if (rc) return rc;
  HmatOp op(H);
  const uint64_t n = H->tree.n;
  DevBuf bb, xb;
  const double* Bd = nullptr;
  if ((rc = stage_in(B, ldB, n, p, bb, Bd, H->stream))) return rc;
  const double* Xc = nullptr;
  if ((rc = stage_in(X, ldX, n, p, xb, Xc, H->stream))) return rc;
  double* Xd = const_cast<double*>(Xc);
  int status = AHX_OK;
  rc = cg_driver(op, p, Bd, Xd, tol, maxit, iters, resid, status);
  if (rc) return rc;
  if (Xd != X) AHX_CUDA(cudaMemcpy2DAsync(X, ldX * 8, Xd, n * 8, n * 8, p, cudaMemcpyDefault, H->stream));
  AHX_CUDA(cudaStreamSynchronize(H->stream));
  return status;
}

int ahx_batch_create(ahx_hmat* const* mats, uint32_t count, int precision, ahx_batch** out) {
  if (!mats || !out || count == 0 || precision < 0 || precision >= kNumPrecisions) {
    set_error("ahx_batch_create: invalid argument");
    return AHX_ERR_ARG;
  }
  *out = nullptr;
  for (uint32_t i = 0; i < count; ++i) {
    if (!mats[i] || !mats[i]->assembled) {
      set_error("ahx_batch_create: every instance must be assembled");
      return AHX_ERR_STATE;
    }
    if (mats[i]->tree.sym) {
      set_error("ahx_batch_create: symmetric instances are not batched");
      return AHX_ERR_ARG;
    }
    if (mats[i]->device != mats[0]->device) {
      set_error("ahx_batch_create: instances on different devices");
      return AHX_ERR_ARG;
    }
  }
  ahx_batch* b = new (std::nothrow) ahx_batch;
  if (!b) return AHX_ERR_NOMEM;
  b->mats.assign(mats, mats + count);
  b->prec = precision;
  b->device = mats[0]->device;
  int rc = ensure_device(mats[0]);
  if (rc) {
    delete b;
    return rc;
  }
  {
    cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
      delete b;
      return cuda_fail(e, "cudaStreamCreate");
    }
    b->own_stream = true;
  }
  b->nseg = count;
  b->seg_off.assign(count + 1, 0);
  for (uint32_t i = 0; i < count; ++i) b->seg_off[i + 1] = b->seg_off[i] + mats[i]->tree.n;
  b->ntot = b->seg_off[count];
  if (b->ntot >= (1ull << 32)) {
    delete b;
    set_error("ahx_batch_create: total length exceeds 2^32");
    return AHX_ERR_ARG;
  }
  for (uint32_t i = 0; i < count; ++i) {
    // instances share the first instance's stream for the duration of the batch
    if ((rc = ensure_device(mats[i]))) {
      delete b;
      return rc;
    }
  }
  if ((rc = b->init_segments()) || (rc = b->build_tab(kFP64)) ||
      (precision != kFP64 && (rc = b->build_tab(precision)))) {
    ahx_batch_destroy(b);
    return rc;
  }
  *out = b;
  return AHX_OK;
}

int ahx_batch_destroy(ahx_batch* b) {
  if (!b) return AHX_OK;
  cudaSetDevice(b->device);
  if (b->own_stream && b->stream) cudaStreamSynchronize(b->stream);
  for (auto& T : b->tab) {
    T.leaves.release();
    T.order.release();
    T.lr.release();
    T.dn.release();
    T.plan.release_all();
  }
  b->stx.release();
  b->sty.release();
  if (b->own_stream && b->stream) cudaStreamDestroy(b->stream);
  b->stream = nullptr;
  delete b;
  return AHX_OK;
}

uint64_t ahx_batch_n(const ahx_batch* b) { return b ? b->ntot : 0; }

int ahx_batch_prepare(ahx_batch* b, int precision) {
  if (!b || precision < 0 || precision >= kNumPrecisions) return AHX_ERR_ARG;
  AHX_CUDA(cudaSetDevice(b->device));
  if (precision == kFP64) return AHX_OK;
  if (precision == kDF64) return b->prepare(kDF64, 1);
  if (b->tab[precision].plan.valid) return AHX_OK;
  return b->build_tab(precision);
}

int ahx_batch_matvec(ahx_batch* b, double d, uint32_t p, const double* X, double* Y) {
  if (!b || !X || !Y) return AHX_ERR_ARG;
  if (p == 0) return AHX_OK;
  AHX_CUDA(cudaSetDevice(b->device));
  const uint64_t n = b->ntot;
  const double* Xd = nullptr;
  int rc = stage_in(X, n, n, p, b->stx, Xd, b->stream);
  if (rc) return rc;
  const bool yd = is_device_ptr(Y);
  double* Yd = Y;
  if (!yd) {
    if ((rc = b->sty.reserve(n * p * 8))) return rc;
    AHX_CUDA(cudaMemcpyAsync(b->sty.p, Y, n * p * 8, cudaMemcpyHostToDevice, b->stream));
    Yd = b->sty.as<double>();
  }
  if ((rc = b->apply(b->prec, d, p, Xd, Yd))) return rc;
  if (!yd) AHX_CUDA(cudaMemcpyAsync(Y, Yd, n * p * 8, cudaMemcpyDeviceToHost, b->stream));
  if (!yd || Xd != X) AHX_CUDA(cudaStreamSynchronize(b->stream));
  return AHX_OK;
}

int ahx_batch_gmres(ahx_batch* b, const double* B, double* X, double tol, uint32_t m,
                    uint32_t maxit, uint32_t* iters, double* resid) {
  if (!b || !B || !X) return AHX_ERR_ARG;
  AHX_CUDA(cudaSetDevice(b->device));
  const uint64_t n = b->ntot;
  DevBuf bb, xb;
  const double* Bd = nullptr;
  int rc = stage_in(B, n, n, 1, bb, Bd, b->stream);
  if (rc) return rc;
  const double* Xc = nullptr;
  if ((rc = stage_in(X, n, n, 1, xb, Xc, b->stream))) return rc;
  double* Xd = const_cast<double*>(Xc);
  int status = AHX_OK;
  rc = gmres_driver(*b, b->prec, 1, Bd, Xd, tol, m, maxit, iters, resid, status);
  if (rc) return rc;
  if (Xd != X) AHX_CUDA(cudaMemcpyAsync(X, Xd, n * 8, cudaMemcpyDefault, b->stream));
  AHX_CUDA(cudaStreamSynchronize(b->stream));
  return status;
}

}  // extern "C"
