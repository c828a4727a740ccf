// ahx_ahmed.hpp -- the reference's C++ entry points for the H-matrix hot path,
// implemented over the C ABI of libahx (include/ahx.h).
//
// A program written against AHMED's hot path
//
//   bemcluster<dof>* cl = new bemcluster<dof>(dofs, op_perm, 0, N);   // Include/bemcluster.h:25
//   cl->createClusterTree(bmin, op_perm, po_perm);                     // Include/cluster_pca.h:204
//   bemblcluster<dof,dof>* bl = new bemblcluster<dof,dof>(0, 0, N, N); // Include/bemblcluster.h:23
//   bl->subdivide(cl, cl, eta * eta, nblcks);                          // Include/blcluster.h:382
//   mblock<double>** A; allocmbls(bl, A);                              // Include/H.h:28
//   matgenGeH_omp(MatGen, nblcks, bl, eps, rankmax, A);                // Include/matgen_omp.h:197
//   mltaGeHVec(1.0, bl, A, x, y);                                      // H/mltaGeHVec.cpp:567
//   GMRes(Op, b, x, eps, m, nsteps);                                   // solvers/GMRES.cpp:80
//   savembls(eta, bmin, bl, A, os); loadmbls(eta, bmin, A, is);        // Include/H.h:60-103
//   freembls(bl, A);                                                   // Include/H.h:42
//
// compiles against this header by replacing the AHMED includes with it and
// `using namespace ahx_ahmed;`.  The clusters, the block-cluster tree and the
// leaves live in one libahx handle (trees on the host, bit-identical to the
// reference's; leaves on the GPU).  mblock<T> objects are host views that
// copy a leaf back from the device when their data is asked for.
// MATGEN_T: the kernels are evaluated on the GPU by this library, not through the
// generator object's cmpbl / scale (Include/matgen_omp.h:27-33).  The matgen_*
// functions therefore accept only the library's generator types (or types derived
// from them), and refuse any other MATGEN_T at compile time:
//   LaplaceGenerator{h}        K = 1/(4 pi r), diagonal 1/(4 pi h)  (mblock<double>, mblock<float>)
//   HelmholtzGenerator{h, k}   K = exp(ikr)/(4 pi r), diagonal exp(ikh)/(4 pi h)
//                              (mblock<dcomp>, mblock<scomp>)
// GMRes / CG run on the GPU for the library's operators (HMatrixOperator,
// ZHMatrixOperator) only; a call with any other Matrix<T> does not compile.  The
// operators have no preconditioner: the reference's Matrix::precond_apply
// (solvers/GMRES.cpp:73,128, solvers/CG.cpp:71) is the identity for them.
#ifndef AHX_AHMED_HPP
#define AHX_AHMED_HPP

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <iterator>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "ahx.h"

namespace ahx_ahmed {

using dcomp = std::complex<double>;  // the reference's dcomp (Include/cmplx.h)
using scomp = std::complex<float>;   // the reference's scomp

inline void check(int rc) {
  if (rc != AHX_OK && rc != AHX_NOT_CONVERGED)
    throw std::runtime_error(std::string("ahx: ") + ahx_last_error());
}

// Geometry shared by the clusters and the block-cluster tree of one matrix.
struct Geometry {
  std::vector<double> pts;  // original order, xyz
  int kind = AHX_TREE_PCA;
  unsigned bmin = 0;
  unsigned* op_perm = nullptr;
  unsigned* po_perm = nullptr;
};

// cluster tree root (the reference's bemcluster / cluster3d_bbx)
template <class DOF, int KIND>
class cluster_root {
 public:
  cluster_root(DOF* dofs, unsigned* op_perm, unsigned k, unsigned l) : geo_(new Geometry) {
    if (k != 0) throw std::invalid_argument("ahx_ahmed: only root clusters (k = 0) are built");
    geo_->kind = KIND;
    geo_->pts.resize(3 * (size_t)l);
    for (unsigned i = 0; i < l; ++i)
      for (unsigned j = 0; j < 3; ++j) geo_->pts[3 * (size_t)i + j] = dofs[i].getcenter(j);
    geo_->op_perm = op_perm;
    n_ = l;
  }
  // Include/cluster_pca.h:204 / Include/cluster_bbx.h:100: the permutation is
  // written when the block-cluster tree is built (the tree needs eta as well).
  void createClusterTree(unsigned bmin, unsigned* op_perm, unsigned* po_perm) {
    geo_->bmin = bmin;
    geo_->op_perm = op_perm;
    geo_->po_perm = po_perm;
  }
  unsigned size() const { return n_; }
  std::shared_ptr<Geometry> geometry() const { return geo_; }

 private:
  std::shared_ptr<Geometry> geo_;
  unsigned n_ = 0;
};

template <class DOF>
using bemcluster = cluster_root<DOF, AHX_TREE_PCA>;
template <class DOF>
using cluster3d_bbx = cluster_root<DOF, AHX_TREE_BBX>;

// root of the block-cluster tree (the reference's bemblcluster / blcluster_geo)
class blcluster {
 public:
  blcluster(unsigned i1, unsigned i2, unsigned m1, unsigned m2) : n_(m1) {
    if (i1 != 0 || i2 != 0 || m1 != m2)
      throw std::invalid_argument("ahx_ahmed: the root block must be (0, 0, N, N)");
  }
  ~blcluster() {
    if (h_) ahx_hmat_destroy(h_);
  }
  blcluster(const blcluster&) = delete;
  blcluster& operator=(const blcluster&) = delete;

  // Include/blcluster.h:382: builds the trees and numbers the leaves in DFS order
  template <class CL>
  void subdivide(CL* cl1, CL* cl2, double eta2, unsigned& nblcks, unsigned maxdepth = 0) {
    if (cl1 != cl2 || maxdepth != 0)
      throw std::invalid_argument("ahx_ahmed: square trees over one cluster tree, maxdepth 0");
    std::shared_ptr<Geometry> g = cl1->geometry();
    check(ahx_hmat_create(g->pts.data(), n_, g->kind, g->bmin, eta2, 0, nullptr, &h_));
    check(ahx_hmat_perm(h_, g->op_perm, g->po_perm));
    nblcks = ahx_hmat_nleaves(h_);
    leaves_.resize(7 * (size_t)nblcks);
    check(ahx_hmat_leaves(h_, leaves_.data()));
  }

  // Include/blcluster.h:388 (cluster/blcluster.cpp:90-113): the symmetric block
  // tree, diagonal and upper blocks (assembled by matgenHeH_omp, applied by mltaHeHVec)
  template <class CL>
  void subdivide_sym(CL* cl, double eta2, unsigned& nblcks, unsigned maxdepth = 0) {
    if (maxdepth != 0) throw std::invalid_argument("ahx_ahmed: maxdepth 0");
    std::shared_ptr<Geometry> g = cl->geometry();
    check(ahx_hmat_create_sym(g->pts.data(), n_, g->kind, g->bmin, eta2, 0, nullptr, &h_));
    check(ahx_hmat_perm(h_, g->op_perm, g->po_perm));
    nblcks = ahx_hmat_nleaves(h_);
    leaves_.resize(7 * (size_t)nblcks);
    check(ahx_hmat_leaves(h_, leaves_.data()));
  }

  unsigned long nleaves() const { return ahx_hmat_nleaves(h_); }
  unsigned long nadmleaves() const {
    unsigned long c = 0;
    for (size_t l = 0; l < leaves_.size() / 7; ++l) c += leaves_[7 * l + 4];
    return c;
  }
  unsigned getn1() const { return n_; }
  unsigned getn2() const { return n_; }
  ahx_hmat* handle() const { return h_; }
  const uint32_t* leaf(unsigned l) const { return &leaves_[7 * (size_t)l]; }
  // per-leaf ranks after an assembly (-1 dense)
  void refresh_ranks() {
    ranks_.resize(ahx_hmat_nleaves(h_));
    check(ahx_hmat_ranks(h_, ranks_.data()));
  }
  // leaves and ranks again (after an agglomeration changed the leaves)
  void refresh_leaves() {
    leaves_.resize(7 * (size_t)ahx_hmat_nleaves(h_));
    check(ahx_hmat_leaves(h_, leaves_.data()));
  }
  void refresh() {
    refresh_leaves();
    refresh_ranks();
  }
  int rank_of(unsigned l) const { return ranks_.at(l); }
  // per-leaf ranks of the Helmholtz (mblock<dcomp>) leaves
  void refresh_zranks() {
    zranks_.resize(ahx_hmat_nleaves(h_));
    check(ahx_helm_ranks(h_, zranks_.data()));
  }
  int zrank_of(unsigned l) const { return zranks_.at(l); }
  int rank_of(unsigned l, const double*) const { return rank_of(l); }
  int rank_of(unsigned l, const dcomp*) const { return zrank_of(l); }
  int rank_of(unsigned l, const float*) const { return rank_of(l); }
  int rank_of(unsigned l, const scomp*) const { return zrank_of(l); }

 private:
  unsigned n_;
  ahx_hmat* h_ = nullptr;
  std::vector<uint32_t> leaves_;
  std::vector<int32_t> ranks_, zranks_;
};

template <class T1, class T2>
using bemblcluster = blcluster;

// Host view of one leaf (Include/mblock.h:29-97): U then V for a low-rank
// block, n1 x n2 column-major for a dense one.
template <class T>
class mblock {
  static constexpr bool kComplex = std::is_same<T, dcomp>::value || std::is_same<T, scomp>::value;

 public:
  mblock(const blcluster* bl, unsigned idx) : bl_(bl), idx_(idx) {}
  // a leaf read by loadmbls, not yet uploaded into a block-cluster tree
  mblock(std::shared_ptr<std::string> file, unsigned idx) : bl_(nullptr), idx_(idx), file_(file) {}
  bool pending() const { return !bl_; }
  const std::shared_ptr<std::string>& file() const { return file_; }
  void attach(const blcluster* bl) {
    bl_ = bl;
    file_.reset();
  }
  unsigned getn1() const { return bound()->leaf(idx_)[1]; }
  unsigned getn2() const { return bound()->leaf(idx_)[3]; }
  bool isLrM() const { return bound()->rank_of(idx_, (const T*)nullptr) >= 0; }
  bool isGeM() const { return !isLrM(); }
  // dense diagonal block of a symmetric tree: packed upper triangle (Include/mblock.h:314)
  bool isHeM() const { return !kComplex && diag_dense(); }
  // dense diagonal block of a complex symmetric matrix: packed upper triangle (SyM)
  bool isSyM() const { return kComplex && diag_dense(); }
  unsigned rank() const { return (unsigned)bound()->rank_of(idx_, (const T*)nullptr); }
  T* getdata() {
    if (data_.empty()) fetch(bound()->handle(), idx_, data_);
    return data_.data();
  }

 private:
  bool diag_dense() const {
    return isGeM() && ahx_hmat_symmetric(bound()->handle()) && bound()->leaf(idx_)[0] == bound()->leaf(idx_)[2];
  }
  static void fetch(ahx_hmat* h, unsigned l, std::vector<double>& d) {
    d.resize(ahx_hmat_leaf_size(h, l));
    if (!d.empty()) check(ahx_hmat_get_leaf(h, l, d.data()));
  }
  // mblock<float> / mblock<scomp>: the FP64 / complex128 leaf rounded to single precision
  static void fetch(ahx_hmat* h, unsigned l, std::vector<float>& d) {
    std::vector<double> w;
    fetch(h, l, w);
    d.assign(w.begin(), w.end());
  }
  static void fetch(ahx_hmat* h, unsigned l, std::vector<scomp>& d) {
    std::vector<dcomp> w;
    fetch(h, l, w);
    d.resize(w.size());
    for (size_t i = 0; i < w.size(); ++i) d[i] = scomp((float)w[i].real(), (float)w[i].imag());
  }
  static void fetch(ahx_hmat* h, unsigned l, std::vector<dcomp>& d) {
    d.resize(ahx_helm_leaf_size(h, l));
    if (!d.empty()) check(ahx_helm_get_leaf(h, l, reinterpret_cast<double*>(d.data())));
  }
  const blcluster* bound() const {
    if (!bl_)
      throw std::logic_error("ahx_ahmed: leaves from loadmbls are bound to a tree by bind_mbls or the first product");
    return bl_;
  }
  const blcluster* bl_;
  unsigned idx_;
  std::vector<T> data_;
  std::shared_ptr<std::string> file_;
};

template <class T>
void allocmbls(blcluster* bl, mblock<T>**& A) {
  const unsigned n = (unsigned)bl->nleaves();
  A = new mblock<T>*[n];
  for (unsigned i = 0; i < n; ++i) A[i] = nullptr;
}

template <class T>
void freembls(blcluster* bl, mblock<T>**& A) {
  if (!A) return;
  const unsigned n = (unsigned)bl->nleaves();
  for (unsigned i = 0; i < n; ++i) delete A[i];
  delete[] A;
  A = nullptr;
}

// The generators whose kernels this library evaluates on the GPU.  A program's own
// MATGEN_T may derive from one of them (keeping its other members); any other
// generator type is refused at compile time, since its cmpbl / scale would not be
// called.
struct LaplaceGenerator {
  double h;  // diagonal 1/(4 pi h)
  double geth() const { return h; }
};
struct HelmholtzGenerator {
  double h;  // diagonal exp(ikh)/(4 pi h)
  double k;  // wavenumber
  double geth() const { return h; }
  double getk() const { return k; }
};

template <class T, class MATGEN_T>
inline void check_generator() {
  constexpr bool real = std::is_same<T, double>::value || std::is_same<T, float>::value;
  constexpr bool cplx = std::is_same<T, dcomp>::value || std::is_same<T, scomp>::value;
  static_assert(real || cplx, "ahx_ahmed: mblock<T> with T = double, float, dcomp or scomp");
  static_assert(!real || std::is_base_of<LaplaceGenerator, MATGEN_T>::value,
                "ahx_ahmed: real leaves are assembled from ahx_ahmed::LaplaceGenerator (or a type derived "
                "from it); a generator's own cmpbl/scale are not evaluated on the GPU");
  static_assert(!cplx || std::is_base_of<HelmholtzGenerator, MATGEN_T>::value,
                "ahx_ahmed: complex leaves are assembled from ahx_ahmed::HelmholtzGenerator (or a type "
                "derived from it); a generator's own cmpbl/scale are not evaluated on the GPU");
}

template <class MATGEN_T>
void assemble_leaves(MATGEN_T& MatGen, blcluster* bl, double eps, unsigned rankmax, const double*) {
  check(ahx_assemble(bl->handle(), MatGen.geth(), eps, rankmax));
  bl->refresh_ranks();
}
// mblock<dcomp>: the Helmholtz kernel (apprx_unsym with T = dcomp)
// mblock<float> / mblock<scomp>: assembled in FP64 / complex128 (the reference's
// ACA<float> runs in single precision); the products use the FP32 / complex64 copies
template <class MATGEN_T>
void assemble_leaves(MATGEN_T& MatGen, blcluster* bl, double eps, unsigned rankmax, const float*) {
  assemble_leaves(MatGen, bl, eps, rankmax, (const double*)nullptr);
}
template <class MATGEN_T>
void assemble_leaves(MATGEN_T& MatGen, blcluster* bl, double eps, unsigned rankmax, const scomp*) {
  assemble_leaves(MatGen, bl, eps, rankmax, (const dcomp*)nullptr);
}
template <class MATGEN_T>
void assemble_leaves(MATGEN_T& MatGen, blcluster* bl, double eps, unsigned rankmax, const dcomp*) {
  check(ahx_helm_assemble(bl->handle(), MatGen.getk(), MatGen.geth(), eps, rankmax));
  bl->refresh_zranks();
}

// Include/matgen_omp.h:197-213: ACA assembly of every leaf (on the GPU)
template <class T, class MATGEN_T>
void matgenGeH_omp(MATGEN_T& MatGen, unsigned nblcks, blcluster* bl, double eps, unsigned rankmax,
                   mblock<T>** A) {
  check_generator<T, MATGEN_T>();
  assemble_leaves(MatGen, bl, eps, rankmax, (const T*)nullptr);
  for (unsigned i = 0; i < nblcks; ++i) {
    delete A[i];
    A[i] = new mblock<T>(bl, i);
  }
}

// Include/matgen_omp.h:96-101: HeH assembly of a symmetric block tree (ACAr,
// Hermitian diagonal blocks)
template <class T, class MATGEN_T>
void matgenHeH_omp(MATGEN_T& MatGen, unsigned nblcks, blcluster* bl, double eps, unsigned rankmax,
                   mblock<T>** A) {
  if (!ahx_hmat_symmetric(bl->handle()))
    throw std::invalid_argument("ahx_ahmed: matgenHeH_omp needs a tree from subdivide_sym");
  matgenGeH_omp(MatGen, nblcks, bl, eps, rankmax, A);
}

// Include/matgen_omp.h:102-107: the complex symmetric assembly of a symmetric block
// tree (ACAr<dcomp>, symmetric dense diagonal blocks)
template <class T, class MATGEN_T>
void matgenSyH_omp(MATGEN_T& MatGen, unsigned nblcks, blcluster* bl, double eps, unsigned rankmax,
                   mblock<T>** A) {
  static_assert(std::is_same<T, dcomp>::value, "ahx_ahmed: matgenSyH_omp assembles mblock<dcomp> leaves");
  if (!ahx_hmat_symmetric(bl->handle()))
    throw std::invalid_argument("ahx_ahmed: matgenSyH_omp needs a tree from subdivide_sym");
  matgenGeH_omp(MatGen, nblcks, bl, eps, rankmax, A);
}

// H/agglH.cpp:253-272: agglomeration of the assembled leaves (unions of low-rank sons)
inline void agglomerate_leaves(blcluster* bl, double eps, unsigned max_rank, const double*) {
  check(ahx_agglomerate(bl->handle(), eps, max_rank, nullptr));
  bl->refresh();
}
inline void agglomerate_leaves(blcluster* bl, double eps, unsigned max_rank, const float*) {
  agglomerate_leaves(bl, eps, max_rank, (const double*)nullptr);
}
inline void agglomerate_leaves(blcluster* bl, double eps, unsigned max_rank, const scomp*);
inline void agglomerate_leaves(blcluster* bl, double eps, unsigned max_rank, const dcomp*) {
  check(ahx_helm_agglomerate(bl->handle(), eps, max_rank, nullptr));
  bl->refresh_leaves();
  bl->refresh_zranks();
}
inline void agglomerate_leaves(blcluster* bl, double eps, unsigned max_rank, const scomp*) {
  agglomerate_leaves(bl, eps, max_rank, (const dcomp*)nullptr);
}

template <class T>
void agglH(blcluster* bl, mblock<T>**& A, double eps, unsigned max_rank) {
  const unsigned before = (unsigned)bl->nleaves();
  agglomerate_leaves(bl, eps, max_rank, (const T*)nullptr);
  for (unsigned i = 0; i < before; ++i) delete A[i];
  delete[] A;
  const unsigned n = (unsigned)bl->nleaves();
  A = new mblock<T>*[n];
  for (unsigned i = 0; i < n; ++i) A[i] = new mblock<T>(bl, i);
}

// Include/matgen_sqntl.h:88-102: the assembly; recmpr agglomerates afterwards
template <class T, class MATGEN_T>
void matgenGeH_sqntl(MATGEN_T& MatGen, blcluster* root, blcluster* bl, bool recmpr, double eps,
                     unsigned rankmax, mblock<T>**& A) {
  if (root != bl) throw std::invalid_argument("ahx_ahmed: sub-blocks not built");
  matgenGeH_omp(MatGen, (unsigned)bl->nleaves(), bl, eps, rankmax, A);
  if (recmpr) agglH(bl, A, eps, rankmax);
}

// Include/H.h:89-103: the leaves of bl in the reference's file layout
inline int save_leaves(blcluster* bl, double eta, unsigned bmin, ahx_io_fn put, void* ctx, const double*) {
  return ahx_hmat_save_stream(bl->handle(), eta, bmin, put, ctx);
}
inline int save_leaves(blcluster* bl, double eta, unsigned bmin, ahx_io_fn put, void* ctx, const dcomp*) {
  return ahx_helm_save_stream(bl->handle(), eta, bmin, put, ctx);
}

template <class T>
void savembls(const double eta, const unsigned bmin, blcluster* bl, mblock<T>**&, std::ofstream& os) {
  auto put = [](void* ctx, void* buf, uint64_t bytes) -> int64_t {
    std::ostream& o = *static_cast<std::ostream*>(ctx);
    o.write(static_cast<const char*>(buf), (std::streamsize)bytes);
    return o ? (int64_t)bytes : -1;
  };
  check(save_leaves(bl, eta, bmin, put, &os, (const T*)nullptr));
}

// Include/H.h:60-73 ("loadmbls does not need allocmbls"): eta and bmin come
// back at once; the leaves wait in host memory until the block-cluster tree
// built with them is given to bind_mbls or to the first product with A.
template <class T>
void loadmbls(double& eta, unsigned& bmin, mblock<T>**& A, std::ifstream& is) {
  if (!is) throw std::runtime_error("ahx_ahmed: InputStream not found");
  auto file = std::make_shared<std::string>(std::istreambuf_iterator<char>(is),
                                            std::istreambuf_iterator<char>());
  uint32_t n = 0, b = 0;
  if (file->size() < 16) throw std::runtime_error("ahx_ahmed: loadmbls: truncated header");
  std::memcpy(&eta, file->data(), 8);
  std::memcpy(&b, file->data() + 8, 4);
  std::memcpy(&n, file->data() + 12, 4);
  bmin = b;
  A = new mblock<T>*[n];
  for (uint32_t i = 0; i < n; ++i) A[i] = new mblock<T>(file, i);
}

inline void load_leaves(blcluster* bl, ahx_io_fn get, void* ctx, const double*) {
  check(ahx_hmat_load_stream(bl->handle(), get, ctx, nullptr, nullptr));
  bl->refresh_ranks();
}
// files of single-precision leaves (4 or 8 bytes per element) are not read
inline void load_leaves(blcluster*, ahx_io_fn, void*, const float*) {
  throw std::logic_error("ahx_ahmed: loadmbls of mblock<float> leaves is not supported");
}
inline void load_leaves(blcluster*, ahx_io_fn, void*, const scomp*) {
  throw std::logic_error("ahx_ahmed: loadmbls of mblock<scomp> leaves is not supported");
}
inline void load_leaves(blcluster* bl, ahx_io_fn get, void* ctx, const dcomp*) {
  check(ahx_helm_load_stream(bl->handle(), get, ctx, nullptr, nullptr));
  bl->refresh_zranks();
}

// Uploads leaves read by loadmbls into bl (no-op for leaves already bound).
template <class T>
void bind_mbls(blcluster* bl, mblock<T>** A) {
  if (!A || !bl->nleaves() || !A[0] || !A[0]->pending()) return;
  struct Src {
    const std::string* s;
    size_t pos;
  } src{A[0]->file().get(), 0};
  auto get = [](void* ctx, void* buf, uint64_t bytes) -> int64_t {
    Src& c = *static_cast<Src*>(ctx);
    const size_t m = std::min<size_t>(bytes, c.s->size() - c.pos);
    std::memcpy(buf, c.s->data() + c.pos, m);
    c.pos += m;
    return (int64_t)m;
  };
  load_leaves(bl, get, &src, (const T*)nullptr);
  for (unsigned long i = 0; i < bl->nleaves(); ++i) A[i]->attach(bl);
}

// H/mltaGeHVec.cpp:567-577: y += d A x, Y += d A X (permuted ordering)
inline bool mltaGeHVec(double d, blcluster* bl, mblock<double>** A, double* x, double* y) {
  bind_mbls(bl, A);
  check(ahx_matvec(bl->handle(), AHX_FP64, d, 1, x, bl->getn1(), y, bl->getn1()));
  return true;
}

inline bool mltaGeHGeM(double d, blcluster* bl, mblock<double>** A, unsigned p, double* X,
                       unsigned ldX, double* Y, unsigned ldY) {
  bind_mbls(bl, A);
  check(ahx_matvec(bl->handle(), AHX_FP64, d, p, X, ldX, Y, ldY));
  return true;
}

// H/mltaGeHVec.cpp:654-662 (mltaHeHVec_/mltaHeHGeM_ :421-475): y += d A x for a
// symmetric tree (its upper blocks applied as A and A^T)
inline void mltaHeHVec(double d, blcluster* bl, mblock<double>** A, double* x, double* y) {
  mltaGeHVec(d, bl, A, x, y);
}

inline void mltaHeHGeM(double d, blcluster* bl, mblock<double>** A, unsigned p, double* X, unsigned ldX,
                       double* Y, unsigned ldY) {
  mltaGeHGeM(d, bl, A, p, X, ldX, Y, ldY);
}

// H/mltaGeHVec.cpp:579-589 (mltaGeHhVec_/mltaGeHhGeM_ :62-105): y += d A^H x, Y += d A^H X (A^T for double)
inline bool mltaGeHhVec(double d, blcluster* bl, mblock<double>** A, double* x, double* y) {
  bind_mbls(bl, A);
  check(ahx_matvec_transposed(bl->handle(), d, 1, x, bl->getn1(), y, bl->getn1()));
  return true;
}

inline bool mltaGeHhGeM(double d, blcluster* bl, mblock<double>** A, unsigned p, double* X,
                        unsigned ldX, double* Y, unsigned ldY) {
  bind_mbls(bl, A);
  check(ahx_matvec_transposed(bl->handle(), d, p, X, ldX, Y, ldY));
  return true;
}

// H/mltaGeHVec.cpp:770-805: the dcomp products of the Helmholtz leaves,
// op 0: A, 1: A^H, 2: A^T
inline bool zproduct(int op, dcomp d, blcluster* bl, unsigned p, dcomp* X, unsigned ldX, dcomp* Y,
                     unsigned ldY) {
  check(ahx_helm_matvec(bl->handle(), AHX_FP64, op, d.real(), d.imag(), p, reinterpret_cast<double*>(X), ldX,
                        reinterpret_cast<double*>(Y), ldY));
  return true;
}
inline bool mltaGeHVec(dcomp d, blcluster* bl, mblock<dcomp>** A, dcomp* x, dcomp* y) {
  bind_mbls(bl, A);
  return zproduct(0, d, bl, 1, x, bl->getn1(), y, bl->getn1());
}
inline bool mltaGeHGeM(dcomp d, blcluster* bl, mblock<dcomp>** A, unsigned p, dcomp* X, unsigned ldX, dcomp* Y,
                       unsigned ldY) {
  bind_mbls(bl, A);
  return zproduct(0, d, bl, p, X, ldX, Y, ldY);
}
inline bool mltaGeHhVec(dcomp d, blcluster* bl, mblock<dcomp>**, dcomp* x, dcomp* y) {
  return zproduct(1, d, bl, 1, x, bl->getn1(), y, bl->getn1());
}
inline bool mltaGeHhGeM(dcomp d, blcluster* bl, mblock<dcomp>**, unsigned p, dcomp* X, unsigned ldX, dcomp* Y,
                        unsigned ldY) {
  return zproduct(1, d, bl, p, X, ldX, Y, ldY);
}
inline bool mltaGeHtVec(dcomp d, blcluster* bl, mblock<dcomp>**, dcomp* x, dcomp* y) {
  return zproduct(2, d, bl, 1, x, bl->getn1(), y, bl->getn1());
}
inline bool mltaGeHtGeM(dcomp d, blcluster* bl, mblock<dcomp>**, unsigned p, dcomp* X, unsigned ldX, dcomp* Y,
                        unsigned ldY) {
  return zproduct(2, d, bl, p, X, ldX, Y, ldY);
}

// H/mltaGeHVec.cpp:885-895: y += d A x for a complex symmetric H-matrix (its upper
// blocks applied as A and A^T)
inline void mltaSyHVec(dcomp d, blcluster* bl, mblock<dcomp>** A, dcomp* x, dcomp* y) { mltaGeHVec(d, bl, A, x, y); }
inline void mltaSyHGeM(dcomp d, blcluster* bl, mblock<dcomp>** A, unsigned p, dcomp* X, unsigned ldX, dcomp* Y,
                       unsigned ldY) {
  mltaGeHGeM(d, bl, A, p, X, ldX, Y, ldY);
}

// H/mltaGeHVec.cpp:671-691 (float) and 908-940 (scomp): the single-precision
// instantiations, on the FP32 / complex64 copies of the leaves (FP32 accumulation);
// the vectors pass through double precision
inline bool sproduct(int op, double d, blcluster* bl, unsigned p, const float* X, unsigned ldX, float* Y,
                     unsigned ldY) {
  const unsigned n = bl->getn1();
  std::vector<double> x((size_t)n * p), y((size_t)n * p);
  for (unsigned c = 0; c < p; ++c)
    for (unsigned i = 0; i < n; ++i) {
      x[(size_t)c * n + i] = X[(size_t)c * ldX + i];
      y[(size_t)c * n + i] = Y[(size_t)c * ldY + i];
    }
  if (op == 0) check(ahx_matvec(bl->handle(), AHX_FP32, d, p, x.data(), n, y.data(), n));
  else check(ahx_matvec_transposed(bl->handle(), d, p, x.data(), n, y.data(), n));
  for (unsigned c = 0; c < p; ++c)
    for (unsigned i = 0; i < n; ++i) Y[(size_t)c * ldY + i] = (float)y[(size_t)c * n + i];
  return true;
}
inline bool mltaGeHVec(float d, blcluster* bl, mblock<float>** A, float* x, float* y) {
  bind_mbls(bl, A);
  return sproduct(0, d, bl, 1, x, bl->getn1(), y, bl->getn1());
}
inline bool mltaGeHGeM(float d, blcluster* bl, mblock<float>** A, unsigned p, float* X, unsigned ldX, float* Y,
                       unsigned ldY) {
  bind_mbls(bl, A);
  return sproduct(0, d, bl, p, X, ldX, Y, ldY);
}
// real leaves: A^H = A^T (the FP64 leaves)
inline bool mltaGeHhVec(float d, blcluster* bl, mblock<float>** A, float* x, float* y) {
  bind_mbls(bl, A);
  return sproduct(1, d, bl, 1, x, bl->getn1(), y, bl->getn1());
}
inline bool mltaGeHhGeM(float d, blcluster* bl, mblock<float>** A, unsigned p, float* X, unsigned ldX, float* Y,
                        unsigned ldY) {
  bind_mbls(bl, A);
  return sproduct(1, d, bl, p, X, ldX, Y, ldY);
}
inline bool cproduct(int op, scomp d, blcluster* bl, unsigned p, const scomp* X, unsigned ldX, scomp* Y,
                     unsigned ldY) {
  const unsigned n = bl->getn1();
  std::vector<dcomp> x((size_t)n * p), y((size_t)n * p);
  for (unsigned c = 0; c < p; ++c)
    for (unsigned i = 0; i < n; ++i) {
      x[(size_t)c * n + i] = dcomp(X[(size_t)c * ldX + i].real(), X[(size_t)c * ldX + i].imag());
      y[(size_t)c * n + i] = dcomp(Y[(size_t)c * ldY + i].real(), Y[(size_t)c * ldY + i].imag());
    }
  check(ahx_helm_matvec(bl->handle(), AHX_FP32, op, d.real(), d.imag(), p, reinterpret_cast<double*>(x.data()), n,
                        reinterpret_cast<double*>(y.data()), n));
  for (unsigned c = 0; c < p; ++c)
    for (unsigned i = 0; i < n; ++i)
      Y[(size_t)c * ldY + i] = scomp((float)y[(size_t)c * n + i].real(), (float)y[(size_t)c * n + i].imag());
  return true;
}
inline bool mltaGeHVec(scomp d, blcluster* bl, mblock<scomp>**, scomp* x, scomp* y) {
  return cproduct(0, d, bl, 1, x, bl->getn1(), y, bl->getn1());
}
inline bool mltaGeHGeM(scomp d, blcluster* bl, mblock<scomp>**, unsigned p, scomp* X, unsigned ldX, scomp* Y,
                       unsigned ldY) {
  return cproduct(0, d, bl, p, X, ldX, Y, ldY);
}
inline bool mltaGeHhVec(scomp d, blcluster* bl, mblock<scomp>**, scomp* x, scomp* y) {
  return cproduct(1, d, bl, 1, x, bl->getn1(), y, bl->getn1());
}
inline bool mltaGeHhGeM(scomp d, blcluster* bl, mblock<scomp>**, unsigned p, scomp* X, unsigned ldX, scomp* Y,
                        unsigned ldY) {
  return cproduct(1, d, bl, p, X, ldX, Y, ldY);
}
inline bool mltaGeHtVec(scomp d, blcluster* bl, mblock<scomp>**, scomp* x, scomp* y) {
  return cproduct(2, d, bl, 1, x, bl->getn1(), y, bl->getn1());
}
inline bool mltaGeHtGeM(scomp d, blcluster* bl, mblock<scomp>**, unsigned p, scomp* X, unsigned ldX, scomp* Y,
                        unsigned ldY) {
  return cproduct(2, d, bl, p, X, ldX, Y, ldY);
}

// Include/matrix.h:20-32
template <class T>
struct Matrix {
  unsigned m, n;
  Matrix(unsigned n1, unsigned n2) : m(n1), n(n2) {}
  Matrix() : m(0), n(0) {}
  virtual void amux(T d, T* x, T* y) const = 0;
  virtual void atmux(T d, T* x, T* y) const { amux(d, x, y); }
  virtual void precond_apply(T*) const {}
  virtual ~Matrix() {}
};

// The H-matrix as a Matrix<double>: GMRes/CG on it run on the GPU.
struct HMatrixOperator : public Matrix<double> {
  blcluster* bl;
  explicit HMatrixOperator(blcluster* b) : Matrix<double>(b->getn1(), b->getn1()), bl(b) {}
  void amux(double d, double* x, double* y) const override { mltaGeHVec(d, bl, nullptr, x, y); }
  void atmux(double d, double* x, double* y) const override { mltaGeHhVec(d, bl, nullptr, x, y); }
};

// Include/matrix.h:50-75: sqrt of the largest eigenvalue of A^H A by it_num power steps;
// on the GPU for the H-matrix operator, else with the operator's own amux / atmux
template <class T>
double spctrlnrm(Matrix<T>& A, const unsigned it_num = 10) {
  if (HMatrixOperator* h = dynamic_cast<HMatrixOperator*>(&A)) {
    double v = 0.0;
    check(ahx_spctrlnrm(h->bl->handle(), it_num, &v));
    return v;
  }
  std::vector<T> x(A.n, (T)1), y(A.m);
  double d = 0.0;
  for (unsigned i = 0; i < it_num; ++i) {
    std::fill(y.begin(), y.end(), (T)0);
    A.amux((T)1, x.data(), y.data());
    std::fill(x.begin(), x.end(), (T)0);
    A.atmux((T)1, y.data(), x.data());
    d = 0.0;
    for (const T& v : x) d += (double)(v * v);
    d = std::sqrt(d);
    for (T& v : x) v = (T)(v / d);
  }
  return std::sqrt(d);
}

// The solvers run on the GPU for the library's operators only: the overloads
// below take HMatrixOperator / ZHMatrixOperator, and this template (an exact
// match for every other type, preferred over a derived-to-base conversion) is
// deleted, so GMRes / CG on a program's own Matrix<T> do not compile.
template <class M, class T>
unsigned GMRes(const M& A, T* const b, T* const x, double& eps, const unsigned m, unsigned& nsteps) = delete;
template <class M, class T>
unsigned CG(const M& A, T* const b, T* const x, double& eps, unsigned& nsteps) = delete;

// solvers/GMRES.cpp:80: returns 0 converged, 1 not; eps and nsteps updated
inline unsigned GMRes(const HMatrixOperator& A, double* const b, double* const x, double& eps,
                      const unsigned m, unsigned& nsteps) {
  const HMatrixOperator* H = &A;
  uint32_t its = 0;
  double res = 0.0;
  const int rc = ahx_gmres(H->bl->handle(), AHX_FP64, 1, b, A.n, x, A.n, eps, m, nsteps, &its, &res);
  check(rc);
  eps = res;
  nsteps = its;
  return rc == AHX_OK ? 0u : 1u;
}

// The Helmholtz H-matrix as a Matrix<dcomp> (complex symmetric: A^T = A)
struct ZHMatrixOperator : public Matrix<dcomp> {
  blcluster* bl;
  explicit ZHMatrixOperator(blcluster* b) : Matrix<dcomp>(b->getn1(), b->getn1()), bl(b) {}
  void amux(dcomp d, dcomp* x, dcomp* y) const override { mltaGeHVec(d, bl, nullptr, x, y); }
  void atmux(dcomp d, dcomp* x, dcomp* y) const override { mltaGeHtVec(d, bl, nullptr, x, y); }
};

// solvers/GMRES.cpp:246: complex GMRes
inline unsigned GMRes(const ZHMatrixOperator& A, dcomp* const b, dcomp* const x, double& eps, const unsigned m,
                      unsigned& nsteps) {
  const ZHMatrixOperator* H = &A;
  uint32_t its = 0;
  double res = 0.0;
  const int rc = ahx_helm_gmres(H->bl->handle(), AHX_FP64, 1, reinterpret_cast<const double*>(b), A.n,
                                reinterpret_cast<double*>(x), A.n, eps, m, nsteps, &its, &res);
  check(rc);
  eps = res;
  nsteps = its;
  return rc == AHX_OK ? 0u : 1u;
}

// solvers/CG.cpp:31
inline unsigned CG(const HMatrixOperator& A, double* const b, double* const x, double& eps,
                   unsigned& nsteps) {
  const HMatrixOperator* H = &A;
  uint32_t its = 0;
  double res = 0.0;
  const int rc = ahx_cg(H->bl->handle(), 1, b, A.n, x, A.n, eps, nsteps, &its, &res);
  check(rc);
  eps = res;
  nsteps = its;
  return rc == AHX_OK ? 0u : 1u;
}

}  // namespace ahx_ahmed

#endif  // AHX_AHMED_HPP
