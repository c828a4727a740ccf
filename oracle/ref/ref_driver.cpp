// Driver over the reference library's own hot-path code (AHMED 1.0), built only
// where the reference sources are present.  It is test infrastructure: it
// produces golden vectors from the unmodified reference templates and library
// objects, and is never part of the shipped library.
//
// Entry points used (all from the reference, called unchanged):
//   cluster3d_bbx::createClusterTree   Include/cluster_bbx.h:100-128
//   bemcluster / cluster_pca tree      Include/bemcluster.h:25-50, Include/cluster_pca.h:204-217
//   blcluster::subdivide               Include/blcluster.h:382-387, cluster/blcluster.cpp:40-66
//   gen_BlSequence                     parallel/gen_blseq.cpp:68-75
//   matgenGeH_omp / apprx_unsym        Include/matgen_omp.h:197-213, Include/apprx.h:136-172
//   ::ACA + mblock::cpyLrM_cmpr        Include/ACA.h:217-350, Include/mblock.h:822-826
//   mltaGeHVec / mltaGeHGeM            H/mltaGeHVec.cpp:567-577
//   GMRes / CG                         solvers/GMRES.cpp:80-181, solvers/CG.cpp:31-113
//   savembls                           Include/H.h:89-103, Include/mblock.h:737-773
//   subdivide_sym / matgenHeH_omp / ACAr / mltaHeHVec  cluster/blcluster.cpp:90-113,
//     Include/matgen_omp.h:96-101, Include/apprx.h:86-132, Include/ACA.h:579-720,
//     H/mltaGeHVec.cpp:421-475
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <sstream>
#include <vector>
#include "bemblcluster.h"
#include "cluster_bbx.h"
#include "apprx.h"
#include "matgen_omp.h"
#include "H.h"
#include "matrix.h"
#include "solvers.h"
#include "bllist.h"

struct Pt {
  double c[3];
  double getcenter(unsigned j) const { return c[j]; }
  double getradius2() const { return 0.0; }
};

// Laplace single-layer collocation generator: K(x,y) = 1/(4 pi |x-y|) and
// 1/(4 pi h) on the diagonal; rows/columns in permuted (cluster) order.
struct LaplaceGen {
  const Pt* dofs;
  const unsigned* op_perm;
  double h;
  double entry(unsigned i, unsigned j) const {
    const unsigned a = op_perm[i], b = op_perm[j];
    if (a == b) return 1.0 / (4.0 * M_PI * h);
    const double dx = dofs[a].c[0] - dofs[b].c[0];
    const double dy = dofs[a].c[1] - dofs[b].c[1];
    const double dz = dofs[a].c[2] - dofs[b].c[2];
    const double r2 = dx * dx + dy * dy + dz * dz;
    return 1.0 / (4.0 * M_PI * sqrt(r2));
  }
  void cmpbl(unsigned b1, unsigned n1, unsigned b2, unsigned n2, double* data) const {
    for (unsigned j = 0; j < n2; ++j)
      for (unsigned i = 0; i < n1; ++i) data[i + j * n1] = entry(b1 + i, b2 + j);
  }
  double scale(unsigned b1, unsigned, unsigned b2, unsigned) const {
    return fabs(entry(b1, b2));
  }
  // packed upper triangle of the diagonal block, column by column (blas::hemva "U")
  void cmpblsym(unsigned b1, unsigned n1, double* data) const {
    for (unsigned j = 0; j < n1; ++j)
      for (unsigned i = 0; i <= j; ++i) data[i + j * (j + 1) / 2] = entry(b1 + i, b1 + j);
  }
};

// Helmholtz single-layer collocation generator (complex): exp(i k r) / (4 pi r),
// exp(i k h) / (4 pi h) on the diagonal.
struct HelmGen {
  const Pt* dofs;
  const unsigned* op_perm;
  double h, k;
  dcomp entry(unsigned i, unsigned j) const {
    const unsigned a = op_perm[i], b = op_perm[j];
    double r = h;
    if (a != b) {
      const double dx = dofs[a].c[0] - dofs[b].c[0];
      const double dy = dofs[a].c[1] - dofs[b].c[1];
      const double dz = dofs[a].c[2] - dofs[b].c[2];
      r = sqrt(dx * dx + dy * dy + dz * dz);
    }
    const double s = 1.0 / (4.0 * M_PI * r);
    return dcomp(cos(k * r) * s, sin(k * r) * s);
  }
  void cmpbl(unsigned b1, unsigned n1, unsigned b2, unsigned n2, dcomp* data) const {
    for (unsigned j = 0; j < n2; ++j)
      for (unsigned i = 0; i < n1; ++i) data[i + j * n1] = entry(b1 + i, b2 + j);
  }
  double scale(unsigned b1, unsigned, unsigned b2, unsigned) const { return abs(entry(b1, b2)); }
  // packed upper triangle of a diagonal block, column by column (symva "U")
  void cmpblsym(unsigned b1, unsigned n1, dcomp* data) const {
    for (unsigned j = 0; j < n1; ++j)
      for (unsigned i = 0; i <= j; ++i) data[i + j * (j + 1) / 2] = entry(b1 + i, b1 + j);
  }
};

struct RefH {
  unsigned n = 0, kind = 0;
  std::vector<Pt> dofs;
  std::vector<unsigned> op_perm, po_perm;
  cluster* root_cl = nullptr;
  blcluster* root_bl = nullptr;
  unsigned nblcks = 0;
  std::vector<blcluster*> leaves;
  mblock<double>** A = nullptr;
  LaplaceGen gen;
  bool sym = false;  // symmetric block tree (subdivide_sym), HeH leaves
  mblock<dcomp>** Az = nullptr;  // Helmholtz leaves (mblock<dcomp>)
};

// The Helmholtz H-matrix as the reference's complex GMRes sees it.
struct ZMatrixOp : public Matrix<dcomp> {
  RefH* H;
  explicit ZMatrixOp(RefH* h) : Matrix<dcomp>(h->n, h->n), H(h) {}
  void amux(dcomp d, dcomp* x, dcomp* y) const {
    if (H->sym) mltaSyHVec(d, H->root_bl, H->Az, x, y);
    else mltaGeHVec(d, H->root_bl, H->Az, x, y);
  }
};

struct HMatrixOp : public Matrix<double> {
  RefH* H;
  explicit HMatrixOp(RefH* h) : Matrix<double>(h->n, h->n), H(h) {}
  void amux(double d, double* x, double* y) const {
    if (H->sym) mltaHeHVec(d, H->root_bl, H->A, x, y);
    else mltaGeHVec(d, H->root_bl, H->A, x, y);
  }
};

// apprx_sym (Include/apprx.h:86-132) with the ACA start row 0 of bounding-box trees;
// cmplx_sym: complex symmetric dense diagonal blocks (SyM) instead of Hermitian ones
template <class T, class MATGEN_T>
static void apprx_sym_bbx(MATGEN_T& MatGen, mblock<T>*& mbl, blcluster* bl, double eps,
                          unsigned rankmax, bool cmplx_sym = false) {
  unsigned n1 = bl->getn1(), n2 = bl->getn2();
  unsigned b1 = bl->getb1(), b2 = bl->getb2();
  unsigned maxk = n1 * n2 / (n1 + n2) + 4;
  if (maxk > rankmax) maxk = rankmax;
  mbl = new mblock<T>(n1, n2);
  bool succ = false;
  if (bl->isadm() && maxk) {
    unsigned k;
    T *U, *V;
    succ = ::ACAr(MatGen, b1, n1, b2, n2, eps, maxk, 0u, k, U, V);
    if (succ) mbl->cpyLrM_cmpr(k, U, n1, V, n2, eps, k);
    delete[] V;
    delete[] U;
  }
  if (!succ) {
    if (bl->isdbl()) {
      if (cmplx_sym) mbl->setSyM();
      else mbl->setHeM();
      MatGen.cmpblsym(b1, n1, mbl->getdata());
    } else {
      mbl->setGeM();
      MatGen.cmpbl(b1, n1, b2, n2, mbl->getdata());
    }
  }
}

// ACA start row for bounding-box trees (they carry no centroid index): row 0.
template <class T, class MATGEN_T>
static void apprx_unsym_bbx(MATGEN_T& MatGen, mblock<T>*& mbl, blcluster* bl,
                            double eps, unsigned rankmax) {
  unsigned n1 = bl->getn1(), n2 = bl->getn2();
  unsigned b1 = bl->getb1(), b2 = bl->getb2();
  unsigned maxk = n1 * n2 / (n1 + n2) + 4;
  if (maxk > rankmax) maxk = rankmax;
  mbl = new mblock<T>(n1, n2);
  bool succ = false;
  if (bl->isadm() && maxk) {
    unsigned k;
    T *U, *V;
    succ = ::ACA(MatGen, b1, n1, b2, n2, eps, maxk, 0u, k, U, V);
    if (succ) mbl->cpyLrM_cmpr(k, U, n1, V, n2, eps, k);
    delete[] V;
    delete[] U;
  }
  if (!succ) {
    mbl->setGeM();
    MatGen.cmpbl(b1, n1, b2, n2, mbl->getdata());
  }
}

extern "C" {

// kind 0: cluster3d_bbx tree + blcluster_geo; kind 1: bemcluster (PCA) + bemblcluster;
// sym: the symmetric block tree (blcluster::subdivide_sym, cluster/blcluster.cpp:90-113)
static void* build_impl(const double* pts, unsigned n, int kind, unsigned bmin, double eta2, double h,
                        bool sym) {
  RefH* H = new RefH;
  H->n = n;
  H->kind = kind;
  H->dofs.resize(n);
  for (unsigned i = 0; i < n; ++i)
    for (int j = 0; j < 3; ++j) H->dofs[i].c[j] = pts[3 * i + j];
  H->op_perm.resize(n);
  H->po_perm.resize(n);
  for (unsigned i = 0; i < n; ++i) H->op_perm[i] = H->po_perm[i] = i;
  if (kind == 0) {
    cluster3d_bbx<Pt>* cl = new cluster3d_bbx<Pt>(H->dofs.data(), H->op_perm.data(), 0, n);
    cl->createClusterTree(bmin, H->op_perm.data(), H->po_perm.data());
    H->root_cl = cl;
    blcluster_geo* bl = new blcluster_geo(0, 0, n, n);
    if (sym) bl->subdivide_sym(cl, eta2, H->nblcks);
    else bl->subdivide(cl, cl, eta2, H->nblcks);
    H->root_bl = bl;
  } else {
    bemcluster<Pt>* cl = new bemcluster<Pt>(H->dofs.data(), H->op_perm.data(), 0, n);
    cl->createClusterTree(bmin, H->op_perm.data(), H->po_perm.data());
    H->root_cl = cl;
    bemblcluster<Pt, Pt>* bl = new bemblcluster<Pt, Pt>(0, 0, n, n);
    if (sym) bl->subdivide_sym(cl, eta2, H->nblcks);
    else bl->subdivide(cl, cl, eta2, H->nblcks);
    H->root_bl = bl;
  }
  blcluster** list;
  gen_BlSequence(H->root_bl, list);
  H->leaves.assign(list, list + H->nblcks);
  delete[] list;
  H->gen.dofs = H->dofs.data();
  H->gen.op_perm = H->op_perm.data();
  H->gen.h = h;
  H->sym = sym;
  return H;
}

void* ref_build(const double* pts, unsigned n, int kind, unsigned bmin, double eta2, double h) {
  return build_impl(pts, n, kind, bmin, eta2, h, false);
}

void* ref_build_sym(const double* pts, unsigned n, int kind, unsigned bmin, double eta2, double h) {
  return build_impl(pts, n, kind, bmin, eta2, h, true);
}

unsigned ref_nleaves(void* p) { return ((RefH*)p)->nblcks; }

void ref_perm(void* p, unsigned* op_perm, unsigned* po_perm) {
  RefH* H = (RefH*)p;
  memcpy(op_perm, H->op_perm.data(), H->n * sizeof(unsigned));
  memcpy(po_perm, H->po_perm.data(), H->n * sizeof(unsigned));
}

// per leaf (DFS order): b1, n1, b2, n2, adm, idx, i0 (ACA start row, 0 if inadmissible)
void ref_leaves(void* p, unsigned* out) {
  RefH* H = (RefH*)p;
  for (unsigned l = 0; l < H->nblcks; ++l) {
    blcluster* b = H->leaves[l];
    unsigned* o = out + 7 * l;
    o[0] = b->getb1(); o[1] = b->getn1(); o[2] = b->getb2(); o[3] = b->getn2();
    o[4] = b->isadm(); o[5] = b->getidx(); o[6] = 0;
    if (H->kind == 1 && b->isadm())
      o[6] = ((bemblcluster<Pt, Pt>*)b)->getcl1()->geticom() - b->getb1();
  }
}

void ref_assemble(void* p, double eps, unsigned rankmax, int nthreads) {
  RefH* H = (RefH*)p;
  if (nthreads > 0) omp_set_num_threads(nthreads);
  allocmbls(H->nblcks, H->A);
  std::streambuf* old = std::cout.rdbuf();
  std::ostringstream sink;
  std::cout.rdbuf(sink.rdbuf());   // progressbar output is not wanted
  if (H->sym && H->kind == 1) {
    matgenHeH_omp(H->gen, H->nblcks, (bemblcluster<Pt, Pt>*)H->root_bl, eps, rankmax, H->A);
  } else if (H->sym) {
#pragma omp parallel for schedule(dynamic)
    for (int l = 0; l < (int)H->nblcks; ++l) {
      blcluster* b = H->leaves[l];
      apprx_sym_bbx(H->gen, H->A[b->getidx()], b, eps, rankmax);
    }
  } else if (H->kind == 1) {
    matgenGeH_omp(H->gen, H->nblcks, (bemblcluster<Pt, Pt>*)H->root_bl, eps, rankmax, H->A);
  } else {
#pragma omp parallel for schedule(dynamic)
    for (int l = 0; l < (int)H->nblcks; ++l) {
      blcluster* b = H->leaves[l];
      apprx_unsym_bbx(H->gen, H->A[b->getidx()], b, eps, rankmax);
    }
  }
  std::cout.rdbuf(old);
}

// per leaf: rank (LrM) or -1 (dense GeM)
void ref_ranks(void* p, int* out) {
  RefH* H = (RefH*)p;
  for (unsigned l = 0; l < H->nblcks; ++l) {
    mblock<double>* m = H->A[H->leaves[l]->getidx()];
    out[l] = m->isLrM() ? (int)m->rank() : -1;
  }
}

// copies leaf l's data (LrM: U n1*k then V n2*k; GeM: n1*n2 column-major); returns count
unsigned long ref_leaf_data(void* p, unsigned l, double* out) {
  RefH* H = (RefH*)p;
  blcluster* b = H->leaves[l];
  mblock<double>* m = H->A[b->getidx()];
  unsigned long cnt = m->isLrM() ? (unsigned long)m->rank() * (b->getn1() + b->getn2())
                    : m->isHeM() ? (unsigned long)b->getn1() * (b->getn1() + 1) / 2
                                 : (unsigned long)b->getn1() * b->getn2();
  if (out && cnt) memcpy(out, m->getdata(), cnt * sizeof(double));
  return cnt;
}

// Y += d A X   (p columns, leading dimension n)
void ref_matvec(void* p, double d, unsigned nrhs, double* X, double* Y) {
  RefH* H = (RefH*)p;
  if (H->sym) {
    if (nrhs == 1) mltaHeHVec(d, H->root_bl, H->A, X, Y);
    else mltaHeHGeM(d, H->root_bl, H->A, nrhs, X, H->n, Y, H->n);
  } else if (nrhs == 1) {
    mltaGeHVec(d, H->root_bl, H->A, X, Y);
  } else {
    mltaGeHGeM(d, H->root_bl, H->A, nrhs, X, H->n, Y, H->n);
  }
}

unsigned ref_gmres(void* p, double* b, double* x, double* eps, unsigned m, unsigned* nsteps) {
  RefH* H = (RefH*)p;
  HMatrixOp op(H);
  double e = *eps;
  unsigned ns = *nsteps;
  std::streambuf* old = std::cout.rdbuf();
  std::ostringstream sink;
  std::cout.rdbuf(sink.rdbuf());   // per-step residual prints are not wanted
  unsigned r = GMRes(op, b, x, e, m, ns);
  std::cout.rdbuf(old);
  *eps = e;
  *nsteps = ns;
  return r;
}

unsigned ref_cg(void* p, double* b, double* x, double* eps, unsigned* nsteps) {
  RefH* H = (RefH*)p;
  HMatrixOp op(H);
  double e = *eps;
  unsigned ns = *nsteps;
  std::streambuf* old = std::cout.rdbuf();
  std::ostringstream sink;
  std::cout.rdbuf(sink.rdbuf());
  unsigned r = CG(op, b, x, e, ns);
  std::cout.rdbuf(old);
  *eps = e;
  *nsteps = ns;
  return r;
}

// one generator entry in permuted order (for dense checks)
double ref_entry(void* p, unsigned i, unsigned j) { return ((RefH*)p)->gen.entry(i, j); }

// ACA ranks of the Helmholtz matrix (bounding-box trees: start row 0), the
// reference's complex ::ACA (Include/ACA.h:217-350 with T = dcomp) per
// admissible leaf: out[l] = k on success, -2 when ACA fails, -1 inadmissible.
void ref_helm_ranks(void* p, double wavenumber, double h, double eps, unsigned rankmax, int* out) {
  RefH* H = (RefH*)p;
  HelmGen gen{H->dofs.data(), H->op_perm.data(), h, wavenumber};
#pragma omp parallel for schedule(dynamic, 16)
  for (long l = 0; l < (long)H->nblcks; ++l) {
    blcluster* bl = H->leaves[l];
    out[l] = -1;
    const unsigned n1 = bl->getn1(), n2 = bl->getn2();
    unsigned maxk = n1 * n2 / (n1 + n2) + 4;
    if (maxk > rankmax) maxk = rankmax;
    if (!bl->isadm() || !maxk) continue;
    unsigned k = 0;
    dcomp *U, *V;
    const bool succ = ::ACA(gen, bl->getb1(), n1, bl->getb2(), n2, eps, maxk, 0u, k, U, V);
    delete[] V;
    delete[] U;
    out[l] = succ ? (int)k : -2;
  }
}

// Helmholtz H-matrix: the reference's assembly with T = dcomp (apprx_unsym,
// Include/apprx.h:136-172: ::ACA<dcomp> then mblock<dcomp>::cpyLrM_cmpr ->
// addtrll, H/mblock_Z.cpp:200-300; dense leaves from cmpbl).
void ref_helm_assemble(void* p, double wavenumber, double h, double eps, unsigned rankmax, int nthreads) {
  RefH* H = (RefH*)p;
  if (nthreads > 0) omp_set_num_threads(nthreads);
  if (H->Az) freembls(H->nblcks, H->Az);
  allocmbls(H->nblcks, H->Az);
  HelmGen gen{H->dofs.data(), H->op_perm.data(), h, wavenumber};
  std::streambuf* old = std::cout.rdbuf();
  std::ostringstream sink;
  std::cout.rdbuf(sink.rdbuf());
  if (H->sym && H->kind == 1) {
    matgenSyH_omp(gen, H->nblcks, (bemblcluster<Pt, Pt>*)H->root_bl, eps, rankmax, H->Az);
  } else if (H->sym) {
#pragma omp parallel for schedule(dynamic)
    for (int l = 0; l < (int)H->nblcks; ++l) {
      blcluster* b = H->leaves[l];
      apprx_sym_bbx(gen, H->Az[b->getidx()], b, eps, rankmax, true);
    }
  } else if (H->kind == 1) {
    matgenGeH_omp(gen, H->nblcks, (bemblcluster<Pt, Pt>*)H->root_bl, eps, rankmax, H->Az);
  } else {
#pragma omp parallel for schedule(dynamic)
    for (int l = 0; l < (int)H->nblcks; ++l) {
      blcluster* b = H->leaves[l];
      apprx_unsym_bbx(gen, H->Az[b->getidx()], b, eps, rankmax);
    }
  }
  std::cout.rdbuf(old);
}

// per leaf of the Helmholtz matrix: rank (LrM) or -1 (dense)
void ref_helm_ranks_assembled(void* p, int* out) {
  RefH* H = (RefH*)p;
  for (unsigned l = 0; l < H->nblcks; ++l) {
    mblock<dcomp>* m = H->Az[H->leaves[l]->getidx()];
    out[l] = m->isLrM() ? (int)m->rank() : -1;
  }
}

// complex entries of Helmholtz leaf l (U then V, or the dense block) as
// interleaved (re, im) doubles in out; returns the complex count
unsigned long ref_helm_leaf_data(void* p, unsigned l, double* out) {
  RefH* H = (RefH*)p;
  blcluster* b = H->leaves[l];
  mblock<dcomp>* m = H->Az[b->getidx()];
  unsigned long cnt = m->isLrM() ? (unsigned long)m->rank() * (b->getn1() + b->getn2())
                   : m->isSyM() ? (unsigned long)b->getn1() * (b->getn1() + 1) / 2
                                : (unsigned long)b->getn1() * b->getn2();
  if (out && cnt) memcpy(out, m->getdata(), cnt * sizeof(dcomp));
  return cnt;
}

// Y += d op(A) X, op 0: A (mltaGeHGeM), 1: A^H (mltaGeHhGeM), 2: A^T (mltaGeHtGeM);
// X, Y: n x nrhs complex, interleaved doubles, leading dimension n
void ref_helm_matvec(void* p, int op, double dre, double dim, unsigned nrhs, double* X, double* Y) {
  RefH* H = (RefH*)p;
  const dcomp d(dre, dim);
  dcomp* x = (dcomp*)X;
  dcomp* y = (dcomp*)Y;
  if (H->sym) {  // complex symmetric: A^T = A (mltaSyHVec / mltaSyHGeM, H/mltaGeHVec.cpp:885-895)
    if (op == 1) return;  // the adjoint is not exported for SyH matrices
    if (nrhs == 1) mltaSyHVec(d, H->root_bl, H->Az, x, y);
    else mltaSyHGeM(d, H->root_bl, H->Az, nrhs, x, H->n, y, H->n);
  } else if (op == 1) mltaGeHhGeM(d, H->root_bl, H->Az, nrhs, x, H->n, y, H->n);
  else if (op == 2) mltaGeHtGeM(d, H->root_bl, H->Az, nrhs, x, H->n, y, H->n);
  else if (nrhs == 1) mltaGeHVec(d, H->root_bl, H->Az, x, y);
  else mltaGeHGeM(d, H->root_bl, H->Az, nrhs, x, H->n, y, H->n);
}

// the reference's complex GMRes (solvers/GMRES.cpp:246-366) with the Helmholtz leaves
unsigned ref_helm_gmres(void* p, double* b, double* x, double* eps, unsigned m, unsigned* nsteps) {
  RefH* H = (RefH*)p;
  ZMatrixOp op(H);
  double e = *eps;
  unsigned ns = *nsteps;
  std::streambuf* old = std::cout.rdbuf();
  std::ostringstream sink;
  std::cout.rdbuf(sink.rdbuf());
  unsigned r = GMRes(op, (dcomp*)b, (dcomp*)x, e, m, ns);
  std::cout.rdbuf(old);
  *eps = e;
  *nsteps = ns;
  return r;
}

// The reference's agglH with T = dcomp (H/agglH.cpp:291-305) of the Helmholtz leaves;
// the leaf list is rebuilt in DFS order (indices as agglH left them).
void ref_helm_agglomerate(void* p, double eps, unsigned rankmax) {
  RefH* H = (RefH*)p;
  agglH(H->root_bl, H->Az, eps, rankmax, (contBasis<dcomp>*)NULL);
  blcluster** list;
  H->nblcks = H->root_bl->nleaves();
  gen_BlSequence(H->root_bl, list);
  H->leaves.assign(list, list + H->nblcks);
  delete[] list;
}

// The reference's savembls (Include/H.h:89-103) of the Helmholtz (mblock<dcomp>) leaves
int ref_helm_save(void* p, double eta, unsigned bmin, const char* path) {
  RefH* H = (RefH*)p;
  if (!H->Az) return 1;
  std::ofstream os(path, std::ios::binary);
  if (!os) return 1;
  savembls(eta, bmin, H->root_bl, H->Az, os);
  return os.good() ? 0 : 1;
}

// The reference's agglomeration agglH (H/agglH.cpp:253-272) of the assembled
// leaves; the leaf list is rebuilt in DFS order (indices as agglH left them).
void ref_agglomerate(void* p, double eps, unsigned rankmax) {
  RefH* H = (RefH*)p;
  agglH(H->root_bl, H->A, eps, rankmax, (contBasis<double>*)NULL);
  blcluster** list;
  H->nblcks = H->root_bl->nleaves();
  gen_BlSequence(H->root_bl, list);
  H->leaves.assign(list, list + H->nblcks);
  delete[] list;
}

// The reference's savembls (Include/H.h:89-103, mblock::save Include/mblock.h:737-773)
// of the assembled leaves; returns 0 on success.
int ref_save(void* p, double eta, unsigned bmin, const char* path) {
  RefH* H = (RefH*)p;
  if (!H->A) return 1;
  std::ofstream os(path, std::ios::binary);
  if (!os) return 1;
  savembls(eta, bmin, H->root_bl, H->A, os);
  return os.good() ? 0 : 1;
}

void ref_free(void* p) {
  RefH* H = (RefH*)p;
  if (H->A) freembls(H->nblcks, H->A);
  if (H->Az) freembls(H->nblcks, H->Az);
  delete H->root_bl;
  delete H->root_cl;
  delete H;
}

}  // extern "C"
