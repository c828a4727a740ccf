/* CPU oracle for the AHMED H-matrix hot path (test infrastructure only).
 *
 * A plain-C restatement of the reference algorithms, used by the tests, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline leg as the checker.
 * It is never linked into the shipped library.  Each function cites the
 * reference file:line it follows (paths relative to the AHMED source tree).
 *
 * Pinning: the tree/permutation/leaf outputs are compared bit-for-bit, and
 * the ACA ranks, block errors and products are compared with tolerances,
 * against golden vectors produced by the reference library itself
 * (tests/golden/make_golden.py driving oracle/ref/ref_driver.cpp).
 *
 * Conventions (same as the reference): op_perm[permuted] = original index,
 * po_perm[original] = permuted index; leaf data is column-major; a low-rank
 * leaf stores U (n1 x k) followed by V (n2 x k) and represents U V^T.
 */
#ifndef AHX_ORACLE_H
#define AHX_ORACLE_H
#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { OR_TREE_BBX = 0, OR_TREE_PCA = 1 };

typedef struct or_hmat or_hmat;

/* Build cluster tree + block-cluster tree.  pts: 3*n doubles (original order).
 * eta2 is the squared admissibility parameter (callers pass eta*eta). */
or_hmat* or_build(const double* pts, uint32_t n, int kind, uint32_t bmin, double eta2);
void or_free(or_hmat* H);
uint32_t or_nleaves(const or_hmat* H);
void or_perm(const or_hmat* H, uint32_t* op_perm, uint32_t* po_perm);
/* 7 words per leaf in DFS order: b1, n1, b2, n2, adm, idx, i0 */
void or_leaves(const or_hmat* H, uint32_t* out);

/* Mean nearest-neighbour distance of the points (exact, grid search). */
double or_mean_nn(const double* pts, uint32_t n);

/* Laplace collocation entry in permuted order: 1/(4 pi |x_i - x_j|), diag 1/(4 pi h). */
double or_entry(const or_hmat* H, double h, uint32_t i, uint32_t j);

/* Assemble all leaves (ACA + recompression, dense fallback).  nthreads<=0: all. */
void or_assemble(or_hmat* H, double h, double eps, uint32_t rankmax, int nthreads);
/* Same, restricted to leaves [l0, l1) of the DFS list (bounded CPU samples). */
void or_assemble_range(or_hmat* H, double h, double eps, uint32_t rankmax, int nthreads,
                       uint32_t l0, uint32_t l1);
/* rank per leaf, -1 for dense leaves */
void or_ranks(const or_hmat* H, int32_t* out);
/* ACA rank before recompression per leaf (-1 dense / failed) */
void or_aca_ranks(const or_hmat* H, int32_t* out);
uint64_t or_leaf_data(const or_hmat* H, uint32_t l, double* out);
/* Replace leaf l's data: rank>=0 low rank (U then V), rank<0 dense. */
void or_set_leaf(or_hmat* H, uint32_t l, int32_t rank, const double* data);

/* Y += d A X, X/Y column-major n x p with leading dimension n. nthreads<=0: all */
void or_matvec(const or_hmat* H, double d, uint32_t p, const double* X, double* Y, int nthreads);

/* ---- CPU baseline of bounded samples (bench.py's reference arm) ---------- */
/* Fortran BLAS dgemm_/dgemv_ supplied by the caller (e.g. the OpenBLAS that
 * scipy bundles), used by or_matvec_layers as the reference uses BLAS in
 * mltaLrMGeM_/mltaGeMGeM (H/mblock.cpp:141-154, Include/mblock.h:105-109).
 * NULL: plain C loops. */
void or_set_blas(void* dgemm, void* dgemv);
/* Assemble the listed leaves only (apprx_unsym per leaf, OpenMP dynamic). */
void or_assemble_list(or_hmat* H, double h, double eps, uint32_t rankmax, int nthreads,
                      const uint32_t* leaves, uint32_t count);
/* Y += d A_S X over a set S of assembled leaves, X/Y column-major with leading
 * dimensions ldX/ldY.  S is given as groups of leaves that share one row
 * cluster (leaves[group_start[g] .. group_start[g+1]-1]), and the groups as
 * layers (groups layer_start[q] .. layer_start[q+1]-1) whose row clusters are
 * pairwise disjoint: the threads share the groups of one layer, so no two
 * threads write the same rows and no private accumulators are needed.  Per
 * leaf, mltaGeM_ (H/mblock.cpp:141-154, 225-238): low rank T = V^T X then
 * Y += d U T; dense Y += d A X (p = 1: the vector forms scpr/axpy and gemv). */
void or_matvec_layers(const or_hmat* H, double d, uint32_t p, const double* X, uint64_t ldX, double* Y,
                      uint64_t ldY, int nthreads, const uint32_t* leaves, const uint32_t* group_start,
                      uint32_t ngroups, const uint32_t* layer_start, uint32_t nlayers);

/* GMRES(m) and CG as the reference solvers (return 0 converged, 1 not). */
uint32_t or_gmres(const or_hmat* H, const double* b, double* x, double* eps, uint32_t m,
                  uint32_t* nsteps, int nthreads);
uint32_t or_cg(const or_hmat* H, const double* b, double* x, double* eps, uint32_t* nsteps,
               int nthreads);

/* Single-block ACA (ACA.h:217-350) on the Laplace generator; returns success.
 * U, V must hold (kmax+1)*n1 and (kmax+1)*n2 doubles. */
int or_aca_block(const or_hmat* H, double h, uint32_t b1, uint32_t n1, uint32_t b2, uint32_t n2,
                 double eps, uint32_t kmax, uint32_t i0, uint32_t* k, double* U, double* V);
/* addtrll recompression (mblock_D.cpp:356-465) of U (n1 x k), V (n2 x k) in place;
 * returns the new rank kt; results in U[:, :kt], V[:, :kt]. */
uint32_t or_recompress(uint32_t n1, uint32_t n2, uint32_t k, double* U, double* V,
                       double delta, uint32_t kgoal);

#ifdef __cplusplus
}
#endif
#endif
