/* ahx -- GB300-native H-matrix hot path (ACA assembly, H-matvec, GMRES/CG).
 *
 * C ABI of libahx.so.  Plain pointers and sizes only.  Every function returns
 * an int status (AHX_OK on success) and never aborts; ahx_last_error() gives
 * the message of the last failure on the calling thread.  Vectors are in the
 * permuted (cluster) ordering, exactly as the reference's products expect
 * them; ahx_hmat_perm() gives the permutation.
 *
 * Each entry point names the reference interface (AHMED 1.0, paths relative
 * to its source tree) that it replaces on the GPU.
 */
#ifndef AHX_H
#define AHX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define AHX_OK 0
#define AHX_ERR_ARG 1      /* invalid argument / size */
#define AHX_ERR_CUDA 2     /* CUDA runtime error (message in ahx_last_error) */
#define AHX_ERR_STATE 3    /* call order (e.g. product before assembly) */
#define AHX_ERR_NOMEM 4    /* device allocation failed */
#define AHX_NOT_CONVERGED 5 /* solver stopped at its iteration limit */

/* cluster-tree kinds */
#define AHX_TREE_BBX 0 /* bounding-box bisection: Include/cluster_bbx.h:24-133 (cluster3d_bbx) */
#define AHX_TREE_PCA 1 /* PCA bisection + centroid ACA start: Include/bemcluster.h:16-59 */

/* storage precisions of the product */
#define AHX_FP64 0      /* plain form: FP64 leaves (mblock<double>) */
#define AHX_FP32 1      /* all leaves FP32, FP32 accumulation */
#define AHX_BF16_FP32 2 /* low-rank factors BF16, dense leaves FP32, FP32 accumulation */
#define AHX_DF64 3      /* FP64 leaves as float pairs, double-float arithmetic on the FP32
                           pipes (about 2^-44 relative; FP64-class): the refinement's outer
                           residual from two right-hand sides per system on (one: the FP64
                           product; AHX_REFINE_RESIDUAL=fp64 / df64 forces either) */

typedef struct ahx_hmat ahx_hmat;
typedef struct ahx_batch ahx_batch;

const char* ahx_last_error(void);
int ahx_version(void);

/* Mean nearest-neighbour distance h of a point cloud (3*n doubles, xyz). */
double ahx_mean_nn(const double* pts, uint32_t n);
/* Smallest nearest-neighbour distance of the points (the diagonal 1/(4 pi h)
 * with this h makes the Laplace matrix of a random point cloud positive
 * definite enough for GMRES; the mean spacing leaves it indefinite). */
double ahx_min_nn(const double* pts, uint32_t n);
/* Product kernels launched by this process so far (plain and mixed forms). */
uint64_t ahx_kernel_launches(void);

/* Cluster tree + block-cluster tree.  Replaces
 *   cluster3d_bbx / bemcluster ctor + createClusterTree  Include/cluster_bbx.h:100,
 *                                                         Include/cluster_pca.h:204
 *   blcluster::subdivide(cl1, cl2, eta2, nblcks)          Include/blcluster.h:382
 *   gen_BlSequence                                        parallel/gen_blseq.cpp:68
 * pts: 3*n doubles in the original order; eta2 = eta*eta as the reference
 * callers pass it.  device: CUDA device ordinal; stream: cudaStream_t or NULL
 * (a private stream is created). */
int ahx_hmat_create(const double* pts, uint32_t n, int tree_kind, uint32_t bmin, double eta2,
                    int device, void* stream, ahx_hmat** out);
/* The same trees with the symmetric block tree: diagonal and upper blocks only
 * (blcluster::subdivide_sym, cluster/blcluster.cpp:90-113).  Its assembly is
 * matgenHeH_omp (Include/matgen_omp.h:96-101: ACAr for admissible blocks,
 * Include/ACA.h:657-720; Hermitian dense diagonal blocks, Include/apprx.h:86-132)
 * and its products are mltaHeHVec / mltaHeHGeM (H/mltaGeHVec.cpp:421-475:
 * upper blocks applied as A and A^T).  ahx_hmat_get_leaf returns the packed
 * upper triangle of a dense diagonal leaf (mblock HeM data); ahx_hmat_set_leaves
 * takes it packed or full.  Symmetric handles are not batched. */
int ahx_hmat_create_sym(const double* pts, uint32_t n, int tree_kind, uint32_t bmin, double eta2,
                        int device, void* stream, ahx_hmat** out);
/* 1 for a symmetric handle, else 0 */
int ahx_hmat_symmetric(const ahx_hmat* H);
int ahx_hmat_destroy(ahx_hmat* H);
int ahx_hmat_set_stream(ahx_hmat* H, void* stream);
void* ahx_hmat_stream(const ahx_hmat* H);
uint32_t ahx_hmat_n(const ahx_hmat* H);
uint32_t ahx_hmat_nleaves(const ahx_hmat* H);
/* op_perm[permuted] = original, po_perm[original] = permuted (either may be NULL) */
int ahx_hmat_perm(const ahx_hmat* H, uint32_t* op_perm, uint32_t* po_perm);
/* 7 words per leaf in DFS (idx) order: b1, n1, b2, n2, adm, idx, i0 */
int ahx_hmat_leaves(const ahx_hmat* H, uint32_t* out);

/* ACA assembly of all leaves with the Laplace collocation generator
 * K(x,y) = 1/(4 pi |x-y|), diagonal 1/(4 pi h); replaces
 *   matgenGeH_omp(MatGen, nblcks, bl, eps, rankmax, A)  Include/matgen_omp.h:197-213
 *   matgenGeH_sqntl(..., recmpr = false, ...)           Include/matgen_sqntl.h:88-102
 *   apprx_unsym / ::ACA / mblock::cpyLrM_cmpr           Include/apprx.h:136-172
 * The assembled leaves live on the device in FP64. */
int ahx_assemble(ahx_hmat* H, double h, double eps, uint32_t rankmax);
/* Assembly with a rank hint per leaf (e.g. from the learned predictor below;
 * NULL or a negative entry: no hint).  The hint only sizes each leaf's ACA
 * workspace and orders the work; ACA with its own stopping rule decides every
 * rank, so the result is the same as ahx_assemble's. */
int ahx_assemble_hinted(ahx_hmat* H, double h, double eps, uint32_t rankmax,
                        const float* rank_hint);
/* {largest ACA workspace batch in bytes, leaves re-run with a larger rank
 * capacity, workspace batches} of the last assembly */
int ahx_hmat_assembly_stats(const ahx_hmat* H, uint64_t* out3);
/* 8 geometric features per leaf (DFS order) for the rank predictor:
 * log diam1, log diam2, log centre distance, min diam / distance, log n1,
 * log n2, wavenumber * max diam, -log10(eps) (diam: Include/cluster.h:194) */
int ahx_hmat_features(const ahx_hmat* H, double wavenumber, double eps, float* out);

/* Autotuner of the mixed-precision product (AHX_FP32 or AHX_BF16_FP32): times
 * candidate stream bucketings (right-hand-side width the units are sized for,
 * unit byte cap) on p right-hand sides and keeps the fastest for this matrix.
 * out4 (may be NULL): chosen width, chosen unit bytes, best ns per product,
 * candidates timed. */
int ahx_hmat_autotune(ahx_hmat* H, int precision, uint32_t p, uint32_t* out4);

/* Helmholtz exp(i k r) / (4 pi r) (diagonal exp(i k h) / (4 pi h)): complex
 * ACA of every admissible leaf with the reference's ACA<dcomp> stopping rule
 * (Include/ACA.h:217-350), ranks[l] = rank (-1 inadmissible, -2 ACA failed).
 * rank_hint (may be NULL; negative: none) sizes the workspaces as in
 * ahx_assemble_hinted; ahx_hmat_assembly_stats reports the batches.
 * Bounding-box trees (ACA start row 0). */
int ahx_helm_aca_ranks(ahx_hmat* H, double wavenumber, double h, double eps, uint32_t rankmax,
                       const float* rank_hint, int32_t* ranks);
/* Helmholtz H-matrix on the handle's block tree: the same kernel and diagonal,
 * assembled as the reference's mblock<dcomp> leaves.  General tree: apprx_unsym
 * with T = dcomp (Include/apprx.h:136-172: ACA<dcomp> from the leaf's start row
 * i0, recompression mblock<dcomp>::addtrll H/mblock_Z.cpp:200-300, dense leaves
 * from the generator where ACA fails).  Symmetric tree (ahx_hmat_create_sym): the
 * complex symmetric form of matgenSyH_omp (Include/matgen_omp.h:102-107:
 * ACAr<dcomp>, dense diagonal blocks symmetric, mblock SyM) whose products are
 * mltaSyHVec / mltaSyHGeM (H/mltaGeHVec.cpp:490-545, 885-895: upper blocks
 * applied as A and A^T; A^T = A, A^H = conj(A)); ahx_helm_get_leaf gives those
 * diagonal blocks packed (upper triangle by columns).  Independent of the real
 * assembly of the same handle.  Complex vectors are interleaved (re, im)
 * doubles, the layout of dcomp; leading dimensions count complex elements. */
int ahx_helm_assemble(ahx_hmat* H, double wavenumber, double h, double eps, uint32_t rankmax);
/* per leaf: rank after recompression, -1 for dense leaves */
int ahx_helm_ranks(const ahx_hmat* H, int32_t* ranks);
/* complex elements of leaf l (U then V, or the dense block) */
uint64_t ahx_helm_leaf_size(const ahx_hmat* H, uint32_t l);
/* copy leaf l (mblock<dcomp>::getdata() layout) into out (2 * size doubles) */
int ahx_helm_get_leaf(const ahx_hmat* H, uint32_t l, double* out);
/* bytes of the complex leaves: AHX_FP64 complex128, AHX_FP32 complex64 */
uint64_t ahx_helm_storage_bytes(const ahx_hmat* H, int precision);
/* Y += d op(A) X, op 0: A (mltaGeHVec / mltaGeHGeM with T = dcomp,
 * H/mltaGeHVec.cpp:770-780), 1: A^H (mltaGeHhVec / mltaGeHhGeM, :782-792),
 * 2: A^T (mltaGeHtVec / mltaGeHtGeM, :794-805); d = d_re + i d_im.  precision
 * AHX_FP64: complex128 leaves; AHX_FP32: complex64 leaves, FP32 accumulation
 * (the reference's scomp instantiation).  X, Y: n x p complex, host or device. */
int ahx_helm_matvec(ahx_hmat* H, int precision, int op, double d_re, double d_im, uint32_t p, const double* X,
                    uint64_t ldX, double* Y, uint64_t ldY);
/* Restarted complex GMRES(m) per right-hand side: GMRes(const Matrix<dcomp>&, b,
 * x, eps, m, nsteps) solvers/GMRES.cpp:246-366 (tol, maxit, iters and resid as in
 * ahx_gmres).  AHX_FP32: FP64 iterative refinement around complex64 inner solves.
 * B, X: n x p complex, host or device; X holds the initial guess. */
int ahx_helm_gmres(ahx_hmat* H, int precision, uint32_t p, const double* B, uint64_t ldB, double* X, uint64_t ldX,
                   double tol, uint32_t m, uint32_t maxit, uint32_t* iters, double* resid);
/* Agglomeration (agglH, H/agglH.cpp:111-272; the recmpr branch of matgenGeH_sqntl,
 * Include/matgen_sqntl.h:32-55): bottom up, a non-diagonal block whose sons are all
 * leaves becomes one low-rank leaf when the recompressed union (relative threshold
 * eps, rank <= max_rank; unify_sons_, H/agglH.cpp:14-107) stores no more; leaf
 * indices are then compacted as fill_gaps does.  As in the reference, the two
 * sons of each block row are united first and truncated, then the two block
 * rows.  Dense sons enter the unions in factored form (D times the identity).
 * Once per assembly.  nmerged (may be NULL): blocks merged. */
int ahx_agglomerate(ahx_hmat* H, double eps, uint32_t max_rank, uint32_t* nmerged);
/* The same for the Helmholtz leaves (agglH with T = dcomp, H/agglH.cpp:291-305).
 * Agglomeration changes the block tree: the handle's other kind of leaves (real
 * after this call, Helmholtz after ahx_agglomerate) is dropped and must be
 * assembled again on the new leaves if needed. */
int ahx_helm_agglomerate(ahx_hmat* H, double eps, uint32_t max_rank, uint32_t* nmerged);
/* per leaf: rank after recompression, -1 for dense leaves (mblock::isLrM/rank) */
int ahx_hmat_ranks(const ahx_hmat* H, int32_t* ranks);
/* per leaf: ACA rank before recompression, -1 for dense */
int ahx_hmat_aca_ranks(const ahx_hmat* H, int32_t* ranks);
/* number of doubles of leaf l (mblock data: U then V, or the dense block) */
uint64_t ahx_hmat_leaf_size(const ahx_hmat* H, uint32_t l);
/* copy leaf l into out (mblock<double>::getdata() layout) */
int ahx_hmat_get_leaf(const ahx_hmat* H, uint32_t l, double* out);
/* upload a whole leaf set (e.g. from host mblock<double>** A): ranks[l] (-1 dense),
 * data = concatenation in leaf order, offsets[l] = start of leaf l in data (nleaves+1). */
int ahx_hmat_set_leaves(ahx_hmat* H, const int32_t* ranks, const double* data,
                        const uint64_t* offsets);
/* bytes of the leaf arena used by the product at a precision */
uint64_t ahx_hmat_storage_bytes(ahx_hmat* H, int precision);
/* prepare the product copy at a precision (done lazily by the product otherwise) */
int ahx_hmat_prepare(ahx_hmat* H, int precision);
/* free the product copy of a precision (AHX_FP32, AHX_BF16, AHX_DF64; the FP64
 * leaves stay); the next product at that precision prepares it again.  No
 * reference counterpart: freembls (Include/H.h:34-45) frees the leaves themselves. */
int ahx_hmat_release(ahx_hmat* H, int precision);
/* bytes of the FP32 tcgen05 product streams (leaf images, chunk heads, padding) */
int ahx_hmat_stream_bytes(ahx_hmat* H, int precision, uint64_t* out);
/* CUDA-event timing of the product sweeps (measurement instrumentation, no
 * reference counterpart): enable != 0 records events around every launch of the
 * FP32 tensor-core sweeps; ahx_timing_read returns per kind (0 = V sweep,
 * 1 = rows sweep) the summed milliseconds and launch counts (it synchronises),
 * and forgets them when reset != 0. */
int ahx_timing(int enable);
int ahx_timing_read(double* ms2, uint64_t* count2, int reset);

/* Y += d A X for p right-hand sides, column-major with leading dimensions ldX, ldY.
 * X and Y may be host or device pointers (host data are staged through the
 * device; pinned host memory is copied asynchronously).  Replaces
 *   mltaGeHVec(d, bl, A, x, y)                     H/mltaGeHVec.cpp:567-571 (p == 1)
 *   mltaGeHGeM(d, bl, A, p, X, ldX, Y, ldY)        H/mltaGeHVec.cpp:573-577 */
int ahx_matvec(ahx_hmat* H, int precision, double d, uint32_t p, const double* X, uint64_t ldX,
               double* Y, uint64_t ldY);
/* Y += d A^T X with the FP64 leaves (mltaGeHtVec / mltaGeHtGeM, and for real
 * leaves mltaGeHhVec / mltaGeHhGeM: H/mltaGeHVec.cpp:62-150).  X, Y: n x p,
 * column-major, host or device. */
int ahx_matvec_transposed(ahx_hmat* H, double d, uint32_t p, const double* X, uint64_t ldX, double* Y,
                          uint64_t ldY);

/* Persistent leaves in the reference's file layout (native byte order):
 *   double eta, uint32 bmin, uint32 nleaves; per leaf in leaf order uint8 present,
 *   then uint32 n1, n2, status and status 0: uint32 rank + rank*(n1+n2) doubles (U, V),
 *   status 4: n1*n2 doubles column-major (1 / 5: packed upper triangle, load only).
 * Replaces savembls  Include/H.h:76-103 with mblock::save Include/mblock.h:737-773
 *          loadmbls  Include/H.h:47-74  with mblock::load Include/mblock.h:775-806.
 * eta and bmin are stored for the caller (the reference stores what it is given).
 * Loading needs the handle of the same tree (points, kind, bmin, eta): every
 * leaf's n1 x n2 is checked; a block marked absent loads as a zero block; on
 * failure the handle is left unassembled.  ahx_mbls_header reads eta, bmin and
 * the leaf count (host only) so the tree can be built first. */
typedef int64_t (*ahx_io_fn)(void* ctx, void* buf, uint64_t bytes); /* bytes moved, <0 error */
int ahx_mbls_header(const char* path, double* eta, uint32_t* bmin, uint32_t* nleaves);
int ahx_hmat_save(ahx_hmat* H, double eta, uint32_t bmin, const char* path);
int ahx_hmat_load(ahx_hmat* H, const char* path, double* eta, uint32_t* bmin);
int ahx_hmat_save_stream(ahx_hmat* H, double eta, uint32_t bmin, ahx_io_fn write, void* ctx);
int ahx_hmat_load_stream(ahx_hmat* H, ahx_io_fn read, void* ctx, double* eta, uint32_t* bmin);
/* The same for the Helmholtz leaves (savembls / loadmbls of mblock<dcomp>: every
 * element two doubles, re and im; a symmetric tree's dense diagonal blocks are
 * written packed with status 5, SyM).  Loading fills the handle's Helmholtz
 * leaves; packed status-1 records load as Hermitian blocks, status 5 as symmetric. */
int ahx_helm_save(ahx_hmat* H, double eta, uint32_t bmin, const char* path);
int ahx_helm_load(ahx_hmat* H, const char* path, double* eta, uint32_t* bmin);
int ahx_helm_save_stream(ahx_hmat* H, double eta, uint32_t bmin, ahx_io_fn write, void* ctx);
int ahx_helm_load_stream(ahx_hmat* H, ahx_io_fn read, void* ctx, double* eta, uint32_t* bmin);

/* Restarted GMRES(m) for p right-hand sides (each with its own Krylov space),
 * right-preconditioner free.  Replaces GMRes(A, b, x, eps, m, nsteps)
 * solvers/GMRES.cpp:80-181.  B, X column-major n x p (host or device), X holds
 * the initial guess.  tol: relative residual target; maxit: iteration limit
 * (the reference's nsteps on input).  precision: storage of the inner
 * product; with AHX_FP32 or AHX_BF16_FP32 the solve is wrapped in FP64
 * iterative refinement (residual and orthogonalisation in FP64 with the FP64
 * leaves).  iters[p], resid[p] (may be NULL) receive per-RHS iteration counts
 * and final relative residuals (the reference's nsteps and eps on output).
 * Returns AHX_OK if every RHS converged, AHX_NOT_CONVERGED otherwise. */
int ahx_gmres(ahx_hmat* H, int precision, uint32_t p, const double* B, uint64_t ldB, double* X,
              uint64_t ldX, double tol, uint32_t m, uint32_t maxit, uint32_t* iters,
              double* resid);

/* Spectral norm sqrt(lambda_max(A^T A)) by it_num power steps from x = 1 with the
 * FP64 leaves; replaces spctrlnrm(A, it_num) Include/matrix.h:50-75. */
int ahx_spctrlnrm(ahx_hmat* H, uint32_t it_num, double* out);

/* Conjugate gradients for p right-hand sides; replaces CG(A, b, x, eps, nsteps)
 * solvers/CG.cpp:31-113 (FP64 product). */
int ahx_cg(ahx_hmat* H, uint32_t p, const double* B, uint64_t ldB, double* X, uint64_t ldX,
           double tol, uint32_t maxit, uint32_t* iters, double* resid);

/* Many independent H-matrices of uneven size as one product: all leaves of all
 * instances run in one launch per product.  Vectors are the concatenation of
 * the instances' vectors (instance i at offset sum_{j<i} n_j), p columns with
 * leading dimension = total length.  The instances must be assembled. */
int ahx_batch_create(ahx_hmat* const* mats, uint32_t count, int precision, ahx_batch** out);
int ahx_batch_destroy(ahx_batch* b);
uint64_t ahx_batch_n(const ahx_batch* b);
int ahx_batch_matvec(ahx_batch* b, double d, uint32_t p, const double* X, double* Y);
/* builds the batch's product copy of a precision ahead of use (e.g. AHX_DF64, the
 * refinement's outer residual, before a timed or captured solve) */
int ahx_batch_prepare(ahx_batch* b, int precision);
/* batched GMRES(m): one right-hand side per instance (b: concatenated), FP64
 * refinement around the batch's storage precision; iters/resid per instance. */
int ahx_batch_gmres(ahx_batch* b, const double* B, double* X, double tol, uint32_t m,
                    uint32_t maxit, uint32_t* iters, double* resid);

/* Learned ACA-rank predictor: an 8 -> 64 -> 64 -> 1 ReLU network trained on
 * the GPU by the library's own forward / backward / Adam kernels; the target
 * is log(1 + ACA rank).  New component of this library (the reference sizes
 * every ACA by its maxk, Include/apprx.h:143). */
typedef struct ahx_mlp ahx_mlp;
uint32_t ahx_mlp_nparams(void);
int ahx_mlp_create(int device, uint64_t seed, ahx_mlp** out);
int ahx_mlp_destroy(ahx_mlp* M);
int ahx_mlp_get_params(const ahx_mlp* M, float* out);
int ahx_mlp_set_params(ahx_mlp* M, const float* in);
int ahx_mlp_set_norm(ahx_mlp* M, const float* mean8, const float* std8);
/* gradient of the mean squared error over n samples (host X n x 8, Y n) */
int ahx_mlp_gradients(ahx_mlp* M, const float* X, const float* Y, uint32_t n, float* grad,
                      float* loss);
int ahx_mlp_train(ahx_mlp* M, const float* X, const float* Y, uint32_t n, uint32_t epochs,
                  uint32_t batch, float lr, uint64_t seed, float* loss_per_epoch);
int ahx_mlp_predict(ahx_mlp* M, const float* X, uint32_t n, float* out);

/* ACA + recompression of ONE admissible block without allocating device
 * memory.  This entry point has no counterpart in the reference.  It is for
 * callers that cannot call cudaMalloc: code running while a framework's
 * caching allocator holds the device memory, paths that cannot afford the
 * device synchronisation of cudaMalloc/cudaFree, and hosts that own every
 * device allocation and only lend buffers.  The scratch comes from a fixed
 * 8 MiB array inside the library (present on every GPU that loads it, until
 * exit); with c = kmax + 1 ACA columns (the reference's capacity) a block needs
 * 256 + 8*(2*(n1+n2)*c + 2*c^2 + 3*c) + 4*(n1+n2) bytes; larger requests, and
 * n1 or n2 above 2^20 or kmax above 2^16, return AHX_ERR_ARG.
 * Inputs (device): px/py/pz = point coordinates in permuted order; the block
 * is rows b1..b1+n1-1, columns b2..b2+n2-1, ACA start row i0 (< n1), kernel
 * diagonal 1/(4 pi h), accuracy eps, at most kmax ACA steps (the reference's
 * maxk).  Outputs (device): U (n1*kmax doubles) and V (n2*kmax) receive the
 * recompressed factors (kt columns, mblock layout), info[3] = {status
 * (1 = low rank, 0 = ACA failed: fill the block densely), ACA rank, kt}.
 * The kernel is queued on `stream` (NULL = default stream); the call does not
 * wait for it.  The first call on a device (and the first after its context was
 * created again, e.g. after cudaDeviceReset) resolves the array's device address:
 * make it before any stream capture.  All calls share the array: calls whose
 * kernels overlap on the GPU race, so serialise them. */
int ahx_aca_block_noalloc(const double* px, const double* py, const double* pz, uint32_t b1,
                          uint32_t n1, uint32_t b2, uint32_t n2, uint32_t i0, double h, double eps,
                          uint32_t kmax, double* U, double* V, int32_t* info, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* AHX_H */
