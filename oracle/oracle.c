/* CPU oracle for the AHMED H-matrix hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * Plain-C restatement of the reference algorithms (AHMED 1.0); only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg load it, and only
 * as the checker.  See oracle.h for conventions and how it is pinned.
 *
 * Build: gcc -O2 -fopenmp -ffp-contract=off -fPIC -shared (oracle/build_oracle.sh).
 * -ffp-contract=off keeps the tree arithmetic identical to the reference's
 * x86-64 build on every host (GCC contracts to FMA by default on AArch64).
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OR_MIN(a, b) ((a) < (b) ? (a) : (b))
#define OR_MAX(a, b) ((a) > (b) ? (a) : (b))

/* ------------------------------------------------------------------------ */
/* cluster trees                                                             */

typedef struct or_cl {
  uint32_t nbeg, nend;
  struct or_cl* son[2];
  int nsons;
  double diam2;
  double com[3];      /* PCA: centre of mass */
  uint32_t icom;      /* PCA: bemcluster centroid index (original numbering) */
  double xmm[6];      /* bbx: xmin[3], xmax[3] */
  uint32_t maindir;
  double cntrdir;
} or_cl;

typedef struct {
  uint32_t b1, n1, b2, n2, adm, idx, i0;
} or_leaf;

struct or_hmat {
  uint32_t n;
  int kind;
  uint32_t bmin;
  double eta2;
  const double* pts; /* copy, original order, 3 per point */
  double* pts_own;
  uint32_t *op_perm, *po_perm;
  or_cl* root;
  or_leaf* leaves;
  uint32_t nleaves, cap;
  /* assembled data */
  double** data;
  int32_t* rank;     /* -1 dense */
  int32_t* aca_rank; /* -1 dense / failed */
};

static double pc(const or_hmat* H, uint32_t orig, int j) { return H->pts[3 * orig + j]; }

/* bbx init: Include/cluster_bbx.h:52-98 (radius 0 collocation points) */
static void bbx_init(const or_hmat* H, or_cl* c) {
  const uint32_t n = 3;
  for (uint32_t i = 0; i < n; ++i) {
    const double x = pc(H, H->op_perm[c->nbeg], i);
    c->xmm[i] = x - 0.0;
    c->xmm[i + n] = x + 0.0;
  }
  for (uint32_t j = c->nbeg + 1; j < c->nend; ++j) {
    for (uint32_t i = 0; i < n; ++i) {
      const double x = pc(H, H->op_perm[j], i);
      const double r = 0.0;
      if (x - r < c->xmm[i]) c->xmm[i] = x - r;
      else if (x + r > c->xmm[i + n]) c->xmm[i + n] = x + r;
    }
  }
  c->diam2 = 0.0;
  uint32_t imax = 0;
  double mx = 0.0;
  for (uint32_t i = 0; i < n; ++i) {
    const double e = c->xmm[i + n] - c->xmm[i];
    c->diam2 += e * e;
    if (e > mx) { mx = e; imax = i; }
  }
  if (c->xmm[n] - c->xmm[0] > 0.8 * mx) c->maindir = 0;
  else c->maindir = imax;
  c->cntrdir = 0.5 * (c->xmm[c->maindir] + c->xmm[c->maindir + n]);
}

static void swap_u32(uint32_t* a, uint32_t* b) { uint32_t t = *a; *a = *b; *b = t; }

static or_cl* new_cl(uint32_t b, uint32_t e) {
  or_cl* c = (or_cl*)calloc(1, sizeof(or_cl));
  c->nbeg = b;
  c->nend = e;
  return c;
}

/* bbx createClusterTree: Include/cluster_bbx.h:100-128 */
static void bbx_tree(or_hmat* H, or_cl* c, uint32_t bmin) {
  uint32_t nnbeg = c->nend;
  for (uint32_t i = c->nbeg; i < nnbeg;) {
    if (pc(H, H->op_perm[i], c->maindir) < c->cntrdir) ++i;
    else {
      swap_u32(&H->op_perm[i], &H->op_perm[--nnbeg]);
      H->po_perm[H->op_perm[i]] = i;
      H->po_perm[H->op_perm[nnbeg]] = nnbeg;
    }
  }
  if (nnbeg - c->nbeg > bmin && c->nend - nnbeg > bmin) {
    c->son[0] = new_cl(c->nbeg, nnbeg);
    bbx_init(H, c->son[0]);
    bbx_tree(H, c->son[0], bmin);
    c->son[1] = new_cl(nnbeg, c->nend);
    bbx_init(H, c->son[1]);
    bbx_tree(H, c->son[1], bmin);
    c->nsons = 2;
  }
}

/* PCA init (Include/cluster_pca.h:84-116) and bemcluster icom (Include/bemcluster.h:27-50) */
static void pca_init(const or_hmat* H, or_cl* c) {
  const uint32_t n = 3;
  for (uint32_t j = 0; j < n; ++j) c->com[j] = 0.0;
  for (uint32_t i = c->nbeg; i < c->nend; ++i)
    for (uint32_t j = 0; j < n; ++j) c->com[j] += pc(H, H->op_perm[i], j);
  const double d = 1.0 / (c->nend - c->nbeg);
  for (uint32_t j = 0; j < n; ++j) c->com[j] *= d;
  c->diam2 = 0.0;
  for (uint32_t i = c->nbeg; i < c->nend; ++i) {
    double d2 = 0.0;
    for (uint32_t j = 0; j < n; ++j) {
      const double d1 = 2 * (pc(H, H->op_perm[i], j) - c->com[j]);
      d2 += d1 * d1;
    }
    if (d2 > c->diam2) c->diam2 = d2;
  }
  /* icom over ORIGINAL indices nbeg..nend-1 (reference quirk, bemcluster.h:35,42) */
  c->icom = c->nbeg;
  double smin = 0.0;
  for (uint32_t j = 0; j < n; ++j) {
    const double e = c->com[j] - pc(H, c->nbeg, j);
    smin += e * e;
  }
  for (uint32_t i = c->nbeg + 1; i < c->nend; ++i) {
    double s = 0.0;
    for (uint32_t j = 0; j < n; ++j) {
      const double e = c->com[j] - pc(H, i, j);
      s += e * e;
    }
    if (s < smin) { c->icom = i; smin = s; }
  }
}

/* PCA subdivide: Include/cluster_pca.h:119-201 */
static uint32_t pca_split(or_hmat* H, or_cl* c) {
  const uint32_t n = 3, m = 6;
  double cv[6] = {0, 0, 0, 0, 0, 0}, d[3], u[3];
  for (uint32_t i = c->nbeg; i < c->nend; i++) {
    for (uint32_t j = 0; j < n; ++j) d[j] = pc(H, H->op_perm[i], j) - c->com[j];
    uint32_t l = 0;
    for (uint32_t j = 0; j < n; ++j)
      for (uint32_t k = j; k < n; ++k) cv[l++] += d[j] * d[k];
  }
  (void)m;
  for (uint32_t i = 0; i < n; ++i) u[i] = 1.0 / sqrt((double)n);
  uint32_t it = 0;
  do {
    for (uint32_t j = 0; j < n; ++j) d[j] = u[j];
    for (uint32_t j = 0; j < n; ++j) {
      uint32_t k;
      u[j] = 0.0;
      for (k = 0; k < j; ++k) u[j] += cv[k * n - k * (k + 1) / 2 + j] * d[k];
      for (; k < n; ++k) u[j] += cv[j * n - j * (j + 1) / 2 + k] * d[k];
    }
    double modu = 0.0;
    for (uint32_t j = 0; j < n; ++j) modu += u[j] * u[j];
    modu = 1.0 / sqrt(modu);
    for (uint32_t j = 0; j < n; ++j) u[j] *= modu;
  } while (++it < 10);
  double mdtcl = 0.0;
  for (uint32_t i = 0; i < n; ++i) mdtcl += u[i] * c->com[i];
  uint32_t nsep = c->nend;
  for (uint32_t i = c->nbeg; i < nsep;) {
    double skp = 0.0;
    for (uint32_t j = 0; j < n; ++j) skp += pc(H, H->op_perm[i], j) * u[j];
    if (skp < mdtcl) ++i;
    else {
      swap_u32(&H->op_perm[i], &H->op_perm[--nsep]);
      H->po_perm[H->op_perm[i]] = i;
      H->po_perm[H->op_perm[nsep]] = nsep;
    }
  }
  if (nsep == c->nbeg || nsep == c->nend) nsep = (c->nend + c->nbeg) / 2;
  return nsep;
}

/* PCA createClusterTree: Include/cluster_pca.h:204-217 */
static void pca_tree(or_hmat* H, or_cl* c, uint32_t bmin) {
  uint32_t nsep = pca_split(H, c);
  if (nsep >= c->nbeg + bmin && c->nend >= nsep + bmin) {
    c->son[0] = new_cl(c->nbeg, nsep);
    pca_init(H, c->son[0]);
    pca_tree(H, c->son[0], bmin);
    c->son[1] = new_cl(nsep, c->nend);
    pca_init(H, c->son[1]);
    pca_tree(H, c->son[1], bmin);
    c->nsons = 2;
  }
}

/* admissibility: PCA Include/cluster_pca.h:54-80; bbx 3-D Include/cluster_bbx.h:33-47,245-297 */
static int isadm(const or_hmat* H, const or_cl* a, const or_cl* b) {
  const double d2 = OR_MIN(a->diam2, b->diam2);
  if (H->kind == OR_TREE_PCA) {
    double dd = 0.0;
    for (int j = 0; j < 3; ++j) {
      const double e = a->com[j] - b->com[j];
      dd += e * e;
    }
    return d2 < H->eta2 * dd;
  }
  double dd = 0.0;
  for (int i = 0; i < 3; ++i) {
    const double e = b->xmm[i] - a->xmm[i + 3];
    if (e > 0.0) dd += e * e;
    else {
      const double e1 = a->xmm[i] - b->xmm[i + 3];
      if (e1 > 0.0) dd += e1 * e1;
    }
  }
  if (d2 < H->eta2 * dd) return 1;
  /* weak admissibility: boxes touching in all three coordinates' faces */
  const double* x = a->xmm;
  const double* p = b->xmm;
  if (x[3] == p[0] || p[3] == x[0]) {
    if (x[4] == p[1] || p[4] == x[1]) {
      if (x[5] == p[2] || p[5] == x[2]) return 1;
    }
  }
  return 0;
}

static void push_leaf(or_hmat* H, const or_cl* a, const or_cl* b, int adm) {
  if (H->nleaves == H->cap) {
    H->cap = H->cap ? 2 * H->cap : 1024;
    H->leaves = (or_leaf*)realloc(H->leaves, H->cap * sizeof(or_leaf));
  }
  or_leaf* L = &H->leaves[H->nleaves];
  L->b1 = a->nbeg; L->n1 = a->nend - a->nbeg;
  L->b2 = b->nbeg; L->n2 = b->nend - b->nbeg;
  L->adm = (uint32_t)adm;
  L->idx = H->nleaves;
  L->i0 = (adm && H->kind == OR_TREE_PCA) ? a->icom - a->nbeg : 0;
  H->nleaves++;
}

/* blcluster::subdivide_: cluster/blcluster.cpp:40-66 (maxdepth 0); DFS leaf numbering */
static void subdivide(or_hmat* H, const or_cl* a, const or_cl* b) {
  if (isadm(H, a, b)) { push_leaf(H, a, b, 1); return; }
  if (a->nsons && b->nsons) {
    for (int i = 0; i < a->nsons; ++i)
      for (int j = 0; j < b->nsons; ++j) subdivide(H, a->son[i], b->son[j]);
  } else {
    push_leaf(H, a, b, 0);
  }
}

static void free_cl(or_cl* c) {
  if (!c) return;
  free_cl(c->son[0]);
  free_cl(c->son[1]);
  free(c);
}

or_hmat* or_build(const double* pts, uint32_t n, int kind, uint32_t bmin, double eta2) {
  or_hmat* H = (or_hmat*)calloc(1, sizeof(or_hmat));
  H->n = n;
  H->kind = kind;
  H->bmin = bmin;
  H->eta2 = eta2;
  H->pts_own = (double*)malloc(sizeof(double) * 3 * (size_t)n);
  memcpy(H->pts_own, pts, sizeof(double) * 3 * (size_t)n);
  H->pts = H->pts_own;
  H->op_perm = (uint32_t*)malloc(sizeof(uint32_t) * n);
  H->po_perm = (uint32_t*)malloc(sizeof(uint32_t) * n);
  for (uint32_t i = 0; i < n; ++i) H->op_perm[i] = H->po_perm[i] = i;
  H->root = new_cl(0, n);
  if (kind == OR_TREE_BBX) {
    bbx_init(H, H->root);
    bbx_tree(H, H->root, bmin);
  } else {
    pca_init(H, H->root);
    pca_tree(H, H->root, bmin);
  }
  subdivide(H, H->root, H->root);
  H->data = (double**)calloc(H->nleaves, sizeof(double*));
  H->rank = (int32_t*)malloc(sizeof(int32_t) * H->nleaves);
  H->aca_rank = (int32_t*)malloc(sizeof(int32_t) * H->nleaves);
  for (uint32_t l = 0; l < H->nleaves; ++l) H->rank[l] = H->aca_rank[l] = -1;
  return H;
}

void or_free(or_hmat* H) {
  if (!H) return;
  for (uint32_t l = 0; l < H->nleaves; ++l) free(H->data[l]);
  free(H->data);
  free(H->rank);
  free(H->aca_rank);
  free(H->leaves);
  free_cl(H->root);
  free(H->op_perm);
  free(H->po_perm);
  free(H->pts_own);
  free(H);
}

uint32_t or_nleaves(const or_hmat* H) { return H->nleaves; }

void or_perm(const or_hmat* H, uint32_t* op, uint32_t* po) {
  memcpy(op, H->op_perm, sizeof(uint32_t) * H->n);
  memcpy(po, H->po_perm, sizeof(uint32_t) * H->n);
}

void or_leaves(const or_hmat* H, uint32_t* out) {
  for (uint32_t l = 0; l < H->nleaves; ++l) {
    const or_leaf* L = &H->leaves[l];
    uint32_t* o = out + 7 * (size_t)l;
    o[0] = L->b1; o[1] = L->n1; o[2] = L->b2; o[3] = L->n2;
    o[4] = L->adm; o[5] = L->idx; o[6] = L->i0;
  }
}

/* ------------------------------------------------------------------------ */
/* generator (user-supplied MATGEN_T in the reference: contract in           */
/* Include/matgen_omp.h:164-172)                                             */

static double nn_dist2(const double* a, const double* b) {
  const double dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
  return dx * dx + dy * dy + dz * dz;
}

double or_mean_nn(const double* pts, uint32_t n) {
  if (n < 2) return 0.0;
  double lo[3], hi[3];
  for (int j = 0; j < 3; ++j) lo[j] = hi[j] = pts[j];
  for (uint32_t i = 1; i < n; ++i)
    for (int j = 0; j < 3; ++j) {
      if (pts[3 * i + j] < lo[j]) lo[j] = pts[3 * i + j];
      if (pts[3 * i + j] > hi[j]) hi[j] = pts[3 * i + j];
    }
  double ext = 0.0;
  for (int j = 0; j < 3; ++j) ext = OR_MAX(ext, hi[j] - lo[j]);
  int g = (int)ceil(cbrt((double)n));
  if (g < 1) g = 1;
  const double cs = ext > 0.0 ? ext / g * (1.0 + 1e-12) : 1.0;
  const size_t ncell = (size_t)g * g * g;
  uint32_t* head = (uint32_t*)malloc(sizeof(uint32_t) * (ncell + 1));
  uint32_t* list = (uint32_t*)malloc(sizeof(uint32_t) * n);
  int* cell = (int*)malloc(sizeof(int) * 3 * (size_t)n);
  memset(head, 0, sizeof(uint32_t) * (ncell + 1));
  for (uint32_t i = 0; i < n; ++i) {
    size_t id = 0;
    for (int j = 0; j < 3; ++j) {
      int c = (int)((pts[3 * i + j] - lo[j]) / cs);
      if (c >= g) c = g - 1;
      if (c < 0) c = 0;
      cell[3 * i + j] = c;
    }
    id = ((size_t)cell[3 * i] * g + cell[3 * i + 1]) * g + cell[3 * i + 2];
    head[id + 1]++;
  }
  for (size_t c = 0; c < ncell; ++c) head[c + 1] += head[c];
  uint32_t* fill = (uint32_t*)malloc(sizeof(uint32_t) * ncell);
  memcpy(fill, head, sizeof(uint32_t) * ncell);
  for (uint32_t i = 0; i < n; ++i) {
    size_t id = ((size_t)cell[3 * i] * g + cell[3 * i + 1]) * g + cell[3 * i + 2];
    list[fill[id]++] = i;
  }
  double* dmin = (double*)malloc(sizeof(double) * n);
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t ii = 0; ii < (int64_t)n; ++ii) {
    const uint32_t i = (uint32_t)ii;
    double best = INFINITY;
    for (int s = 0; s <= g; ++s) {
      for (int a = cell[3 * i] - s; a <= cell[3 * i] + s; ++a) {
        if (a < 0 || a >= g) continue;
        for (int b = cell[3 * i + 1] - s; b <= cell[3 * i + 1] + s; ++b) {
          if (b < 0 || b >= g) continue;
          for (int c = cell[3 * i + 2] - s; c <= cell[3 * i + 2] + s; ++c) {
            if (c < 0 || c >= g) continue;
            if (OR_MAX(OR_MAX(abs(a - cell[3 * i]), abs(b - cell[3 * i + 1])),
                       abs(c - cell[3 * i + 2])) != s)
              continue;
            const size_t id = ((size_t)a * g + b) * g + c;
            for (uint32_t q = head[id]; q < head[id + 1]; ++q) {
              const uint32_t jj = list[q];
              if (jj == i) continue;
              const double d2 = nn_dist2(pts + 3 * (size_t)i, pts + 3 * (size_t)jj);
              if (d2 < best) best = d2;
            }
          }
        }
      }
      /* every point outside rings 0..s is at least s*cs away */
      const double r = (double)s * cs;
      if (best <= r * r) break;
    }
    dmin[i] = sqrt(best);
  }
  double sum = 0.0;
  for (uint32_t i = 0; i < n; ++i) sum += dmin[i];
  free(dmin);
  free(fill);
  free(cell);
  free(list);
  free(head);
  return sum / n;
}

static const double OR_FOURPI = 4.0 * M_PI;

/* K(x,y) = 1/(4 pi |x-y|), diagonal 1/(4 pi h), permuted indices */
static inline double lap_entry(const or_hmat* H, double h, uint32_t i, uint32_t j) {
  const uint32_t a = H->op_perm[i], b = H->op_perm[j];
  if (a == b) return 1.0 / (OR_FOURPI * h);
  const double r2 = nn_dist2(H->pts + 3 * (size_t)a, H->pts + 3 * (size_t)b);
  return 1.0 / (OR_FOURPI * sqrt(r2));
}

double or_entry(const or_hmat* H, double h, uint32_t i, uint32_t j) { return lap_entry(H, h, i, j); }

static void lap_cmpbl(const or_hmat* H, double h, uint32_t b1, uint32_t n1, uint32_t b2,
                      uint32_t n2, double* data) {
  for (uint32_t j = 0; j < n2; ++j)
    for (uint32_t i = 0; i < n1; ++i) data[i + (size_t)j * n1] = lap_entry(H, h, b1 + i, b2 + j);
}

/* expected entry size of a block: |K| at its first row and column */
static double lap_scale(const or_hmat* H, double h, uint32_t b1, uint32_t b2) {
  return fabs(lap_entry(H, h, b1, b2));
}

/* ------------------------------------------------------------------------ */
/* ACA: Include/ACA.h:29-350                                                */

static uint32_t nexti(uint32_t n, const int* Z, uint32_t j) {
  for (uint32_t t = 0; t < n; ++t) {
    if (Z[j] != -1) return j;
    j = (j + 1 < n) ? j + 1 : 0;
  }
  return j;
}

static double dot(uint32_t n, const double* a, const double* b) {
  double s = 0.0;
  for (uint32_t i = 0; i < n; ++i) s += a[i] * b[i];
  return s;
}

/* ACA_row_step: Include/ACA.h:46-130 */
static int aca_row_step(const or_hmat* H, double h, uint32_t b1, uint32_t n1, uint32_t b2,
                        uint32_t n2, uint32_t* klast, uint32_t* i0, uint32_t k, uint32_t* no,
                        int* Z, int* S, double* U, double* V, double* nrmlsk2, double scale) {
  uint32_t l, j0 = 0;
  double nrmu2, nrmv2, absmax;
  double* const pu = U + (size_t)k * n1;
  double* const pv = V + (size_t)k * n2;
  do {
    for (l = 0; l < n2; ++l) pv[l] = lap_entry(H, h, b1 + *i0, b2 + l);
    for (l = 0; l < k; ++l) {
      const double d = -U[(size_t)l * n1 + *i0];
      const double* vl = V + (size_t)l * n2;
      for (uint32_t j = 0; j < n2; ++j) pv[j] += d * vl[j];
    }
    absmax = 0.0;
    for (l = 0; l < n2; ++l) {
      if (S[l] >= 0) {
        const double eabs = fabs(pv[l]);
        if (eabs > absmax) { absmax = eabs; j0 = l; }
      }
    }
    if (absmax < 1e-14 * scale) {
      Z[*i0] = -1;
      if (++(*no) < n1) *i0 = nexti(n1, Z, *i0);
    }
  } while (absmax < 1e-14 * scale && *no < n1);
  if (absmax < 1e-14 * scale) return 0;

  const double sqrtpiv = sqrt(absmax);
  nrmv2 = 0.0;
  const double sca = sqrtpiv / pv[j0];
  for (l = 0; l < n2; ++l) {
    if (S[l] >= 0) {
      const double e = (pv[l] *= sca);
      nrmv2 += e * e;
      if (fabs(e) > 1e-8 * scale * sqrtpiv) ++S[l];
    }
  }
  for (l = 0; l < n1; ++l) pu[l] = lap_entry(H, h, b1 + l, b2 + j0);
  for (l = 0; l < k; ++l) {
    const double d = -V[(size_t)l * n2 + j0];
    const double* ul = U + (size_t)l * n1;
    for (uint32_t i = 0; i < n1; ++i) pu[i] += d * ul[i];
  }
  *klast = (uint32_t)Z[*i0];
  Z[*i0] = S[j0] = -1;
  ++(*no);
  const double dsca = 1.0 / sqrtpiv;
  absmax = nrmu2 = 0.0;
  for (l = 0; l < n1; ++l) {
    const double eabs = fabs(pu[l] *= dsca);
    if (Z[l] >= 0 && eabs > 1e-8 * scale * sqrtpiv) ++Z[l];
    nrmu2 += eabs * eabs;
    if (Z[l] >= 0 && eabs > absmax) { *i0 = l; absmax = eabs; }
  }
  *nrmlsk2 = nrmu2 * nrmv2;
  return 1;
}

/* ACA_col_step: Include/ACA.h:134-213 */
static int aca_col_step(const or_hmat* H, double h, uint32_t b1, uint32_t n1, uint32_t b2,
                        uint32_t n2, uint32_t* j0, uint32_t k, uint32_t* no, int* Z, int* S,
                        double* U, double* V, double* nrmlsk2, double scale) {
  double nrmu2, nrmv2, absmax;
  double* const pu = U + (size_t)k * n1;
  double* const pv = V + (size_t)k * n2;
  uint32_t l, i0 = 0;
  do {
    for (l = 0; l < n1; ++l) pu[l] = lap_entry(H, h, b1 + l, b2 + *j0);
    for (l = 0; l < k; ++l) {
      const double d = -V[(size_t)l * n2 + *j0];
      const double* ul = U + (size_t)l * n1;
      for (uint32_t i = 0; i < n1; ++i) pu[i] += d * ul[i];
    }
    absmax = 0.0;
    for (l = 0; l < n1; ++l) {
      if (Z[l] >= 0) {
        const double eabs = fabs(pu[l]);
        if (eabs > absmax) { absmax = eabs; i0 = l; }
      }
    }
    if (absmax < 1e-14 * scale) {
      S[*j0] = -1;
      if (++(*no) < n2) *j0 = nexti(n2, S, *j0);
    }
  } while (absmax < 1e-14 * scale && *no < n2);
  if (absmax < 1e-14 * scale) return 0;

  const double sqrtpiv = sqrt(absmax);
  nrmu2 = 0.0;
  const double sca = sqrtpiv / pu[i0];
  for (l = 0; l < n1; ++l) {
    if (Z[l] >= 0) {
      const double e = (pu[l] *= sca);
      nrmu2 += e * e;
      if (fabs(e) > 1e-8 * scale * sqrtpiv) ++Z[l];
    }
  }
  for (l = 0; l < n2; ++l) pv[l] = lap_entry(H, h, b1 + i0, b2 + l);
  for (l = 0; l < k; ++l) {
    const double d = -U[(size_t)l * n1 + i0];
    const double* vl = V + (size_t)l * n2;
    for (uint32_t j = 0; j < n2; ++j) pv[j] += d * vl[j];
  }
  Z[i0] = S[*j0] = -1;
  ++(*no);
  const double dsca = 1.0 / sqrtpiv;
  absmax = nrmv2 = 0.0;
  for (l = 0; l < n2; ++l) {
    const double eabs = fabs(pv[l] *= dsca);
    if (S[l] >= 0 && eabs > 1e-8 * scale * sqrtpiv) ++S[l];
    nrmv2 += eabs * eabs;
    if (eabs > absmax) { *j0 = l; absmax = eabs; }
  }
  *nrmlsk2 = nrmu2 * nrmv2;
  return 1;
}

/* ACA driver: Include/ACA.h:217-350 */
int or_aca_block(const or_hmat* H, double h, uint32_t b1, uint32_t n1, uint32_t b2, uint32_t n2,
                 double eps, uint32_t kmax, uint32_t i0, uint32_t* kout, double* U, double* V) {
  uint32_t l, no = 0, j0, inext, klast = 0, k = 0;
  int kmin = -2, keps = -1, ok, stpcrit;
  double nrmlsk2 = 0.0, nrms2 = 0.0, sum;
  double scale = lap_scale(H, h, b1, b2);
  int* Z = (int*)calloc(n1, sizeof(int));
  int* S = (int*)calloc(n2, sizeof(int));
  int result;
  do {
    inext = i0;
    ok = aca_row_step(H, h, b1, n1, b2, n2, &klast, &inext, k, &no, Z, S, U, V, &nrmlsk2, scale);
    if (!ok) { nrmlsk2 = 0.0; goto SUCC; }
    sum = 0.0;
    for (l = 0; l < k; ++l)
      sum += dot(n1, U + (size_t)l * n1, U + (size_t)k * n1) *
             dot(n2, V + (size_t)l * n2, V + (size_t)k * n2);
    nrms2 += 2.0 * sum + nrmlsk2;
    stpcrit = (nrmlsk2 < eps * eps * nrms2);
    if (stpcrit && keps == -1) keps = (int)klast + 1;
    ++k;
    scale = sqrt(nrmlsk2 / (n1 * n2));
    if (keps > 0) {
      for (i0 = 0; i0 < n1 && Z[i0] < 0; ++i0);
      if (i0 == n1) { nrmlsk2 = 0.0; goto SUCC; }
      kmin = Z[i0];
      for (uint32_t i = i0 + 1; i < n1; ++i)
        if (Z[i] >= 0 && Z[i] < kmin) kmin = Z[i0 = i];
      if ((uint32_t)kmin == k) i0 = inext;
    } else
      i0 = inext;
  } while (no < n1 && k < kmax && kmin < keps);

  if ((no == n1 || k == kmax) && kmin < keps) goto NSUCC;

  do {
    for (j0 = 0; j0 < n2 && S[j0] < 0; ++j0);
    if (j0 == n2) { nrmlsk2 = 0.0; goto SUCC; }
    kmin = S[j0];
    for (uint32_t j = j0 + 1; j < n2; ++j)
      if (S[j] >= 0 && S[j] < kmin) kmin = S[j0 = j];
    if (kmin >= keps) goto SUCC;
    ok = aca_col_step(H, h, b1, n1, b2, n2, &j0, k, &no, Z, S, U, V, &nrmlsk2, scale);
    if (!ok) { nrmlsk2 = 0.0; goto SUCC; }
    ++k;
  } while (no < n2 && k < kmax);

NSUCC:
  result = 0;
  goto DONE;
SUCC: {
    const double epsa = sqrt(nrmlsk2 / nrms2);
    result = !(epsa >= eps); /* NaN (0/0) counts as success, as in the reference */
  }
DONE:
  free(S);
  free(Z);
  *kout = k;
  return result;
}

/* ------------------------------------------------------------------------ */
/* recompression: mblock<double>::addtrll, H/mblock_D.cpp:356-465            */
/* LAPACK dgeqrf/dgesvd/dormqr replaced by Householder QR and one-sided       */
/* (Hestenes) Jacobi SVD; factors may differ by signs/rotations, products and */
/* truncated ranks agree.                                                     */

/* Householder QR of A (m x n, lda m) in place; reflectors below the diagonal */
static void hh_qr(uint32_t m, uint32_t n, double* A, double* tau) {
  const uint32_t kk = OR_MIN(m, n);
  for (uint32_t j = 0; j < kk; ++j) {
    double* a = A + (size_t)j * m;
    double xn2 = 0.0;
    for (uint32_t i = j + 1; i < m; ++i) xn2 += a[i] * a[i];
    const double alpha = a[j];
    if (xn2 == 0.0) { tau[j] = 0.0; continue; }
    const double nrm = sqrt(alpha * alpha + xn2);
    const double beta = alpha >= 0.0 ? -nrm : nrm;
    tau[j] = (beta - alpha) / beta;
    const double sc = 1.0 / (alpha - beta);
    for (uint32_t i = j + 1; i < m; ++i) a[i] *= sc;
    a[j] = beta;
    for (uint32_t c = j + 1; c < n; ++c) {
      double* b = A + (size_t)c * m;
      double s = b[j];
      for (uint32_t i = j + 1; i < m; ++i) s += a[i] * b[i];
      s *= tau[j];
      b[j] -= s;
      for (uint32_t i = j + 1; i < m; ++i) b[i] -= s * a[i];
    }
  }
}

/* C (m x nc, ldc m) := Q C with Q = H_0 ... H_{kr-1} from hh_qr */
static void hh_apply(uint32_t m, uint32_t kr, const double* A, const double* tau, uint32_t nc,
                     double* C) {
  for (int j = (int)kr - 1; j >= 0; --j) {
    if (tau[j] == 0.0) continue;
    const double* a = A + (size_t)j * m;
    for (uint32_t c = 0; c < nc; ++c) {
      double* b = C + (size_t)c * m;
      double s = b[j];
      for (uint32_t i = (uint32_t)j + 1; i < m; ++i) s += a[i] * b[i];
      s *= tau[j];
      b[j] -= s;
      for (uint32_t i = (uint32_t)j + 1; i < m; ++i) b[i] -= s * a[i];
    }
  }
}

/* one-sided Jacobi on the columns of A (m x n); on exit the columns of A are
 * A V (= U Sigma) and V (n x n) is orthogonal; columns sorted by norm, desc. */
static void jacobi_svd(uint32_t m, uint32_t n, double* A, double* Vm, double* sig) {
  for (uint32_t i = 0; i < n * n; ++i) Vm[i] = 0.0;
  for (uint32_t i = 0; i < n; ++i) Vm[i + (size_t)i * n] = 1.0;
  for (int sweep = 0; sweep < 60; ++sweep) {
    int rotated = 0;
    for (uint32_t p = 0; p + 1 < n; ++p)
      for (uint32_t q = p + 1; q < n; ++q) {
        double* ap = A + (size_t)p * m;
        double* aq = A + (size_t)q * m;
        double al = 0.0, be = 0.0, ga = 0.0;
        for (uint32_t i = 0; i < m; ++i) {
          al += ap[i] * ap[i];
          be += aq[i] * aq[i];
          ga += ap[i] * aq[i];
        }
        if (ga == 0.0 || fabs(ga) <= 1e-15 * sqrt(al * be)) continue;
        rotated = 1;
        const double zeta = (be - al) / (2.0 * ga);
        const double t = (zeta >= 0.0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
        const double c = 1.0 / sqrt(1.0 + t * t);
        const double s = c * t;
        for (uint32_t i = 0; i < m; ++i) {
          const double x = ap[i], y = aq[i];
          ap[i] = c * x - s * y;
          aq[i] = s * x + c * y;
        }
        double* vp = Vm + (size_t)p * n;
        double* vq = Vm + (size_t)q * n;
        for (uint32_t i = 0; i < n; ++i) {
          const double x = vp[i], y = vq[i];
          vp[i] = c * x - s * y;
          vq[i] = s * x + c * y;
        }
      }
    if (!rotated) break;
  }
  for (uint32_t j = 0; j < n; ++j) sig[j] = sqrt(dot(m, A + (size_t)j * m, A + (size_t)j * m));
  /* selection sort, descending */
  for (uint32_t j = 0; j < n; ++j) {
    uint32_t b = j;
    for (uint32_t q = j + 1; q < n; ++q)
      if (sig[q] > sig[b]) b = q;
    if (b != j) {
      double t = sig[j]; sig[j] = sig[b]; sig[b] = t;
      for (uint32_t i = 0; i < m; ++i) {
        t = A[i + (size_t)j * m]; A[i + (size_t)j * m] = A[i + (size_t)b * m]; A[i + (size_t)b * m] = t;
      }
      for (uint32_t i = 0; i < n; ++i) {
        t = Vm[i + (size_t)j * n]; Vm[i + (size_t)j * n] = Vm[i + (size_t)b * n]; Vm[i + (size_t)b * n] = t;
      }
    }
  }
}

uint32_t or_recompress(uint32_t n1, uint32_t n2, uint32_t k, double* U, double* V, double delta,
                       uint32_t kgoal) {
  if (k == 0) return 0;
  const uint32_t mmin = OR_MIN(n1, k), nmin = OR_MIN(n2, k), amin = OR_MIN(mmin, nmin);
  double* tau1 = (double*)malloc(sizeof(double) * (mmin + nmin));
  double* tau2 = tau1 + mmin;
  hh_qr(n1, k, U, tau1);
  hh_qr(n2, k, V, tau2);
  double* R = (double*)malloc(sizeof(double) * ((size_t)mmin * nmin + (size_t)nmin * nmin + nmin));
  double* Vm = R + (size_t)mmin * nmin;
  double* sig = Vm + (size_t)nmin * nmin;
  /* R = R1 R2^T (blas::utrmmh, Include/blas.h:2767-2781) */
  for (uint32_t j = 0; j < nmin; ++j)
    for (uint32_t i = 0; i < mmin; ++i) {
      double d = 0.0;
      for (uint32_t l = OR_MAX(i, j); l < k; ++l) d += U[i + (size_t)l * n1] * V[j + (size_t)l * n2];
      R[i + (size_t)j * mmin] = d;
    }
  const double thresh =
      delta * sqrt(dot(mmin * nmin, R, R)) / (double)sqrtf((float)mmin * (float)nmin);
  for (uint32_t i = 0; i < mmin * nmin; ++i)
    if (fabs(R[i]) < thresh) R[i] = 0.0;
  jacobi_svd(mmin, nmin, R, Vm, sig);
  uint32_t kt = OR_MIN(amin, kgoal);
  while (kt > 0 && (sig[kt - 1] <= delta * sig[0] || sig[kt - 1] < 1e-64)) --kt;
  if (kt > 0) {
    double* nu = (double*)calloc((size_t)n1 * kt + (size_t)n2 * kt, sizeof(double));
    double* nv = nu + (size_t)n1 * kt;
    for (uint32_t j = 0; j < kt; ++j) {
      for (uint32_t i = 0; i < mmin; ++i) nu[i + (size_t)j * n1] = R[i + (size_t)j * mmin];
      for (uint32_t i = 0; i < nmin; ++i) nv[i + (size_t)j * n2] = Vm[i + (size_t)j * nmin];
    }
    hh_apply(n1, mmin, U, tau1, kt, nu);
    hh_apply(n2, nmin, V, tau2, kt, nv);
    memcpy(U, nu, sizeof(double) * n1 * kt);
    memcpy(V, nv, sizeof(double) * n2 * kt);
    free(nu);
  }
  free(R);
  free(tau1);
  return kt;
}

/* apprx_unsym: Include/apprx.h:136-172 (i0 from the tree) */
static void apprx_leaf(or_hmat* H, double h, double eps, uint32_t rankmax, uint32_t l) {
  const or_leaf* L = &H->leaves[l];
  const uint32_t n1 = L->n1, n2 = L->n2;
  uint32_t maxk = n1 * n2 / (n1 + n2) + 4;
  if (maxk > rankmax) maxk = rankmax;
  free(H->data[l]);
  H->data[l] = NULL;
  H->aca_rank[l] = -1;
  int succ = 0;
  if (L->adm && maxk) {
    uint32_t k = 0;
    double* U = (double*)malloc(sizeof(double) * (size_t)(maxk + 1) * n1);
    double* V = (double*)malloc(sizeof(double) * (size_t)(maxk + 1) * n2);
    succ = or_aca_block(H, h, L->b1, n1, L->b2, n2, eps, maxk, L->i0, &k, U, V);
    if (succ) {
      H->aca_rank[l] = (int32_t)k;
      const uint32_t kt = or_recompress(n1, n2, k, U, V, eps, k);
      H->rank[l] = (int32_t)kt;
      if (kt) {
        double* d = (double*)malloc(sizeof(double) * (size_t)kt * (n1 + n2));
        memcpy(d, U, sizeof(double) * (size_t)kt * n1);
        memcpy(d + (size_t)kt * n1, V, sizeof(double) * (size_t)kt * n2);
        H->data[l] = d;
      }
    }
    free(V);
    free(U);
  }
  if (!succ) {
    H->rank[l] = -1;
    H->data[l] = (double*)malloc(sizeof(double) * (size_t)n1 * n2);
    lap_cmpbl(H, h, L->b1, n1, L->b2, n2, H->data[l]);
  }
}

static void set_threads(int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
}

/* matgenGeH_omp: Include/matgen_omp.h:197-213 (dynamic schedule over the DFS leaf list) */
void or_assemble_range(or_hmat* H, double h, double eps, uint32_t rankmax, int nthreads,
                       uint32_t l0, uint32_t l1) {
  set_threads(nthreads);
#pragma omp parallel for schedule(dynamic)
  for (int64_t l = (int64_t)l0; l < (int64_t)l1; ++l) apprx_leaf(H, h, eps, rankmax, (uint32_t)l);
}

void or_assemble(or_hmat* H, double h, double eps, uint32_t rankmax, int nthreads) {
  or_assemble_range(H, h, eps, rankmax, nthreads, 0, H->nleaves);
}

void or_ranks(const or_hmat* H, int32_t* out) { memcpy(out, H->rank, sizeof(int32_t) * H->nleaves); }
void or_aca_ranks(const or_hmat* H, int32_t* out) {
  memcpy(out, H->aca_rank, sizeof(int32_t) * H->nleaves);
}

uint64_t or_leaf_data(const or_hmat* H, uint32_t l, double* out) {
  const or_leaf* L = &H->leaves[l];
  const uint64_t cnt = H->rank[l] >= 0 ? (uint64_t)H->rank[l] * (L->n1 + L->n2)
                                       : (uint64_t)L->n1 * L->n2;
  if (out && cnt && H->data[l]) memcpy(out, H->data[l], sizeof(double) * cnt);
  return cnt;
}

void or_set_leaf(or_hmat* H, uint32_t l, int32_t rank, const double* data) {
  const or_leaf* L = &H->leaves[l];
  free(H->data[l]);
  H->data[l] = NULL;
  H->rank[l] = rank;
  const uint64_t cnt = rank >= 0 ? (uint64_t)rank * (L->n1 + L->n2) : (uint64_t)L->n1 * L->n2;
  if (cnt) {
    H->data[l] = (double*)malloc(sizeof(double) * cnt);
    memcpy(H->data[l], data, sizeof(double) * cnt);
  }
}

/* ------------------------------------------------------------------------ */
/* product: mltaGeHVec_ / mblock::mltaLrMVec_ / mltaGeMVec                    */
/* (H/mltaGeHVec.cpp:16-35, H/mblock.cpp:126-138, Include/mblock.h:99-102)    */

/* one leaf, all p right-hand sides: low rank as mltaLrMGeM_ (t = V^T X, Y += d U t,
 * H/mblock.cpp:141-154), dense as mltaGeMGeM (Include/mblock.h:105-109) */
static void leaf_mm(const or_hmat* H, uint32_t l, double d, uint32_t p, const double* X,
                    double* Y, size_t ld) {
  const or_leaf* L = &H->leaves[l];
  const double* A = H->data[l];
  const uint32_t n1 = L->n1, n2 = L->n2;
  if (H->rank[l] > 0) {
    const uint32_t k = (uint32_t)H->rank[l];
    const double* V = A + (size_t)k * n1;
    double tb[256];
    double* t = (size_t)k * p <= 256 ? tb : (double*)malloc(sizeof(double) * (size_t)k * p);
    for (uint32_t c = 0; c < p; ++c)
      for (uint32_t r = 0; r < k; ++r)
        t[r + (size_t)c * k] = d * dot(n2, V + (size_t)r * n2, X + c * ld + L->b2);
    for (uint32_t c = 0; c < p; ++c) {
      double* yp = Y + c * ld + L->b1;
      for (uint32_t r = 0; r < k; ++r) {
        const double e = t[r + (size_t)c * k];
        const double* u = A + (size_t)r * n1;
        for (uint32_t i = 0; i < n1; ++i) yp[i] += e * u[i];
      }
    }
    if (t != tb) free(t);
  } else if (H->rank[l] < 0) {
    for (uint32_t c = 0; c < p; ++c) {
      const double* xp = X + c * ld + L->b2;
      double* yp = Y + c * ld + L->b1;
      for (uint32_t j = 0; j < n2; ++j) {
        const double t = d * xp[j];
        const double* a = A + (size_t)j * n1;
        for (uint32_t i = 0; i < n1; ++i) yp[i] += t * a[i];
      }
    }
  }
}

/* H/mltaGeHVec.cpp:16-59 visits every leaf once; here the leaves are shared
 * among threads with private accumulators summed in thread order. */
void or_matvec(const or_hmat* H, double d, uint32_t p, const double* X, double* Y, int nthreads) {
  const size_t n = H->n;
  set_threads(nthreads);
  int nt = 1;
#ifdef _OPENMP
  nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#endif
  if (nt <= 1) {
    for (uint32_t l = 0; l < H->nleaves; ++l) leaf_mm(H, l, d, p, X, Y, n);
    return;
  }
  double* acc = (double*)malloc(sizeof(double) * (size_t)nt * n * p);
#pragma omp parallel num_threads(nt)
  {
    int t = 0;
#ifdef _OPENMP
    t = omp_get_thread_num();
#endif
    double* ya = acc + (size_t)t * n * p;
    memset(ya, 0, sizeof(double) * n * p);
#pragma omp for schedule(dynamic, 8)
    for (int64_t l = 0; l < (int64_t)H->nleaves; ++l) leaf_mm(H, (uint32_t)l, d, p, X, ya, n);
#pragma omp for schedule(static)
    for (int64_t i = 0; i < (int64_t)(n * p); ++i) {
      double s = 0.0;
      for (int q = 0; q < nt; ++q) s += acc[(size_t)q * n * p + i];
      Y[i] += s;
    }
  }
  free(acc);
}

/* ------------------------------------------------------------------------ */
/* CPU baseline of bounded samples                                            */

typedef void (*or_dgemm_t)(const char*, const char*, const int*, const int*, const int*, const double*,
                           const double*, const int*, const double*, const int*, const double*, double*,
                           const int*);
typedef void (*or_dgemv_t)(const char*, const int*, const int*, const double*, const double*, const int*,
                           const double*, const int*, const double*, double*, const int*);
static or_dgemm_t g_dgemm = NULL;
static or_dgemv_t g_dgemv = NULL;

void or_set_blas(void* dgemm, void* dgemv) {
  g_dgemm = (or_dgemm_t)dgemm;
  g_dgemv = (or_dgemv_t)dgemv;
}

void or_assemble_list(or_hmat* H, double h, double eps, uint32_t rankmax, int nthreads,
                      const uint32_t* leaves, uint32_t count) {
  set_threads(nthreads);
#pragma omp parallel for schedule(dynamic)
  for (int64_t q = 0; q < (int64_t)count; ++q) apprx_leaf(H, h, eps, rankmax, leaves[q]);
}

/* C = alpha op(A) B + beta C with op = T (transa 'T') or N, column-major */
static void mm(char ta, int m, int n, int k, double alpha, const double* A, int lda, const double* B, int ldb,
               double beta, double* Cm, int ldc) {
  if (g_dgemm) {
    const char tb = 'N';
    g_dgemm(&ta, &tb, &m, &n, &k, &alpha, A, &lda, B, &ldb, &beta, Cm, &ldc);
    return;
  }
  for (int c = 0; c < n; ++c)
    for (int i = 0; i < m; ++i) {
      double s = 0.0;
      for (int l = 0; l < k; ++l) s += (ta == 'T' ? A[l + (size_t)i * lda] : A[i + (size_t)l * lda]) * B[l + (size_t)c * ldb];
      /* beta = 0 ignores C (BLAS semantics: it may hold anything) */
      Cm[i + (size_t)c * ldc] = alpha * s + (beta != 0.0 ? beta * Cm[i + (size_t)c * ldc] : 0.0);
    }
}

/* y = alpha op(A) x + y */
static void mv(char ta, int m, int n, double alpha, const double* A, int lda, const double* x, double* y) {
  if (g_dgemv) {
    const int one = 1;
    const double b1 = 1.0;
    g_dgemv(&ta, &m, &n, &alpha, A, &lda, x, &one, &b1, y, &one);
    return;
  }
  if (ta == 'N') {
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < m; ++i) y[i] += alpha * A[i + (size_t)j * lda] * x[j];
  } else {
    for (int j = 0; j < n; ++j) {
      double s = 0.0;
      for (int i = 0; i < m; ++i) s += A[i + (size_t)j * lda] * x[i];
      y[j] += alpha * s;
    }
  }
}

static void leaf_gem(const or_hmat* H, uint32_t l, double d, uint32_t p, const double* X, uint64_t ldX,
                     double* Y, uint64_t ldY, double* tmp) {
  const or_leaf* L = &H->leaves[l];
  const double* A = H->data[l];
  const int n1 = (int)L->n1, n2 = (int)L->n2, lx = (int)ldX, ly = (int)ldY;
  if (!A) return;
  const double* x = X + L->b2;
  double* y = Y + L->b1;
  if (H->rank[l] > 0) {
    const int k = H->rank[l];
    const double* V = A + (size_t)k * n1;
    if (p == 1) { /* mltaLrMVec_: t = V^T x, y += d U t */
      for (int r = 0; r < k; ++r) tmp[r] = 0.0;
      mv('T', n2, k, 1.0, V, n2, x, tmp);
      mv('N', n1, k, d, A, n1, tmp, y);
    } else { /* mltaLrMGeM_: gemhm then gemma */
      mm('T', k, (int)p, n2, 1.0, V, n2, x, lx, 0.0, tmp, k);
      mm('N', n1, (int)p, k, d, A, n1, tmp, k, 1.0, y, ly);
    }
  } else if (H->rank[l] < 0) {
    if (p == 1) mv('N', n1, n2, d, A, n1, x, y);
    else mm('N', n1, (int)p, n2, d, A, n1, x, lx, 1.0, y, ly);
  }
}

void or_matvec_layers(const or_hmat* H, double d, uint32_t p, const double* X, uint64_t ldX, double* Y,
                      uint64_t ldY, int nthreads, const uint32_t* leaves, const uint32_t* group_start,
                      uint32_t ngroups, const uint32_t* layer_start, uint32_t nlayers) {
  set_threads(nthreads);
  uint32_t kmax = 1;
  for (uint32_t q = 0; q < group_start[ngroups]; ++q)
    if (H->rank[leaves[q]] > (int32_t)kmax) kmax = (uint32_t)H->rank[leaves[q]];
#pragma omp parallel
  {
    double* tmp = (double*)malloc(sizeof(double) * (size_t)kmax * p);
    for (uint32_t q = 0; q < nlayers; ++q) {
#pragma omp for schedule(dynamic, 4)
      for (int64_t g = (int64_t)layer_start[q]; g < (int64_t)layer_start[q + 1]; ++g)
        for (uint32_t e = group_start[g]; e < group_start[g + 1]; ++e)
          leaf_gem(H, leaves[e], d, p, X, ldX, Y, ldY, tmp);
      /* the implicit barrier of the omp for ends the layer */
    }
    free(tmp);
  }
}

/* ------------------------------------------------------------------------ */
/* solvers: GMRes (solvers/GMRES.cpp:32-181), CG (solvers/CG.cpp:31-113)      */

static double nrm2(size_t n, const double* x) { return sqrt(dot((uint32_t)n, x, x)); }

static void gen_rot(double dx, double dy, double* cs, double* sn) {
  if (dy == 0.0) { *cs = 1.0; *sn = 0.0; }
  else if (fabs(dy) > fabs(dx)) {
    const double t = dx / dy;
    *sn = 1.0 / sqrt(1.0 + t * t);
    *cs = t * *sn;
  } else {
    const double t = dy / dx;
    *cs = 1.0 / sqrt(1.0 + t * t);
    *sn = t * *cs;
  }
}

static void appl_rot(double* dx, double* dy, double cs, double sn) {
  const double t = cs * *dx + sn * *dy;
  *dy = cs * *dy - sn * *dx;
  *dx = t;
}

/* solve H y = s (upper triangular, ldH) and x += V y  (GMRES.cpp:59-78) */
static void gm_update(size_t n, uint32_t k, const double* Hm, uint32_t ldH, const double* s,
                      const double* V, double* x) {
  double* y = (double*)malloc(sizeof(double) * k);
  memcpy(y, s, sizeof(double) * k);
  for (int j = (int)k - 1; j >= 0; --j) {
    y[j] /= Hm[j + (size_t)j * ldH];
    for (int i = 0; i < j; ++i) y[i] -= y[j] * Hm[i + (size_t)j * ldH];
  }
  for (uint32_t j = 0; j < k; ++j)
    for (size_t i = 0; i < n; ++i) x[i] += y[j] * V[i + j * n];
  free(y);
}

uint32_t or_gmres(const or_hmat* H, const double* b, double* x, double* eps, uint32_t m,
                  uint32_t* nsteps, int nthreads) {
  const size_t n = H->n;
  double resid;
  uint32_t j = 1;
  double* r = (double*)malloc(sizeof(double) * (n + n * (m + 1) + (size_t)(m + 1) * m + 3 * (m + 1)));
  double* V = r + n;
  double* Hm = V + n * (m + 1);
  double* cs = Hm + (size_t)(m + 1) * m;
  double* sn = cs + m + 1;
  double* s = sn + m + 1;
  const double normb = nrm2(n, b);
  if (normb == 0.0) {
    memset(x, 0, sizeof(double) * n);
    *eps = 0.0;
    *nsteps = 0;
    free(r);
    return 0;
  }
  memcpy(r, b, sizeof(double) * n);
  or_matvec(H, -1.0, 1, x, r, nthreads);
  double beta = nrm2(n, r);
  if ((resid = beta / normb) <= *eps) {
    *eps = resid;
    *nsteps = 0;
    free(r);
    return 0;
  }
  while (j <= *nsteps) {
    for (size_t i = 0; i < n; ++i) V[i] = r[i] * (1.0 / beta);
    s[0] = beta;
    memset(s + 1, 0, sizeof(double) * m);
    for (uint32_t i = 0; i < m && j <= *nsteps; i++, j++) {
      double* w = V + (i + 1) * n;
      memset(w, 0, sizeof(double) * n);
      or_matvec(H, 1.0, 1, V + i * n, w, nthreads);
      for (uint32_t k = 0; k <= i; k++) {
        const double hk = dot((uint32_t)n, w, V + k * n);
        Hm[k + i * (m + 1)] = hk;
        for (size_t q = 0; q < n; ++q) w[q] += -hk * V[q + k * n];
      }
      Hm[i * (m + 2) + 1] = nrm2(n, w);
      const double inv = 1.0 / Hm[i * (m + 2) + 1];
      for (size_t q = 0; q < n; ++q) w[q] *= inv;
      for (uint32_t k = 0; k < i; k++)
        appl_rot(&Hm[k + i * (m + 1)], &Hm[k + 1 + i * (m + 1)], cs[k], sn[k]);
      gen_rot(Hm[i * (m + 2)], Hm[i * (m + 2) + 1], &cs[i], &sn[i]);
      appl_rot(&Hm[i * (m + 2)], &Hm[i * (m + 2) + 1], cs[i], sn[i]);
      appl_rot(&s[i], &s[i + 1], cs[i], sn[i]);
      if ((resid = fabs(s[i + 1] / normb)) < *eps) {
        gm_update(n, i + 1, Hm, m + 1, s, V, x);
        *eps = resid;
        *nsteps = j;
        free(r);
        return 0;
      }
    }
    gm_update(n, m, Hm, m + 1, s, V, x);
    memcpy(r, b, sizeof(double) * n);
    or_matvec(H, -1.0, 1, x, r, nthreads);
    beta = nrm2(n, r);
    if ((resid = beta / normb) < *eps) {
      *eps = resid;
      *nsteps = j;
      free(r);
      return 0;
    }
  }
  *eps = resid;
  free(r);
  return 1;
}

uint32_t or_cg(const or_hmat* H, const double* b, double* x, double* eps, uint32_t* nsteps,
               int nthreads) {
  const size_t N = H->n;
  double rho, rho1 = 0.0;
  double* p = (double*)malloc(sizeof(double) * 4 * N);
  double *q = p + N, *r = q + N, *rhat = r + N;
  const double nrmb = nrm2(N, b);
  if (nrmb < 1e-16) {
    memset(x, 0, sizeof(double) * N);
    *eps = 0.0;
    *nsteps = 0;
    free(p);
    return 0;
  }
  memcpy(r, b, sizeof(double) * N);
  or_matvec(H, -1.0, 1, x, r, nthreads);
  double resid = nrm2(N, r);
  if (resid <= *eps * nrmb) {
    *eps = resid / nrmb;
    *nsteps = 0;
    free(p);
    return 0;
  }
  for (uint32_t l = 1; l <= *nsteps; ++l) {
    memcpy(rhat, r, sizeof(double) * N);
    rho = dot((uint32_t)N, r, rhat);
    if (l > 1) {
      const double beta = rho / rho1;
      for (size_t i = 0; i < N; ++i) p[i] = beta * p[i] + rhat[i];
    } else
      memcpy(p, rhat, sizeof(double) * N);
    memset(q, 0, sizeof(double) * N);
    or_matvec(H, 1.0, 1, p, q, nthreads);
    const double alpha = rho / dot((uint32_t)N, p, q);
    for (size_t i = 0; i < N; ++i) x[i] += alpha * p[i];
    for (size_t i = 0; i < N; ++i) r[i] += -alpha * q[i];
    resid = nrm2(N, r);
    if (resid <= *eps * nrmb) {
      *eps = resid / nrmb;
      *nsteps = l;
      free(p);
      return 0;
    }
    rho1 = rho;
  }
  *eps = resid / nrmb;
  free(p);
  return 1;
}
