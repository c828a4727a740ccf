// Cluster trees, block-cluster tree and DFS leaf list (host, bit-exact with
// the reference; compiled with -ffp-contract=off).
#include "ahx_tree.hpp"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>

namespace ahx {
namespace {

struct Builder {
  Tree& T;
  const double* P;  // original order

  double c(uint32_t orig, uint32_t j) const { return P[3 * (size_t)orig + j]; }

  int32_t add_node(uint32_t b, uint32_t e, uint32_t level) {
    ClusterNode nd{};
    nd.nbeg = b;
    nd.nend = e;
    nd.son[0] = nd.son[1] = -1;
    nd.level = level;
    T.nodes.push_back(nd);
    return (int32_t)T.nodes.size() - 1;
  }

  // Include/cluster_bbx.h:52-98 (point DOFs carry radius 0)
  void bbx_init(ClusterNode& nd) {
    const uint32_t n = 3;
    const uint32_t* op = T.op_perm.data();
    for (uint32_t i = 0; i < n; ++i) {
      const double x = c(op[nd.nbeg], i);
      nd.xmm[i] = x - 0.0;
      nd.xmm[i + n] = x + 0.0;
    }
    for (uint32_t j = nd.nbeg + 1; j < nd.nend; ++j) {
      for (uint32_t i = 0; i < n; ++i) {
        const double x = c(op[j], i);
        const double r = 0.0;
        if (x - r < nd.xmm[i]) nd.xmm[i] = x - r;
        else if (x + r > nd.xmm[i + n]) nd.xmm[i + n] = x + r;
      }
    }
    nd.diam2 = 0.0;
    uint32_t imax = 0;
    double mx = 0.0;
    for (uint32_t i = 0; i < n; ++i) {
      const double e = nd.xmm[i + n] - nd.xmm[i];
      nd.diam2 += e * e;
      if (e > mx) {
        mx = e;
        imax = i;
      }
    }
    nd.maindir = (nd.xmm[n] - nd.xmm[0] > 0.8 * mx) ? 0u : imax;
    nd.cntrdir = 0.5 * (nd.xmm[nd.maindir] + nd.xmm[nd.maindir + n]);
  }

  // Include/cluster_pca.h:84-116 and Include/bemcluster.h:27-50
  void pca_init(ClusterNode& nd) {
    const uint32_t n = 3;
    const uint32_t* op = T.op_perm.data();
    for (uint32_t j = 0; j < n; ++j) nd.com[j] = 0.0;
    for (uint32_t i = nd.nbeg; i < nd.nend; ++i)
      for (uint32_t j = 0; j < n; ++j) nd.com[j] += c(op[i], j);
    const double d = 1.0 / (nd.nend - nd.nbeg);
    for (uint32_t j = 0; j < n; ++j) nd.com[j] *= d;
    nd.diam2 = 0.0;
    for (uint32_t i = nd.nbeg; i < nd.nend; ++i) {
      double d2 = 0.0;
      for (uint32_t j = 0; j < n; ++j) {
        const double d1 = 2 * (c(op[i], j) - nd.com[j]);
        d2 += d1 * d1;
      }
      if (d2 > nd.diam2) nd.diam2 = d2;
    }
    // The reference measures the distance to dofs[i] in the ORIGINAL numbering
    // for i in [nbeg, nend) (bemcluster.h:35,42); kept as is.
    nd.icom = nd.nbeg;
    double smin = 0.0;
    for (uint32_t j = 0; j < n; ++j) {
      const double e = nd.com[j] - c(nd.nbeg, j);
      smin += e * e;
    }
    for (uint32_t i = nd.nbeg + 1; i < nd.nend; ++i) {
      double s = 0.0;
      for (uint32_t j = 0; j < n; ++j) {
        const double e = nd.com[j] - c(i, j);
        s += e * e;
      }
      if (s < smin) {
        nd.icom = i;
        smin = s;
      }
    }
  }

  void swap_perm(uint32_t a, uint32_t b) {
    std::swap(T.op_perm[a], T.op_perm[b]);
    T.po_perm[T.op_perm[a]] = a;
    T.po_perm[T.op_perm[b]] = b;
  }

  // Include/cluster_bbx.h:100-128
  void bbx_tree(int32_t id) {
    const uint32_t nbeg = T.nodes[id].nbeg, nend = T.nodes[id].nend;
    const uint32_t dir = T.nodes[id].maindir;
    const double cd = T.nodes[id].cntrdir;
    uint32_t nnbeg = nend;
    for (uint32_t i = nbeg; i < nnbeg;) {
      if (c(T.op_perm[i], dir) < cd) ++i;
      else swap_perm(i, --nnbeg);
    }
    if (nnbeg - nbeg > T.bmin && nend - nnbeg > T.bmin) {
      const uint32_t lvl = T.nodes[id].level + 1;
      int32_t s0 = add_node(nbeg, nnbeg, lvl);
      bbx_init(T.nodes[s0]);
      bbx_tree(s0);
      int32_t s1 = add_node(nnbeg, nend, lvl);
      bbx_init(T.nodes[s1]);
      bbx_tree(s1);
      T.nodes[id].son[0] = s0;
      T.nodes[id].son[1] = s1;
    }
  }

  // Include/cluster_pca.h:119-201
  uint32_t pca_split(int32_t id) {
    const ClusterNode nd = T.nodes[id];
    const uint32_t n = 3;
    double cv[6] = {0, 0, 0, 0, 0, 0}, d[3], u[3];
    for (uint32_t i = nd.nbeg; i < nd.nend; i++) {
      for (uint32_t j = 0; j < n; ++j) d[j] = c(T.op_perm[i], j) - nd.com[j];
      uint32_t l = 0;
      for (uint32_t j = 0; j < n; ++j)
        for (uint32_t k = j; k < n; ++k) cv[l++] += d[j] * d[k];
    }
    for (uint32_t i = 0; i < n; ++i) u[i] = 1.0 / std::sqrt((double)n);
    for (int it = 0; it < 10; ++it) {
      for (uint32_t j = 0; j < n; ++j) d[j] = u[j];
      for (uint32_t j = 0; j < n; ++j) {
        uint32_t k;
        u[j] = 0.0;
        for (k = 0; k < j; ++k) u[j] += cv[k * n - k * (k + 1) / 2 + j] * d[k];
        for (; k < n; ++k) u[j] += cv[j * n - j * (j + 1) / 2 + k] * d[k];
      }
      double modu = 0.0;
      for (uint32_t j = 0; j < n; ++j) modu += u[j] * u[j];
      modu = 1.0 / std::sqrt(modu);
      for (uint32_t j = 0; j < n; ++j) u[j] *= modu;
    }
    double mdtcl = 0.0;
    for (uint32_t i = 0; i < n; ++i) mdtcl += u[i] * nd.com[i];
    uint32_t nsep = nd.nend;
    for (uint32_t i = nd.nbeg; i < nsep;) {
      double skp = 0.0;
      for (uint32_t j = 0; j < n; ++j) skp += c(T.op_perm[i], j) * u[j];
      if (skp < mdtcl) ++i;
      else swap_perm(i, --nsep);
    }
    if (nsep == nd.nbeg || nsep == nd.nend) nsep = (nd.nend + nd.nbeg) / 2;
    return nsep;
  }

  // Include/cluster_pca.h:204-217
  void pca_tree(int32_t id) {
    const uint32_t nsep = pca_split(id);
    const uint32_t nbeg = T.nodes[id].nbeg, nend = T.nodes[id].nend;
    if (nsep >= nbeg + T.bmin && nend >= nsep + T.bmin) {
      const uint32_t lvl = T.nodes[id].level + 1;
      int32_t s0 = add_node(nbeg, nsep, lvl);
      pca_init(T.nodes[s0]);
      pca_tree(s0);
      int32_t s1 = add_node(nsep, nend, lvl);
      pca_init(T.nodes[s1]);
      pca_tree(s1);
      T.nodes[id].son[0] = s0;
      T.nodes[id].son[1] = s1;
    }
  }

  // Include/cluster_pca.h:54-80; Include/cluster_bbx.h:33-47, 245-297
  bool isadm(const ClusterNode& a, const ClusterNode& b) const {
    const double d2 = std::min(a.diam2, b.diam2);
    if (T.kind == kTreePca) {
      double dd = 0.0;
      for (int j = 0; j < 3; ++j) {
        const double e = a.com[j] - b.com[j];
        dd += e * e;
      }
      return d2 < T.eta2 * dd;
    }
    double dd = 0.0;
    for (int i = 0; i < 3; ++i) {
      const double e = b.xmm[i] - a.xmm[i + 3];
      if (e > 0.0) dd += e * e;
      else {
        const double e1 = a.xmm[i] - b.xmm[i + 3];
        if (e1 > 0.0) dd += e1 * e1;
      }
    }
    if (d2 < T.eta2 * dd) return true;
    // weak admissibility: boxes whose faces coincide in all three directions
    const bool t0 = a.xmm[3] == b.xmm[0] || b.xmm[3] == a.xmm[0];
    const bool t1 = a.xmm[4] == b.xmm[1] || b.xmm[4] == a.xmm[1];
    const bool t2 = a.xmm[5] == b.xmm[2] || b.xmm[5] == a.xmm[2];
    return t0 && t1 && t2;
  }

  void push_leaf(int32_t ia, int32_t ib, bool adm) {
    const ClusterNode& a = T.nodes[ia];
    const ClusterNode& b = T.nodes[ib];
    Leaf L;
    L.b1 = a.nbeg;
    L.n1 = a.nend - a.nbeg;
    L.b2 = b.nbeg;
    L.n2 = b.nend - b.nbeg;
    L.adm = adm ? 1u : 0u;
    L.idx = (uint32_t)T.leaves.size();
    // bbx trees have no centroid index: their ACA starts at the block's first row
    L.i0 = (adm && T.kind == kTreePca) ? a.icom - a.nbeg : 0u;
    L.row_cl = ia;
    L.col_cl = ib;
    T.leaves.push_back(L);
  }

  // cluster/blcluster.cpp:90-113: diagonal blocks recurse symmetrically, the
  // blocks above them are general subtrees, the blocks below are absent
  void subdivide_sym(int32_t ia) {
    const ClusterNode& a = T.nodes[ia];
    if (a.son[0] >= 0) {
      const int32_t s0 = a.son[0], s1 = a.son[1];
      subdivide_sym(s0);
      subdivide(s0, s1);
      subdivide_sym(s1);
    } else {
      push_leaf(ia, ia, false);
    }
  }

  // cluster/blcluster.cpp:40-66
  void subdivide(int32_t ia, int32_t ib) {
    if (isadm(T.nodes[ia], T.nodes[ib])) {
      push_leaf(ia, ib, true);
      return;
    }
    const ClusterNode& a = T.nodes[ia];
    const ClusterNode& b = T.nodes[ib];
    if (a.son[0] >= 0 && b.son[0] >= 0) {
      const int32_t as[2] = {a.son[0], a.son[1]};
      const int32_t bs[2] = {b.son[0], b.son[1]};
      for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j) subdivide(as[i], bs[j]);
    } else {
      push_leaf(ia, ib, false);
    }
  }
};

}  // namespace

void build_tree(Tree& T, const double* pts, uint32_t n, int kind, uint32_t bmin, double eta2, bool sym) {
  T.n = n;
  T.sym = sym;
  T.kind = kind;
  T.bmin = bmin;
  T.eta2 = eta2;
  T.pts.assign(pts, pts + 3 * (size_t)n);
  T.op_perm.resize(n);
  T.po_perm.resize(n);
  for (uint32_t i = 0; i < n; ++i) T.op_perm[i] = T.po_perm[i] = i;
  T.nodes.clear();
  T.leaves.clear();
  T.nodes.reserve(4 * (n / (bmin ? bmin : 1) + 1));
  Builder B{T, T.pts.data()};
  int32_t root = B.add_node(0, n, 0);
  if (kind == kTreeBbx) {
    B.bbx_init(T.nodes[root]);
    B.bbx_tree(root);
  } else {
    B.pca_init(T.nodes[root]);
    B.pca_tree(root);
  }
  if (sym) B.subdivide_sym(root);
  else B.subdivide(root, root);
}

void leaf_features(const Tree& T, const Leaf& L, double wavenumber, double eps, float out[8]) {
  const ClusterNode& a = T.nodes[L.row_cl];
  const ClusterNode& b = T.nodes[L.col_cl];
  double ca[3], cb[3];
  for (int j = 0; j < 3; ++j) {
    ca[j] = T.kind == kTreePca ? a.com[j] : 0.5 * (a.xmm[j] + a.xmm[j + 3]);
    cb[j] = T.kind == kTreePca ? b.com[j] : 0.5 * (b.xmm[j] + b.xmm[j + 3]);
  }
  const double dist = std::sqrt((ca[0] - cb[0]) * (ca[0] - cb[0]) + (ca[1] - cb[1]) * (ca[1] - cb[1]) +
                                (ca[2] - cb[2]) * (ca[2] - cb[2]));
  const double da = std::sqrt(a.diam2), db = std::sqrt(b.diam2);
  // a block on the diagonal has distance 0: floor it at 1e-6 of the larger
  // diameter so that every feature stays finite
  const double tiny = 1e-300;
  const double dfl = std::max(dist, std::max(1e-6 * std::max(da, db), tiny));
  out[0] = (float)std::log(std::max(da, tiny));
  out[1] = (float)std::log(std::max(db, tiny));
  out[2] = (float)std::log(dfl);
  out[3] = (float)(std::min(da, db) / dfl);
  out[4] = (float)std::log((double)L.n1);
  out[5] = (float)std::log((double)L.n2);
  out[6] = (float)(wavenumber * std::max(da, db));
  out[7] = (float)(-std::log10(eps));
}

double mean_nn(const double* pts, uint32_t n, double* min_out) {
  if (min_out) *min_out = 0.0;
  if (n < 2) return 0.0;
  double lo[3], hi[3];
  for (int j = 0; j < 3; ++j) lo[j] = hi[j] = pts[j];
  for (uint32_t i = 1; i < n; ++i)
    for (int j = 0; j < 3; ++j) {
      lo[j] = std::min(lo[j], pts[3 * (size_t)i + j]);
      hi[j] = std::max(hi[j], pts[3 * (size_t)i + j]);
    }
  double ext = 0.0;
  for (int j = 0; j < 3; ++j) ext = std::max(ext, hi[j] - lo[j]);
  int g = (int)std::ceil(std::cbrt((double)n));
  if (g < 1) g = 1;
  const double cs = ext > 0.0 ? ext / g * (1.0 + 1e-12) : 1.0;
  const size_t ncell = (size_t)g * g * g;
  std::vector<uint32_t> start(ncell + 1, 0), list(n);
  std::vector<int> cell(3 * (size_t)n);
  for (uint32_t i = 0; i < n; ++i) {
    for (int j = 0; j < 3; ++j) {
      int cc = (int)((pts[3 * (size_t)i + j] - lo[j]) / cs);
      cell[3 * (size_t)i + j] = std::min(std::max(cc, 0), g - 1);
    }
    const size_t id = ((size_t)cell[3 * i] * g + cell[3 * i + 1]) * g + cell[3 * i + 2];
    start[id + 1]++;
  }
  for (size_t q = 0; q < ncell; ++q) start[q + 1] += start[q];
  std::vector<uint32_t> fill(start.begin(), start.end() - 1);
  for (uint32_t i = 0; i < n; ++i) {
    const size_t id = ((size_t)cell[3 * i] * g + cell[3 * i + 1]) * g + cell[3 * i + 2];
    list[fill[id]++] = i;
  }
  std::vector<double> dmin(n);
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t ii = 0; ii < (int64_t)n; ++ii) {
    const uint32_t i = (uint32_t)ii;
    const int* ci = &cell[3 * (size_t)i];
    const double* pi = pts + 3 * (size_t)i;
    double best = INFINITY;
    for (int s = 0; s <= g; ++s) {
      for (int a = ci[0] - s; a <= ci[0] + s; ++a) {
        if (a < 0 || a >= g) continue;
        for (int b = ci[1] - s; b <= ci[1] + s; ++b) {
          if (b < 0 || b >= g) continue;
          for (int q = ci[2] - s; q <= ci[2] + s; ++q) {
            if (q < 0 || q >= g) continue;
            if (std::max(std::max(std::abs(a - ci[0]), std::abs(b - ci[1])), std::abs(q - ci[2])) != s)
              continue;
            const size_t id = ((size_t)a * g + b) * g + q;
            for (uint32_t t = start[id]; t < start[id + 1]; ++t) {
              const uint32_t jj = list[t];
              if (jj == i) continue;
              const double* pj = pts + 3 * (size_t)jj;
              const double dx = pi[0] - pj[0], dy = pi[1] - pj[1], dz = pi[2] - pj[2];
              const double d2 = dx * dx + dy * dy + dz * dz;
              if (d2 < best) best = d2;
            }
          }
        }
      }
      const double r = (double)s * cs;
      if (best <= r * r) break;
    }
    dmin[i] = std::sqrt(best);
  }
  double sum = 0.0, mn = INFINITY;
  for (uint32_t i = 0; i < n; ++i) {
    sum += dmin[i];
    mn = std::min(mn, dmin[i]);
  }
  if (min_out) *min_out = mn;
  return sum / n;
}

}  // namespace ahx
