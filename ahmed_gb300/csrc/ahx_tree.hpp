// Host-side cluster trees and block-cluster trees of the H-matrix.
//
// These reproduce the reference's trees bit for bit (same floating-point
// expressions in the same order; the file is compiled with -ffp-contract=off):
//   bounding-box bisection   Include/cluster_bbx.h:33-128, 245-297
//   PCA bisection            Include/cluster_pca.h:54-217, Include/bemcluster.h:25-50
//   block-cluster tree       cluster/blcluster.cpp:40-66 (DFS leaf numbering)
//   leaf sequence            parallel/gen_blseq.cpp:15-75
#pragma once
#include <cstdint>
#include <vector>

namespace ahx {

enum TreeKind : int { kTreeBbx = 0, kTreePca = 1 };

struct ClusterNode {
  uint32_t nbeg, nend;
  int32_t son[2];  // -1: none
  double diam2;
  double com[3];   // PCA centre of mass
  uint32_t icom;   // PCA: centroid-nearest index (reference numbering quirk)
  double xmm[6];   // bbx: min[3], max[3]
  uint32_t maindir;
  double cntrdir;
  uint32_t level;
};

struct Leaf {
  uint32_t b1, n1, b2, n2;
  uint32_t adm;
  uint32_t idx;
  uint32_t i0;         // ACA start row relative to b1
  int32_t row_cl, col_cl;
};

struct Tree {
  uint32_t n = 0;
  int kind = kTreeBbx;
  uint32_t bmin = 0;
  double eta2 = 0.0;
  bool sym = false;                 // symmetric (HeH) block tree
  std::vector<double> pts;          // original order, xyz interleaved
  std::vector<uint32_t> op_perm;    // permuted -> original
  std::vector<uint32_t> po_perm;    // original -> permuted
  std::vector<ClusterNode> nodes;   // nodes[0] = root
  std::vector<Leaf> leaves;         // DFS order == idx order
};

// Builds the cluster tree over `pts` (3*n doubles, original order) and the
// block-cluster tree with the admissibility parameter eta2 (= eta^2).
// sym: the symmetric block tree (blcluster::subdivide_sym): diagonal and upper blocks only
void build_tree(Tree& T, const double* pts, uint32_t n, int kind, uint32_t bmin, double eta2,
                bool sym = false);

// Mean nearest-neighbour distance (exact; uniform-grid search; deterministic
// sum order); *min_out (if given) receives the smallest one.
double mean_nn(const double* pts, uint32_t n, double* min_out = nullptr);

// Geometric features of a leaf for the rank predictor (8 floats):
//   log diam(row cluster), log diam(col cluster), log centre distance,
//   min(diam) / distance, log n1, log n2, wavenumber * max(diam), -log10(eps)
// diam = sqrt(diam2) of the cluster (Include/cluster.h:194); centres are the
// PCA centres of mass or the bounding-box centres.
void leaf_features(const Tree& T, const Leaf& L, double wavenumber, double eps, float out[8]);

}  // namespace ahx
