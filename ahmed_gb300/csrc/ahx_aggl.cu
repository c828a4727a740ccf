// Agglomeration of an assembled H-matrix: agglH (H/agglH.cpp:111-272), the
// recmpr branch of matgenGeH_sqntl (Include/matgen_sqntl.h:32-55, 88-102).
//
// Bottom up, a block that is not diagonal and whose sons are all leaves is
// replaced by one low-rank leaf when the recompressed union of its sons
// (unify_sons_, H/agglH.cpp:14-107: relative threshold eps, at most max_rank)
// stores no more than the sons did.  The block tree is rebuilt from the
// cluster tree; the candidates of one height are merged as one batch on the
// GPU (factors gathered into workspaces, QR + SVD recompression per block);
// the merged leaf takes its first son's index and the indices are then
// compacted like fill_gaps_ (H/agglH.cpp:185-211).  The leaf arena is
// rewritten in leaf order.
//
// A dense son D enters a union in factored form D I^T (its columns as U, an
// identity as V), so that every union is one QR + SVD recompression of
// [U_cat][V_cat]^T; the reference forms the dense block and takes its SVD
// (mblock::unify_cols, H/mblock_D.cpp:804-860) with the same truncation rule.
// As in the reference, the sons are united pairwise: the two sons of each
// block row first (unify_cols), then the two truncated block rows (unify_rows),
// with a truncation after each step.  Unions wider than kMaxUnion columns are
// not formed.
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "ahx_aca.cuh"
#include "ahx_hmat.hpp"

namespace ahx {
namespace {

constexpr uint32_t kMaxUnion = 1024;

struct BNode {
  uint32_t b1, n1, b2, n2;
  int32_t rc, cc;
  int32_t son[4];  // row-major 2 x 2 (son[2 i + j]); -1: absent
  int32_t leaf;    // leaf index while a leaf, else -1
  bool dbl;        // diagonal block (never merged)
  bool decided;    // tried (merged or kept)
};

struct TreeBuilder {
  const Tree& T;
  std::vector<BNode> nodes;
  uint32_t next_leaf = 0;
  bool failed = false;  // the leaves are not those of the cluster tree's block tree

  int32_t add(int32_t ia, int32_t ib) {
    const ClusterNode& a = T.nodes[ia];
    const ClusterNode& b = T.nodes[ib];
    BNode n{};
    n.b1 = a.nbeg;
    n.n1 = a.nend - a.nbeg;
    n.b2 = b.nbeg;
    n.n2 = b.nend - b.nbeg;
    n.rc = ia;
    n.cc = ib;
    n.son[0] = n.son[1] = n.son[2] = n.son[3] = -1;
    n.leaf = -1;
    n.dbl = n.b1 == n.b2;
    n.decided = false;
    nodes.push_back(n);
    return (int32_t)nodes.size() - 1;
  }
  // the recursion of Tree's own builder: its leaves come out in leaf order
  int32_t general(int32_t ia, int32_t ib) {
    const int32_t id = add(ia, ib);
    const uint32_t l = next_leaf;
    if (l < T.leaves.size() && T.leaves[l].row_cl == ia && T.leaves[l].col_cl == ib) {
      nodes[id].leaf = (int32_t)next_leaf++;
      return id;
    }
    const ClusterNode& a = T.nodes[ia];
    const ClusterNode& b = T.nodes[ib];
    if (failed || a.son[0] < 0 || b.son[0] < 0) {
      failed = true;
      return id;
    }
    const int32_t as[2] = {a.son[0], a.son[1]}, bs[2] = {b.son[0], b.son[1]};
    for (int i = 0; i < 2; ++i)
      for (int j = 0; j < 2; ++j) {
        const int32_t s = general(as[i], bs[j]);
        nodes[id].son[2 * i + j] = s;
      }
    return id;
  }
  int32_t sym(int32_t ia) {
    const int32_t id = add(ia, ia);
    const uint32_t l = next_leaf;
    if (l < T.leaves.size() && T.leaves[l].row_cl == ia && T.leaves[l].col_cl == ia) {
      nodes[id].leaf = (int32_t)next_leaf++;
      return id;
    }
    const ClusterNode& a = T.nodes[ia];
    if (failed || a.son[0] < 0) {
      failed = true;
      return id;
    }
    const int32_t s0 = sym(a.son[0]);
    nodes[id].son[0] = s0;
    const int32_t s1 = general(a.son[0], a.son[1]);
    nodes[id].son[1] = s1;
    const int32_t s3 = sym(a.son[1]);
    nodes[id].son[3] = s3;
    return id;
  }
};

}  // namespace
}  // namespace ahx

using namespace ahx;

namespace {

// cplx: the Helmholtz (mblock<dcomp>) leaves, two doubles per element; the block
// tree changes, so the other kind of leaves of the handle is dropped.
int agglomerate_impl(ahx_hmat* H, double eps, uint32_t max_rank, uint32_t* nmerged, bool cplx) {
  if (!H || !(eps >= 0.0)) return AHX_ERR_ARG;
  if (!(cplx ? H->z.assembled : H->assembled)) {
    set_error("agglomerate: H-matrix not assembled");
    return AHX_ERR_STATE;
  }
  int rc = ensure_device(H);
  if (rc) return rc;
  Tree& T = H->tree;
  if (T.nodes.empty() || T.leaves.empty()) return AHX_OK;
  // the block tree of the current leaves (the root is the node of cluster 0 with itself)
  TreeBuilder B{T};
  const int32_t root = T.sym ? B.sym(0) : B.general(0, 0);
  if (B.failed || B.next_leaf != T.leaves.size()) {
    set_error("ahx_agglomerate: the leaves do not form the block tree (agglomerate once per assembly)");
    return AHX_ERR_STATE;
  }
  std::vector<BNode>& N = B.nodes;
  const uint32_t nl0 = (uint32_t)T.leaves.size();
  // leaf state, indexed by the reference's leaf index (idx)
  std::vector<int32_t> rank(cplx ? H->z.rank : H->rank);
  std::vector<uint64_t> off(cplx ? H->z.off : H->off);
  const uint64_t ew = cplx ? 2 : 1;  // doubles per element
  auto arena = [&]() -> double* { return cplx ? H->z.arena.as<double>() : H->arena64.as<double>(); };
  std::vector<int32_t> leaf_node(nl0, -1);
  for (int32_t i = 0; i < (int32_t)N.size(); ++i)
    if (N[i].leaf >= 0) leaf_node[N[i].leaf] = i;
  auto size_of = [&](int32_t leaf) -> uint64_t {
    const BNode& q = N[leaf_node[leaf]];
    const int32_t r = rank[leaf];
    return r < 0 ? (uint64_t)q.n1 * q.n2 : (uint64_t)r * (q.n1 + q.n2);
  };
  // columns of a union's factored form: the sons' ranks and the widths of dense
  // sons; a union of four dense sons is the parent block itself (n2 columns)
  auto dense_sons = [&](const BNode& q) -> bool {
    for (int s = 0; s < 4; ++s)
      if (rank[N[q.son[s]].leaf] >= 0) return false;
    return true;
  };
  auto union_width = [&](const BNode& q) -> uint32_t {
    if (dense_sons(q)) return q.n2;
    uint32_t k = 0;
    for (int s = 0; s < 4; ++s) {
      const BNode& c = N[q.son[s]];
      k += rank[c.leaf] < 0 ? c.n2 : (uint32_t)rank[c.leaf];
    }
    return k;
  };
  uint32_t merged = 0;
  ScopedBuf ws, zs, dtasks, dres, dsegs, dcopy;
  const size_t budget = aca_ws_budget();
  const char* tr = std::getenv("AHX_TRACE");
  const bool trace = tr && *tr && *tr != '0';
  int round = 0;
  for (;;) {
    const auto t0 = std::chrono::steady_clock::now();
    const uint32_t merged0 = merged;
    // candidates of this height: undecided, not diagonal, all sons leaves
    std::vector<int32_t> cand;
    for (int32_t i = 0; i < (int32_t)N.size(); ++i) {
      BNode& q = N[i];
      if (q.leaf >= 0 || q.decided || q.dbl) continue;
      bool all_leaves = true;
      for (int s = 0; s < 4; ++s) {
        if (q.son[s] < 0 || N[q.son[s]].leaf < 0) {
          all_leaves = false;
          break;
        }
      }
      if (!all_leaves) continue;
      if (union_width(q) > kMaxUnion) {
        q.decided = true;
        continue;
      }
      cand.push_back(i);
    }
    if (cand.empty()) break;
    uint64_t kmax_round = 0;
    // union widths (columns of the factored union)
    auto width = [&](int32_t c) -> uint32_t { return union_width(N[c]); };
    // batches under the workspace budget: one warp per union, one CTA for unions
    // wider than 64 columns (the SVD's column pairs in parallel) or blocks over 4096
    // rows; the costliest first so that they spread over the SMs
    std::vector<uint64_t> cost(N.size(), 0);
    for (int32_t c : cand) {
      const uint64_t w = width(c);
      cost[c] = w * w * (N[c].n1 + N[c].n2);
    }
    // a warp per union hides its loads' latency only among many unions: a round of
    // fewer unions than warp slots runs its unions of more than 256 rows on CTAs
    const bool few = cand.size() < 8u * 152u;
    std::vector<int32_t> parts[2];
    for (int32_t c : cand) {
      const uint32_t rows = std::max(N[c].n1, N[c].n2);
      parts[(width(c) > 64u || rows > 4096u || (few && rows > 256u)) ? 1 : 0].push_back(c);
    }
    for (int large = 0; large < 2; ++large) {
      std::vector<int32_t>& todo = parts[large];
      std::stable_sort(todo.begin(), todo.end(), [&](int32_t a, int32_t b) { return cost[a] > cost[b]; });
      size_t at = 0;
      while (at < todo.size()) {
        // Pairwise unions as the reference's unify_sons_ (H/agglH.cpp:40-86):
        // phase A unites the sons of each block row (unify_cols: [U0 U1],
        // diag(V0, V1), a dense son as (D, I)) and truncates; phase B unites the
        // two truncated block rows (unify_rows: diag(U_top, U_bot), [V_top V_bot])
        // and truncates again.  Both phases run as batches of merge tasks.
        std::vector<MergeTask> tasksA, tasksB;
        std::vector<Seg2D> segsA;
        std::vector<int32_t> which;
        std::vector<int32_t> pairA[2];  // per candidate: its phase-A task (-1: empty pair)
        uint64_t wszA = 0, zszA = 0, wszB = 0, zszB = 0;
        const uint32_t e32 = (uint32_t)ew;
        for (; at < todo.size(); ++at) {
          const BNode& q = N[todo[at]];
          uint32_t kp[2] = {0, 0};
          for (int i = 0; i < 2; ++i)
            for (int j = 0; j < 2; ++j) {
              const BNode& c = N[q.son[2 * i + j]];
              kp[i] += rank[c.leaf] < 0 ? c.n2 : (uint32_t)rank[c.leaf];
            }
          const uint32_t m0 = N[q.son[0]].n1, m1 = N[q.son[2]].n1;
          const uint64_t needA = aca_ws_doubles(m0, q.n2, std::max(kp[0], 1u)) + merge_qrcp_doubles(kp[0]) +
                                 aca_ws_doubles(m1, q.n2, std::max(kp[1], 1u)) + merge_qrcp_doubles(kp[1]);
          const uint32_t kb = std::min(kp[0] + kp[1], 2 * max_rank);
          const uint64_t needB = aca_ws_doubles(q.n1, q.n2, std::max(kb, 1u)) + merge_qrcp_doubles(kb);
          if (!which.empty() && (wszA + needA + wszB + needB) * ew * sizeof(double) > budget) break;
          kmax_round = std::max<uint64_t>(kmax_round, std::max(kp[0], kp[1]));
          for (int i = 0; i < 2; ++i) {
            if (kp[i] == 0) {
              pairA[i].push_back(-1);
              continue;
            }
            const uint32_t m = i ? m1 : m0, k = kp[i];
            const uint32_t rb = N[q.son[2 * i]].b1;  // first row of this block row
            MergeTask t{m, q.n2, k, 0u, wszA, zszA};
            uint32_t col = 0;
            for (int j = 0; j < 2; ++j) {
              const BNode& c = N[q.son[2 * i + j]];
              const bool dense = rank[c.leaf] < 0;
              const uint32_t kc = dense ? c.n2 : (uint32_t)rank[c.leaf];
              if (kc == 0) continue;
              const uint32_t ro = c.b1 - rb, co = c.b2 - q.b2;
              const uint64_t o = off[c.leaf];
              const uint64_t vdst = wszA + (uint64_t)m * k + (uint64_t)col * q.n2 + co;
              segsA.push_back(Seg2D{o * ew, (wszA + (uint64_t)col * m + ro) * ew, c.n1 * e32, kc, m * e32, 0u});
              if (dense) segsA.push_back(Seg2D{kSegIdentity, vdst * ew, kc, kc, q.n2 * e32, cplx ? 1u : 0u});
              else segsA.push_back(Seg2D{(o + (uint64_t)c.n1 * kc) * ew, vdst * ew, c.n2 * e32, kc, q.n2 * e32, 0u});
              col += kc;
            }
            pairA[i].push_back((int32_t)tasksA.size());
            tasksA.push_back(t);
            wszA += aca_ws_doubles(m, q.n2, std::max(k, 1u)) + merge_qrcp_doubles(k);
            zszA += m + q.n2 + 1;
          }
          which.push_back(todo[at]);
          wszB += needB;
          zszB += q.n1 + q.n2 + 1;
        }
        auto run_merge = [&](ScopedBuf& w, uint64_t wsz, uint64_t zsz, std::vector<MergeTask>& tasks,
                             std::vector<Seg2D>& segs, const double* src,
                             std::vector<AcaResult>& res) -> int {
          res.assign(tasks.size(), AcaResult{});
          if (tasks.empty()) return AHX_OK;
          int r;
          if ((r = w.reserve(std::max<uint64_t>(wsz, 1) * ew * sizeof(double)))) return r;
          if ((r = zs.reserve(std::max<uint64_t>(zsz, 1) * sizeof(int)))) return r;
          AHX_CUDA(cudaMemsetAsync(w.p, 0, wsz * ew * sizeof(double), H->stream));
          if ((r = upload(dsegs, segs, H->stream))) return r;
          AHX_CUDA(launch_copy2d(dsegs.as<Seg2D>(), (uint32_t)segs.size(), src, w.as<double>(), H->stream));
          if ((r = upload(dtasks, tasks, H->stream))) return r;
          if ((r = dres.reserve(tasks.size() * sizeof(AcaResult)))) return r;
          MergeParams p;
          p.tasks = dtasks.as<MergeTask>();
          p.ntasks = (uint32_t)tasks.size();
          p.ws = w.as<double>();
          p.zs = zs.as<int>();
          p.eps = eps;
          p.res = dres.as<AcaResult>();
          AHX_CUDA(cplx ? launch_zmerge(p, H->stream) : launch_merge(p, large == 1, H->stream));
          AHX_CUDA(cudaMemcpyAsync(res.data(), dres.p, res.size() * sizeof(AcaResult), cudaMemcpyDeviceToHost,
                                   H->stream));
          AHX_CUDA(cudaStreamSynchronize(H->stream));
          return AHX_OK;
        };
        std::vector<AcaResult> resA, resB;
        if ((rc = run_merge(ws, wszA, zszA, tasksA, segsA, arena(), resA))) return rc;
        // phase B: gather the truncated block rows (first kt columns of Un, Vn)
        std::vector<Seg2D> segsB;
        std::vector<int32_t> taskB(which.size(), -1);
        uint64_t offB = 0;
        for (size_t w = 0; w < which.size(); ++w) {
          const BNode& q = N[which[w]];
          uint32_t kt[2] = {0, 0};
          for (int i = 0; i < 2; ++i)
            if (pairA[i][w] >= 0) kt[i] = std::min(resA[pairA[i][w]].kt, max_rank);
          const uint32_t k = kt[0] + kt[1];
          const uint64_t needB = aca_ws_doubles(q.n1, q.n2, std::max(k, 1u)) + merge_qrcp_doubles(k);
          if (k > 0) {
            MergeTask t{q.n1, q.n2, k, 0u, offB, 0u};
            uint32_t col = 0;
            for (int i = 0; i < 2; ++i) {
              if (kt[i] == 0) continue;
              const MergeTask& ta = tasksA[pairA[i][w]];
              const uint64_t un = ta.ws + (uint64_t)(ta.m + ta.n) * ta.k;  // Un (m x k), then Vn (n x k)
              const uint64_t vn = un + (uint64_t)ta.m * ta.k;
              const uint32_t ro = i ? N[q.son[0]].n1 : 0u;
              segsB.push_back(Seg2D{un * ew, (offB + (uint64_t)col * q.n1 + ro) * ew, ta.m * e32, kt[i],
                                    q.n1 * e32, 0u});
              segsB.push_back(Seg2D{vn * ew, (offB + (uint64_t)q.n1 * k + (uint64_t)col * q.n2) * ew,
                                    q.n2 * e32, kt[i], q.n2 * e32, 0u});
              col += kt[i];
            }
            taskB[w] = (int32_t)tasksB.size();
            tasksB.push_back(t);
          }
          offB += needB;
        }
        // zs offsets of phase B
        {
          uint64_t z = 0;
          for (MergeTask& t : tasksB) {
            t.zs = z;
            z += t.m + t.n + 1;
          }
          zszB = z;
        }
        ScopedBuf wsB;
        if ((rc = run_merge(wsB, offB, zszB, tasksB, segsB, ws.as<double>(), resB))) return rc;
        std::vector<CopyTask> copies;
        for (size_t w = 0; w < which.size(); ++w) {
          BNode& nd = N[which[w]];
          nd.decided = true;
          const uint32_t kt = taskB[w] >= 0 ? std::min(resB[taskB[w]].kt, max_rank) : 0u;
          uint64_t pre = 0;
          for (int s = 0; s < 4; ++s) pre += size_of(N[nd.son[s]].leaf);
          const uint64_t post = (uint64_t)kt * (nd.n1 + nd.n2);
          if (pre < post) continue;  // H/agglH.cpp:86: merge when it does not cost more
          // the merged block takes its first son's index; the other sons' are freed
          const int32_t first = N[nd.son[0]].leaf;
          uint64_t dst = 0;
          if (post && (rc = cplx ? zarena_append(H, post, dst) : arena_append(H, post, dst))) return rc;
          if (post) {
            const MergeTask& t = tasksB[taskB[w]];
            const uint64_t un = t.ws + (uint64_t)(t.m + t.n) * t.k;  // Un follows U and V
            copies.push_back(CopyTask{un * ew, (un + (uint64_t)t.m * t.k) * ew, dst * ew, t.m * e32, t.n * e32, kt, 0u});
          }
          rank[first] = (int32_t)kt;
          off[first] = dst;
          leaf_node[first] = which[w];
          nd.leaf = first;
          ++merged;
        }
        if (!copies.empty()) {
          if ((rc = upload(dcopy, copies, H->stream))) return rc;
          AHX_CUDA(launch_copy_factors(dcopy.as<CopyTask>(), (uint32_t)copies.size(), wsB.as<double>(), arena(),
                                       H->stream));
          AHX_CUDA(cudaStreamSynchronize(H->stream));
        }
      }
    }
    if (trace) {
      const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
      std::fprintf(stderr, "ahx agglomerate round %d: %zu unions tried, %u merged, widest union %llu, %.1f ms\n",
                   round, cand.size(), merged - merged0, (unsigned long long)kmax_round, ms);
    }
    ++round;
  }
  for (ScopedBuf* b : {&ws, &zs, &dtasks, &dres, &dsegs, &dcopy}) b->release();
  (void)round;
  if (nmerged) *nmerged = merged;
  if (!merged) return AHX_OK;
  // fill_gaps_ (H/agglH.cpp:185-211): in DFS order, leaves whose index is past the new
  // count move to the lowest free index
  std::vector<int32_t> dfs;  // leaf indices of the final tree in DFS order
  {
    std::vector<int32_t> stack{root};
    while (!stack.empty()) {
      const int32_t i = stack.back();
      stack.pop_back();
      const BNode& q = N[i];
      if (q.leaf >= 0) {
        dfs.push_back(q.leaf);
        continue;
      }
      for (int s = 3; s >= 0; --s)
        if (q.son[s] >= 0) stack.push_back(q.son[s]);
    }
  }
  const uint32_t nnew = (uint32_t)dfs.size();
  std::vector<uint8_t> taken(nl0, 0);
  for (int32_t l : dfs)
    if ((uint32_t)l < nnew) taken[l] = 1;
  std::vector<int32_t> final_idx(nl0, -1);
  uint32_t gap = 0;
  for (int32_t l : dfs) {
    if ((uint32_t)l < nnew) {
      final_idx[l] = l;
    } else {
      while (taken[gap]) ++gap;
      taken[gap] = 1;
      final_idx[l] = (int32_t)gap;
    }
  }
  // new leaf list in index order; the arena rewritten in that order
  std::vector<Leaf> leaves(nnew);
  std::vector<int32_t> nrank(nnew);
  std::vector<uint64_t> noff(nnew);
  std::vector<CopyTask> moves;
  uint64_t total = 0;
  std::vector<int32_t> at_idx(nnew, -1);
  for (int32_t l : dfs) at_idx[final_idx[l]] = l;
  for (uint32_t k = 0; k < nnew; ++k) {
    const int32_t l = at_idx[k];
    const BNode& q = N[leaf_node[l]];
    Leaf L{};
    if ((uint32_t)l < nl0 && leaf_node[l] >= 0 && N[leaf_node[l]].son[0] < 0) {
      L = T.leaves[l];  // an original leaf
    } else {
      L.b1 = q.b1;
      L.n1 = q.n1;
      L.b2 = q.b2;
      L.n2 = q.n2;
      L.adm = 0;  // the merged block keeps its (inadmissible) tree flag
      L.i0 = 0;
      L.row_cl = q.rc;
      L.col_cl = q.cc;
    }
    L.idx = k;
    leaves[k] = L;
    nrank[k] = rank[l];
    const uint64_t cnt = rank[l] < 0 ? (uint64_t)q.n1 * q.n2 : (uint64_t)rank[l] * (q.n1 + q.n2);
    noff[k] = total;
    if (cnt) {
      // dense: n1 x n2 as "U" with kt = n2 columns and an empty "V" (doubles: ew per element)
      const uint32_t e32 = (uint32_t)ew;
      if (rank[l] < 0)
        moves.push_back(CopyTask{off[l] * ew, off[l] * ew, total * ew, q.n1 * e32, 0u, q.n2, 0u});
      else
        moves.push_back(CopyTask{off[l] * ew, (off[l] + (uint64_t)q.n1 * rank[l]) * ew, total * ew, q.n1 * e32,
                                 q.n2 * e32, (uint32_t)rank[l], 0u});
    }
    total += cnt;
  }
  DevBuf fresh;
  ScopedBuf dm;
  if ((rc = fresh.reserve(std::max<uint64_t>(total, 1) * ew * sizeof(double)))) return rc;
  if ((rc = upload(dm, moves, H->stream))) {
    fresh.release();
    return rc;
  }
  {
    cudaError_t e = launch_copy_factors(dm.as<CopyTask>(), (uint32_t)moves.size(), arena(), fresh.as<double>(),
                                        H->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(H->stream);
    if (e != cudaSuccess) {
      fresh.release();
      return cuda_fail(e, "agglomerate: arena compaction");
    }
  }
  T.leaves = leaves;
  if (cplx) {
    ZState& Z = H->z;
    Z.arena.release();
    Z.arena = fresh;
    Z.elems = total;
    Z.valid32 = Z.table = false;
    Z.arena32.release();
    Z.rank = nrank;
    Z.aca_rank = nrank;
    Z.off = noff;
    // the real leaves belong to the old block tree
    invalidate_products(H);
    H->assembled = false;
    H->rank.clear();
    H->aca_rank.clear();
    H->off.clear();
  } else {
    H->arena64.release();
    H->arena64 = fresh;
    H->arena64_elems = total;
    invalidate_products(H);
    H->rank = nrank;
    H->aca_rank = nrank;
    H->off = noff;
    H->z.release_all();  // Helmholtz leaves of the old block tree
  }
  return AHX_OK;
}

}  // namespace

extern "C" int ahx_agglomerate(ahx_hmat* H, double eps, uint32_t max_rank, uint32_t* nmerged) {
  return agglomerate_impl(H, eps, max_rank, nmerged, false);
}

extern "C" int ahx_helm_agglomerate(ahx_hmat* H, double eps, uint32_t max_rank, uint32_t* nmerged) {
  return agglomerate_impl(H, eps, max_rank, nmerged, true);
}
