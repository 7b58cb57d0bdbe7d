// inspect.cu -- host-side schedule inspectors for the load-balanced level
// coarsening (LBC) executors: the tree level set, the tree LBC, and the
// DAG LBC built from the elimination tree of L.
//
// The reference produces LBC schedules on the CPU in its ParSy inspector:
//   parsy::getLevelSet          sparse_blas/parsy/common/TreeUtils.cpp:89-140
//   parsy::getCoarseLevelSet_6  sparse_blas/parsy/symbolic/InspectionLevel_06.cpp:17-400
//     heightPartitioning        sparse_blas/parsy/common/TreeUtils.cpp:284-362
//     postOrderSpliting         sparse_blas/parsy/symbolic/PostOrderSpliting.cpp:13-142
//     worstFitBinPack           sparse_blas/parsy/common/TreeUtils.cpp:184-221
// and its demo calls get_coarse_levelSet_DAG_CSC_tree on the CSR of L
// (demo/sptrsv_demo_utils.h:78-90), a function of the unvendored
// aggregation dependency.  These are O(n + nnz) integer passes over the
// tree, run once per matrix, so they stay on the host.  The schedules
// must match the reference's bit for bit, so the steps are the
// reference's steps, including the choices that shape the output: which
// cut levels the height partitioning takes, the post-order walk's stack
// discipline, the worst-fit packing's tie order (the same std::sort on
// the same costs), and the packing's bin costs carrying over from one
// coarse level to the next.
//
// The DAG builder takes the elimination tree of the symmetric pattern of L
// (Liu's algorithm over the rows of L).  Every nonzero L_ij, i > j, has i
// as an ancestor of j in that tree, so a schedule that respects the tree
// respects every dependency of the solve.
#include <algorithm>
#include <climits>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <vector>

#include "gbsym.h"

namespace gbsym {
namespace {

// Level set of a forest, leaves first, ascending index within a level.
// The reference builds it by sweeps over a shrinking index window, each
// sweep taking in ascending order every node whose children earlier sweeps
// placed; so a node's level is 0 for a leaf and otherwise one more than its
// highest child.  With parent[v] > v every child precedes its parent, so
// one ascending pass finds the levels and a counting sort lists them: O(n)
// where the sweeps cost O(n * levels), which on the path-shaped
// elimination tree of a naturally ordered grid is quadratic.
int forest_levels(int n, const int *parent, int *lptr, int *lset) {
  std::vector<int> lev(n, 0);
  int nl = 0;
  for (int v = 0; v < n; ++v) {
    nl = std::max(nl, lev[v] + 1);
    if (parent[v] >= 0) lev[parent[v]] = std::max(lev[parent[v]], lev[v] + 1);
  }
  std::fill(lptr, lptr + nl + 1, 0);
  for (int v = 0; v < n; ++v) lptr[lev[v] + 1]++;
  for (int l = 0; l < nl; ++l) lptr[l + 1] += lptr[l];
  std::vector<int> fill(lptr, lptr + nl);
  for (int v = 0; v < n; ++v) lset[fill[lev[v]]++] = v;
  return nl;
}

// Largest depth (edges to the root) in a forest with parent[v] > v: one
// descending pass, each node one deeper than its parent.
int forest_height(int n, const int *parent) {
  std::vector<int> depth(n, 0);
  int h = 0;
  for (int v = n - 1; v >= 0; --v) {
    if (parent[v] >= 0) depth[v] = depth[parent[v]] + 1;
    h = std::max(h, depth[v]);
  }
  return h;
}

// Children lists of a forest (children in ascending index); nchild must be
// zero on entry and receives the child counts.
void child_lists(int n, const int *parent, std::vector<int> &cptr, std::vector<int> &cidx,
                 std::vector<int> &nchild) {
  for (int v = 0; v < n; ++v)
    if (parent[v] >= 0) nchild[parent[v]]++;
  cptr.assign(n + 1, 0);
  for (int v = 0; v < n; ++v) cptr[v + 1] = cptr[v] + nchild[v];
  cidx.assign(std::max(1, cptr[n]), 0);
  std::vector<int> fill(cptr.begin(), cptr.end() - 1);
  for (int v = 0; v < n; ++v)
    if (parent[v] >= 0) cidx[fill[parent[v]]++] = v;
}

// Cut levels of the tree into coarse levels (sw = false form): starting at
// the root end, skip levels no wider than the target part count, cut
// min_level_dist below, and divide the part count by div_rate for the next
// cut; the last coarse level reaches the root.
int height_cuts(int nlev, const int *lptr, int height, int inner_parts, int min_level_dist, int div_rate,
                std::vector<int> &parts_per_cut, std::vector<int> &cut) {
  cut.assign(nlev + 2, 0);
  if (nlev <= 2) {
    cut[1] = nlev;
    parts_per_cut.push_back(1);
    return 1;
  }
  std::vector<int> width(nlev);
  for (int l = 0; l < nlev; ++l) width[l] = lptr[l + 1] - lptr[l];
  int cnt = 0, parts = inner_parts;
  while (parts > 1) {
    int skip = 0;
    while (width[height - skip - 1] <= parts && skip < nlev) {
      ++skip;
      if (height - skip - 1 < 0 || height - skip - 1 >= nlev) break;
    }
    parts_per_cut.push_back(parts);
    const int c = height - skip - min_level_dist;
    if (c > cut[cnt] && c < nlev) cut[++cnt] = c;
    parts /= div_rate;
  }
  if (cnt + 1 >= (int)cut.size()) cut.resize(cnt + 2);
  cut[++cnt] = height + 1;
  parts_per_cut.push_back(1);
  return cnt;
}

// Split a forest (tree[v] == -2: not in it) into connected post-order
// pieces.  The work list is used from its front, and it outlives one start
// node: a walk that reaches a root stops there and leaves the rest of the
// list for the next start node.
void post_order_pieces(int n, const int *tree, const double *cost, const std::vector<int> &cptr,
                       const std::vector<int> &cidx, std::vector<int> &nchild, std::vector<double> &piece_cost,
                       std::vector<std::vector<int>> &pieces) {
  std::vector<char> visited(n, 0), mark(n, 0);
  std::deque<int> work;  // taken from the front; pushed at either end
  pieces.clear();
  pieces.emplace_back();
  int cur = 0;
  for (int start = 0; start < n; ++start) {
    if (tree[start] == -2 || visited[start]) continue;
    work.push_back(start);
    while (!work.empty()) {
      const int k = work[0];
      if (nchild[k] == 0) {
        work.pop_front();
        pieces[cur].push_back(k);
        piece_cost[cur] += cost[k];
        visited[k] = 1;
        const int p = tree[k];
        if (p < 0) break;
        nchild[p]--;
        if (!visited[p]) {
          if (!mark[p]) work.push_front(p);
          mark[p] = 1;
        }
      } else {
        for (int q = cptr[k]; q < cptr[k + 1]; ++q) {
          const int c = cidx[q];
          if (visited[c]) continue;
          if (nchild[c] == 0) {
            if (!visited[k]) {
              int a = k;
              if (!work.empty())
                while (a >= 0 && a != work.back()) {
                  mark[a] = 1;
                  a = tree[a];
                }
              if (a >= 0) mark[a] = 1;
            }
            pieces[cur].push_back(c);
            piece_cost[cur] += cost[c];
            visited[c] = 1;
            nchild[tree[c]]--;
          } else {
            work.push_front(c);
          }
        }
      }
    }
    ++cur;
    pieces.emplace_back();
  }
  pieces.pop_back();
}

// Worst-fit packing: pieces by decreasing cost (std::sort, as the
// reference sorts them) each go to the currently cheapest bin.  bin_cost
// is not cleared here: it carries the bins' totals from earlier calls.
void worst_fit(const std::vector<std::vector<int>> &pieces, const std::vector<double> &piece_cost,
               std::vector<double> &bin_cost, int nbins, std::vector<std::vector<int>> &bins) {
  struct Item {
    double cost;
    int idx;
  };
  std::vector<Item> order(pieces.size());
  for (size_t i = 0; i < pieces.size(); ++i) order[i] = Item{piece_cost[i], (int)i};
  std::sort(order.begin(), order.end(), [](const Item &a, const Item &b) { return a.cost > b.cost; });
  bins.assign(nbins, {});
  for (const Item &it : order) {
    double best = (double)INT_MAX;
    int b = 0;
    for (int j = 0; j < nbins; ++j)
      if (bin_cost[j] < best) {
        best = bin_cost[j];
        b = j;
      }
    bin_cost[b] += it.cost;
    bins[b].insert(bins[b].end(), pieces[it.idx].begin(), pieces[it.idx].end());
  }
}

// Tree LBC.  Outputs: level_ptr[level_no+1] into part_ptr, part_ptr[part_no+1]
// into node_ptr[n].  The arrays are sized n+1, n+1 and n.
int tree_lbc(int n, const int *parent, const double *cost, int inner_parts, int min_level_dist, int div_rate,
             int *level_ptr, int *part_ptr, int *node_ptr, int *part_no) {
  level_ptr[0] = 0;
  part_ptr[0] = 0;
  std::vector<int> nchild(n, 0);
  for (int v = 0; v < n; ++v)
    if (parent[v] >= 0) nchild[parent[v]]++;
  const int height = forest_height(n, parent);
  if (height == 0 && n == 1) {
    level_ptr[1] = 1;
    part_ptr[1] = 1;
    node_ptr[0] = 0;
    *part_no = 1;
    return 1;
  }
  std::vector<int> lptr(n + 1), lset(n), node_level(n);
  const int nlev = forest_levels(n, parent, lptr.data(), lset.data());
  for (int l = 0; l < nlev; ++l)
    for (int q = lptr[l]; q < lptr[l + 1]; ++q) node_level[lset[q]] = l;
  std::vector<double> level_cost(nlev, 0.0);
  for (int v = 0; v < n; ++v) level_cost[node_level[v]] += cost[v];

  std::vector<int> parts_per_cut, cut;
  const int ncut = height_cuts(nlev, lptr.data(), height, inner_parts, min_level_dist, div_rate, parts_per_cut, cut);

  std::vector<int> sub(n, -2), cptr, cidx, sub_nchild(n);
  std::vector<double> piece_cost(n, 0.0), bin_cost(n, 0.0);
  std::vector<std::vector<int>> pieces, bins;
  int nparts = 0;
  for (int l = 0; l < ncut; ++l) {
    const int parts = parts_per_cut[l];
    // the subforest of this coarse level: tree edges with both ends inside
    for (int lev = cut[l]; lev < cut[l + 1]; ++lev)
      for (int q = lptr[lev]; q < lptr[lev + 1]; ++q) {
        const int v = lset[q];
        const int p = parent[v];
        const int pl = p >= 0 ? node_level[p] : height + 1;
        sub[v] = (pl < cut[l + 1] && l + 1 <= ncut && pl >= cut[l]) ? p : -1;
      }
    std::fill(sub_nchild.begin(), sub_nchild.end(), 0);
    child_lists(n, sub.data(), cptr, cidx, sub_nchild);
    std::fill(piece_cost.begin(), piece_cost.end(), 0.0);
    post_order_pieces(n, sub.data(), cost, cptr, cidx, sub_nchild, piece_cost, pieces);
    const std::vector<std::vector<int>> *out = &pieces;
    if ((int)pieces.size() > parts) {
      worst_fit(pieces, piece_cost, bin_cost, parts_per_cut[l], bins);
      out = &bins;
    }
    level_ptr[l + 1] = level_ptr[l] + (int)out->size();
    for (const auto &part : *out) {
      int e = part_ptr[nparts];
      for (int v : part) node_ptr[e++] = v;
      part_ptr[nparts + 1] = e;
      ++nparts;
    }
    std::fill(sub.begin(), sub.end(), -2);
  }
  *part_no = nparts;
  return ncut;
}

// Elimination tree of the symmetric pattern whose lower triangle is the CSR
// of L (Liu's algorithm with path compression over the rows in order).
void etree_lower_csr(int n, const int *Lp, const int *Li, int *parent) {
  std::vector<int> anc(n, -1);
  for (int i = 0; i < n; ++i) {
    parent[i] = -1;
    for (int q = Lp[i]; q < Lp[i + 1]; ++q) {
      int j = Li[q];
      while (j != -1 && j < i) {
        const int next = anc[j];
        anc[j] = i;
        if (next == -1) parent[j] = i;
        j = next;
      }
    }
  }
}

bool forest_ok(int n, const int *parent) {
  for (int v = 0; v < n; ++v)
    if (parent[v] < -1 || parent[v] >= n || (parent[v] >= 0 && parent[v] <= v)) return false;
  return true;
}

bool csr_lower_ok(int n, const int *Lp, const int *Li) {
  if (Lp[0] != 0) return false;
  for (int i = 0; i < n; ++i) {
    if (Lp[i + 1] < Lp[i]) return false;
    for (int q = Lp[i]; q < Lp[i + 1]; ++q)
      if (Li[q] < 0 || Li[q] > i) return false;
  }
  return true;
}

template <class T>
T *host_array(size_t count) {
  return static_cast<T *>(std::malloc(sizeof(T) * std::max<size_t>(count, 1)));
}

int lbc_outputs(int n, const int *parent, const double *cost, int inner_parts, int min_level_dist, int div_rate,
                int *level_no, int **level_ptr, int *part_no, int **part_ptr, int **node_ptr) {
  int *lp = host_array<int>((size_t)n + 1), *pp = host_array<int>((size_t)n + 1), *np = host_array<int>(n);
  if (!lp || !pp || !np) {
    std::free(lp);
    std::free(pp);
    std::free(np);
    return GBSYM_ERR_SIZE;  // host allocation failed
  }
  int parts = 0;
  *level_no = tree_lbc(n, parent, cost, inner_parts, min_level_dist, div_rate, lp, pp, np, &parts);
  *part_no = parts;
  *level_ptr = lp;
  *part_ptr = pp;
  *node_ptr = np;
  return GBSYM_OK;
}

}  // namespace
}  // namespace gbsym

using namespace gbsym;

extern "C" int gbsym_etree_lower_csr(int n, const int *Lp, const int *Li, int *parent) {
  if (n < 0) return GBSYM_ERR_SIZE;
  if (n == 0) return GBSYM_OK;
  if (!Lp || !Li || !parent) return GBSYM_ERR_NULL_ARG;
  if (!csr_lower_ok(n, Lp, Li)) return GBSYM_ERR_BAD_MATRIX;
  etree_lower_csr(n, Lp, Li, parent);
  return GBSYM_OK;
}

extern "C" int gbsym_tree_levelset(int n, const int *parent, int *level_ptr, int *level_set) {
  if (n < 0) return -GBSYM_ERR_SIZE;
  if (n == 0) {
    if (level_ptr) level_ptr[0] = 0;
    return 0;
  }
  if (!parent || !level_ptr || !level_set) return -GBSYM_ERR_NULL_ARG;
  if (!forest_ok(n, parent)) return -GBSYM_ERR_BAD_SCHEDULE;
  return forest_levels(n, parent, level_ptr, level_set);
}

extern "C" int gbsym_coarse_levelset_tree(int n, const int *parent, const double *node_cost, int inner_parts,
                                          int min_level_dist, int div_rate, int *level_no, int **level_ptr,
                                          int *part_no, int **part_ptr, int **node_ptr) {
  if (!level_no || !level_ptr || !part_no || !part_ptr || !node_ptr) return GBSYM_ERR_NULL_ARG;
  *level_ptr = *part_ptr = *node_ptr = nullptr;
  *level_no = *part_no = 0;
  if (n < 0 || inner_parts < 1 || div_rate < 1) return GBSYM_ERR_SIZE;
  if (n == 0) return GBSYM_OK;
  if (!parent || !node_cost) return GBSYM_ERR_NULL_ARG;
  if (!forest_ok(n, parent)) return GBSYM_ERR_BAD_SCHEDULE;
  return lbc_outputs(n, parent, node_cost, inner_parts, min_level_dist, div_rate, level_no, level_ptr, part_no,
                     part_ptr, node_ptr);
}

extern "C" int gbsym_build_lbc(int n, const int *Lp, const int *Li, const double *cost, int inner_parts,
                               int min_level_dist, int div_rate, int *level_no, int **level_ptr, int *part_no,
                               int **part_ptr, int **node_ptr) {
  if (!level_no || !level_ptr || !part_no || !part_ptr || !node_ptr) return GBSYM_ERR_NULL_ARG;
  *level_ptr = *part_ptr = *node_ptr = nullptr;
  *level_no = *part_no = 0;
  if (n < 0 || inner_parts < 1 || div_rate < 1) return GBSYM_ERR_SIZE;
  if (n == 0) return GBSYM_OK;
  if (!Lp || !Li) return GBSYM_ERR_NULL_ARG;
  if (!csr_lower_ok(n, Lp, Li)) return GBSYM_ERR_BAD_MATRIX;
  std::vector<int> parent(n);
  etree_lower_csr(n, Lp, Li, parent.data());
  std::vector<double> rowlen;
  if (!cost) {  // the demo's cost: entries per row of L (sptrsv_demo_utils.h:78-81)
    rowlen.resize(n);
    for (int i = 0; i < n; ++i) rowlen[i] = Lp[i + 1] - Lp[i];
    cost = rowlen.data();
  }
  return lbc_outputs(n, parent.data(), cost, inner_parts, min_level_dist, div_rate, level_no, level_ptr, part_no,
                     part_ptr, node_ptr);
}
