// topology.cpp -- host construction of a cloth's static structure: block
// pattern, 1-ring, BVH, traversal order, assembly source lists and the block
// ILU(0) level schedule.  Built once per cloth when it is admitted.
//
// Compiled with -ffp-contract=off: the BVH split planes come from centroid
// arithmetic that must round like the reference's (bvh_aabb.cpp:141-290).
#include "topology.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <exception>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <thread>
#include <utility>

namespace cs {
namespace {

// element lists per vertex, elements ascending (CJaggedArray::SetNodeToElem,
// jagged_array.h:96-126)
void incident(int n, int ne, int k, const int* el, std::vector<int>& ptr, std::vector<int>& arr) {
  ptr.assign(n + 1, 0);
  for (int e = 0; e < ne * k; e++) ptr[el[e] + 1]++;
  for (int v = 0; v < n; v++) ptr[v + 1] += ptr[v];
  arr.resize(ptr[n]);
  std::vector<int> fill(ptr.begin(), ptr.end() - 1);
  for (int e = 0; e < ne; e++)
    for (int a = 0; a < k; a++) arr[fill[el[e * k + a]]++] = e;
}

// vertex neighbours through elements, self excluded, in discovery order
// (CJaggedArray::SetEdgeOfElem with is_dia = false, jagged_array.h:158-207)
void adjacency(int n, int ne, int k, const int* el, std::vector<int>& ptr, std::vector<int>& arr) {
  std::vector<int> eptr, earr;
  incident(n, ne, k, el, eptr, earr);
  std::vector<int> seen(n, -1);
  ptr.assign(n + 1, 0);
  arr.clear();
  for (int v = 0; v < n; v++) {
    seen[v] = v;
    for (int i = eptr[v]; i < eptr[v + 1]; i++) {
      const int e = earr[i];
      for (int a = 0; a < k; a++) {
        const int w = el[e * k + a];
        if (seen[w] != v) {
          seen[w] = v;
          arr.push_back(w);
        }
      }
    }
    ptr[v + 1] = (int)arr.size();
  }
}

struct P3 {
  double x, y, z;
};

// --- BVH (MakeBVHTopology_TopDown, bvh_aabb.cpp:109-313) ---------------------
class BvhBuilder {
 public:
  BvhBuilder(const ClothTopo& t) : t_(t) {}

  void build(std::vector<int>& node) {
    static const int kEdge[3][2] = {{1, 2}, {2, 0}, {0, 1}};
    const int nt = t_.nt;
    std::vector<int> eptr, earr;
    incident(t_.np, nt, 3, t_.tri.data(), eptr, earr);
    // neighbour across each edge: first triangle (ascending) holding the
    // reversed edge (MakeTriSurTri, bvh_aabb.cpp:109-138)
    across_.assign(3 * nt, -1);
    for (int tr = 0; tr < nt; tr++)
      for (int e = 0; e < 3; e++) {
        const int a = t_.tri[tr * 3 + kEdge[e][0]], b = t_.tri[tr * 3 + kEdge[e][1]];
        for (int i = eptr[a]; i < eptr[a + 1] && across_[tr * 3 + e] < 0; i++) {
          const int u = earr[i];
          if (u == tr) continue;
          for (int f = 0; f < 3; f++)
            if (a == t_.tri[u * 3 + kEdge[f][1]] && b == t_.tri[u * 3 + kEdge[f][0]]) {
              across_[tr * 3 + e] = u;
              break;
            }
        }
      }
    cen_.resize(nt);
    for (int tr = 0; tr < nt; tr++) {
      const int* v = &t_.tri[tr * 3];
      const double* X = t_.X0.data();
      cen_[tr] = {(X[v[0] * 3 + 0] + X[v[1] * 3 + 0] + X[v[2] * 3 + 0]) / 3.0,
                  (X[v[0] * 3 + 1] + X[v[1] * 3 + 1] + X[v[2] * 3 + 1]) / 3.0,
                  (X[v[0] * 3 + 2] + X[v[1] * 3 + 2] + X[v[2] * 3 + 2]) / 3.0};
    }
    owner_.reset(new std::atomic<int>[nt]);
    for (int i = 0; i < nt; i++) owner_[i].store(0, std::memory_order_relaxed);
    node.assign(3 * (size_t)(2 * nt - 1), -1);
    if (nt == 1) {
      node[1] = 0;
      return;
    }
    std::vector<int> all(nt);
    for (int i = 0; i < nt; i++) all[i] = i;
    unsigned hc = std::thread::hardware_concurrency();
    spawn_depth_ = 0;
    while (spawn_depth_ < 4 && (2u << spawn_depth_) <= hc) spawn_depth_++;
    subtree(node, 0, std::move(all), 1, 0);
    if (error_) std::rethrow_exception(error_);
  }

  // The subtree below node `self`, whose triangles are `list` (more than one).
  // The reference numbers nodes depth first, child 0's subtree before child 1
  // is split.  A subtree of m triangles has 2m - 1 nodes, so after a split
  // into c0 = base and c1 = base + 1, c0's descendants are numbered from
  // base + 2 and c1's from base + 2 |l0|: subtrees are independent, and the
  // large ones near the root are built on threads of their own.
  void subtree(std::vector<int>& node, int self, std::vector<int> list, int base, int depth) {
    struct Job {
      int self;
      std::vector<int> list;
      int base, depth;
    };
    std::vector<std::thread> threads;
    try {
      std::vector<Job> work;
      work.push_back({self, std::move(list), base, depth});
      while (!work.empty()) {
        Job w = std::move(work.back());
        work.pop_back();
        std::vector<int> l0, l1;
        const int c0 = w.base, c1 = w.base + 1;
        split(node, w.self, w.list, c0, c1, l0, l1);
        const int b0 = w.base + 2, b1 = w.base + 2 * (int)l0.size();
        if (l1.size() == 1) {
          node[c1 * 3 + 1] = l1[0];
        } else if (w.depth < spawn_depth_ && l1.size() >= kParallelMin) {
          threads.emplace_back([this, &node, c1, b1, d = w.depth + 1, l = std::move(l1)]() mutable {
            subtree(node, c1, std::move(l), b1, d);
          });
        } else {
          work.push_back({c1, std::move(l1), b1, w.depth + 1});
        }
        if (l0.size() == 1)
          node[c0 * 3 + 1] = l0[0];
        else
          work.push_back({c0, std::move(l0), b0, w.depth + 1});
      }
    } catch (...) {
      std::lock_guard<std::mutex> lk(error_mu_);
      if (!error_) error_ = std::current_exception();
    }
    for (std::thread& th : threads) th.join();
  }

 private:
  static double dotp(P3 a, P3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
  static P3 subp(P3 a, P3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }

  // seed on the positive side of the plane (org, dir); flips dir toward it
  int seed(const std::vector<int>& list, P3 org, P3& dir) const {
    for (int t : list) {
      const P3 g = cen_[t];
      if (std::fabs(dotp(subp(g, org), dir)) < 1.0e-10) continue;
      if (dotp(subp(g, org), dir) < 0) dir = {dir.x * -1.0, dir.y * -1.0, dir.z * -1.0};
      return t;
    }
    return -1;
  }

  // DevideTriAryConnex, bvh_aabb.cpp:156-290
  void split(std::vector<int>& node, int self, const std::vector<int>& list, int c0, int c1, std::vector<int>& l0,
             std::vector<int>& l1) {
    const double eps = 1.0e-10;
    double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    bool full = false;
    for (int t : list) {  // AddPoint(eps) over the centroids, aabb.h:102-122
      const double q[3] = {cen_[t].x, cen_[t].y, cen_[t].z};
      for (int k = 0; k < 3; k++) {
        if (full) {
          lo[k] = (lo[k] < q[k] - eps) ? lo[k] : q[k] - eps;
          hi[k] = (hi[k] > q[k] + eps) ? hi[k] : q[k] + eps;
        } else {
          lo[k] = q[k] - eps;
          hi[k] = q[k] + eps;
        }
      }
      full = true;
    }
    const double lx = hi[0] - lo[0], ly = hi[1] - lo[1], lz = hi[2] - lo[2];
    P3 dir = {0, 0, 0};
    if (lx > ly && lx > lz) dir = {1, 0, 0};
    if (ly > lz && ly > lx) dir = {0, 1, 0};
    if (lz > lx && lz > ly) dir = {0, 0, 1};
    P3 org = {(lo[0] + hi[0]) * 0.5, (lo[1] + hi[1]) * 0.5, (lo[2] + hi[2]) * 0.5};
    int s = seed(list, org, dir);
    if (s == -1) {  // principal axis of the centroids by 10 power iterations
      org = {0, 0, 0};
      for (int t : list) org = {org.x + cen_[t].x, org.y + cen_[t].y, org.z + cen_[t].z};
      const double n = (double)list.size();
      if (!(std::fabs(n) < 1.e-16)) org = {org.x / n, org.y / n, org.z / n};
      double M[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
      for (int t : list) {
        const P3 g = subp(cen_[t], org);
        const double gv[3] = {g.x, g.y, g.z};
        for (int r = 0; r < 3; r++)
          for (int c = 0; c < 3; c++) M[r][c] += gv[r] * gv[c];
      }
      double d[3] = {1, 1, 1};
      for (int it = 0; it < 10; it++) {
        const double tv[3] = {M[0][0] * d[0] + M[0][1] * d[1] + M[0][2] * d[2],
                              M[1][0] * d[0] + M[1][1] * d[1] + M[1][2] * d[2],
                              M[2][0] * d[0] + M[2][1] * d[1] + M[2][2] * d[2]};
        const double len = std::sqrt(tv[0] * tv[0] + tv[1] * tv[1] + tv[2] * tv[2]);
        d[0] = tv[0] / len;
        d[1] = tv[1] / len;
        d[2] = tv[2] / len;
      }
      dir = {d[0], d[1], d[2]};
      s = seed(list, org, dir);
      if (s == -1) s = list[0];  // every centroid on the plane: not met on sheets
    }
    node[c0 * 3 + 0] = self;
    node[c1 * 3 + 0] = self;
    node[self * 3 + 1] = c0;
    node[self * 3 + 2] = c1;
    // flood fill over edge neighbours on the positive side, LIFO (a neighbour
    // in another subtree has an owner other than `self`, whatever its thread
    // writes there)
    owner_[s].store(c0, std::memory_order_relaxed);
    l0.push_back(s);
    std::vector<int> stack(1, s);
    while (!stack.empty()) {
      const int t = stack.back();
      stack.pop_back();
      for (int e = 0; e < 3; e++) {
        const int u = across_[t * 3 + e];
        if (u == -1 || owner_[u].load(std::memory_order_relaxed) != self) continue;
        if (dotp(subp(cen_[u], org), dir) < 0) continue;
        stack.push_back(u);
        owner_[u].store(c0, std::memory_order_relaxed);
        l0.push_back(u);
      }
    }
    for (int t : list) {
      if (owner_[t].load(std::memory_order_relaxed) == c0) continue;
      owner_[t].store(c1, std::memory_order_relaxed);
      l1.push_back(t);
    }
    if (l1.empty()) throw std::runtime_error("BVH split produced an empty half");
  }

  static constexpr size_t kParallelMin = 8192;  // triangles of a subtree worth a thread

  const ClothTopo& t_;
  std::vector<int> across_;
  std::unique_ptr<std::atomic<int>[]> owner_;  // node that holds each triangle
  std::vector<P3> cen_;
  int spawn_depth_ = 0;
  std::mutex error_mu_;
  std::exception_ptr error_;
};

}  // namespace

void build_pattern_only(ClothTopo& t, int np, int nq, const int* quad) {
  for (int i = 0; i < 4 * nq; i++)
    if (quad[i] < 0 || quad[i] >= np) throw std::runtime_error("stencil index out of range");
  t.np = np;
  t.nq = nq;
  // bending-stencil adjacency with sorted rows (self_contact_sparse/main.cpp:578-581)
  adjacency(np, nq, 4, quad, t.row_ptr, t.col_idx);
  for (int v = 0; v < np; v++) std::sort(t.col_idx.begin() + t.row_ptr[v], t.col_idx.begin() + t.row_ptr[v + 1]);
  t.nb = t.row_ptr[np];
  t.dia_split.resize(np);
  for (int v = 0; v < np; v++) {
    const int* b = t.col_idx.data() + t.row_ptr[v];
    const int* e = t.col_idx.data() + t.row_ptr[v + 1];
    t.dia_split[v] = (int)(std::upper_bound(b, e, v) - t.col_idx.data());
  }
}

void build_topology(ClothTopo& t, int np, const double* X0, const int* bc, int nt, const int* tri, int nq,
                    const int* quad, bool with_ilu) {
  t.np = np;
  t.nt = nt;
  t.nq = nq;
  t.X0.assign(X0, X0 + 3 * np);
  t.bc.assign(bc, bc + np);
  t.tri.assign(tri, tri + 3 * nt);
  t.quad.assign(quad, quad + 4 * nq);
  for (int i = 0; i < 3 * nt; i++)
    if (tri[i] < 0 || tri[i] >= np) throw std::runtime_error("triangle index out of range");
  for (int i = 0; i < 4 * nq; i++)
    if (quad[i] < 0 || quad[i] >= np) throw std::runtime_error("stencil index out of range");
  if (nt < 1) throw std::runtime_error("a cloth needs at least one triangle");

  build_pattern_only(t, np, nq, quad);

  // 1-ring over triangles (self_contact_sparse/main.cpp:577) and its edges
  adjacency(np, nt, 3, tri, t.ring_ptr, t.ring);
  t.edge_uv.clear();
  for (int v = 0; v < np; v++)
    for (int i = t.ring_ptr[v]; i < t.ring_ptr[v + 1]; i++)
      if (v < t.ring[i]) {
        t.edge_uv.push_back(v);
        t.edge_uv.push_back(t.ring[i]);
      }

  // BVH and its depth-first traversal tables
  BvhBuilder(t).build(t.node);
  t.nnode = (int)t.node.size() / 3;
  t.pre.clear();
  t.skip.assign(t.nnode, 0);
  t.leaf_lo.assign(t.nnode, 0);
  t.leaf_hi.assign(t.nnode, 0);
  t.depth.assign(t.nnode, 0);
  {
    std::vector<int> pos_of(t.nnode, 0);
    std::vector<int> st(1, 0);
    while (!st.empty()) {
      const int n = st.back();
      st.pop_back();
      pos_of[n] = (int)t.pre.size();
      t.pre.push_back(n);
      if (t.node[n * 3 + 2] != -1) {
        const int c0 = t.node[n * 3 + 1], c1 = t.node[n * 3 + 2];
        t.depth[c0] = t.depth[c1] = t.depth[n] + 1;
        st.push_back(c1);
        st.push_back(c0);
      }
    }
    // subtree extents from a reverse preorder sweep
    std::vector<int> size(t.nnode, 1);
    int leaf = 0;
    for (int k = 0; k < t.nnode; k++) {
      const int n = t.pre[k];
      if (t.node[n * 3 + 2] == -1) t.leaf_lo[n] = t.leaf_hi[n] = leaf++;
    }
    for (int k = t.nnode - 1; k >= 0; k--) {
      const int n = t.pre[k];
      if (t.node[n * 3 + 2] != -1) {
        const int c0 = t.node[n * 3 + 1], c1 = t.node[n * 3 + 2];
        size[n] = 1 + size[c0] + size[c1];
        t.leaf_lo[n] = t.leaf_lo[c0];
        t.leaf_hi[n] = t.leaf_hi[c1];
      }
      t.skip[k] = k + size[n];
    }
  }

  // assembly source lists in element order (AddWdWddW_Cloth, solve_internal_sparse.h:19-76,
  // merged like CMatrixSquareSparse::Mearge, matrix_square_sparse.cpp:88-138)
  auto slot_of = [&](int i, int j) -> int {
    const int* b = t.col_idx.data() + t.row_ptr[i];
    const int* e = t.col_idx.data() + t.row_ptr[i + 1];
    const int* p = std::lower_bound(b, e, j);
    return (p != e && *p == j) ? (int)(p - t.col_idx.data()) : -1;
  };
  // Counted twice over the same element order (count, then fill), so each list
  // keeps the order in which the reference merges the blocks.
  const int nslot = t.nb + np;
  std::vector<int> tslot(9 * (size_t)nt), qslot(16 * (size_t)nq);
  t.slot_ptr.assign(nslot + 1, 0);
  t.grad_ptr.assign(np + 1, 0);
  for (int e = 0; e < nt; e++)
    for (int a = 0; a < 3; a++) {
      const int i = tri[e * 3 + a];
      t.grad_ptr[i + 1]++;
      for (int b = 0; b < 3; b++) {
        const int s = (a == b) ? t.nb + i : slot_of(i, tri[e * 3 + b]);
        tslot[e * 9 + a * 3 + b] = s;
        if (s >= 0) t.slot_ptr[s + 1]++;
      }
    }
  for (int e = 0; e < nq; e++)
    for (int a = 0; a < 4; a++) {
      const int i = quad[e * 4 + a];
      t.grad_ptr[i + 1]++;
      for (int b = 0; b < 4; b++) {
        const int s = (a == b) ? t.nb + i : slot_of(i, quad[e * 4 + b]);
        qslot[e * 16 + a * 4 + b] = s;
        if (s >= 0) t.slot_ptr[s + 1]++;
      }
    }
  for (int s = 0; s < nslot; s++) t.slot_ptr[s + 1] += t.slot_ptr[s];
  for (int v = 0; v < np; v++) t.grad_ptr[v + 1] += t.grad_ptr[v];
  t.slot_src.resize(t.slot_ptr[nslot]);
  t.grad_src.resize(t.grad_ptr[np]);
  {
    std::vector<int> fill(t.slot_ptr.begin(), t.slot_ptr.end() - 1);
    std::vector<int> gfill(t.grad_ptr.begin(), t.grad_ptr.end() - 1);
    for (int e = 0; e < nt; e++) {
      for (int a = 0; a < 3; a++) t.grad_src[gfill[tri[e * 3 + a]]++] = e * 3 + a;
      for (int k = 0; k < 9; k++) {
        const int s = tslot[e * 9 + k];
        if (s >= 0) t.slot_src[fill[s]++] = e * 9 + k;
      }
    }
    for (int e = 0; e < nq; e++) {
      for (int a = 0; a < 4; a++) t.grad_src[gfill[quad[e * 4 + a]]++] = -(e * 4 + a) - 1;
      for (int k = 0; k < 16; k++) {
        const int s = qslot[e * 16 + k];
        if (s >= 0) t.slot_src[fill[s]++] = -(e * 16 + k) - 1;
      }
    }
  }

  // block ILU(0) schedule (DoILUDecomp, ilu_sparse.cpp:507-569): row i waits for
  // the rows of its lower part; the backward sweep for the rows of its upper part
  t.lev_ptr.clear();
  t.lev_rows.clear();
  t.blev_ptr.clear();
  t.blev_rows.clear();
  t.fac_ptr.assign(np + 1, 0);
  t.fac_ops.clear();
  if (with_ilu) {
    std::vector<int> lev(np, 0), blev(np, 0);
    int nlev = 0, nblev = 0;
    for (int i = 0; i < np; i++) {
      int l = 0;
      for (int s = t.row_ptr[i]; s < t.dia_split[i]; s++) l = std::max(l, lev[t.col_idx[s]] + 1);
      lev[i] = l;
      nlev = std::max(nlev, l + 1);
    }
    for (int i = np - 1; i >= 0; i--) {
      int l = 0;
      for (int s = t.dia_split[i]; s < t.row_ptr[i + 1]; s++) l = std::max(l, blev[t.col_idx[s]] + 1);
      blev[i] = l;
      nblev = std::max(nblev, l + 1);
    }
    auto bucket = [np](const std::vector<int>& L, int n, std::vector<int>& ptr, std::vector<int>& rows) {
      ptr.assign(n + 1, 0);
      for (int i = 0; i < np; i++) ptr[L[i] + 1]++;
      for (int k = 0; k < n; k++) ptr[k + 1] += ptr[k];
      rows.resize(np);
      std::vector<int> fill(ptr.begin(), ptr.end() - 1);
      for (int i = 0; i < np; i++) rows[fill[L[i]]++] = i;
    };
    bucket(lev, nlev, t.lev_ptr, t.lev_rows);
    bucket(blev, nblev, t.blev_ptr, t.blev_rows);
    for (int i = 0; i < np; i++) {
      for (int s = t.row_ptr[i]; s < t.dia_split[i]; s++) {
        const int k = t.col_idx[s];
        for (int ks = t.dia_split[k]; ks < t.row_ptr[k + 1]; ks++) {
          const int j = t.col_idx[ks];
          int target;
          if (j != i) {
            target = slot_of(i, j);
            if (target < 0) continue;
          } else {
            target = -1;
          }
          t.fac_ops.push_back(s);
          t.fac_ops.push_back(ks);
          t.fac_ops.push_back(target);
        }
      }
      t.fac_ptr[i + 1] = (int)t.fac_ops.size() / 3;
    }
  }
}

}  // namespace cs
