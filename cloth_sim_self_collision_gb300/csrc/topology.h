// topology.h -- host-side, build-once structure of one cloth.
#pragma once
#include <vector>

namespace cs {

struct ClothTopo {
  int np = 0, nt = 0, nq = 0, nb = 0, nnode = 0;
  std::vector<double> X0;
  std::vector<int> bc, tri, quad;

  // 3x3 block pattern, diagonal apart (rows sorted ascending)
  std::vector<int> row_ptr, col_idx, dia_split;

  // vertex 1-ring through triangles, and its undirected edges (u < v)
  std::vector<int> ring_ptr, ring, edge_uv;

  // BVH: 3 ints per node (parent, child0, child1; child1 == -1 at a leaf)
  std::vector<int> node;
  // depth-first (child0 first) traversal: pre[k] = node at preorder k,
  // skip[k] = preorder position after its subtree; leaf order range per node
  std::vector<int> pre, skip, leaf_lo, leaf_hi, depth;

  // assembly: for every slot (nb off-diagonal, then np diagonal) the element
  // blocks summed into it, in the reference's order (triangles then stencils).
  // code >= 0: triangle block t*9 + a*3 + b;  code < 0: stencil entry
  // -(q*16 + a*4 + b) - 1.
  std::vector<int> slot_ptr, slot_src;
  // gradient: for every vertex, t*3 + a (triangles) then -(q*4 + a) - 1 (stencils)
  std::vector<int> grad_ptr, grad_src;

  // block ILU(0) schedule in natural row order
  std::vector<int> lev_ptr, lev_rows;    // forward levels (factor and L sweep)
  std::vector<int> blev_ptr, blev_rows;  // backward levels (U sweep)
  std::vector<int> fac_ptr, fac_ops;     // per row: (ik slot, kj slot, target slot or -1 = diagonal)
};

// Builds everything above from the mesh.  The BVH follows the reference's
// MakeBVHTopology_TopDown node for node.
void build_topology(ClothTopo& t, int np, const double* X0, const int* bc, int nt, const int* tri, int nq,
                    const int* quad, bool with_ilu);

// Only the block pattern (row_ptr, col_idx, dia_split, nb) from the stencils.
void build_pattern_only(ClothTopo& t, int np, int nq, const int* quad);

}  // namespace cs
