// DoF enumeration. Reference: Domain::from_mesh (src/fem_domain/domain.rs:69-159), gen_basis_specs
// (domain.rs:201-235), BasisSpec::new (basis_spec.rs:41-75), matches_with_edge (basis_spec.rs:80-110),
// PolyOrders::permutations (p_refinement.rs:49-64).
//
// Numbering rule (bit-exact with the reference):
//   1. leaf Elems in ascending id; within an Elem the interior U specs (i < ni, 2 <= j <= nj, i >= 2)
//      then interior V specs, each in (i, j) lexicographic order -> one DoF per spec;
//   2. Edges in ascending id that have an active Elem pair: the U/V edge specs of the two active Elems,
//      in (Elem id, U before V, (i, j)) order, are paired first-match -> one DoF per pair.
// Non-leaf Elems keep only their matched edge specs. W-directed and node-type specs never become DoFs.
#include "domain.h"

#include <algorithm>

#include "common.h"

namespace fem2d {

namespace {
struct EdgeSpec {
  int64_t elem;
  uint8_t i, j, dir, slot;   // slot: the Elem's edge index the spec lives on
};

// BasisSpec::new location rule for U and V specs: returns the edge slot, or -1 for an interior spec
inline int edge_slot(int i, int j, int dir) {
  if (i >= 2 && j >= 2) return -1;
  if (dir == 0 && j <= 1) return j;
  if (dir == 1 && i <= 1) return i + 2;
  return -1;
}

inline bool edge_match(const EdgeSpec& a, const EdgeSpec& b) {
  if (a.dir != b.dir) return false;
  if (a.dir == 0) return a.i == b.i && a.j + b.j == 1 && a.slot + b.slot == 1;
  return a.j == b.j && a.i + b.i == 1 && a.slot + b.slot == 5;
}
}  // namespace

Domain Domain::from_mesh(const Mesh& m, int cc) {
  Domain d;
  d.mesh = m;
  d.cc = cc;
  if (cc != FEM2D_CC_HCURL) {   // only H(curl) basis specs exist (basis_spec.rs:71 unimplemented!)
    d.spec_ptr.assign(m.elems.size() + 1, 0);
    return d;
  }
  Mesh& mesh = d.mesh;
  mesh.set_edge_activation();
  const int64_t ne = (int64_t)mesh.elems.size();
  std::vector<std::vector<Spec>> per(ne);
  std::vector<std::vector<EdgeSpec>> on_edge(mesh.edges.size());
  int32_t next = 0;
  // spec generation in (Elem, dir, (i, j)) order; interior specs of leaves become DoFs at once
  for (int64_t e = 0; e < ne; e++) {
    const MElem& el = mesh.elems[e];
    for (int dir = 0; dir < 2; dir++) {
      int imax = dir == 0 ? el.ni - 1 : el.ni;
      int jmax = dir == 0 ? el.nj : el.nj - 1;
      for (int i = 0; i <= imax; i++)
        for (int j = 0; j <= jmax; j++) {
          int slot = edge_slot(i, j, dir);
          if (slot >= 0) on_edge[el.edges[slot]].push_back({e, (uint8_t)i, (uint8_t)j, (uint8_t)dir, (uint8_t)slot});
        }
    }
  }
  for (int64_t e = 0; e < ne; e++) {
    const MElem& el = mesh.elems[e];
    if (!el.leaf()) continue;
    for (int dir = 0; dir < 2; dir++) {
      int imax = dir == 0 ? el.ni - 1 : el.ni;
      int jmax = dir == 0 ? el.nj : el.nj - 1;
      for (int i = 0; i <= imax; i++)
        for (int j = 0; j <= jmax; j++)
          if (edge_slot(i, j, dir) < 0) per[e].push_back({(uint8_t)i, (uint8_t)j, (uint8_t)dir, next++});
    }
  }
  std::vector<EdgeSpec> rel;
  std::vector<char> used;
  for (size_t ed = 0; ed < mesh.edges.size(); ed++) {
    const MEdge& E = mesh.edges[ed];
    if (!E.active || on_edge[ed].empty()) continue;
    rel.clear();
    for (auto& s : on_edge[ed])
      if (s.elem == E.act[0] || s.elem == E.act[1]) rel.push_back(s);
    for (size_t a = 0; a < rel.size(); a++)
      for (size_t b = a + 1; b < rel.size(); b++)
        if (edge_match(rel[a], rel[b])) {
          int32_t dof = next++;
          per[rel[a].elem].push_back({rel[a].i, rel[a].j, rel[a].dir, dof});
          per[rel[b].elem].push_back({rel[b].i, rel[b].j, rel[b].dir, dof});
          break;
        }
  }
  d.ndofs = next;
  d.spec_ptr.resize(ne + 1);
  d.spec_ptr[0] = 0;
  for (int64_t e = 0; e < ne; e++) d.spec_ptr[e + 1] = d.spec_ptr[e] + (int64_t)per[e].size();
  d.specs.reserve(d.spec_ptr[ne]);
  for (auto& v : per) d.specs.insert(d.specs.end(), v.begin(), v.end());
  return d;
}

}  // namespace fem2d
