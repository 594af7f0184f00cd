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
  const int64_t nedges = (int64_t)mesh.edges.size();
  // the U/V specs an Elem generates, in (dir, (i, j)) order; f(i, j, dir, edge slot or -1)
  auto for_specs = [](const MElem& el, auto&& f) {
    for (int dir = 0; dir < 2; dir++) {
      const int imax = dir == 0 ? el.ni - 1 : el.ni;
      const int jmax = dir == 0 ? el.nj : el.nj - 1;
      for (int i = 0; i <= imax; i++)
        for (int j = 0; j <= jmax; j++) f(i, j, dir, edge_slot(i, j, dir));
    }
  };
  // edge specs grouped by Edge (flat, counted then filled), each group in (Elem, dir, (i, j)) order
  std::vector<int64_t> eptr(nedges + 1, 0);
  for (int64_t e = 0; e < ne; e++)
    for_specs(mesh.elems[e], [&](int, int, int, int slot) {
      if (slot >= 0) eptr[mesh.elems[e].edges[slot] + 1]++;
    });
  for (int64_t ed = 0; ed < nedges; ed++) eptr[ed + 1] += eptr[ed];
  std::vector<EdgeSpec> on_edge(eptr[nedges]);
  {
    std::vector<int64_t> fill(eptr.begin(), eptr.end() - 1);
    for (int64_t e = 0; e < ne; e++)
      for_specs(mesh.elems[e], [&](int i, int j, int dir, int slot) {
        if (slot >= 0)
          on_edge[fill[mesh.elems[e].edges[slot]]++] = {e, (uint8_t)i, (uint8_t)j, (uint8_t)dir, (uint8_t)slot};
      });
  }
  // interior specs of leaves become DoFs in Elem order; matched edge-spec pairs follow in Edge order.
  // Each Elem's spec list is its interior specs, then its matched edge specs in the order matched.
  std::vector<int64_t> nint(ne, 0), nmatch(ne, 0);
  for (int64_t e = 0; e < ne; e++)
    if (mesh.elems[e].leaf())
      for_specs(mesh.elems[e], [&](int, int, int, int slot) { nint[e] += slot < 0; });
  struct Match { int64_t ea, eb, sa, sb; int32_t dof; };   // sa, sb: indices into on_edge
  std::vector<Match> matches;
  int32_t next = 0;
  for (int64_t e = 0; e < ne; e++) next += (int32_t)nint[e];
  std::vector<int64_t> rel;   // indices into on_edge of the specs of the Edge's active Elems
  for (int64_t ed = 0; ed < nedges; ed++) {
    const MEdge& E = mesh.edges[ed];
    if (!E.active || eptr[ed] == eptr[ed + 1]) continue;
    rel.clear();
    for (int64_t q = eptr[ed]; q < eptr[ed + 1]; q++)
      if (on_edge[q].elem == E.act[0] || on_edge[q].elem == E.act[1]) rel.push_back(q);
    for (size_t a = 0; a < rel.size(); a++)
      for (size_t b = a + 1; b < rel.size(); b++)
        if (edge_match(on_edge[rel[a]], on_edge[rel[b]])) {
          const EdgeSpec &sa = on_edge[rel[a]], &sb = on_edge[rel[b]];
          matches.push_back({sa.elem, sb.elem, rel[a], rel[b], next++});
          nmatch[sa.elem]++;
          nmatch[sb.elem]++;
          break;
        }
  }
  d.ndofs = next;
  d.spec_ptr.resize(ne + 1);
  d.spec_ptr[0] = 0;
  for (int64_t e = 0; e < ne; e++) d.spec_ptr[e + 1] = d.spec_ptr[e] + nint[e] + nmatch[e];
  d.specs.resize(d.spec_ptr[ne]);
  std::vector<int64_t> pos(ne);
  int32_t dof = 0;
  for (int64_t e = 0; e < ne; e++) {
    pos[e] = d.spec_ptr[e];
    if (!mesh.elems[e].leaf()) continue;
    for_specs(mesh.elems[e], [&](int i, int j, int dir, int slot) {
      if (slot < 0) d.specs[pos[e]++] = {(uint8_t)i, (uint8_t)j, (uint8_t)dir, dof++};
    });
  }
  for (const Match& mt : matches) {
    const EdgeSpec &sa = on_edge[mt.sa], &sb = on_edge[mt.sb];
    d.specs[pos[mt.ea]++] = {sa.i, sa.j, sa.dir, mt.dof};
    d.specs[pos[mt.eb]++] = {sb.i, sb.j, sb.dir, mt.dof};
  }
  return d;
}

}  // namespace fem2d
