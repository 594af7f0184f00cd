// Multifrontal factorization of the shifted pencil A + alpha B over a nested dissection of the
// base-Elem trees.
//
// DoFs of different base-Elem trees couple only through the edge DoFs their trees share
// (galerkin.rs visits pairs within one Elem tree only). A nested dissection of the base Elems by
// coordinate bisection therefore gives an exact elimination tree: a leaf front holds the DoFs
// interior to one tree, an inner front the DoFs shared between its two halves. Fronts are dense;
// each partial LU (partial pivoting within the fully-summed rows) leaves a Schur complement that is
// extend-added into the parent front.
#pragma once
#include <cstdint>
#include <vector>

#include "gep.h"

namespace fem2d {

struct Domain;
struct HostGEP;

struct MFSymbolic {
  int64_t n = 0;
  int nfronts = 0;
  // per front (postorder: children before parents)
  std::vector<int32_t> parent;            // -1 for the root
  std::vector<int32_t> level;             // distance from the deepest leaf level (0 = processed first)
  std::vector<int32_t> f, p;              // front size, pivot count
  std::vector<int64_t> dof_ptr;           // front dofs (pivots first, then struct), nfronts + 1
  std::vector<int32_t> dofs;
  std::vector<int64_t> mat_off;           // offset of the dense f x f front in the factor buffer
  int64_t mat_total = 0;
  // assembly from the CSR: (front-local row*f + col, csr index), grouped per front
  std::vector<int64_t> asm_ptr;
  HostVec<int64_t> asm_pos;               // row * f + col (written in full by the fill pass: no zeroing)
  HostVec<int64_t> asm_csr;
  // extend-add of each front's Schur complement into its parent: positions of struct(C) in F_parent
  std::vector<int64_t> ea_ptr;            // per front
  std::vector<int32_t> ea_map;
  // grouping by level, children-before-parents order
  int nlevels = 0;
  std::vector<int32_t> level_ptr;         // nlevels + 1
  std::vector<int32_t> level_fronts;      // fronts ordered by level
  int max_f = 0, max_p = 0;
  double flops = 0;                        // factorization flop estimate
};

// lift (optional, one entry per DoF): eliminate that DoF so many tree levels above its natural front
void mf_symbolic(const Domain& d, const HostGEP& g, MFSymbolic& s, const std::vector<uint8_t>* lift = nullptr);
// one dense front with every DoF (full partial pivoting)
void mf_symbolic_dense(const HostGEP& g, MFSymbolic& s);

}  // namespace fem2d
