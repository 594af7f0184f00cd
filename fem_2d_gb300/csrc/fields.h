// Field evaluation over the leaf Elems of a Domain (UniformFieldSpace, fields.rs:17-122).
//
// The reference samples, on every leaf Elem, a d0 x d1 grid of uniformly spaced parametric points
// and sums over the leaf and all its ancestors the curl-conforming basis functions times the
// solution coefficients (fields.rs:83-119). For the affine, axis-aligned Elems the leaf grid maps
// to an ancestor's parametric square by a scale and offset per axis, and the inverse Jacobian is
// diagonal, so one (leaf, ancestor) pair is described by six numbers and a spec range.
#pragma once
#include <cstdint>
#include <vector>

#include "device.h"
#include "domain.h"

namespace fem2d {

// one (leaf, ancestor) pair of the evaluation plan
struct alignas(16) FieldItem {
  double su, ou, sv, ov;   // leaf parametric point x -> ancestor point x * s + o, per axis
  double jiu, jiv;         // ancestor inverse-Jacobian diagonal (jac_inv.u.x, jac_inv.v.y)
  int32_t sp0, sp1;        // the ancestor's spec range in the Domain's spec order
};

struct FieldSpace {
  Ctx* ctx = nullptr;
  int device = 0;
  int basis = 0, d0 = 0, d1 = 0;
  int imax = 0, jmax = 0;             // Mesh::max_expansion_orders
  int64_t ndofs = 0;
  std::vector<int64_t> leaves;        // leaf Elem ids, ascending
  std::vector<double> leaf_bounds;    // per leaf: x and y of nodes[0], then of nodes[3]
  std::vector<FieldItem> h_items;
  std::vector<int32_t> h_item_ptr;    // leaves + 1
  DBuf<FieldItem> items;
  DBuf<int32_t> item_ptr, dofs;
  DBuf<uint32_t> codes;               // i | j << 8 | dir << 16
  DBuf<double> sol, out;              // staging for the host-pointer entry point
  size_t smem = 0;
  int64_t h2d_bytes = 0;
};

// host plan (leaf order, ancestors leaf first, spec ranges) and its upload
void fields_plan(Ctx& c, const Domain& d, int basis, int d0, int d1, FieldSpace& f);
// x and y values of every leaf grid, [leaf][m][n] with m along u (d0) and n along v (d1); device
// pointers, asynchronous on the context's stream
void fields_eval(FieldSpace& f, const double* d_solution, double* d_x, double* d_y);

}  // namespace fem2d
