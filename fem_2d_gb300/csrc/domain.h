// Domain: DoF enumeration over an RBS mesh (src/fem_domain/domain.rs:69-159).
#pragma once
#include <cstdint>
#include <vector>

#include "common.h"
#include "mesh.h"

namespace fem2d {

// One basis function bound to a DoF: orders (i, j), direction (0 = U, 1 = V).
struct Spec {
  uint8_t i, j, dir;
  int32_t dof;
};

struct Domain {
  Mesh mesh;
  int cc = FEM2D_CC_HCURL;
  int64_t ndofs = 0;
  // spec lists per Elem in Domain::basis_specs order, stored CSR-style
  std::vector<int64_t> spec_ptr;   // elems + 1
  std::vector<Spec> specs;

  static Domain from_mesh(const Mesh& m, int cc);
  int64_t nspecs(int64_t e) const { return spec_ptr[e + 1] - spec_ptr[e]; }
};

}  // namespace fem2d
