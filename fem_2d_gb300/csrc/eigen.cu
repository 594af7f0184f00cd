#include "eigen.h"

namespace fem2d {

void dense_solve(Ctx&, const HostGEP&, const DeviceGEP&, double, double*, double*) {
  fail(FEM2D_E_NOT_CONVERGED, "dense solve not available in this build");
}
void sparse_solve(Ctx&, const HostGEP&, const DeviceGEP&, double, int, const fem2d_solve_opts&, double*, double*,
                  double*, fem2d_solve_stats*) {
  fail(FEM2D_E_NOT_CONVERGED, "sparse solve not available in this build");
}

}  // namespace fem2d
