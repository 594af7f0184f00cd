// Eigensolvers on the device: dense (nalgebra_solve_gep restated) and sparse shift-invert.
#pragma once
#include "device.h"

namespace fem2d {

struct Domain;
void dense_solve(Ctx& c, const Domain& dom, const HostGEP& h, const DeviceGEP& d, double target, double* value,
                 double* vector);
void sparse_solve(Ctx& c, const Domain& dom, const HostGEP& h, const DeviceGEP& d, double target, int n_pairs,
                  const fem2d_solve_opts& o, double* values, double* vectors, double* residuals,
                  fem2d_solve_stats* st);

void shifted_solve(Ctx& c, const Domain& dom, const HostGEP& h, const DeviceGEP& d, double ca, double cb, bool spd,
                   int nrhs, const double* rhs, double* x);

}  // namespace fem2d
