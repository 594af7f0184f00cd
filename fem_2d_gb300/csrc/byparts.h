// integrate_by_parts over the Galerkin visit set (byparts.cu).
#pragma once
#include "device.h"
#include "gep.h"

namespace fem2d {

// per upper-triangle entry in (row, col) order, 6 doubles: the CurlCurl face term, its edge terms 0..3
// and the L2Inner value, each summed over the entry's visits
void gep_by_parts(Ctx& c, const HostGEP& h, const DeviceGEP& d, double* out6);
void glq_points(int n, std::vector<double>& x, std::vector<double>& w);

}  // namespace fem2d
