// Shape-function families evaluated on the device (HierPoly and KOLeg), shared by the assembly and
// field kernels. Families: 0 N (normal, "norm"), 1 N', 2 T (tangential, "tang"), 3 T'.
#pragma once
#include <cuda_runtime.h>

#include "../../include/fem2d_gb300.h"

namespace fem2d {
namespace {

// Shape families at x: 0 N (norm), 1 N', 2 T (tang), 3 T'.
// HierPoly: hierarchical_basis_fns.rs:102-162. KOLeg (Legendre, restating HierMaxOrtho):
// hierarchical_basis_fns.rs:201-647.
__constant__ double c_euc[12] = {0.968246, 2.561738, 0.838525, 4.248161, 0.816397, 5.882766,
                                 0.808509, 1.0, 1.0, 1.0, 1.0, 1.0};
__constant__ int c_qden[12] = {1, 3, 6, 10, 15, 21, 28, 36, 40, 55, 66, 72};

// numerator k of Q-function row idx (idx = order - 2): entries alternate with zeros; the odd/even
// pattern is -1, -5, -9, ... (even rows) or -3, -7, -11, ... (odd rows), the last entry is positive.
__device__ __forceinline__ double q_numerator(int idx, int k) {
  const int dim = idx + 3;
  if (k == dim - 1) {
    const int tops[12] = {1, 3, 6, 10, 15, 21, 28, 36, 40, 55, 66, 72};
    return (double)tops[idx];
  }
  if ((idx & 1) == 0) return (k & 1) ? 0.0 : -(double)(2 * k + 1);
  return (k & 1) ? -(double)(2 * k + 1) : 0.0;
}

__device__ double shape(int basis, int family, int a, double x) {
  if (basis == FEM2D_BASIS_HIERPOLY) {
    if (a == 0) {
      switch (family) { case 0: return 1.0; case 1: return 0.0; case 2: return 1.0 - x; default: return -1.0; }
    }
    if (a == 1) {
      switch (family) { case 0: return x; case 1: return 1.0; case 2: return 1.0 + x; default: return 1.0; }
    }
    double prev = x, pw = x;   // pows[a-1], pows[a]
    for (int k = 2; k <= a; k++) {
      prev = pw;
      pw = prev * x;
    }
    const double d1 = (double)a * prev;
    const bool even = (a % 2) == 0;
    switch (family) {
      case 0: return pw;
      case 1: return d1;
      case 2: return even ? pw - 1.0 : pw - x;
      default: return even ? d1 : d1 - 1.0;
    }
  }
  // KOLeg
  if (family == 2 || family == 3) {
    if (a == 0) return family == 2 ? 1.0 - x : -1.0;
    if (a == 1) return family == 2 ? 1.0 + x : 1.0;
  }
  double l0 = 1.0, l1 = x, d1 = 1.0;
  double accv = 0.0, accd = 0.0;
  const bool want_q = family >= 2;
  const int idx = a - 2;
  const int top = want_q ? a : a;   // Q_a uses L_0 .. L_a
  for (int k = 0; k <= top; k++) {
    double lk, dk;
    if (k == 0) { lk = 1.0; dk = 0.0; }
    else if (k == 1) { lk = x; dk = 1.0; }
    else {
      const double f = (double)k;
      lk = ((2.0 * f - 1.0) * x * l1 - (f - 1.0) * l0) / f;
      dk = f * l1 + x * d1;
      l0 = l1; l1 = lk; d1 = dk;
    }
    if (want_q) {
      const double w = q_numerator(idx, k) / (double)c_qden[idx];
      accv += w * lk;
      accd += w * dk;
    } else if (k == a) {
      return family == 0 ? lk : dk;
    }
  }
  return family == 2 ? accv * c_euc[idx] : accd * c_euc[idx];
}

}  // namespace
}  // namespace fem2d
