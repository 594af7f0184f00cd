// Dense symmetric eigen-decomposition on the host for the small projected (Rayleigh-Ritz) matrices:
// Householder reduction to tridiagonal form with accumulated transforms, then the implicit-shift QL
// iteration (Golub & Van Loan, "Matrix Computations", 8.3; the tred2/tql2 pair).
#pragma once
#include <vector>

namespace fem2d {

// a: n x n row-major symmetric (only read); w: eigenvalues ascending; z: n x n row-major, column k
// is the eigenvector of w[k]. Returns false if QL did not converge.
bool symeig(int n, const std::vector<double>& a, std::vector<double>& w, std::vector<double>& z);

}  // namespace fem2d
