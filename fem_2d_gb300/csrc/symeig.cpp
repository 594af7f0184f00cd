#include "symeig.h"

#include <algorithm>
#include <cmath>
#include <numeric>

namespace fem2d {

bool symeig(int n, const std::vector<double>& a, std::vector<double>& w, std::vector<double>& z) {
  w.assign(n, 0.0);
  z.assign((size_t)n * n, 0.0);
  if (n == 0) return true;
  // V holds the working matrix; after reduction it is the orthogonal transform Q (column-major in V[i][j] = V[i*n+j])
  std::vector<double> V(a), d(n), e(n, 0.0);
  auto at = [&](int i, int j) -> double& { return V[(size_t)i * n + j]; };
  for (int i = 0; i < n; i++)
    for (int j = 0; j < i; j++) at(j, i) = at(i, j) = 0.5 * (at(i, j) + at(j, i));
  // Householder tridiagonalization (lower triangle), rows processed from the bottom
  for (int i = n - 1; i > 0; i--) {
    int l = i - 1;
    double h = 0.0, scale = 0.0;
    if (l > 0) {
      for (int k = 0; k <= l; k++) scale += std::fabs(at(i, k));
      if (scale == 0.0) {
        e[i] = at(i, l);
      } else {
        for (int k = 0; k <= l; k++) {
          at(i, k) /= scale;
          h += at(i, k) * at(i, k);
        }
        double f = at(i, l);
        double g = f >= 0.0 ? -std::sqrt(h) : std::sqrt(h);
        e[i] = scale * g;
        h -= f * g;
        at(i, l) = f - g;
        f = 0.0;
        for (int j = 0; j <= l; j++) {
          at(j, i) = at(i, j) / h;
          g = 0.0;
          for (int k = 0; k <= j; k++) g += at(j, k) * at(i, k);
          for (int k = j + 1; k <= l; k++) g += at(k, j) * at(i, k);
          e[j] = g / h;
          f += e[j] * at(i, j);
        }
        double hh = f / (h + h);
        for (int j = 0; j <= l; j++) {
          f = at(i, j);
          e[j] = g = e[j] - hh * f;
          for (int k = 0; k <= j; k++) at(j, k) -= (f * e[k] + g * at(i, k));
        }
      }
    } else {
      e[i] = at(i, l);
    }
    d[i] = h;
  }
  d[0] = 0.0;
  e[0] = 0.0;
  // accumulate the transforms
  for (int i = 0; i < n; i++) {
    int l = i - 1;
    if (d[i] != 0.0) {
      for (int j = 0; j <= l; j++) {
        double g = 0.0;
        for (int k = 0; k <= l; k++) g += at(i, k) * at(k, j);
        for (int k = 0; k <= l; k++) at(k, j) -= g * at(k, i);
      }
    }
    d[i] = at(i, i);
    at(i, i) = 1.0;
    for (int j = 0; j <= l; j++) at(j, i) = at(i, j) = 0.0;
  }
  // implicit QL with shifts on (d, e)
  for (int i = 1; i < n; i++) e[i - 1] = e[i];
  e[n - 1] = 0.0;
  for (int l = 0; l < n; l++) {
    int iter = 0, m;
    do {
      for (m = l; m < n - 1; m++) {
        double dd = std::fabs(d[m]) + std::fabs(d[m + 1]);
        if (std::fabs(e[m]) <= 1e-300 || std::fabs(e[m]) <= 2.3e-16 * dd) break;
      }
      if (m != l) {
        if (++iter > 60) return false;
        double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
        double r = std::hypot(g, 1.0);
        g = d[m] - d[l] + e[l] / (g + (g >= 0.0 ? std::fabs(r) : -std::fabs(r)));
        double s = 1.0, c = 1.0, p = 0.0;
        int i;
        for (i = m - 1; i >= l; i--) {
          double f = s * e[i], b = c * e[i];
          r = std::hypot(f, g);
          e[i + 1] = r;
          if (r == 0.0) {
            d[i + 1] -= p;
            e[m] = 0.0;
            break;
          }
          s = f / r;
          c = g / r;
          g = d[i + 1] - p;
          r = (d[i] - g) * s + 2.0 * c * b;
          p = s * r;
          d[i + 1] = g + p;
          g = c * r - b;
          for (int k = 0; k < n; k++) {
            f = at(k, i + 1);
            at(k, i + 1) = s * at(k, i) + c * f;
            at(k, i) = c * at(k, i) - s * f;
          }
        }
        if (r == 0.0 && i >= l) continue;
        d[l] -= p;
        e[l] = g;
        e[m] = 0.0;
      }
    } while (m != l);
  }
  std::vector<int> idx(n);
  std::iota(idx.begin(), idx.end(), 0);
  std::sort(idx.begin(), idx.end(), [&](int x, int y) { return d[x] < d[y]; });
  for (int k = 0; k < n; k++) {
    w[k] = d[idx[k]];
    for (int i = 0; i < n; i++) z[(size_t)i * n + k] = at(i, idx[k]);
  }
  return true;
}

}  // namespace fem2d
