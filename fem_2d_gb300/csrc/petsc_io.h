// Binary files of the reference's hand-off to an external SLEPc solver (see petsc_io.cpp).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace fem2d {

struct AIJ {
  int64_t n = 0;
  std::vector<int64_t> row_ptr;
  std::vector<int32_t> col;
  std::vector<double> val;
};

void aij_write(const std::string& path, int64_t n, const int64_t* row_ptr, const int32_t* col, const double* val);
void aij_read(const std::string& path, AIJ& m);
void vec_write(const std::string& path, const double* v, int64_t n);
void vec_read(const std::string& path, std::vector<double>& v);
void scalar_write(const std::string& path, double x);
double scalar_read(const std::string& path);

}  // namespace fem2d
