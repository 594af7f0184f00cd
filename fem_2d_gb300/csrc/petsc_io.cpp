// PETSc-style binary files of the reference's external-solver hand-off (host code, big-endian).
//
// Matrices: AIJMatrixBinary::print_to_petsc_binary_file (sparse_matrix.rs:184-265) writes the bytes
// "\0{P" (three bytes where PETSc has the four-byte class id 1211216), then rows, cols and nnz as
// u32, the per-row entry counts as u32, the column indices as u32 and the values as f64, rows in
// ascending order and columns ascending within a row, both triangles present. The reader accepts that
// layout and the standard one (four-byte class id 0x00124850).
// Vectors: retrieve_eigenvector (slepc_solve.rs:114-135): class id 1211214 (i32), m (i32), m f64.
// Scalars: retrieve_eigenvalue (slepc_solve.rs:137-147): one f64.
#include "petsc_io.h"

#include <cstdio>
#include <cstring>
#include <fstream>
#include <memory>

#include "common.h"

namespace fem2d {

namespace {

void put_u32(std::vector<unsigned char>& b, uint32_t v) {
  for (int s = 24; s >= 0; s -= 8) b.push_back((unsigned char)((v >> s) & 0xffu));
}

void put_f64(std::vector<unsigned char>& b, double v) {
  uint64_t u;
  std::memcpy(&u, &v, 8);
  for (int s = 56; s >= 0; s -= 8) b.push_back((unsigned char)((u >> s) & 0xffu));
}

uint32_t get_u32(const unsigned char* p) {
  return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | (uint32_t)p[3];
}

double get_f64(const unsigned char* p) {
  uint64_t u = 0;
  for (int k = 0; k < 8; k++) u = (u << 8) | p[k];
  double v;
  std::memcpy(&v, &u, 8);
  return v;
}

void write_file(const std::string& path, const std::vector<unsigned char>& bytes) {
  std::ofstream f(path, std::ios::binary | std::ios::trunc);
  if (!f) fail(FEM2D_E_IO, "cannot create " + path);
  f.write(reinterpret_cast<const char*>(bytes.data()), (std::streamsize)bytes.size());
  if (!f) fail(FEM2D_E_IO, "write failed: " + path);
}

std::vector<unsigned char> read_file(const std::string& path) {
  std::ifstream f(path, std::ios::binary);
  if (!f) fail(FEM2D_E_IO, "cannot open " + path);
  return std::vector<unsigned char>((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
}

}  // namespace

void aij_write(const std::string& path, int64_t n, const int64_t* row_ptr, const int32_t* col, const double* val) {
  if (n < 0 || n > 0xffffffffLL) fail(FEM2D_E_INVALID_ARG, "matrix dimension out of range");
  const int64_t nnz = n > 0 ? row_ptr[n] : 0;
  if (nnz > 0xffffffffLL) fail(FEM2D_E_TOO_LARGE, "more than 2^32 entries");
  std::vector<unsigned char> b;
  b.reserve(15 + 4 * (size_t)n + 12 * (size_t)nnz);
  b.push_back(0x00);
  b.push_back('{');
  b.push_back('P');
  put_u32(b, (uint32_t)n);
  put_u32(b, (uint32_t)n);
  put_u32(b, (uint32_t)nnz);
  for (int64_t r = 0; r < n; r++) {
    const int64_t cnt = row_ptr[r + 1] - row_ptr[r];
    if (cnt < 0) fail(FEM2D_E_INVALID_ARG, "row pointers decrease");
    for (int64_t k = row_ptr[r] + 1; k < row_ptr[r + 1]; k++)
      if (col[k] <= col[k - 1]) fail(FEM2D_E_INVALID_ARG, "columns must ascend within a row");
    put_u32(b, (uint32_t)cnt);
  }
  for (int64_t k = 0; k < nnz; k++) {
    if (col[k] < 0 || col[k] >= n) fail(FEM2D_E_INVALID_ARG, "column index out of range");
    put_u32(b, (uint32_t)col[k]);
  }
  for (int64_t k = 0; k < nnz; k++) put_f64(b, val[k]);
  write_file(path, b);
}

void aij_read(const std::string& path, AIJ& m) {
  std::vector<unsigned char> b = read_file(path);
  size_t off;
  if (b.size() >= 16 && get_u32(b.data()) == 1211216u) off = 4;   // standard class id
  else if (b.size() >= 15 && b[0] == 0x00 && b[1] == '{' && b[2] == 'P') off = 3;
  else fail(FEM2D_E_IO, "not an AIJ matrix file: " + path);
  const uint32_t rows = get_u32(&b[off]), cols = get_u32(&b[off + 4]), nnz = get_u32(&b[off + 8]);
  off += 12;
  if (rows != cols) fail(FEM2D_E_IO, "matrix is not square");
  const size_t need = off + 4 * (size_t)rows + 12 * (size_t)nnz;
  if (b.size() < need) fail(FEM2D_E_IO, "truncated matrix file: " + path);
  m.n = rows;
  m.row_ptr.assign(rows + 1, 0);
  for (uint32_t r = 0; r < rows; r++) m.row_ptr[r + 1] = m.row_ptr[r] + get_u32(&b[off + 4 * (size_t)r]);
  off += 4 * (size_t)rows;
  if (m.row_ptr[rows] != (int64_t)nnz) fail(FEM2D_E_IO, "row counts do not add up to nnz");
  m.col.resize(nnz);
  m.val.resize(nnz);
  for (uint32_t k = 0; k < nnz; k++) {
    const uint32_t c = get_u32(&b[off + 4 * (size_t)k]);
    if (c >= cols) fail(FEM2D_E_IO, "column index out of range");
    m.col[k] = (int32_t)c;
  }
  off += 4 * (size_t)nnz;
  for (uint32_t k = 0; k < nnz; k++) m.val[k] = get_f64(&b[off + 8 * (size_t)k]);
}

void vec_write(const std::string& path, const double* v, int64_t n) {
  if (n < 0 || n > 0x7fffffffLL) fail(FEM2D_E_INVALID_ARG, "vector length out of range");
  std::vector<unsigned char> b;
  b.reserve(8 + 8 * (size_t)n);
  put_u32(b, 1211214u);
  put_u32(b, (uint32_t)n);
  for (int64_t k = 0; k < n; k++) put_f64(b, v[k]);
  write_file(path, b);
}

void vec_read(const std::string& path, std::vector<double>& v) {
  std::vector<unsigned char> b = read_file(path);
  if (b.size() < 8 || get_u32(b.data()) != 1211214u) fail(FEM2D_E_IO, "not a PETSc vector file: " + path);
  const int32_t m = (int32_t)get_u32(&b[4]);
  if (m < 0 || b.size() < 8 + 8 * (size_t)m) fail(FEM2D_E_IO, "truncated vector file: " + path);
  v.resize(m);
  for (int32_t k = 0; k < m; k++) v[k] = get_f64(&b[8 + 8 * (size_t)k]);
}

void scalar_write(const std::string& path, double x) {
  std::vector<unsigned char> b;
  put_f64(b, x);
  write_file(path, b);
}

double scalar_read(const std::string& path) {
  std::vector<unsigned char> b = read_file(path);
  if (b.size() < 8) fail(FEM2D_E_IO, "truncated scalar file: " + path);
  return get_f64(b.data());
}

}  // namespace fem2d
