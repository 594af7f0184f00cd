// FP64 block Gram products on the tensor cores (tcgen05) by exact integer slicing (ozaki.cu).
#pragma once
#include <cstddef>
#include <cstdint>
#include <vector>

#include "device.h"

namespace fem2d {


// number of row-range partial tiles the Gram kernel writes for an (n, a, b) product
int ozaki_gram_partials(int64_t n, int a, int b, int num_sms);
// FP64 workspace (doubles) ozaki_gram needs for an (n, a, b) product
size_t ozaki_gram_workspace(int64_t n, int a, int b, int num_sms);
// C (device, row-major a x b) = X^T Y for row-major X (n x a, ldx) and Y (n x b, ldy), accurate to
// FP64 rounding in the normwise sense; a <= 512, b <= 256. Queued on c.stream; *err (device) is set
// nonzero if a bounded wait inside the kernel expired.
void ozaki_gram(Ctx& c, int64_t n, const double* X, int64_t ldx, int a, const double* Y, int64_t ldy, int b,
                double* C, double* work, size_t work_doubles, int* err);

// Z (row-major n x b, ldz) = beta Z + alpha X C for X (n x a, ldx) and C (device, row-major a x b);
// a <= 256, b <= 32; FP64 emulated on the tensor cores (one exponent per row of X and per column of C,
// normwise accuracy at FP64 rounding level). Queued on c.stream; *err as ozaki_gram.
void ozaki_gemm(Ctx& c, int64_t n, const double* X, int64_t ldx, int a, const double* C, int b, double alpha,
                double beta, double* Z, int64_t ldz, int* rowexp /* n ints of scratch */, int* err);

// Y = coef M X for one matrix M of a pencil (its values sliced once into digit planes), X and Y
// row-major n x nb (nb <= 32), Y accumulated (zero it first). Built per pattern (row runs of at most
// 64 rows with one column list), sliced per value array: which = 0 (A) or 1 (B).
struct TcSpmm {
  int nitems = 0;
  int64_t plane_units = 0, exp_count = 0;
  DBuf<int4> items;
  DBuf<int64_t> poff, eoff;
  DBuf<uint4> planesA, planesB;
  DBuf<int> expA, expB;
  bool readyA = false, readyB = false;
  void build(Ctx& c, int64_t n, const std::vector<int32_t>& grp, const std::vector<int64_t>& row_ptr);
  void slice(Ctx& c, const int32_t* grp, const int64_t* rp, const double* v, int which);
  void apply(Ctx& c, int which, double coef, const int32_t* grp, const int64_t* rp, const int32_t* col,
             const double* X, int64_t ldx, int nb, double* Y, int64_t ldy, int* err);
};

}  // namespace fem2d
