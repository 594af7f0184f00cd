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

// measured issue cost (ns per instruction and SM) of tcgen05.mma kind::f16 with M = 128, K = 16 and the
// given N (16..256, multiple of 16)
double measure_mma_ns(Ctx& c, int n);

// Y = coef M X for a matrix M = ca A + cb B of a pencil (its values sliced once into digit planes: a
// slot), X and Y row-major n x nb (nb <= 32); every row of Y is written (overwritten), bitwise
// reproducibly. Built per pattern (row runs of at most 64 rows with one column list, 64-column items),
// sliced per slot.
// one item of the product kernel (a run and 64 columns of its list), in a CTA's processing order
struct alignas(16) TcSpmmItem {
  int64_t cbase;    // CSR position of the item's first column in the run's first row
  int64_t poff;     // its digit planes (uint4 units)
  int32_t eoff;     // its row exponents
  int32_t r0;       // the run's first row
  int16_t R, Lc;    // rows of the run, columns of the item
  int32_t last;     // 1 for the last item of its run
};

struct TcSpmm {
  static constexpr int kSlots = 4;
  int nitems = 0, grid = 0, nzero = 0;
  int64_t plane_units = 0, exp_count = 0;
  DBuf<int4> items;            // (run, first column, rows, columns) in run order, for slicing
  DBuf<int64_t> poff, eoff;
  DBuf<TcSpmmItem> citems;     // the same items in the product kernel's order: CTA by CTA
  DBuf<int32_t> cta_ptr;       // first item of each CTA (grid + 1)
  DBuf<int2> zruns;            // (first row, rows) of the runs without columns
  struct Slot {
    double ca = 0, cb = 0;
    bool ready = false;
    DBuf<uint4> planes;
    DBuf<int> exps;
  } slot[kSlots];
  void build(Ctx& c, int64_t n, const std::vector<int32_t>& grp, const std::vector<int64_t>& row_ptr);
  // slot k holds ca va + cb vb (vb may be null when cb = 0)
  void slice(Ctx& c, int k, const int32_t* grp, const int64_t* rp, const double* va, const double* vb, double ca,
             double cb);
  // the slot and factor with ca A + cb B = coef * slot, or -1: slots (1, 0) and (0, 1) serve every product
  // with A or B alone, the others their exact coefficients
  int find(double ca, double cb, double* coef) const;
  void apply(Ctx& c, int k, double coef, const int32_t* grp, const int64_t* rp, const int32_t* col, const double* X,
             int64_t ldx, int nb, double* Y, int64_t ldy, int* err);
};

}  // namespace fem2d
