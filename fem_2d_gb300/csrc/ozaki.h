// FP64 block Gram products on the tensor cores (tcgen05) by exact integer slicing (ozaki.cu).
#pragma once
#include <cstddef>
#include <cstdint>

namespace fem2d {

struct Ctx;

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
                double beta, double* Z, int64_t ldz, int* err);

}  // namespace fem2d
