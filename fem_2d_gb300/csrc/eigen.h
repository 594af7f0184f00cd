// Eigensolvers on the device: dense (nalgebra_solve_gep restated) and sparse shift-invert.
#pragma once
#include "device.h"
#include "mfdev.h"

namespace fem2d {

struct Domain;
struct PatchNet;
void dense_solve(Ctx& c, const Domain& dom, const HostGEP& h, const DeviceGEP& d, MFPlan& plan, double target,
                 double* value, double* vector);
void sparse_solve(Ctx& c, const Domain& dom, const HostGEP& h, const DeviceGEP& d, MFPlan& plan, double target,
                  int n_pairs,
                  const fem2d_solve_opts& o, double* values, double* vectors, double* residuals,
                  fem2d_solve_stats* st, const PatchNet* net = nullptr);

// Y = ca A X + cb B X (device pointers, row-major n x nb, nb <= 32), queued on the context's stream
void gep_spmm(Ctx& c, const HostGEP& h, const DeviceGEP& d, double ca, double cb, const double* X, int64_t ldx, int nb,
              double* Y, int64_t ldy);
// the same on a pencil given by its own value arrays (full CSR order, the GEP's pattern)
void gep_spmm_values(Ctx& c, const HostGEP& h, const DeviceGEP& d, const double* va, const double* vb, double ca,
                     double cb, const double* X, int64_t ldx, int nb, double* Y, int64_t ldy);
void shifted_solve(Ctx& c, const Domain& dom, const HostGEP& h, const DeviceGEP& d, MFPlan& plan, double ca,
                   double cb, bool spd,
                   int nrhs, const double* rhs, double* x);
// C (device, row-major a x b) = X^T Y: method 0 on the tensor cores (ozaki.cu), 1 on the FP64 CUDA cores
// Z = beta Z + alpha X C (device, C row-major a x b): method 0 tensor cores, 1 FP64 CUDA cores
void block_gemm(Ctx& c, int method, int64_t n, const double* X, int64_t ldx, int a, const double* Cd, int b,
                double alpha, double beta, double* Z, int64_t ldz);
// Y = coef M X, M = A (which 0) or B (1), through the tensor-core product; synchronises
void gep_spmm_tensor(Ctx& c, const HostGEP& h, const DeviceGEP& d, int which, double coef, const double* X,
                     int64_t ldx, int nb, double* Y, int64_t ldy);
void block_gram(Ctx& c, int method, int64_t n, const double* X, int64_t ldx, int a, const double* Y, int64_t ldy,
                int b, double* Cd);

}  // namespace fem2d
