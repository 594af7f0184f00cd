// Inner iterative solver of the shifted pencil K = ca A + cb B (SPD shifts) with two preconditioners:
//
//  * plain: additive Schwarz over Elem patches ("block-Jacobi": every Elem's own basis functions, the
//    edge functions it shares included, with the exact inverse of its diagonal block of K);
//  * learned: the same plus a two-level coarse correction whose coarse basis a per-Elem-patch network
//    produces: for every spec (basis function) of an Elem, a small MLP maps 16 geometric and
//    polynomial features to k coefficients, so each Elem contributes k coarse vectors (weighted by a
//    partition of unity on shared functions). The coarse operator Z^T K Z is inverted densely.
//
// The network is trained on the GPU by its own forward/backward/Adam kernels on error vectors that
// the plain solver produces (e = x* - x_i at its iterates, x* from the exact multifrontal solve): the
// loss is the relative distance of each Elem's restriction of e from the span of that Elem's k
// vectors, averaged over Elems and samples. Its gradient with respect to the vectors has the closed
// form -2 (e - Z c*) c*^T / ||e||^2 (c* the least-squares coefficients).
#pragma once
#include <cstdint>
#include <memory>
#include <vector>

#include "device.h"
#include "domain.h"

namespace fem2d {

constexpr int kPatchFeatures = 16;

struct PatchNet {
  int nin = kPatchFeatures, hidden = 192, k = 16;
  std::vector<float> params;   // W1 (nin x H), b1 (H), W2 (H x H), b2 (H), W3 (H x k), b3 (k); row-major
  int64_t size() const { return (int64_t)nin * hidden + hidden + (int64_t)hidden * hidden + hidden + (int64_t)hidden * k + k; }
  void init(uint64_t seed);
};

// Per-Elem patches of a Domain: rows = specs in Domain order, patch p = one Elem with specs.
struct Patches {
  int64_t nrows = 0;
  std::vector<int64_t> ptr;     // npatch + 1
  std::vector<int32_t> dof;     // per row
  std::vector<float> feat;      // per row, kPatchFeatures
  std::vector<float> weight;    // per row: 1 / (number of rows bound to the same DoF)
  int npatch() const { return (int)ptr.size() - 1; }
};
void build_patches(const Domain& d, double shift, Patches& out);

// Loss and gradient of the network on one GEP's patches for S error samples (E: n x S row-major,
// host). Returns the mean loss; grad (size params) is added to.
double patchnet_loss_grad(Ctx& c, const PatchNet& net, const Patches& pt, int64_t n, const double* E, int S,
                          std::vector<float>& grad);

// Adam training over several GEPs' samples; returns the loss of each epoch (mean over GEPs).
std::vector<double> patchnet_train(Ctx& c, PatchNet& net, const std::vector<const Patches*>& pts,
                                   const std::vector<int64_t>& ns, const std::vector<const double*>& Es, int S,
                                   int epochs, double lr);

struct PCGStats {
  int iters = 0;
  double relres = 0, ms = 0, setup_ms = 0;
  int coarse_dim = 0;
};

class PCGSolver {
 public:
  // net: learned coarse basis; else basis (nrows x basis_k floats, rows in patch order) when given; else plain.
  // va, vb: the pencil's values (full CSR order, the GEP's pattern) when not the GEP's own A and B (the
  // eigensolver passes its scaled pencil)
  PCGSolver(Ctx& c, const Domain& dom, const HostGEP& h, const DeviceGEP& d, double ca, double cb,
            const PatchNet* net, const float* basis = nullptr, int basis_k = 0, const double* va = nullptr,
            const double* vb = nullptr);
  ~PCGSolver();
  // device-resident solves of nb <= 32 right-hand sides (row-major n x nb blocks, leading dimensions
  // ldr and ldx), zero start, per column to ||r|| <= tol ||b|| (CG) or ||r||_P <= tol ||b||_P (MINRES):
  //  cg_device:     K = ca A + cb B (the solver's SPD shift) by preconditioned CG
  //  minres_device: ka A + kb B (symmetric, possibly indefinite) by MINRES with this solver's SPD
  //                 preconditioner
  void cg_device(const double* R, int64_t ldr, double* X, int64_t ldx, int nb, double tol, int max_iter,
                 PCGStats* st);
  // (coarse = false: the additive-Schwarz part of the preconditioner only)
  void minres_device(double ka, double kb, const double* R, int64_t ldr, double* X, int64_t ldx, int nb, double tol,
                     int max_iter, PCGStats* st, bool coarse = true);
  // x = K^-1 rhs (n x nrhs row-major, host) by preconditioned CG, per column to ||r|| <= tol ||b||
  void solve(int nrhs, const double* rhs, double* x, double tol, int max_iter, PCGStats* st,
             std::vector<double>* snaps = nullptr, const double* xstar = nullptr, int every = 0, int max_snaps = 0,
             int first = 0);
  int coarse_dim() const;
  double setup_ms() const;

  struct Impl;

 private:
  std::unique_ptr<Impl> p_;
};

}  // namespace fem2d
