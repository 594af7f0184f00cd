// Device side of the multifrontal factorization (mf.cu).
#pragma once
#include <cstring>
#include <memory>
#include <mutex>
#include <vector>

#include "blockscale.h"
#include "device.h"
#include "mf.h"
#include "ozaki.h"

namespace fem2d {

// One numeric factorization: dense fronts and their row pivots.
struct MFFactor {
  DBuf<double> F;
  DBuf<int32_t> piv;
  DBuf<int32_t> perm;    // gather permutation equivalent to the row swaps
  DBuf<int32_t> iperm;   // its inverse
  int flags = 0;   // 1: a zero pivot was perturbed, 2: a non-positive pivot in Cholesky mode
  std::vector<int32_t> weak;   // DoFs whose columns had no stable pivot among their front's fully-summed rows
  // dense single-front plans (small GEPs): F holds the explicit inverse K^-1 (n x n) instead of LU
  // factors (Gauss-Jordan, partial pivoting); solves are then one dense product
  int64_t inv_n = 0;
};

struct MFDevice {
  int nf = 0, nlevels = 0, max_f = 0, max_p = 0, nb_cap = 0;
  int64_t mat_total = 0, piv_total = 0;
  double factor_flops = 0;   // LU flops of all fronts, 2/3 (f^3 - (f - p)^3) each (half for Cholesky)
  std::vector<int32_t> level_ptr;
  std::vector<int64_t> level_off;
  std::vector<int32_t> level_max_f, level_max_p;
  std::vector<double> level_factor_bytes;   // L (forward) or U (backward) bytes read per level
  DBuf<uint8_t> desc;
  DBuf<int32_t> lfronts, dofs, ea_map;
  DBuf<int64_t> asm_pos, asm_csr, piv_off, woff;
  DBuf<double> work;
  DBuf<int> flags;
  DBuf<int32_t> weak_list;   // capacity n: weak-pivot DoFs recorded by the panel kernel
  DBuf<int> weak_count;
  // per level, the fronts solved by one CTA each (inverted diagonal blocks) and the rest (clusters)
  std::vector<int32_t> small_ptr, large_ptr;   // nlevels + 1 offsets into lsmall / llarge
  std::vector<int32_t> level_small_f, level_small_p;
  DBuf<int32_t> lsmall, llarge;
  int nsmall = 0, max_small_p = 0;
  // tiled levels (narrow upper levels solved through the fronts' partitioned inverses, rows spread over
  // many CTAs): per level a flag and offsets into the (front, first row) items of each direction
  std::vector<uint8_t> level_tiled;
  std::vector<int32_t> tf_ptr, tb_ptr;
  DBuf<int32_t> tf_items, tb_items;
  DBuf<int64_t> prow, src_off;   // pull lists of the tiled fronts' right-hand sides
  DBuf<int32_t> src_str;
  // factor-time work of the tiled fronts: diagonal inversion of those outside lsmall (p <= kSmallP:
  // lmid; larger: lwide, 32-column items, scratch squares sq), then the partitioned-inverse items
  DBuf<int32_t> lmid, lwide, wide_items, pinv_items;
  DBuf<double> sq;
  int nmid = 0, max_mid_p = 0, nwide = 0, nwide_items = 0, max_wide_p = 0, npinv = 0, max_tiled_p = 0;

  void setup(Ctx& c, const MFSymbolic& s, int nb_max);
  // factor c_a*A + c_b*B (values in full-CSR order); Cholesky mode skips pivoting (SPD shifts)
  void factor(Ctx& c, const double* va, const double* vb, double ca, double cb, bool cholesky, MFFactor& out);
  // X = K^-1 B for an n x nb row-major block (nb <= nb_cap); B and X must not alias
  void solve(Ctx& c, const MFFactor& fac, const double* B, int64_t ldb, double* X, int64_t ldx, int nb);
  int read_flags(Ctx& c);
};

// The factorization plan of one GEP: the host symbolic phase and its device copy depend on the
// sparsity pattern only, so they are built on the first solve of a GEP and reused by later solves of
// the same GEP (numeric factorizations are always recomputed). mu serialises solves that share the
// plan's solve workspace.
struct MFPlan {
  std::unique_ptr<MFSymbolic> sym;
  std::unique_ptr<MFDevice> mf;
  bool ready = false;
  bool dense = false;   // a single dense front (chosen when the sparse plan's solves are inaccurate)
  std::vector<uint8_t> lift;   // per DoF: levels its elimination was moved up (delayed pivots)
  int device = -1;
  // pattern-only structures of the eigensolver, built on first use on the plan's device: the row-run
  // block scaling's blocks and segments, the tensor-core operator products' items (their values are
  // recomputed, and the pencil re-sliced, by every solve)
  std::unique_ptr<BlockScale> bsc;
  std::unique_ptr<TcSpmm> tcs;
  int aux_device = -1;
  std::mutex mu;
};

// the plan's MFDevice, building the plan on first use (or after a device change); `pre`, when given, is
// the sparse symbolic analysis already computed for this GEP
MFDevice& mf_plan(MFPlan& p, Ctx& c, const Domain& dom, const HostGEP& h, std::unique_ptr<MFSymbolic> pre = nullptr);
// replace the plan by the dense single-front plan
MFDevice& mf_plan_dense(MFPlan& p, Ctx& c, const HostGEP& h);

}  // namespace fem2d
