// Block congruence scaling of the pencil over row runs (blockscale.cu).
#pragma once
#include <cstdint>

#include "device.h"

namespace fem2d {

struct BlockScale {
  int ngrp = 0;
  DBuf<int32_t> grp_d;     // run starts, ngrp + 1
  DBuf<int64_t> soff;      // offset of each run's |g| x |g| block of S
  DBuf<int64_t> seg_ptr;   // per run, its column-run segments
  DBuf<int2> seg;          // (column run, offset of its first column within the run's rows)
  DBuf<double> S;          // blockdiag(L_g^-1), row-major lower-triangular blocks
  bool ready = false;      // the pattern part (runs, block offsets, segments) is set up
  // algorithmic work of one build: A and B read and S A S^T, S B S^T written (32 B per CSR entry), the
  // diagonal blocks of B read and S written and read; per run its Cholesky factor and inverse (R^3 FLOPs)
  // and per (run, column run) block of R x H entries both triangular products, for A and B
  double alg_bytes = 0.0, alg_flops = 0.0;
  // S from B's diagonal blocks; sa = S A S^T, sb = S B S^T (full CSR order, same pattern). The pattern
  // part is set up on the first call and kept.
  void build(Ctx& c, const HostGEP& h, const DeviceGEP& d, double* sa, double* sb);
  // X <- S^T X for an n x nb block (nb <= 32): eigenvectors of the scaled pencil back to the GEP's
  void unscale(Ctx& c, double* X, int64_t ldx, int nb) const;
};

}  // namespace fem2d
