// Device bodies of the two assembly kernels, shared by the single-GEP launches (assemble.cu) and the
// batched persistent launch over many GEPs (assemble_batch.cu), so both compute every value with the
// same operations in the same order.
#pragma once
#include <cuda_runtime.h>

#include "gep.h"
#include "shape.cuh"

namespace fem2d {
namespace {

// kind -> (family of the outer Elem at the scaled points, family of the inner Elem)
__device__ __forceinline__ int2 kind_families(int kind) {
  switch (kind) {
    case 0: return make_int2(0, 0);   // N  N
    case 1: return make_int2(3, 3);   // T' T'
    case 2: return make_int2(2, 2);   // T  T
    case 3: return make_int2(0, 3);   // N  T'
    default: return make_int2(3, 0);  // T' N
  }
}

// One (interval, axis, kind) table of 1-D contractions, P x P entries, strided over the block's threads:
//   G[a][b] = sum_m w_m X_a(s x_m + o) Y_b(x_m)            (glq.rs:19-32 restricted to one axis)
__device__ __forceinline__ void contract1d_table(int basis, int P, int nivl, int iv, int axis, int kind,
                                                 const double* __restrict__ ivl, const double* __restrict__ glq,
                                                 int nq_u, int nq_v, double* __restrict__ tables) {
  const int nq = axis == 0 ? nq_u : nq_v;
  const double* xs = axis == 0 ? glq : glq + 2 * nq_u;
  const double* ws = xs + nq;
  const double s = ivl[2 * iv], o = ivl[2 * iv + 1];
  const int2 fam = kind_families(kind);
  double* out = tables + (((size_t)axis * nivl + iv) * 5 + kind) * P * P;
  for (int t = threadIdx.x; t < P * P; t += blockDim.x) {
    const int a = t / P, b = t % P;
    double acc = 0.0;
    for (int m = 0; m < nq; m++) {
      const double x = xs[m];
      acc += ws[m] * shape(basis, fam.x, a, s * x + o) * shape(basis, fam.y, b, x);
    }
    out[t] = acc;
  }
}

// The value of one full CSR entry of A and B: the sum of its visits k0..k1-1, each the product
// C * Gu * Gv that equals the reference's 2-D Gauss sum (integrals.rs:26-92, 292-354).
__device__ __forceinline__ void entry_values(int64_t k0, int64_t k1, const uint64_t* __restrict__ codes,
                                             const GBlock* __restrict__ blocks, const uint32_t* __restrict__ specs,
                                             const double* __restrict__ tables, int P, int nivl, double& out_a,
                                             double& out_b) {
  const size_t PP = (size_t)P * P;
  const size_t axis_stride = (size_t)nivl * 5 * PP;
  double sa = 0.0, sb = 0.0;
  for (int64_t k = k0; k < k1; k++) {
    const uint64_t code = __ldg(codes + k);
    const GBlock* bl = blocks + (code >> 32);
    const int2 sp = __ldg(reinterpret_cast<const int2*>(bl));
    const int2 iv = __ldg(reinterpret_cast<const int2*>(bl) + 1);
    const uint32_t p = __ldg(specs + sp.x + (int)((code >> 16) & 0xffff));
    const uint32_t q = __ldg(specs + sp.y + (int)(code & 0xffff));
    const int pi = p & 0xff, pj = (p >> 8) & 0xff, pd = (p >> 16) & 0xff;
    const int qi = q & 0xff, qj = (q >> 8) & 0xff, qd = (q >> 16) & 0xff;
    const double* gu = tables + (size_t)iv.x * 5 * PP + (size_t)pi * P + qi;
    const double* gv = tables + axis_stride + (size_t)iv.y * 5 * PP + (size_t)pj * P + qj;
    const int dd = pd * 2 + qd;   // 0 UU, 1 UV, 2 VU, 3 VV
    const double ca = __ldg(bl->ca + dd);
    double va, vb = 0.0;
    if (dd == 0) {
      const double nn = __ldg(gu + G_NN * PP);
      va = ca * nn * __ldg(gv + G_DD * PP);
      vb = __ldg(bl->cb) * nn * __ldg(gv + G_TT * PP);
    } else if (dd == 3) {
      const double nn = __ldg(gv + G_NN * PP);
      va = ca * __ldg(gu + G_DD * PP) * nn;
      vb = __ldg(bl->cb + 1) * __ldg(gu + G_TT * PP) * nn;
    } else if (dd == 1) {
      va = ca * __ldg(gu + G_ND * PP) * __ldg(gv + G_DN * PP);
    } else {
      va = ca * __ldg(gu + G_DN * PP) * __ldg(gv + G_ND * PP);
    }
    sa += va;
    sb += vb;
  }
  out_a = sa;
  out_b = sb;
}

}  // namespace
}  // namespace fem2d
