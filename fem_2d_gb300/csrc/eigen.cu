// Eigensolvers on the device.
//
// gpu_solve_gep (stands beside slepc_solve_gep, slepc_solve.rs:14-68): the n_pairs eigenpairs of
// (A, B) nearest the target sigma among the non-spurious spectrum. The curl-curl operator has a large
// null space (gradients, lambda = 0) which sits at distance |sigma| from the target; the reference
// treats such modes as spurious (nalgebra_solve.rs:24-26). The pencil is first scaled by the Cholesky
// factors of B's row-run diagonal blocks (blockscale.cu; Jacobi scaling as the fallback). The search
// space is generated with
//     T = (A - sigma B)^-1 A (A + c B)^-1 B
// with c = |sigma|: eigenvalue lambda / ((lambda - sigma)(lambda + c)), close to the plain
// shift-invert 1 / (lambda - sigma) for the physical modes, zero on the null space (A kills it
// whatever the accuracy of the SPD solve; rounding smears it to small lambda, damped by
// lambda / (lambda + c)) and small for high-frequency modes; exact multifrontal solves (mf.cu). Each
// cycle builds a block Krylov basis [XL, X, TX, ..., T^s X] (s = 4 by default; XL the locked converged
// pairs, X the active Ritz vectors), B-orthonormalised by CGS2 in FP64, then a Rayleigh-Ritz step on
// the pencil (A, B) itself (FP64) over the active columns; Ritz pairs with a relative residual above 1
// (mixtures of null-space and high-frequency directions that land near sigma) are not selected.
// Residuals ||A x - lambda B x|| / (|lambda| ||B x||) and backward errors are computed in FP64.
//
// nalgebra_solve_gep (nalgebra_solve.rs:14-50) on the device: B is factored (Cholesky mode; a
// non-positive pivot is FailedToInvertB), Z = B^-1 A is formed column block by column block, and
// the eigen-decomposition of the symmetric matrix built from the lower triangle of Z (the triangle
// nalgebra's SymmetricEigen reads) gives the pair nearest the target.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <future>
#include <cmath>
#include <mutex>
#include <numeric>

#include "blockscale.h"
#include <memory>

#include "eigen.h"
#include "ozaki.h"
#include "precond.h"
#include "mf.h"
#include "mfdev.h"
#include "symeig.h"

namespace fem2d {


namespace {

// ---------------------------------------------------------------- dense block kernels
// Y = ca*A*X + cb*B*X; X, Y row-major (ldx, ldy), nb <= 32 columns. One warp per row; the warp's
// lanes split into (32 / G) groups of G >= nb lanes, each group walking a slice of the row's entries.
// Y = (ca A + cb B) X for nb <= 32 columns, one warp per row. The warp first loads up to 128
// (col, value) pairs of its row (four coalesced 32-entry chunks, issued back to back), then lane
// (sub, c) gathers X[col_e][c] for the entries e = sub, sub + 32/G, ... of every chunk (G = columns
// rounded up to a power of two). All gathers of the 128 entries are independent of each other, so a
// row costs about two memory round trips instead of two per chunk. Partial sums of the 32/G entry
// groups are combined with shuffles.
__global__ void __launch_bounds__(256) spmm_kernel(int64_t n, const int64_t* __restrict__ rp,
                                                   const int32_t* __restrict__ col, const double* __restrict__ va,
                                                   const double* __restrict__ vb, double ca, double cb,
                                                   const double* __restrict__ X, int64_t ldx, int nb, int G,
                                                   double* __restrict__ Y, int64_t ldy) {
  constexpr int CH = 4;   // chunks of 32 entries staged per pass
  const int lane = threadIdx.x & 31;
  const int groups = 32 / G;
  const int c = lane % G, sub = lane / G;
  const bool live = c < nb;
  for (int64_t row = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; row < n;
       row += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    double acc = 0.0;
    const int64_t k1 = rp[row + 1];
    for (int64_t k0 = rp[row]; k0 < k1; k0 += 32 * CH) {
      int mc[CH];
      double mv[CH];
#pragma unroll
      for (int q = 0; q < CH; q++) {
        const int64_t kk = k0 + 32 * q + lane;
        mc[q] = 0;
        mv[q] = 0.0;
        if (kk < k1) {
          mc[q] = __ldg(col + kk);
          if (ca != 0.0) mv[q] += ca * __ldg(va + kk);
          if (cb != 0.0) mv[q] += cb * __ldg(vb + kk);
        }
      }
      const int cnt = (int)min((int64_t)(32 * CH), k1 - k0);
#pragma unroll
      for (int q = 0; q < CH; q++) {
        if (32 * q >= cnt) break;   // warp-uniform
#pragma unroll 8
        for (int e0 = 0; e0 < 32; e0 += groups) {
          const int e = e0 + sub;
          const int cj = __shfl_sync(0xffffffffu, mc[q], e);
          const double vj = __shfl_sync(0xffffffffu, mv[q], e);
          if (32 * q + e < cnt && live) acc += vj * __ldg(X + (int64_t)cj * ldx + c);
        }
      }
    }
    for (int off = G; off < 32; off <<= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
    if (sub == 0 && live) Y[row * ldy + c] = acc;
  }
}

// Y = (ca A + cb B) X for nb <= 32 columns over runs of rows with one shared column list (an Elem's
// interior functions couple to the same functions). A work item is one run and one segment of at most
// 256 of its columns, so the long rows of ancestor Elems (over a thousand columns) spread over many
// CTAs. Per pass of 48 columns a CTA stages the gathered X rows (48 x nb) and the run's combined
// values ca*A + cb*B (rows x 48, each row's entries read contiguously) in shared memory, accumulates
// every (row, column) output from shared memory only, and adds its partial sums to Y (zeroed before
// the launch) with FP64 atomics. X is gathered once per run instead of once per row. Up to 64 rows x
// 32 columns = 8 outputs per thread.
constexpr int kGrpChunk = 48;
constexpr int kGrpRows = 64;
constexpr int kGrpSeg = 256;
__global__ void zero_block_kernel(int64_t n, int nb, double* __restrict__ Y, int64_t ldy) {
  const int64_t total = n * nb;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x)
    Y[(t / nb) * ldy + t % nb] = 0.0;
}

__global__ void __launch_bounds__(256) spmm_group_kernel(int nwork, const int2* __restrict__ work,
                                                         const int32_t* __restrict__ grp,
                                                         const int64_t* __restrict__ rp,
                                                         const int32_t* __restrict__ col,
                                                         const double* __restrict__ va, const double* __restrict__ vb,
                                                         double ca, double cb, const double* __restrict__ X,
                                                         int64_t ldx, int nb, double* __restrict__ Y, int64_t ldy) {
  __shared__ double xs[kGrpChunk * 32];
  __shared__ double vs[kGrpRows * (kGrpChunk + 1)];
  for (int w = blockIdx.x; w < nwork; w += gridDim.x) {
    const int2 it = work[w];
    const int r0 = grp[it.x], R = grp[it.x + 1] - r0;
    const int64_t c0 = rp[r0];
    const int cend = min((int)(rp[r0 + 1] - c0), it.y + kGrpSeg);
    const int32_t* cols = col + c0;
    double acc[8];
#pragma unroll
    for (int o = 0; o < 8; o++) acc[o] = 0.0;
    for (int q0 = it.y; q0 < cend; q0 += kGrpChunk) {
      const int qn = min(kGrpChunk, cend - q0);
      __syncthreads();
      for (int t = threadIdx.x; t < qn * nb; t += blockDim.x) {
        const int q = t / nb, j = t - q * nb;
        xs[q * 32 + j] = __ldg(X + (int64_t)__ldg(cols + q0 + q) * ldx + j);
      }
      for (int t = threadIdx.x; t < R * kGrpChunk; t += blockDim.x) {
        const int r = t / kGrpChunk, q = t - r * kGrpChunk;
        double v = 0.0;
        if (q < qn) {
          const int64_t k = rp[r0 + r] + q0 + q;
          if (ca != 0.0) v += ca * __ldg(va + k);
          if (cb != 0.0) v += cb * __ldg(vb + k);
        }
        vs[r * (kGrpChunk + 1) + q] = v;
      }
      __syncthreads();
#pragma unroll
      for (int o = 0; o < 8; o++) {
        const int t = threadIdx.x + o * 256;
        if (t < R * nb) {
          const int r = t / nb, j = t - r * nb;
          const double* vr = vs + r * (kGrpChunk + 1);
          double s = acc[o];
#pragma unroll 8
          for (int q = 0; q < qn; q++) s += vr[q] * xs[q * 32 + j];
          acc[o] = s;
        }
      }
    }
#pragma unroll
    for (int o = 0; o < 8; o++) {
      const int t = threadIdx.x + o * 256;
      if (t < R * nb) {
        const int r = t / nb, j = t - r * nb;
        atomicAdd(Y + (int64_t)(r0 + r) * ldy + j, acc[o]);
      }
    }
  }
}

__global__ void __launch_bounds__(256) gram_partial_kernel(int64_t n, const double* __restrict__ X, int64_t ldx, int a,
                                                           const double* __restrict__ Y, int64_t ldy, int b,
                                                           int64_t rows_per_block, int e0, double* __restrict__ P) {
  extern __shared__ double sm[];
  double* xs = sm;               // 32 x a
  double* ys = sm + 32 * a;      // 32 x b
  const int64_t r0 = blockIdx.x * rows_per_block;
  const int64_t r1 = min(n, r0 + rows_per_block);
  const int ab = a * b;
  double acc[8];
  for (int q = 0; q < 8; q++) acc[q] = 0.0;
  for (int64_t rt = r0; rt < r1; rt += 32) {
    const int nr = (int)min((int64_t)32, r1 - rt);
    __syncthreads();
    for (int t = threadIdx.x; t < 32 * a; t += blockDim.x) {
      const int r = t / a, i = t % a;
      xs[t] = r < nr ? X[(rt + r) * ldx + i] : 0.0;
    }
    for (int t = threadIdx.x; t < 32 * b; t += blockDim.x) {
      const int r = t / b, j = t % b;
      ys[t] = r < nr ? Y[(rt + r) * ldy + j] : 0.0;
    }
    __syncthreads();
    for (int q = 0; q < 8; q++) {
      const int e = e0 + threadIdx.x + q * blockDim.x;
      if (e >= ab) break;
      const int i = e / b, j = e % b;
      double s = acc[q];
      for (int r = 0; r < nr; r++) s += xs[r * a + i] * ys[r * b + j];
      acc[q] = s;
    }
  }
  for (int q = 0; q < 8; q++) {
    const int e = e0 + threadIdx.x + q * blockDim.x;
    if (e < ab) P[(int64_t)blockIdx.x * ab + e] = acc[q];
  }
}

__global__ void reduce_partials_kernel(const double* __restrict__ P, int nblk, int ab, double* __restrict__ C) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ab) return;
  double s = 0.0;
  for (int k = 0; k < nblk; k++) s += P[(int64_t)k * ab + e];
  C[e] = s;
}

// Z = beta*Z + X * C; X n x a (ldx), C a x b row-major (device), Z n x b (ldz)
__global__ void __launch_bounds__(256) gemm_nn_kernel(int64_t n, const double* __restrict__ X, int64_t ldx, int a,
                                                      const double* __restrict__ C, int b, double alpha, double beta,
                                                      double* __restrict__ Z, int64_t ldz) {
  extern __shared__ double cs[];
  for (int t = threadIdx.x; t < a * b; t += blockDim.x) cs[t] = C[t];
  __syncthreads();
  const int64_t total = n * b;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = t / b;
    const int j = (int)(t % b);
    const double* xr = X + r * ldx;
    // four independent accumulators keep several row loads in flight
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
    int i = 0;
#pragma unroll 2
    for (; i + 4 <= a; i += 4) {
      s0 += xr[i] * cs[i * b + j];
      s1 += xr[i + 1] * cs[(i + 1) * b + j];
      s2 += xr[i + 2] * cs[(i + 2) * b + j];
      s3 += xr[i + 3] * cs[(i + 3) * b + j];
    }
    for (; i < a; i++) s0 += xr[i] * cs[i * b + j];
    double s = (s0 + s1) + (s2 + s3);
    if (alpha != 1.0) s *= alpha;
    Z[r * ldz + j] = beta == 0.0 ? s : beta * Z[r * ldz + j] + s;
  }
}

__global__ void copy_block_kernel(int64_t n, int b, const double* __restrict__ X, int64_t ldx, double* __restrict__ Y,
                                  int64_t ldy) {
  const int64_t total = n * b;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = t / b;
    const int j = (int)(t % b);
    Y[r * ldy + j] = X[r * ldx + j];
  }
}

// per CTA the largest absolute row sum of ka A + kb B over its rows (an upper bound of the 2-norm);
// one warp per row (coalesced reads of the row's values)
__global__ void __launch_bounds__(256) rowsum_max_kernel(int64_t n, const int64_t* __restrict__ rp,
                                                         const double* __restrict__ va, const double* __restrict__ vb,
                                                         double ka, double kb, double* __restrict__ part) {
  __shared__ double red[256];
  const int lane = threadIdx.x & 31;
  const int64_t warp0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  double m = 0.0;
  for (int64_t r = warp0; r < n; r += nwarps) {
    double s = 0.0;
    for (int64_t k = rp[r] + lane; k < rp[r + 1]; k += 32) s += fabs(ka * va[k] + kb * vb[k]);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    m = fmax(m, s);
  }
  red[threadIdx.x] = m;
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + st]);
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// Y = alpha X + beta Y on an n x b row-major block
__global__ void axpby_kernel(int64_t n, int b, double alpha, const double* __restrict__ X, int64_t ldx, double beta,
                             double* __restrict__ Y, int64_t ldy) {
  const int64_t total = n * b;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = t / b;
    const int j = (int)(t % b);
    Y[r * ldy + j] = alpha * X[r * ldx + j] + beta * Y[r * ldy + j];
  }
}

// R = AX - BX * diag(theta) column by column, accumulating per CTA the column sums of squares of R, of
// BX and of X: P[cta][0, b) = |R|^2, [b, 2b) = |BX|^2, [2b, 3b) = |X|^2
__global__ void __launch_bounds__(256) resid_partial_kernel(int64_t n, const double* __restrict__ AX,
                                                            const double* __restrict__ BX,
                                                            const double* __restrict__ X, int64_t ld, int b,
                                                            const double* __restrict__ theta, int64_t rows_per_block,
                                                            double* __restrict__ P) {
  __shared__ double sr[256], sb[256], sx[256];
  const int64_t r0 = blockIdx.x * rows_per_block, r1 = min(n, r0 + rows_per_block);
  for (int j = 0; j < b; j++) {
    double a1 = 0.0, a2 = 0.0, a3 = 0.0;
    const double th = theta[j];
    for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
      const double bx = BX[r * ld + j];
      const double res = AX[r * ld + j] - th * bx;
      const double x = X[r * ld + j];
      a1 += res * res;
      a2 += bx * bx;
      a3 += x * x;
    }
    sr[threadIdx.x] = a1;
    sb[threadIdx.x] = a2;
    sx[threadIdx.x] = a3;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
      if (threadIdx.x < s) {
        sr[threadIdx.x] += sr[threadIdx.x + s];
        sb[threadIdx.x] += sb[threadIdx.x + s];
        sx[threadIdx.x] += sx[threadIdx.x + s];
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      P[(int64_t)blockIdx.x * 3 * b + j] = sr[0];
      P[(int64_t)blockIdx.x * 3 * b + b + j] = sb[0];
      P[(int64_t)blockIdx.x * 3 * b + 2 * b + j] = sx[0];
    }
    __syncthreads();
  }
}

// s[i] = 1 / sqrt(B_ii) (B is SPD); one warp per row
// per block of rows and column q < k: the entry of largest magnitude (signed) and its row, the first
// such row in the block's ascending range (ties keep the smaller row)
__global__ void __launch_bounds__(256) colmax_partial_kernel(int64_t n, const double* __restrict__ X, int64_t ldx,
                                                             int k, double* __restrict__ pm, int64_t* __restrict__ pi) {
  __shared__ double sv[256];
  __shared__ int64_t si[256];
  const int64_t per = (n + gridDim.x - 1) / gridDim.x;
  const int64_t r0 = blockIdx.x * per, r1 = min(n, r0 + per);
  for (int q = 0; q < k; q++) {
    double bv = 0.0;
    int64_t bi = INT64_MAX;
    for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
      const double v = X[r * ldx + q];
      if (fabs(v) > fabs(bv) || bi == INT64_MAX) {
        bv = v;
        bi = r;
      }
    }
    sv[threadIdx.x] = bv;
    si[threadIdx.x] = bi;
    __syncthreads();
    for (int off = 128; off > 0; off >>= 1) {
      if (threadIdx.x < off) {
        const double ov = sv[threadIdx.x + off];
        const int64_t oi = si[threadIdx.x + off];
        const double mv = sv[threadIdx.x];
        const int64_t mi = si[threadIdx.x];
        if (oi != INT64_MAX && (mi == INT64_MAX || fabs(ov) > fabs(mv) || (fabs(ov) == fabs(mv) && oi < mi))) {
          sv[threadIdx.x] = ov;
          si[threadIdx.x] = oi;
        }
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      pm[(int64_t)blockIdx.x * k + q] = sv[0];
      pi[(int64_t)blockIdx.x * k + q] = si[0] == INT64_MAX ? INT64_MAX : si[0];
    }
    __syncthreads();
  }
}

// VT[q * n + i] = sgn[q] X[i * ldx + q]: one contiguous vector per pair
__global__ void signed_transpose_kernel(int64_t n, const double* __restrict__ X, int64_t ldx, int k,
                                        const double* __restrict__ sgn, double* __restrict__ VT) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n * k; t += (int64_t)gridDim.x * blockDim.x) {
    const int q = (int)(t / n);
    const int64_t i = t - (int64_t)q * n;
    VT[t] = sgn[q] * X[i * ldx + q];
  }
}

__global__ void jacobi_scale_kernel(int64_t n, const int64_t* __restrict__ rp, const int32_t* __restrict__ col,
                                    const double* __restrict__ vb, double* __restrict__ sc, int* __restrict__ bad) {
  const int lane = threadIdx.x & 31;
  for (int64_t row = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; row < n;
       row += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    for (int64_t k = rp[row] + lane; k < rp[row + 1]; k += 32)
      if (col[k] == row) {
        const double dg = vb[k];
        if (dg > 0.0) sc[row] = 1.0 / sqrt(dg);
        else {
          sc[row] = 1.0;
          atomicOr(bad, 1);
        }
      }
  }
}

// out = diag(s) M diag(s) for M in {A, B}, entry by entry in CSR order; one warp per row
__global__ void scale_csr_kernel(int64_t n, const int64_t* __restrict__ rp, const int32_t* __restrict__ col,
                                 const double* __restrict__ va, const double* __restrict__ vb,
                                 const double* __restrict__ sc, double* __restrict__ oa, double* __restrict__ ob) {
  const int lane = threadIdx.x & 31;
  for (int64_t row = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; row < n;
       row += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const double sr = sc[row];
    for (int64_t k = rp[row] + lane; k < rp[row + 1]; k += 32) {
      const double f = sr * sc[col[k]];
      oa[k] = va[k] * f;
      ob[k] = vb[k] * f;
    }
  }
}

// X[r][c] *= s[r] for a row-major block
__global__ void scale_rows_kernel(int64_t n, int b, const double* __restrict__ sc, double* __restrict__ X, int64_t ld) {
  const int64_t total = n * b;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = t / b;
    X[r * ld + (t % b)] *= sc[r];
  }
}

// dense n x n row-major from the full CSR (ca*A + cb*B)
__global__ void densify_kernel(int64_t n, const int64_t* __restrict__ rp, const int32_t* __restrict__ col,
                               const double* __restrict__ va, const double* __restrict__ vb, double ca, double cb,
                               double* __restrict__ D) {
  for (int64_t r = blockIdx.x; r < n; r += gridDim.x)
    for (int64_t k = rp[r] + threadIdx.x; k < rp[r + 1]; k += blockDim.x) D[r * n + col[k]] = ca * va[k] + cb * vb[k];
}

// ---------------------------------------------------------------- host helpers
void setup_gemm_smem(int device);

struct Dev {
  Ctx& c;
  const HostGEP& h;
  const DeviceGEP& d;
  const double* va;   // values used by spmm (the GEP's, or a scaled copy)
  const double* vb;
  DBuf<double> part;
  DBuf<double> small;
  int dense_mode = 0;    // Gram products: 0 FP64 emulated on the tensor cores (ozaki.cu), 1 FP64 CUDA cores
  TcSpmm* tcs = nullptr;  // products with A or B alone on the tensor cores when set (slices of va, vb)
  DBuf<double> ozw;      // tensor Gram workspace (partial tiles)
  DBuf<int> ozerr;       // set by the tensor Gram kernel when a bounded wait expired
  DBuf<int> ozrow;       // row exponents of the tensor block update
  int grid_rows() const { return std::max(1, c.num_sms * 2); }

  // C (device, a x b) = X^T Y on the tensor cores; false when the FP64 CUDA-core kernels must be used
  bool tensor_gram(const double* X, int64_t ldx, int a, const double* Y, int64_t ldy, int b, double* Cd) {
    if (dense_mode != 0 || a > 512 || b > 256 || a <= 0 || b <= 0) return false;
    ProfScope ps(c, "gram_tc", 8.0 * h.n * (a + b), 2.0 * h.n * a * b);
    const size_t need = ozaki_gram_workspace(h.n, a, b, c.num_sms);
    if (ozw.n < need) ozw.alloc_on(std::max(need, ozaki_gram_workspace(h.n, 160, 160, c.num_sms)), c.stream);
    if (ozerr.n == 0) {
      ozerr.alloc_on(1, c.stream);
      FEM2D_CUDA(cudaMemsetAsync(ozerr.p, 0, sizeof(int), c.stream));
    }
    ozaki_gram(c, h.n, X, ldx, a, Y, ldy, b, Cd, ozw.p, ozw.n, ozerr.p);
    return true;
  }
  // Z = beta Z + alpha X C (C device, a x b) on the tensor cores; false when the FP64 kernel must be used
  bool tensor_gemm(const double* X, int64_t ldx, int a, const double* Cd, int b, double alpha, double beta, double* Z,
                   int64_t ldz) {
    if (dense_mode != 0 || a > 256 || b > 32 || a <= 0 || b <= 0) return false;
    ProfScope ps(c, "gemm_tc", 8.0 * h.n * (a + (beta != 0.0 ? 2.0 : 1.0) * b), 2.0 * h.n * a * b);
    if (ozerr.n == 0) {
      ozerr.alloc_on(1, c.stream);
      FEM2D_CUDA(cudaMemsetAsync(ozerr.p, 0, sizeof(int), c.stream));
    }
    if (ozrow.n < (size_t)std::max<int64_t>(h.n, 1)) ozrow.alloc_on(std::max<int64_t>(h.n, 1), c.stream);
    ozaki_gemm(c, h.n, X, ldx, a, Cd, b, alpha, beta, Z, ldz, ozrow.p, ozerr.p);
    return true;
  }
  // the tensor Gram kernel's error flag (synchronises the stream)
  void check_tensor() {
    if (ozerr.n == 0) return;
    int e = 0;
    FEM2D_CUDA(cudaMemcpyAsync(&e, ozerr.p, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    FEM2D_CUDA(cudaStreamSynchronize(c.stream));
    if (e) fail(FEM2D_E_TIMEOUT, "tensor-core Gram kernel: a bounded wait expired");
  }

  void spmm(double ca, double cb, const double* X, int64_t ldx, int nb, double* Y, int64_t ldy) {
    const double nv = (ca != 0.0) + (cb != 0.0);
    double coef = 1.0;
    const int slot = (tcs && nb <= 32 && nv > 0.0) ? tcs->find(ca, cb, &coef) : -1;
    if (slot >= 0) {
      ProfScope ps(c, "spmm_tc", (double)tcs->plane_units * 16.0 + 4.0 * h.nnz_full + 16.0 * h.n * nb,
                   2.0 * (double)h.nnz_full * nb);
      if (ozerr.n == 0) {
        ozerr.alloc_on(1, c.stream);
        FEM2D_CUDA(cudaMemsetAsync(ozerr.p, 0, sizeof(int), c.stream));
      }
      tcs->apply(c, slot, coef, d.grp.p, d.row_ptr.p, d.col.p, X, ldx, nb, Y, ldy, ozerr.p);
      return;
    }
    ProfScope ps(c, "spmm", (double)h.nnz_full * (4.0 + 8.0 * nv) + 8.0 * (h.n + 1) + 16.0 * h.n * nb,
                 2.0 * (double)h.nnz_full * nb);
    if (d.nwork > 0 && nb <= 32) {
      const int64_t zb = std::min<int64_t>((h.n * nb + 255) / 256, (int64_t)c.num_sms * 8);
      zero_block_kernel<<<(int)std::max<int64_t>(zb, 1), 256, 0, c.stream>>>(h.n, nb, Y, ldy);
      const int grid = std::max(1, std::min(d.nwork, c.num_sms * 6));
      spmm_group_kernel<<<grid, 256, 0, c.stream>>>(d.nwork, d.gwork.p, d.grp.p, d.row_ptr.p, d.col.p, va, vb, ca,
                                                    cb, X, ldx, nb, Y, ldy);
      c.launches += 2;
      return;
    }
    for (int c0 = 0; c0 < nb; c0 += 32) {
      const int w = std::min(32, nb - c0);
      int G = 1;
      while (G < w) G <<= 1;
      const int64_t warps = h.n;
      const int64_t blocks = std::min<int64_t>((warps * 32 + 255) / 256, (int64_t)c.num_sms * 16);
      spmm_kernel<<<(int)std::max<int64_t>(blocks, 1), 256, 0, c.stream>>>(h.n, d.row_ptr.p, d.col.p, va, vb, ca,
                                                                           cb, X + c0, ldx, w, G, Y + c0, ldy);
      c.launches++;
    }
  }
  // C (a x b, host row-major) = X^T Y
  void gram(const double* X, int64_t ldx, int a, const double* Y, int64_t ldy, int b, std::vector<double>& C) {
    const int ab = a * b;
    if (small.n < (size_t)ab) small.alloc_on(std::max<size_t>(ab, 16384), c.stream);
    if (tensor_gram(X, ldx, a, Y, ldy, b, small.p)) {
      C.resize(ab);
      FEM2D_CUDA(cudaMemcpyAsync(C.data(), small.p, ab * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
      check_tensor();
      return;
    }
    ProfScope ps(c, "dense_block", 8.0 * h.n * (a + b), 2.0 * h.n * a * b);
    const int nblk = std::min<int64_t>(grid_rows(), std::max<int64_t>(1, (h.n + 255) / 256));
    const int64_t rpb = (h.n + nblk - 1) / nblk;

    if (part.n < (size_t)nblk * ab) part.alloc_on((size_t)nblk * ab, c.stream);
    if (small.n < (size_t)ab) small.alloc_on(std::max<size_t>(ab, 16384), c.stream);
    const size_t smem = (size_t)32 * (a + b) * sizeof(double);
    for (int e0 = 0; e0 < ab; e0 += 8 * 256) {
      gram_partial_kernel<<<nblk, 256, smem, c.stream>>>(h.n, X, ldx, a, Y, ldy, b, rpb, e0, part.p);
      c.launches++;
    }
    reduce_partials_kernel<<<(ab + 255) / 256, 256, 0, c.stream>>>(part.p, nblk, ab, small.p);
    c.launches++;
    C.resize(ab);
    FEM2D_CUDA(cudaMemcpyAsync(C.data(), small.p, ab * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    FEM2D_CUDA(cudaStreamSynchronize(c.stream));
  }
  // Z = beta Z + X * C (C host a x b), tiled over the columns of C so a tile fits in shared memory
  void gemm(const double* X, int64_t ldx, int a, const std::vector<double>& C, int b, double beta, double* Z,
            int64_t ldz) {
    if (a <= 0 || b <= 0) return;
    if (dense_mode == 0 && a <= 256) {
      // 32 columns of C at a time through the tensor-core kernel
      std::vector<double> Ct;
      for (int j0 = 0; j0 < b; j0 += 32) {
        const int w = std::min(32, b - j0);
        Ct.resize((size_t)a * w);
        for (int i = 0; i < a; i++)
          for (int j = 0; j < w; j++) Ct[(size_t)i * w + j] = C[(size_t)i * b + j0 + j];
        if (small.n < Ct.size()) small.alloc_on(std::max<size_t>(Ct.size(), 16384), c.stream);
        FEM2D_CUDA(cudaMemcpyAsync(small.p, Ct.data(), Ct.size() * sizeof(double), cudaMemcpyHostToDevice, c.stream));
        tensor_gemm(X, ldx, a, small.p, w, 1.0, beta, Z + j0, ldz);
        // (pageable copies are staged before cudaMemcpyAsync returns: Ct may be reused)
      }
      return;
    }
    ProfScope ps(c, "dense_block", 8.0 * h.n * (a + (beta != 0.0 ? 2.0 : 1.0) * b), 2.0 * h.n * a * b);
    const int chunk = std::max(1, std::min(b, (int)((96 * 1024) / (sizeof(double) * a))));
    std::vector<double> Ct;
    for (int j0 = 0; j0 < b; j0 += chunk) {
      const int w = std::min(chunk, b - j0);
      Ct.resize((size_t)a * w);
      for (int i = 0; i < a; i++)
        for (int j = 0; j < w; j++) Ct[(size_t)i * w + j] = C[(size_t)i * b + j0 + j];
      if (small.n < Ct.size()) small.alloc_on(std::max<size_t>(Ct.size(), 16384), c.stream);
      FEM2D_CUDA(cudaMemcpyAsync(small.p, Ct.data(), Ct.size() * sizeof(double), cudaMemcpyHostToDevice, c.stream));
      const size_t smem = Ct.size() * sizeof(double);
      const int64_t blocks = std::min<int64_t>((h.n * w + 255) / 256, (int64_t)c.num_sms * 8);
      gemm_nn_kernel<<<(int)std::max<int64_t>(blocks, 1), 256, smem, c.stream>>>(h.n, X, ldx, a, small.p, w, 1.0, beta,
                                                                                Z + j0, ldz);
      c.launches++;   // (pageable copies are staged before cudaMemcpyAsync returns: Ct may be reused)
    }
  }
  void axpby(double alpha, const double* X, int64_t ldx, int b, double beta, double* Y, int64_t ldy) {
    ProfScope ps(c, "vector_ops", 8.0 * h.n * b * (beta != 0.0 ? 3.0 : 2.0));
    const int64_t blocks = std::min<int64_t>((h.n * b + 255) / 256, (int64_t)c.num_sms * 8);
    axpby_kernel<<<(int)std::max<int64_t>(blocks, 1), 256, 0, c.stream>>>(h.n, b, alpha, X, ldx, beta, Y, ldy);
    c.launches++;
  }
  // C (a x b, device, row-major) = X^T Y without leaving the device
  void gram_dev(const double* X, int64_t ldx, int a, const double* Y, int64_t ldy, int b, double* Cd) {
    if (tensor_gram(X, ldx, a, Y, ldy, b, Cd)) return;
    ProfScope ps(c, "dense_block", 8.0 * h.n * (a + b), 2.0 * h.n * a * b);
    const int nblk = std::min<int64_t>(grid_rows(), std::max<int64_t>(1, (h.n + 255) / 256));
    const int64_t rpb = (h.n + nblk - 1) / nblk;
    const int ab = a * b;
    if (part.n < (size_t)nblk * ab) part.alloc_on((size_t)nblk * ab, c.stream);
    const size_t smem = (size_t)32 * (a + b) * sizeof(double);
    for (int e0 = 0; e0 < ab; e0 += 8 * 256) {
      gram_partial_kernel<<<nblk, 256, smem, c.stream>>>(h.n, X, ldx, a, Y, ldy, b, rpb, e0, part.p);
      c.launches++;
    }
    reduce_partials_kernel<<<(ab + 255) / 256, 256, 0, c.stream>>>(part.p, nblk, ab, Cd);
    c.launches++;
  }
  // Z = beta Z + alpha X C with C (a x b) already on the device (a * b * 8 bytes fit the kernel's smem)
  void gemm_dev(const double* X, int64_t ldx, int a, const double* Cd, int b, double alpha, double beta, double* Z,
                int64_t ldz) {
    if (a <= 0 || b <= 0) return;
    if (tensor_gemm(X, ldx, a, Cd, b, alpha, beta, Z, ldz)) return;
    ProfScope ps(c, "dense_block", 8.0 * h.n * (a + (beta != 0.0 ? 2.0 : 1.0) * b), 2.0 * h.n * a * b);
    const size_t smem = (size_t)a * b * sizeof(double);
    if (smem > 96 * 1024) fail(FEM2D_E_INVALID_ARG, "device-resident projection block too large");
    const int64_t blocks = std::min<int64_t>((h.n * b + 255) / 256, (int64_t)c.num_sms * 8);
    gemm_nn_kernel<<<(int)std::max<int64_t>(blocks, 1), 256, smem, c.stream>>>(h.n, X, ldx, a, Cd, b, alpha, beta, Z,
                                                                              ldz);
    c.launches++;
  }
  void copy(const double* X, int64_t ldx, int b, double* Y, int64_t ldy) {
    ProfScope ps(c, "vector_ops", 16.0 * h.n * b);
    const int64_t blocks = std::min<int64_t>((h.n * b + 255) / 256, (int64_t)c.num_sms * 8);
    copy_block_kernel<<<(int)std::max<int64_t>(blocks, 1), 256, 0, c.stream>>>(h.n, b, X, ldx, Y, ldy);
    c.launches++;
  }
};

// dynamic shared memory limits, once per device (a function attribute lives in the device's context)
void setup_gemm_smem(int device) {
  static std::mutex mu;
  static bool done[256] = {};
  std::lock_guard<std::mutex> lk(mu);
  if (device < 0 || device >= 256 || done[device]) return;
  FEM2D_CUDA(cudaFuncSetAttribute(gemm_nn_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024));
  FEM2D_CUDA(cudaFuncSetAttribute(gram_partial_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024));
  done[device] = true;
}

// splitmix64 -> standard normal (Box-Muller), deterministic start blocks
// deterministic pseudo-random start blocks: a splitmix64 sequence turned into standard normals by
// Box-Muller, generated on the device (element k of the row-major n x b block uses the generator's
// calls 2 floor(k/2) + 1 and + 2, so every element is independent); written with leading dimension ld
__global__ void random_block_kernel(int64_t n, int b, uint64_t seed, double* __restrict__ out, int64_t ld) {
  const uint64_t s0 = seed * 0x9E3779B97F4A7C15ull + 0x2545F4914F6CDD1Dull;
  const int64_t total = n * b;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < total; k += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t pair = (uint64_t)(k >> 1);
    auto mix = [](uint64_t z) {
      z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
      z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
      return z ^ (z >> 31);
    };
    const uint64_t z1 = mix(s0 + (2 * pair + 1) * 0x9E3779B97F4A7C15ull);
    const uint64_t z2 = mix(s0 + (2 * pair + 2) * 0x9E3779B97F4A7C15ull);
    const double u1 = ((double)(z1 >> 11) + 0.5) / 9007199254740992.0;
    const double u2 = ((double)(z2 >> 11) + 0.5) / 9007199254740992.0;
    const double r = sqrt(-2.0 * log(u1));
    const double v = (k & 1) ? r * sinpi(2.0 * u2) : r * cospi(2.0 * u2);
    out[(k / b) * ld + (k % b)] = v;
  }
}

void random_block_device(Ctx& c, int64_t n, int b, uint64_t seed, double* out, int64_t ld) {
  const int64_t blocks = std::min<int64_t>((n * b + 255) / 256, (int64_t)c.num_sms * 16);
  random_block_kernel<<<(int)std::max<int64_t>(blocks, 1), 256, 0, c.stream>>>(n, b, seed, out, ld);
  FEM2D_CUDA(cudaGetLastError());
  c.launches++;
}


}  // namespace

MFDevice& mf_plan(MFPlan& p, Ctx& c, const Domain& dom, const HostGEP& h, std::unique_ptr<MFSymbolic> pre) {
  if (!p.ready || p.device != c.device) {
    p.ready = false;
    p.mf.reset();
    if (pre && !p.dense) {
      p.sym = std::move(pre);   // computed ahead on a host thread
    } else {
      p.sym.reset(new MFSymbolic);
      if (p.dense) mf_symbolic_dense(h, *p.sym);
      else mf_symbolic(dom, h, *p.sym, p.lift.empty() ? nullptr : &p.lift);
    }
    p.mf.reset(new MFDevice);
    p.mf->setup(c, *p.sym, 32);
    p.device = c.device;
    p.ready = true;
  }
  return *p.mf;
}

MFDevice& mf_plan_dense(MFPlan& p, Ctx& c, const HostGEP& h) {
  p.ready = false;
  p.mf.reset();
  p.sym.reset(new MFSymbolic);
  mf_symbolic_dense(h, *p.sym);
  p.mf.reset(new MFDevice);
  p.mf->setup(c, *p.sym, 32);
  p.device = c.device;
  p.dense = true;
  p.ready = true;
  return *p.mf;
}

// ================================================================ sparse shift-invert eigensolver
void sparse_solve(Ctx& c, const Domain& dom, const HostGEP& h, const DeviceGEP& d, MFPlan& plan, double sigma, int k,
                  const fem2d_solve_opts& o, double* values, double* vectors, double* residuals,
                  fem2d_solve_stats* st, const PatchNet* net) {
  auto t0 = std::chrono::steady_clock::now();
  setup_gemm_smem(c.device);
  enable_stream_pool(c.device);
  const int64_t n = h.n;
  // From kDeepN DoFs the cycles are deeper with a small guard block (5 Krylov steps, b = k + 4): on the
  // full-form meshes of 160k and 1.07M DoFs (HierPoly and KOLeg) this took 3-5 cycles instead of 5-8
  // and 13-25% less time; below, the guard of k / 2 and 4 steps are kept.
  constexpr int64_t kDeepN = 100000;
  const bool deep = n >= kDeepN;
  const int guard = deep ? 4 : std::max(4, k / 2);
  int b = o.block > 0 ? o.block : std::min<int64_t>(k + guard, n);
  if (b < k) b = k;
  if (b > 32) fail(FEM2D_E_INVALID_ARG, "block size above 32 (n_pairs too large for one block)");
  const int steps = o.krylov_steps > 0 ? std::min(o.krylov_steps, 8) : (deep ? 5 : 4);
  // basis columns: the Krylov space of a cycle, and room for up to 32 locked pairs, a 32-column active
  // block and its first expansion (96) whatever the block size
  const int mmax = std::max(b * (steps + 1), 96);
  const double tol = o.tol > 0 ? o.tol : 1e-10;
  const int max_cycles = o.max_outer > 0 ? o.max_outer : 40;
  const double spur = 1e-6 * std::max(1.0, std::fabs(sigma));
  if (sigma == 0.0) fail(FEM2D_E_INVALID_ARG, "target 0 is the null space of the curl-curl operator");

  // symmetric Jacobi scaling: the whole solve runs on (D A D, D B D), D = diag(B)^-1/2 (same
  // eigenvalues, eigenvectors x = D x~); it keeps the unnormalised high-order bases well scaled
  DBuf<double> sc, sa, sb;
  DBuf<int> bad;
  sc.alloc_on(n, c.stream);
  sa.alloc_on(h.nnz_full, c.stream);
  sb.alloc_on(h.nnz_full, c.stream);
  bad.alloc_on(1, c.stream);
  FEM2D_CUDA(cudaMemsetAsync(bad.p, 0, sizeof(int), c.stream));
  const int64_t jblocks = std::max<int64_t>(1, std::min<int64_t>((n * 32 + 255) / 256, (int64_t)c.num_sms * 16));
  {
    jacobi_scale_kernel<<<(int)jblocks, 256, 0, c.stream>>>(n, d.row_ptr.p, d.col.p, d.b.p, sc.p, bad.p);
    scale_csr_kernel<<<(int)jblocks, 256, 0, c.stream>>>(n, d.row_ptr.p, d.col.p, d.a.p, d.b.p, sc.p, sa.p, sb.p);
    c.launches += 2;
    int hb = 0;
    FEM2D_CUDA(cudaMemcpyAsync(&hb, bad.p, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    FEM2D_CUDA(cudaStreamSynchronize(c.stream));
    if (hb) fail(FEM2D_E_B_NOT_SPD, "B has a non-positive diagonal entry");
  }
  // Row-run block scaling (default from kLargeN DoFs): S = blockdiag(L_g^-1) over runs of rows with one
  // column list, L_g the Cholesky factor of B's diagonal block of run g; S A S^T and S B S^T keep the
  // pattern, their diagonal blocks of B become identities, and cond(B) drops by orders of magnitude for
  // monomial bases, which lowers the forward error of every shifted solve. A run block that is not
  // numerically positive definite falls back to the Jacobi scaling (unless the block scaling was asked
  // for). Below kLargeN DoFs the Jacobi scaling is kept unless the factorizations prove inaccurate
  // (below): there the rounding smear of the null space is small and the block set-up would cost more
  // than the solve gains (about 8 ms per solve at 2-4k DoFs).
  constexpr int64_t kLargeN = 10000;
  const bool large = n >= kLargeN;
  // the pattern-only structures kept in the plan (block scaling, tensor-core products) belong to the
  // device they were built on
  if (plan.aux_device != c.device) {
    plan.bsc.reset();
    plan.tcs.reset();
    plan.aux_device = c.device;
  }
  if (!plan.bsc) plan.bsc = std::make_unique<BlockScale>();
  BlockScale& bsc = *plan.bsc;
  // precond 1 / 2: T's two shifted solves by preconditioned CG (A + c B) and MINRES (A - sigma B) with
  // the plain additive-Schwarz preconditioner or the learned two-level one, instead of multifrontal LU
  const bool iterative = o.precond == 1 || o.precond == 2;
  // a plan still to be built: its symbolic analysis (host only, pattern only) runs on a host thread
  // while the device computes the scaling below; the future is joined before the plan is set up, and
  // on every exit path by its destructor
  std::future<std::unique_ptr<MFSymbolic>> sym_job;
  if (!iterative && !plan.dense && (!plan.ready || plan.device != c.device)) {
    std::vector<uint8_t> lift = plan.lift;
    sym_job = std::async(std::launch::async, [&dom, &h, lift]() {
      auto s = std::make_unique<MFSymbolic>();
      mf_symbolic(dom, h, *s, lift.empty() ? nullptr : &lift);
      return s;
    });
  }
  bool blocked = false;
  if (o.scaling == 2 || (o.scaling == 0 && large)) {
    try {
      {
        ProfScope ps_bs(c, "block_scale", 0.0);
        bsc.build(c, h, d, sa.p, sb.p);
        ps_bs.bytes = bsc.alg_bytes;
        ps_bs.flops = bsc.alg_flops;
      }
      blocked = true;
    } catch (const Error&) {
      if (o.scaling == 2) throw;
      scale_csr_kernel<<<(int)jblocks, 256, 0, c.stream>>>(n, d.row_ptr.p, d.col.p, d.a.p, d.b.p, sc.p, sa.p, sb.p);
      c.launches++;
    }
  }
  if (o.precond == 2 && !net) fail(FEM2D_E_INVALID_ARG, "precond 2 (learned) needs a trained network");
  if (o.precond < 0 || o.precond > 2) fail(FEM2D_E_INVALID_ARG, "precond must be 0, 1 or 2");
  MFDevice* M = iterative ? nullptr : &mf_plan(plan, c, dom, h, sym_job.valid() ? sym_job.get() : nullptr);
  MFFactor fm, fp;
  // A + c B (c > 0) is SPD: factored without pivoting. c = |sigma| by default from kLargeN DoFs: the null
  // space of the curl-curl operator, smeared by rounding to |lambda| <~ eps ||A|| / lambda_min(B) (which
  // grows with p^4 / h^2), is damped by lambda / (lambda + c) in every application of T, and the
  // physical modes below sigma keep |mu| = lambda / ((lambda + c)(sigma - lambda)) above the far end of
  // a 20-pair window. Smaller GEPs keep c = 0.05 |sigma| (their smear is negligible and the modes below
  // sigma converge faster).
  // (the iterative inner solves keep c = |sigma|: A + c B is then far from singular on the null space,
  // and the same additive-Schwarz preconditioner of A + |sigma| B serves the MINRES solves of A - sigma B)
  const double cshift = (o.damping > 0 ? o.damping : ((large || iterative) ? 1.0 : 0.05)) * std::fabs(sigma);
  int delayed = 0;
  auto factor_both = [&]() {
    M->factor(c, sa.p, sb.p, 1.0, -sigma, false, fm);
    // delayed pivoting: columns of A - sigma B without a stable pivot among their front's fully-summed
    // rows move (their DoFs' elimination) to the parent front; re-plan and refactor, at most 3 rounds
    for (int round = 0; round < 3 && !fm.weak.empty() && !plan.dense; round++) {
      if (plan.lift.empty()) plan.lift.assign(n, 0);
      for (int32_t x : fm.weak)
        if (plan.lift[x] < 255) plan.lift[x]++;
      delayed += (int)fm.weak.size();
      plan.ready = false;
      M = &mf_plan(plan, c, dom, h);
      M->factor(c, sa.p, sb.p, 1.0, -sigma, false, fm);
    }
    M->factor(c, sa.p, sb.p, 1.0, cshift, true, fp);
    if (fp.flags & 2) fail(FEM2D_E_B_NOT_SPD, "A + c B is not positive definite; B is likely ill-conditioned");
  };
  std::unique_ptr<PCGSolver> pcg;
  if (iterative) pcg.reset(new PCGSolver(c, dom, h, d, 1.0, cshift, o.precond == 2 ? net : nullptr, nullptr, 0, sa.p,
                                         sb.p));
  else factor_both();
  FEM2D_CUDA(cudaStreamSynchronize(c.stream));
  auto t1 = std::chrono::steady_clock::now();
  const double inner_tol = o.inner_tol > 0 ? o.inner_tol : 1e-10;
  const int max_inner = o.max_inner > 0 ? o.max_inner : 5000;
  int64_t cg_iters = 0, minres_iters = 0;
  double inner_worst = 0.0;

  Dev D{c, h, d, sa.p, sb.p};
  // Gram products and block updates on the tensor cores by default from kTensorDenseN rows: below, their
  // fixed costs (exponent pre-passes, one CTA per SM) outweigh the FP64 work (256 concurrent small solves
  // of the batching family: 1.51 s per step on the FP64 kernels against 1.74 s); dense = 2 and 3 use
  // them at every size
  constexpr int64_t kTensorDenseN = 50000;
  D.dense_mode = (o.dense == 1 || (o.dense == 0 && n < kTensorDenseN)) ? 1 : 0;
  DBuf<double> V, AV, BV, X, AX, BX, G0, W1, W2, W3;
  V.alloc_on((size_t)n * mmax, c.stream);
  AV.alloc_on((size_t)n * mmax, c.stream);
  BV.alloc_on((size_t)n * mmax, c.stream);
  for (DBuf<double>* buf : {&X, &AX, &BX, &G0, &W1, &W2, &W3}) buf->alloc((size_t)n * 32);
  int64_t spmv = 0, napply = 0;

  // x = K^-1 rhs for K = ka A + kb B (factored as fac) followed by nref steps of iterative refinement
  // in FP64 (r = rhs - K x, x += K^-1 r). The multifrontal LU pivots within each front only, which
  // loses digits on indefinite pencils with ill-conditioned (monomial) bases; refinement restores
  // them. R1, R2 are scratch blocks.
  DBuf<double> R1, R2;
  R1.alloc_on((size_t)n * 32, c.stream);
  R2.alloc_on((size_t)n * 32, c.stream);
  auto solve_ref = [&](const MFFactor& fac, double ka, double kb, const double* rhs, int64_t lr, double* x, int64_t lx,
                       int nb, int nref) {
    M->solve(c, fac, rhs, lr, x, lx, nb);
    for (int r = 0; r < nref; r++) {
      D.spmm(ka, kb, x, lx, nb, R1.p, 32);
      D.axpby(1.0, rhs, lr, nb, -1.0, R1.p, 32);
      M->solve(c, fac, R1.p, 32, R2.p, 32, nb);
      D.axpby(1.0, R2.p, 32, nb, 1.0, x, lx);
      spmv += nb;
    }
  };
  // refinement steps needed by each factorization: measured once on a fixed random block, up to 3
  // steps, while the solves are not backward stable (normwise backward error above kStableBwd) and the
  // relative residual max_j ||rhs_j - K x_j|| / ||rhs_j|| stays above 1e-12.
  // The accuracy measure is the normwise backward error ||b - K x|| / (||K|| ||x|| + ||b||) of the
  // solves (||K|| bounded by the largest absolute row sum): a backward-stable factorization keeps it
  // near the unit roundoff whatever cond(K) is, whereas the plain residual ||b - K x|| / ||b|| cannot
  // fall below about eps * cond(K) even for an exact-in-FP64 solve.
  // ||ka A + kb B||_inf of the pencil in use (largest absolute row sum)
  auto pencil_norm = [&](double ka, double kb) -> double {
    const int nblk = std::max(1, std::min<int>(c.num_sms * 4, (int)((n + 7) / 8)));
    DBuf<double> part;
    part.alloc_on(nblk, c.stream);
    rowsum_max_kernel<<<nblk, 256, 0, c.stream>>>(n, d.row_ptr.p, D.va, D.vb, ka, kb, part.p);
    c.launches++;
    std::vector<double> hp(nblk);
    FEM2D_CUDA(cudaMemcpyAsync(hp.data(), part.p, nblk * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    FEM2D_CUDA(cudaStreamSynchronize(c.stream));
    double m = 0.0;
    for (double v : hp) m = std::max(m, v);
    return m;
  };
  // normwise backward error below which the exact solves are used without refinement
  constexpr double kStableBwd = 1e-13;
  auto calibrate = [&](const MFFactor& fac, double ka, double kb, double& rel_out) -> int {
    const int nb = 4;
    const double knorm = pencil_norm(ka, kb);
    DBuf<double> Rb, Xb, Tb;
    Rb.alloc_on((size_t)n * nb, c.stream);
    Xb.alloc_on((size_t)n * nb, c.stream);
    Tb.alloc_on((size_t)n * nb, c.stream);
    random_block_device(c, n, nb, 777, Rb.p, nb);
    std::vector<double> G;
    D.gram(Rb.p, nb, nb, Rb.p, nb, nb, G);
    std::vector<double> bn(nb);
    for (int j = 0; j < nb; j++) bn[j] = std::sqrt(G[(size_t)j * nb + j]);
    double prev = 1e300;
    for (int nref = 0; nref <= 3; nref++) {
      solve_ref(fac, ka, kb, Rb.p, nb, Xb.p, nb, nb, nref);
      D.spmm(ka, kb, Xb.p, nb, nb, Tb.p, nb);
      D.axpby(1.0, Rb.p, nb, nb, -1.0, Tb.p, nb);
      D.gram(Tb.p, nb, nb, Tb.p, nb, nb, G);
      std::vector<double> GX;
      D.gram(Xb.p, nb, nb, Xb.p, nb, nb, GX);
      double rel = 0, bwd = 0;
      for (int j = 0; j < nb; j++) {
        const double rn = std::sqrt(G[(size_t)j * nb + j]), xn = std::sqrt(GX[(size_t)j * nb + j]);
        rel = std::max(rel, rn / bn[j]);
        bwd = std::max(bwd, rn / (knorm * xn + bn[j]));
      }
      if (nref == 0 || rel <= prev) rel_out = bwd;
      // backward-stable solves apply T to a pencil within rounding of the scaled one: the Krylov space
      // needs nothing more (the Rayleigh-Ritz step and the residuals use exact products), and the plain
      // residual's floor eps * cond(K) is no measure of the factorization
      if (rel < 1e-12 || bwd < kStableBwd) return nref;
      if (rel > 0.5 * prev) return std::max(0, nref - 1);  // refinement no longer improves
      prev = rel;
    }
    return 3;
  };
  double rel_p = 0, rel_m = 0;
  int nref_p = iterative ? 0 : calibrate(fp, 1.0, cshift, rel_p);
  int nref_m = iterative ? 0 : calibrate(fm, 1.0, -sigma, rel_m);
  // a caller-fixed refinement count replaces the calibrated one after the checks below
  if (!iterative && (rel_p > 1e-11 || rel_m > 1e-11) && !blocked && !plan.dense && o.scaling == 0) {
    // the Jacobi-scaled factorizations lose too many digits: scale by row-run blocks of B instead
    try {
      {
        ProfScope ps_bs(c, "block_scale", 0.0);
        bsc.build(c, h, d, sa.p, sb.p);
        ps_bs.bytes = bsc.alg_bytes;
        ps_bs.flops = bsc.alg_flops;
      }
      blocked = true;
      factor_both();
      nref_p = calibrate(fp, 1.0, cshift, rel_p);
      nref_m = calibrate(fm, 1.0, -sigma, rel_m);
    } catch (const Error&) {
      scale_csr_kernel<<<(int)jblocks, 256, 0, c.stream>>>(n, d.row_ptr.p, d.col.p, d.a.p, d.b.p, sc.p, sa.p, sb.p);
      c.launches++;
      factor_both();
      nref_p = calibrate(fp, 1.0, cshift, rel_p);
      nref_m = calibrate(fm, 1.0, -sigma, rel_m);
    }
  }
  // small GEPs whose sparse factorization stays inaccurate after refinement (pivoting restricted to
  // each front's fully-summed rows can grow badly on indefinite pencils of ill-conditioned bases)
  // switch to one dense front with partial pivoting over all rows; the choice is kept in the plan
  constexpr int64_t kDenseMax = 4096;
  if (!iterative && (rel_p > 1e-11 || rel_m > 1e-11) && !plan.dense && n <= kDenseMax) {
    M = &mf_plan_dense(plan, c, h);
    factor_both();
    nref_p = calibrate(fp, 1.0, cshift, rel_p);
    nref_m = calibrate(fm, 1.0, -sigma, rel_m);
  }
  if (o.refine > 0) nref_p = nref_m = std::min(o.refine, 3);
  if (o.refine < 0) nref_p = nref_m = 0;
  // Out (ld lo) = T In (ld li), nb columns; In and Out may not alias W1..W3
  auto apply_T = [&](const double* In, int64_t li, double* Out, int64_t lo, int nb) {
    D.spmm(0.0, 1.0, In, li, nb, W1.p, 32);
    if (iterative) {
      PCGStats s1, s2;
      pcg->cg_device(W1.p, 32, W2.p, 32, nb, inner_tol, max_inner, &s1);
      D.spmm(1.0, 0.0, W2.p, 32, nb, W3.p, 32);
      // the learned coarse space is trained on, and corrects, the SPD system's errors: the MINRES solves
      // of the indefinite system keep the additive-Schwarz preconditioner alone
      pcg->minres_device(1.0, -sigma, W3.p, 32, Out, lo, nb, inner_tol, max_inner, &s2, false);
      cg_iters += s1.iters;
      minres_iters += s2.iters;
      spmv += (int64_t)nb * (s1.iters + s2.iters);
      inner_worst = std::max(inner_worst, std::max(s1.relres, s2.relres));
    } else {
      solve_ref(fp, 1.0, cshift, W1.p, 32, W2.p, 32, nb, nref_p);
      D.spmm(1.0, 0.0, W2.p, 32, nb, W3.p, 32);
      solve_ref(fm, 1.0, -sigma, W3.p, 32, Out, lo, nb, nref_m);
    }
    spmv += 2 * nb;
    napply += nb;
  };
  // W = V[:, m0:m0+r]: B-orthogonalise against V[:, :m0] (CGS2 with the stored B V), form B W once,
  // orthonormalise within the block (eigen-decomposition of its Gram matrix, rank-revealing; the same
  // transforms applied to B W), then store the exact product A*W in AV and B*W in BV. Returns the number
  // of columns kept. Per new column: one product with B and one with A.
  DBuf<double> Cproj;
  Cproj.alloc_on((size_t)mmax * 32, c.stream);
  auto borth_new = [&](int m0, int r) -> int {
    if (r <= 0) return 0;
    double* Wb = V.p + m0;
    double* BWb = BV.p + m0;
    std::vector<double> G, w, z;
    // W -= V ((B V)^T W): the first two CGS passes need no product with B (the basis carries B V);
    // coefficients stay on the device (no host round trip)
    auto project_w = [&](int cols) {
      D.gram_dev(BV.p, mmax, m0, Wb, mmax, cols, Cproj.p);
      D.gemm_dev(V.p, mmax, m0, Cproj.p, cols, -1.0, 1.0, Wb, mmax);
    };
    // W -= V (V^T B W), B W -= (B V)(V^T B W): B W tracked linearly through a late, small correction
    auto project = [&](int cols) {
      D.gram_dev(V.p, mmax, m0, BWb, mmax, cols, Cproj.p);
      D.gemm_dev(V.p, mmax, m0, Cproj.p, cols, -1.0, 1.0, Wb, mmax);
      D.gemm_dev(BV.p, mmax, m0, Cproj.p, cols, -1.0, 1.0, BWb, mmax);
    };
    if (m0 > 0) {
      project_w(r);
      project_w(r);
    }
    // the exact product of the projected block; the orthonormalising transforms below are applied to
    // W and B W alike
    D.spmm(0.0, 1.0, Wb, mmax, r, BWb, mmax);
    spmv += r;
    int keep = r;
    for (int pass = 0; pass < 2; pass++) {
      D.gram(Wb, mmax, keep, BWb, mmax, keep, G);
      for (int i = 0; i < keep; i++)
        for (int j = 0; j < i; j++)
          G[(size_t)i * keep + j] = G[(size_t)j * keep + i] = 0.5 * (G[(size_t)i * keep + j] + G[(size_t)j * keep + i]);
      if (!symeig(keep, G, w, z)) fail(FEM2D_E_NOT_CONVERGED, "Gram eigen-decomposition failed");
      const double wmax = *std::max_element(w.begin(), w.end());
      std::vector<int> kept;
      for (int q = 0; q < keep; q++)
        if (w[q] > (pass == 0 ? 1e-8 : 1e-14) * wmax && w[q] > 0) kept.push_back(q);
      const int nk = (int)kept.size();
      if (nk == 0) return 0;
      std::vector<double> T((size_t)keep * nk);
      for (int i = 0; i < keep; i++)
        for (int q = 0; q < nk; q++) T[(size_t)i * nk + q] = z[(size_t)i * keep + kept[q]] / std::sqrt(w[kept[q]]);
      D.gemm(Wb, mmax, keep, T, nk, 0.0, W2.p, 32);
      D.copy(W2.p, 32, nk, Wb, mmax);
      D.gemm(BWb, mmax, keep, T, nk, 0.0, W2.p, 32);
      D.copy(W2.p, 32, nk, BWb, mmax);
      keep = nk;
      if (pass == 0 && m0 > 0) project(keep);
    }
    D.spmm(1.0, 0.0, Wb, mmax, keep, AV.p + m0, mmax);
    spmv += keep;
    return keep;
  };

  const double norm_a = pencil_norm(1.0, 0.0), norm_b = pencil_norm(0.0, 1.0);
  // products with A or B alone (the T applications, the basis products) on the tensor cores from here
  // on: the scaled pencil is final, so its values are sliced once (by default from kTensorSpmmNnz
  // nonzeros, where the slicing is amortised; always with dense = 2)
  constexpr int64_t kTensorSpmmNnz = 1000000;
  // the sliced pencil lives for this solve only (stream-ordered buffers, released on every exit path)
  struct SliceRelease {
    TcSpmm* t = nullptr;
    ~SliceRelease() {
      if (t)
        for (auto& sl : t->slot) {
          sl.planes.release();
          sl.exps.release();
          sl.ready = false;
        }
    }
  } slice_release;
  if (d.nwork > 0 && (o.dense == 2 || (o.dense == 0 && h.nnz_full >= kTensorSpmmNnz))) {
    ProfScope ps(c, "spmm_slice", 2.0 * (8.0 * h.nnz_full + 16.0 * h.nnz_full), 0.0);
    if (!plan.tcs) {
      plan.tcs = std::make_unique<TcSpmm>();
      plan.tcs->build(c, n, d.grp_h, h.row_ptr);
    }
    TcSpmm& tcs = *plan.tcs;
    slice_release.t = &tcs;
    tcs.slice(c, 0, d.grp.p, d.row_ptr.p, sa.p, nullptr, 1.0, 0.0);
    tcs.slice(c, 1, d.grp.p, d.row_ptr.p, nullptr, sb.p, 0.0, 1.0);
    // the shifted matrices of the refinement residuals (exact solves with refinement steps)
    if (!iterative && nref_p > 0) tcs.slice(c, 2, d.grp.p, d.row_ptr.p, sa.p, sb.p, 1.0, cshift);
    if (!iterative && nref_m > 0) tcs.slice(c, 3, d.grp.p, d.row_ptr.p, sa.p, sb.p, 1.0, -sigma);
    D.tcs = &tcs;
  }
  // start block: T applied to a fixed pseudo-random block
  {
    DBuf<double> R;
    R.alloc_on((size_t)n * b, c.stream);
    random_block_device(c, n, b, 12345, R.p, b);
    apply_T(R.p, b, X.p, 32, b);
  }
  // A pair is converged when its relative residual is below tol or its normwise backward error
  // ||A x - theta B x|| / ((||A|| + |theta| ||B||) ||x||) is below kBackward: the pair is then exact for
  // a pencil within 1e-14 of (A, B). With high-order monomial bases ||A|| grows as p^4 / h^2 and the
  // relative residual attainable in FP64 rises with it.
  constexpr double kBackward = 1e-14;
  // The attainable backward error is set by the forward accuracy of the T applications, which falls
  // with cond(A - sigma B): a pair whose residual stopped falling for one cycle with a backward error
  // below kStuck / 10, or for two cycles below kStuck, is converged too (its Ritz value, second order
  // in the residual, is settled).
  constexpr double kSame = 1e-8, kStuck = 1e-11;
  // Converged pairs are locked: their vectors and exact products are kept as they are, every new
  // direction is B-orthogonalised against them, and the Rayleigh-Ritz step runs on the active part of
  // the basis only. Locked pairs are not expanded again (the expansion of a pair at its attainable
  // accuracy adds only rounding noise, and noise that mixes null-space and high-frequency directions
  // yields spurious Ritz values near sigma) and do not drift through later Rayleigh-Ritz steps.
  DBuf<double> XL, AXL, BXL;
  for (DBuf<double>* buf : {&XL, &AXL, &BXL}) buf->alloc_on((size_t)n * 32, c.stream);
  int nl = 0;
  std::vector<double> theta_l, rel_l, bwd_l;
  std::vector<double> theta_sel, rel_sel, bwd_sel, theta_prev, rel_prev;
  std::vector<int> stuck_sel, stuck_prev;
  int cycles = 0, bx = b;
  bool converged = false;
  double best_worst = 1e300;
  int stall_total = 0;
  bool attained = false;
  // the k pairs nearest sigma among the locked and the selected active ones: (locked?, index)
  std::vector<std::pair<int, int>> nearest;
  auto merge_nearest = [&]() {
    std::vector<std::pair<int, int>> all;
    for (int j = 0; j < nl; j++) all.push_back({1, j});
    for (int j = 0; j < bx; j++) all.push_back({0, j});
    auto th_of = [&](const std::pair<int, int>& e) { return e.first ? theta_l[e.second] : theta_sel[e.second]; };
    std::stable_sort(all.begin(), all.end(), [&](const std::pair<int, int>& x, const std::pair<int, int>& y) {
      return std::fabs(th_of(x) - sigma) < std::fabs(th_of(y) - sigma);
    });
    all.resize(std::min<size_t>(all.size(), (size_t)k));
    nearest = all;
  };
  for (; cycles < max_cycles; cycles++) {
    int m, last0, lastn;
    if (cycles == 0) {
      D.copy(X.p, 32, bx, V.p, mmax);
      m = borth_new(0, bx);
      last0 = 0;
      lastn = m;
    } else {
      // V = [locked | active Ritz vectors | T^j (active)]; every active vector is unconverged
      if (nl > 0) {
        D.copy(XL.p, 32, nl, V.p, mmax);
        D.copy(AXL.p, 32, nl, AV.p, mmax);
        D.copy(BXL.p, 32, nl, BV.p, mmax);
      }
      D.copy(X.p, 32, bx, V.p + nl, mmax);
      D.copy(AX.p, 32, bx, AV.p + nl, mmax);
      D.copy(BX.p, 32, bx, BV.p + nl, mmax);
      m = nl + bx;
      if (m + bx > mmax) fail(FEM2D_E_NOT_CONVERGED, "gpu_solve_gep: basis capacity exceeded");
      // expand with T applied to the active Ritz vectors: T kills their null-space part and damps
      // high-frequency content, which also pushes spurious Ritz vectors out of the basis
      apply_T(X.p, 32, V.p + m, mmax, bx);
      const int r = borth_new(m, bx);
      last0 = m;
      lastn = r;
      m += r;
    }
    for (int st2 = (cycles == 0 ? 0 : 1); st2 < steps && lastn > 0 && m + lastn <= mmax; st2++) {
      apply_T(V.p + last0, mmax, V.p + m, mmax, lastn);
      int r = borth_new(m, lastn);
      if (r == 0) break;
      last0 = m;
      lastn = r;
      m += r;
    }
    // Rayleigh-Ritz on the active columns [nl, m): (V^T A V, V^T B V)
    const int ma = m - nl;
    if (ma <= 0)
      fail(nl > 0 ? FEM2D_E_NOT_CONVERGED : FEM2D_E_SPURIOUS,
           nl > 0 ? "gpu_solve_gep: the search space collapsed onto the locked pairs"
                  : "gpu_solve_gep: T vanishes on the start block (A has only null-space directions); only spurious "
                    "modes exist");
    const double* Va = V.p + nl;
    const double* AVa = AV.p + nl;
    const double* BVa = BV.p + nl;
    std::vector<double> GA, GB, wb, zb;
    D.gram(Va, mmax, ma, AVa, mmax, ma, GA);
    D.gram(Va, mmax, ma, BVa, mmax, ma, GB);
    for (int i = 0; i < ma; i++)
      for (int j = 0; j < i; j++) {
        GA[(size_t)i * ma + j] = GA[(size_t)j * ma + i] = 0.5 * (GA[(size_t)i * ma + j] + GA[(size_t)j * ma + i]);
        GB[(size_t)i * ma + j] = GB[(size_t)j * ma + i] = 0.5 * (GB[(size_t)i * ma + j] + GB[(size_t)j * ma + i]);
      }
    auto hs_rr = std::make_unique<HostScope>(c, "rr_host");
    if (!symeig(ma, GB, wb, zb)) fail(FEM2D_E_NOT_CONVERGED, "Gram eigen-decomposition failed");
    const double wbmax = *std::max_element(wb.begin(), wb.end());
    std::vector<int> kb;
    for (int q = 0; q < ma; q++)
      if (wb[q] > 1e-12 * wbmax) kb.push_back(q);
    const int m2 = (int)kb.size();
    std::vector<double> Wh((size_t)ma * m2);   // GB^-1/2 restricted to its numerical range
    for (int i = 0; i < ma; i++)
      for (int q = 0; q < m2; q++) Wh[(size_t)i * m2 + q] = zb[(size_t)i * ma + kb[q]] / std::sqrt(wb[kb[q]]);
    std::vector<double> S((size_t)m2 * m2, 0.0), tmp((size_t)ma * m2, 0.0);
    for (int i = 0; i < ma; i++)
      for (int q = 0; q < m2; q++) {
        double acc = 0.0;
        for (int k2 = 0; k2 < ma; k2++) acc += GA[(size_t)i * ma + k2] * Wh[(size_t)k2 * m2 + q];
        tmp[(size_t)i * m2 + q] = acc;
      }
    for (int p2 = 0; p2 < m2; p2++)
      for (int q = 0; q < m2; q++) {
        double acc = 0.0;
        for (int i = 0; i < ma; i++) acc += Wh[(size_t)i * m2 + p2] * tmp[(size_t)i * m2 + q];
        S[(size_t)p2 * m2 + q] = acc;
      }
    std::vector<double> th, Z;
    if (!symeig(m2, S, th, Z)) fail(FEM2D_E_NOT_CONVERGED, "Rayleigh-Ritz eigen-decomposition failed");
    std::vector<double> Y((size_t)ma * m2, 0.0);
    for (int i = 0; i < ma; i++)
      for (int q = 0; q < m2; q++) {
        double acc = 0.0;
        for (int k2 = 0; k2 < m2; k2++) acc += Wh[(size_t)i * m2 + k2] * Z[(size_t)k2 * m2 + q];
        Y[(size_t)i * m2 + q] = acc;
      }
    // Ritz residuals AV*y - BV*y*theta of the non-spurious pairs nearest sigma only (twice the block):
    // the selection never reaches further, and the products scale with the number of columns
    std::vector<int> order;
    for (int j = 0; j < m2; j++)
      if (std::fabs(th[j]) > spur) order.push_back(j);
    std::stable_sort(order.begin(), order.end(),
                     [&](int x, int y) { return std::fabs(th[x] - sigma) < std::fabs(th[y] - sigma); });
    if (nl + (int)order.size() < k) fail(FEM2D_E_SPURIOUS, "only spurious (null-space) Ritz values were found");
    const int nc = std::min<int>((int)order.size(), 2 * b);
    std::vector<double> Ysub((size_t)ma * nc), thc(nc);
    for (int i = 0; i < ma; i++)
      for (int q = 0; q < nc; q++) Ysub[(size_t)i * nc + q] = Y[(size_t)i * m2 + order[q]];
    for (int q = 0; q < nc; q++) thc[q] = th[order[q]];
    // the two dense products forming S and the Ritz vectors Y exactly, and 9 n^3 for each symmetric
    // eigen-decomposition (the nominal count of a tridiagonal reduction with eigenvectors)
    hs_rr->flops = 2.0 * ((double)ma * ma * m2 + (double)m2 * m2 * ma + (double)ma * m2 * m2) +
                   9.0 * ((double)ma * ma * ma + (double)m2 * m2 * m2);
    hs_rr.reset();
    DBuf<double> AY, BY, XY, th_d, P;
    AY.alloc_on((size_t)n * nc, c.stream);
    BY.alloc_on((size_t)n * nc, c.stream);
    XY.alloc_on((size_t)n * nc, c.stream);
    D.gemm(AVa, mmax, ma, Ysub, nc, 0.0, AY.p, nc);
    D.gemm(BVa, mmax, ma, Ysub, nc, 0.0, BY.p, nc);
    D.gemm(Va, mmax, ma, Ysub, nc, 0.0, XY.p, nc);
    th_d.upload_on(thc, c.stream);
    const int nblk = std::min<int64_t>(D.grid_rows(), std::max<int64_t>(1, (n + 255) / 256));
    const int64_t rpb = (n + nblk - 1) / nblk;
    P.alloc_on((size_t)nblk * 3 * nc, c.stream);
    {
      ProfScope ps_r(c, "vector_ops", 24.0 * n * nc);
      resid_partial_kernel<<<nblk, 256, 0, c.stream>>>(n, AY.p, BY.p, XY.p, nc, nc, th_d.p, rpb, P.p);
      c.launches++;
    }
    std::vector<double> Ph((size_t)nblk * 3 * nc);
    FEM2D_CUDA(cudaMemcpyAsync(Ph.data(), P.p, Ph.size() * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    FEM2D_CUDA(cudaStreamSynchronize(c.stream));
    std::vector<double> rel(m2, 1e300), bwd(m2, 1e300);
    for (int q = 0; q < nc; q++) {
      double sr = 0, sb = 0, sx = 0;
      for (int t = 0; t < nblk; t++) {
        sr += Ph[(size_t)t * 3 * nc + q];
        sb += Ph[(size_t)t * 3 * nc + nc + q];
        sx += Ph[(size_t)t * 3 * nc + 2 * nc + q];
      }
      rel[order[q]] = std::sqrt(sr) / (std::fabs(thc[q]) * std::sqrt(sb) + 1e-300);
      bwd[order[q]] = std::sqrt(sr) / ((norm_a + std::fabs(thc[q]) * norm_b) * std::sqrt(sx) + 1e-300);
    }
    // the active block keeps b - nl vectors (at least 4): the nearest credible Ritz pairs
    const int ba = std::max(4, b - nl);
    std::vector<int> cand;
    for (int q = 0; q < nc; q++)
      if (rel[order[q]] < 1.0) cand.push_back(order[q]);
    if ((int)cand.size() < std::max(1, k - nl)) {
      // not enough credible Ritz pairs yet: keep the nearest non-spurious ones regardless of residual
      cand.assign(order.begin(), order.begin() + nc);
    }
    std::vector<int> sel(cand.begin(), cand.begin() + std::min<size_t>(cand.size(), (size_t)ba));
    const int ns = (int)sel.size();
    theta_sel.resize(ns);
    rel_sel.resize(ns);
    bwd_sel.resize(ns);
    stuck_sel.assign(ns, 0);
    std::vector<uint8_t> lock(ns, 0);
    for (int q = 0; q < ns; q++) {
      theta_sel[q] = th[sel[q]];
      rel_sel[q] = rel[sel[q]];
      bwd_sel[q] = bwd[sel[q]];
      // the same pair (its Ritz value within kSame of one of the previous cycle) whose residual has not
      // halved for two cycles, with a backward error below kStuck, has reached the accuracy the T
      // applications allow
      for (size_t p = 0; p < theta_prev.size(); p++)
        if (std::fabs(theta_sel[q] - theta_prev[p]) <= kSame * std::fabs(theta_sel[q])) {
          stuck_sel[q] = rel_sel[q] > 0.5 * rel_prev[p] ? stuck_prev[p] + 1 : 0;
          break;
        }
      lock[q] = (rel_sel[q] < tol || bwd_sel[q] < kBackward || (stuck_sel[q] >= 1 && bwd_sel[q] < 0.1 * kStuck) ||
                 (stuck_sel[q] >= 2 && bwd_sel[q] < kStuck))
                    ? 1
                    : 0;
    }
    // newly converged pairs join the locked set (at most 32 locked vectors); the rest stay active
    std::vector<int> to_lock, to_keep;
    for (int q = 0; q < ns; q++) {
      if (lock[q] && nl + (int)to_lock.size() < 32)
        to_lock.push_back(q);
      else
        to_keep.push_back(q);
    }
    auto gather = [&](const std::vector<int>& idx, double* Xd, double* AXd, double* BXd) {
      const int w = (int)idx.size();
      if (w == 0) return;
      std::vector<double> Ys((size_t)ma * w);
      for (int i = 0; i < ma; i++)
        for (int q = 0; q < w; q++) Ys[(size_t)i * w + q] = Y[(size_t)i * m2 + sel[idx[q]]];
      D.gemm(Va, mmax, ma, Ys, w, 0.0, Xd, 32);
      D.gemm(AVa, mmax, ma, Ys, w, 0.0, AXd, 32);
      D.gemm(BVa, mmax, ma, Ys, w, 0.0, BXd, 32);
    };
    gather(to_lock, XL.p + nl, AXL.p + nl, BXL.p + nl);
    for (int q : to_lock) {
      theta_l.push_back(theta_sel[q]);
      rel_l.push_back(rel_sel[q]);
      bwd_l.push_back(bwd_sel[q]);
    }
    nl += (int)to_lock.size();
    gather(to_keep, X.p, AX.p, BX.p);
    {
      std::vector<double> t2, r2, b2;
      std::vector<int> s2;
      for (int q : to_keep) {
        t2.push_back(theta_sel[q]);
        r2.push_back(rel_sel[q]);
        b2.push_back(bwd_sel[q]);
        s2.push_back(stuck_sel[q]);
      }
      theta_sel = t2;
      rel_sel = r2;
      bwd_sel = b2;
      stuck_sel = s2;
    }
    bx = (int)to_keep.size();
    theta_prev = theta_sel;
    rel_prev = rel_sel;
    stuck_prev = stuck_sel;
    merge_nearest();
    double worst = 0, worst_bwd = 0;
    bool all_locked = (int)nearest.size() == k, by_bwd = false;
    for (const auto& e : nearest) {
      const double r = e.first ? rel_l[e.second] : rel_sel[e.second];
      const double bw = e.first ? bwd_l[e.second] : bwd_sel[e.second];
      worst = std::max(worst, r);
      worst_bwd = std::max(worst_bwd, bw);
      all_locked = all_locked && e.first;
      by_bwd = by_bwd || r >= tol;
    }
    if (o.verbose)
      fprintf(stderr, "[gpu_solve_gep] cycle %d basis %d (%d locked) worst residual %.3e backward error %.3e\n",
              cycles, m, nl, worst, worst_bwd);
    if (o.verbose > 1)
      for (const auto& e : nearest)
        fprintf(stderr, "    theta %.12f residual %.3e backward error %.3e%s\n",
                e.first ? theta_l[e.second] : theta_sel[e.second], e.first ? rel_l[e.second] : rel_sel[e.second],
                e.first ? bwd_l[e.second] : bwd_sel[e.second], e.first ? " locked" : "");
    if (all_locked) {
      converged = true;
      attained = by_bwd;
      cycles++;
      break;
    }
    if (worst < 0.5 * best_worst) {
      best_worst = worst;
      stall_total = 0;
    } else {
      stall_total++;
    }
    // last resort: eight cycles without halving the worst residual, below 1e-6, end the solve as
    // converged (eigenvalue errors scale with the squared residual)
    if (stall_total >= 8 && worst < 1e-6) {
      converged = true;
      attained = true;
      cycles++;
      break;
    }
    if (bx == 0) fail(FEM2D_E_NOT_CONVERGED, "gpu_solve_gep: no active Ritz vectors left to expand");
  }
  if (nearest.empty()) merge_nearest();
  FEM2D_CUDA(cudaStreamSynchronize(c.stream));
  auto t2 = std::chrono::steady_clock::now();
  // the k output pairs, nearest sigma first: vectors gathered from the locked and active blocks
  const int kout = (int)nearest.size();
  std::vector<double> theta_out(kout), rel_out(kout), bwd_out(kout);
  DBuf<double> XO;
  XO.alloc_on((size_t)n * 32, c.stream);
  for (int q = 0; q < kout; q++) {
    const auto& e = nearest[q];
    theta_out[q] = e.first ? theta_l[e.second] : theta_sel[e.second];
    D.copy((e.first ? XL.p : X.p) + e.second, 32, 1, XO.p + q, 32);
  }
  if (st) {
    st->outer_iters = cycles;
    st->inner_iters_total = (int)napply;
    st->converged = converged ? 1 : 0;
    st->t_setup_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
    st->t_solve_ms = std::chrono::duration<double, std::milli>(t2 - t1).count();
    st->spmv_count = spmv;
    st->refine_spd = nref_p;
    st->refine_indefinite = nref_m;
    st->dense_plan = plan.dense ? 1 : 0;
    st->inner_cg_iters = cg_iters;
    st->inner_minres_iters = minres_iters;
    st->inner_max_relres = inner_worst;
    st->block_scaled = blocked ? 1 : 0;
    st->delayed_pivots = delayed;
    st->floor_reached = attained ? 1 : 0;
  }
  // back to the original pencil: x = D x~ (B-orthonormal), residuals in the original norms
  {
    if (blocked) {
      bsc.unscale(c, XO.p, 32, kout);
    } else {
      const int64_t blocks = std::min<int64_t>((n * kout + 255) / 256, (int64_t)c.num_sms * 8);
      scale_rows_kernel<<<(int)std::max<int64_t>(blocks, 1), 256, 0, c.stream>>>(n, kout, sc.p, XO.p, 32);
      c.launches++;
    }
    D.tcs = nullptr;   // the final residuals use the unscaled pencil (and FP64 products)
    D.va = d.a.p;
    D.vb = d.b.p;
    D.spmm(1.0, 0.0, XO.p, 32, kout, AX.p, 32);
    D.spmm(0.0, 1.0, XO.p, 32, kout, BX.p, 32);
    DBuf<double> th_d, P;
    th_d.upload_on(theta_out, c.stream);
    const int nblk = std::min<int64_t>(D.grid_rows(), std::max<int64_t>(1, (n + 255) / 256));
    const int64_t rpb = (n + nblk - 1) / nblk;
    P.alloc_on((size_t)nblk * 3 * kout, c.stream);
    resid_partial_kernel<<<nblk, 256, 0, c.stream>>>(n, AX.p, BX.p, XO.p, 32, kout, th_d.p, rpb, P.p);
    c.launches++;
    const double na0 = pencil_norm(1.0, 0.0), nb0 = pencil_norm(0.0, 1.0);
    std::vector<double> Ph((size_t)nblk * 3 * kout);
    FEM2D_CUDA(cudaMemcpyAsync(Ph.data(), P.p, Ph.size() * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    FEM2D_CUDA(cudaStreamSynchronize(c.stream));
    for (int j = 0; j < kout; j++) {
      double sr = 0, sbb = 0, sx = 0;
      for (int q = 0; q < nblk; q++) {
        sr += Ph[(size_t)q * 3 * kout + j];
        sbb += Ph[(size_t)q * 3 * kout + kout + j];
        sx += Ph[(size_t)q * 3 * kout + 2 * kout + j];
      }
      rel_out[j] = std::sqrt(sr) / (std::fabs(theta_out[j]) * std::sqrt(sbb) + 1e-300);
      bwd_out[j] = std::sqrt(sr) / ((na0 + std::fabs(theta_out[j]) * nb0) * std::sqrt(sx) + 1e-300);
    }
    if (st) {
      double w = 0, wb = 0;
      for (int q = 0; q < kout; q++) {
        w = std::max(w, rel_out[q]);
        wb = std::max(wb, bwd_out[q]);
      }
      st->max_rel_residual = w;
      st->max_backward_error = wb;
    }
  }
  // outputs: B-normalised (the Ritz vectors are B-orthonormal), sign fixed by the largest entry (the
  // first of equal magnitude); the signs and the transposition to one contiguous vector per pair are
  // done on the device, so exactly kout x n doubles come back
  for (int q = 0; q < kout; q++) {
    if (values) values[q] = theta_out[q];
    if (residuals) residuals[q] = rel_out[q];
  }
  if (vectors && kout > 0) {
    const int nblk = (int)std::min<int64_t>(D.grid_rows(), std::max<int64_t>(1, (n + 255) / 256));
    DBuf<double> pm;
    DBuf<int64_t> pi;
    pm.alloc_on((size_t)nblk * kout, c.stream);
    pi.alloc_on((size_t)nblk * kout, c.stream);
    colmax_partial_kernel<<<nblk, 256, 0, c.stream>>>(n, XO.p, 32, kout, pm.p, pi.p);
    c.launches++;
    std::vector<double> hm((size_t)nblk * kout);
    std::vector<int64_t> hi((size_t)nblk * kout);
    FEM2D_CUDA(cudaMemcpyAsync(hm.data(), pm.p, hm.size() * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    FEM2D_CUDA(cudaMemcpyAsync(hi.data(), pi.p, hi.size() * sizeof(int64_t), cudaMemcpyDeviceToHost, c.stream));
    FEM2D_CUDA(cudaStreamSynchronize(c.stream));
    std::vector<double> sgn(kout, 1.0);
    for (int q = 0; q < kout; q++) {
      double best = -1.0, val = 0.0;
      int64_t bi = INT64_MAX;
      for (int b = 0; b < nblk; b++) {   // blocks hold ascending row ranges: keep the first maximum
        const double m = std::fabs(hm[(size_t)b * kout + q]);
        if (m > best || (m == best && hi[(size_t)b * kout + q] < bi)) {
          best = m;
          bi = hi[(size_t)b * kout + q];
          val = hm[(size_t)b * kout + q];
        }
      }
      sgn[q] = val < 0 ? -1.0 : 1.0;
    }
    DBuf<double> sg, VT;
    sg.upload_on(sgn, c.stream);
    VT.alloc_on((size_t)kout * n, c.stream);
    const int64_t tb = std::min<int64_t>((n * kout + 255) / 256, (int64_t)c.num_sms * 16);
    signed_transpose_kernel<<<(int)std::max<int64_t>(tb, 1), 256, 0, c.stream>>>(n, XO.p, 32, kout, sg.p, VT.p);
    c.launches++;
    FEM2D_CUDA(cudaMemcpyAsync(vectors, VT.p, (size_t)kout * n * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    FEM2D_CUDA(cudaStreamSynchronize(c.stream));
  }
  if (!converged)
    fail(FEM2D_E_NOT_CONVERGED, "gpu_solve_gep did not reach the residual tolerance (outputs hold the last iterate)");
}

// ================================================================ dense solve (nalgebra_solve_gep)
void dense_solve(Ctx& c, const Domain& dom, const HostGEP& h, const DeviceGEP& d, MFPlan& plan, double target,
                 double* value, double* vector) {
  const int64_t n = h.n;
  if (n > 1000) fail(FEM2D_E_TOO_LARGE, "Matrices Exceeded Maximum Size (1000x1000); Cannot Solve!");
  MFDevice& mf = mf_plan(plan, c, dom, h);
  MFFactor fb;
  mf.factor(c, d.a.p, d.b.p, 0.0, 1.0, true, fb);
  if (fb.flags & 2) fail(FEM2D_E_B_NOT_SPD, "Failed to invert B-matrix (via cholesky); likely ill-conditioned!");
  DBuf<double> Ad, Z;
  Ad.alloc_on((size_t)n * n, c.stream);
  Z.alloc_on((size_t)n * n, c.stream);
  FEM2D_CUDA(cudaMemsetAsync(Ad.p, 0, (size_t)n * n * sizeof(double), c.stream));
  densify_kernel<<<(int)std::min<int64_t>(n, 4096), 128, 0, c.stream>>>(n, d.row_ptr.p, d.col.p, d.a.p, d.b.p, 1.0,
                                                                        0.0, Ad.p);
  c.launches++;
  for (int64_t c0 = 0; c0 < n; c0 += 32) {
    const int w = (int)std::min<int64_t>(32, n - c0);
    mf.solve(c, fb, Ad.p + c0, n, Z.p + c0, n, w);
  }
  std::vector<double> Zh((size_t)n * n);
  FEM2D_CUDA(cudaMemcpyAsync(Zh.data(), Z.p, Zh.size() * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
  FEM2D_CUDA(cudaStreamSynchronize(c.stream));
  // symmetric matrix from the lower triangle of B^-1 A
  std::vector<double> S((size_t)n * n);
  for (int64_t i = 0; i < n; i++)
    for (int64_t j = 0; j <= i; j++) S[(size_t)i * n + j] = S[(size_t)j * n + i] = Zh[(size_t)i * n + j];
  std::vector<double> w, z;
  if (!symeig((int)n, S, w, z)) fail(FEM2D_E_NOT_CONVERGED, "symmetric eigen-decomposition did not converge");
  bool all_spurious = true;
  for (double x : w)
    if (std::fabs(x) >= 1e-12) all_spurious = false;
  if (all_spurious) fail(FEM2D_E_SPURIOUS, "Only spurious modes were found!");
  int64_t best = 0;
  double dmin = HUGE_VAL;
  for (int64_t q = 0; q < n; q++) {
    double dl = std::fabs(w[q] - target);
    if (dl < dmin) {
      dmin = dl;
      best = q;
    }
  }
  if (value) *value = w[best];
  if (vector)
    for (int64_t i = 0; i < n; i++) vector[i] = z[(size_t)i * n + best];
}

}  // namespace fem2d

namespace fem2d {

void gep_spmm(Ctx& c, const HostGEP& h, const DeviceGEP& d, double ca, double cb, const double* X, int64_t ldx, int nb,
              double* Y, int64_t ldy) {
  Dev D{c, h, d, d.a.p, d.b.p};
  D.spmm(ca, cb, X, ldx, nb, Y, ldy);
  FEM2D_CUDA(cudaGetLastError());
}

void gep_spmm_values(Ctx& c, const HostGEP& h, const DeviceGEP& d, const double* va, const double* vb, double ca,
                     double cb, const double* X, int64_t ldx, int nb, double* Y, int64_t ldy) {
  Dev D{c, h, d, va, vb};
  D.spmm(ca, cb, X, ldx, nb, Y, ldy);
  FEM2D_CUDA(cudaGetLastError());
}

void shifted_solve(Ctx& c, const Domain& dom, const HostGEP& h, const DeviceGEP& d, MFPlan& plan, double ca,
                   double cb, bool spd, int nrhs, const double* rhs, double* x) {
  const int64_t n = h.n;
  Dev D{c, h, d, d.a.p, d.b.p};
  DBuf<double> R, X, T, U;
  R.alloc_on((size_t)n * 32, c.stream);
  X.alloc_on((size_t)n * 32, c.stream);
  T.alloc_on((size_t)n * 32, c.stream);
  U.alloc_on((size_t)n * 32, c.stream);
  std::vector<double> hr((size_t)n * 32), hx((size_t)n * 32), G;
  // max over the columns of ||R - K X|| / ||R||, K = ca A + cb B
  auto relres = [&](int w) {
    D.spmm(ca, cb, X.p, 32, w, T.p, 32);
    D.axpby(1.0, R.p, 32, w, -1.0, T.p, 32);
    D.gram(T.p, 32, w, T.p, 32, w, G);
    std::vector<double> tg = G;
    D.gram(R.p, 32, w, R.p, 32, w, G);
    double rel = 0;
    for (int j = 0; j < w; j++)
      rel = std::max(rel, std::sqrt(tg[(size_t)j * w + j] / std::max(G[(size_t)j * w + j], 1e-300)));
    return rel;
  };
  for (int attempt = 0; attempt < 2; attempt++) {
    MFDevice& mf = attempt == 0 ? mf_plan(plan, c, dom, h) : mf_plan_dense(plan, c, h);
    MFFactor fac;
    mf.factor(c, d.a.p, d.b.p, ca, cb, spd, fac);
    if (spd && (fac.flags & 2)) fail(FEM2D_E_B_NOT_SPD, "the shifted matrix is not positive definite");
    double worst = 0;
    for (int c0 = 0; c0 < nrhs; c0 += 32) {
      const int w = std::min(32, nrhs - c0);
      for (int64_t i = 0; i < n; i++)
        for (int k = 0; k < 32; k++) hr[(size_t)i * 32 + k] = k < w ? rhs[(size_t)i * nrhs + c0 + k] : 0.0;
      FEM2D_CUDA(cudaMemcpyAsync(R.p, hr.data(), hr.size() * sizeof(double), cudaMemcpyHostToDevice, c.stream));
      mf.solve(c, fac, R.p, 32, X.p, 32, w);
      // iterative refinement in FP64 while it keeps improving (up to 3 steps)
      double rel = relres(w);
      for (int it = 0; it < 3 && rel > 1e-13; it++) {
        mf.solve(c, fac, T.p, 32, U.p, 32, w);
        D.axpby(1.0, U.p, 32, w, 1.0, X.p, 32);
        const double r2 = relres(w);
        if (r2 > 0.5 * rel) {   // no longer improving: undo the step
          D.axpby(-1.0, U.p, 32, w, 1.0, X.p, 32);
          break;
        }
        rel = r2;
      }
      worst = std::max(worst, rel);
      FEM2D_CUDA(cudaMemcpyAsync(hx.data(), X.p, hx.size() * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
      FEM2D_CUDA(cudaStreamSynchronize(c.stream));
      for (int64_t i = 0; i < n; i++)
        for (int k = 0; k < w; k++) x[(size_t)i * nrhs + c0 + k] = hx[(size_t)i * 32 + k];
    }
    // small systems the sparse plan cannot solve accurately are redone with one dense front
    if (worst <= 1e-10 || plan.dense || n > 4096) break;
  }
}

}  // namespace fem2d

namespace fem2d {

// C (device, row-major a x b) = X^T Y with the FP64 CUDA-core kernels (method 1) or the tensor-core
// emulation (method 0); synchronises
void block_gram(Ctx& c, int method, int64_t n, const double* X, int64_t ldx, int a, const double* Y, int64_t ldy,
                int b, double* Cd) {
  setup_gemm_smem(c.device);
  HostGEP hg;
  hg.n = n;
  DeviceGEP dg;
  Dev D{c, hg, dg, nullptr, nullptr};
  D.dense_mode = method == 0 ? 0 : 1;
  if (method == 0 && (a > 512 || b > 256)) fail(FEM2D_E_INVALID_ARG, "tensor Gram: a <= 512 and b <= 256");
  D.gram_dev(X, ldx, a, Y, ldy, b, Cd);
  D.check_tensor();
  FEM2D_CUDA(cudaStreamSynchronize(c.stream));
}

}  // namespace fem2d

namespace fem2d {

// Z = beta Z + alpha X C (device blocks; C row-major a x b): method 0 tensor cores, 1 FP64 CUDA cores
void block_gemm(Ctx& c, int method, int64_t n, const double* X, int64_t ldx, int a, const double* Cd, int b,
                double alpha, double beta, double* Z, int64_t ldz) {
  setup_gemm_smem(c.device);
  HostGEP hg;
  hg.n = n;
  DeviceGEP dg;
  Dev D{c, hg, dg, nullptr, nullptr};
  D.dense_mode = method == 0 ? 0 : 1;
  if (method == 0 && (a > 256 || b > 32)) fail(FEM2D_E_INVALID_ARG, "tensor update: a <= 256 and b <= 32");
  D.gemm_dev(X, ldx, a, Cd, b, alpha, beta, Z, ldz);
  D.check_tensor();
  FEM2D_CUDA(cudaStreamSynchronize(c.stream));
}

}  // namespace fem2d

namespace fem2d {

// Y = coef M X for M = A (which 0) or B (which 1) of the GEP through the tensor-core product (the GEP's
// values sliced for this call); synchronises
void gep_spmm_tensor(Ctx& c, const HostGEP& h, const DeviceGEP& d, int which, double coef, const double* X,
                     int64_t ldx, int nb, double* Y, int64_t ldy) {
  if (which != 0 && which != 1) fail(FEM2D_E_INVALID_ARG, "which must be 0 (A) or 1 (B)");
  if (nb < 1 || nb > 32) fail(FEM2D_E_INVALID_ARG, "1..32 columns");
  TcSpmm tcs;
  tcs.build(c, h.n, d.grp_h, h.row_ptr);
  tcs.slice(c, 0, d.grp.p, d.row_ptr.p, which == 0 ? d.a.p : nullptr, which == 1 ? d.b.p : nullptr,
            which == 0 ? 1.0 : 0.0, which == 1 ? 1.0 : 0.0);
  Dev D{c, h, d, d.a.p, d.b.p};
  D.tcs = &tcs;
  D.spmm(which == 0 ? coef : 0.0, which == 1 ? coef : 0.0, X, ldx, nb, Y, ldy);
  D.check_tensor();
  FEM2D_CUDA(cudaStreamSynchronize(c.stream));
}

}  // namespace fem2d
