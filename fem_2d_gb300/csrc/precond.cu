// Inner PCG solver, its plain (additive Schwarz over Elem patches) and learned (two-level, network
// coarse basis) preconditioners, and the network's training kernels. See precond.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>

#include "eigen.h"
#include "gep.h"
#include "mf.h"
#include "mfdev.h"
#include "precond.h"

namespace fem2d {

namespace {

constexpr int kMaxK = 32;        // coarse vectors per Elem
constexpr int kMaxSamples = 256;  // error samples per loss launch
constexpr int kMaxPatch = 160;    // specs per Elem handled by the block inverses
constexpr int kNB = 32;           // right-hand sides per PCG block

// ------------------------------------------------------------------ FP32 MLP kernels
// C (M x N) = op(A) (M x K) * op(B) (K x N) + beta C, row-major; 64 x 64 tile per CTA, 4 x 4 per thread.
// op(A)(i, k) = TA ? A[k * lda + i] : A[i * lda + k];  op(B)(k, j) = TB ? B[j * ldb + k] : B[k * ldb + j]
template <bool TA, bool TB>
__global__ void __launch_bounds__(256) sgemm_kernel(int M, int N, int K, const float* __restrict__ A, int lda,
                                                    const float* __restrict__ B, int ldb, float* __restrict__ C,
                                                    int ldc, float beta) {
  __shared__ float As[16][65];
  __shared__ float Bs[16][65];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int i0 = blockIdx.y * 64, j0 = blockIdx.x * 64;
  float acc[4][4];
#pragma unroll
  for (int q = 0; q < 4; q++)
#pragma unroll
    for (int s = 0; s < 4; s++) acc[q][s] = 0.f;
  for (int k0 = 0; k0 < K; k0 += 16) {
    for (int t = threadIdx.x; t < 16 * 64; t += 256) {
      int kk, ii;
      if (TA) { ii = t & 63; kk = t >> 6; } else { kk = t & 15; ii = t >> 4; }
      const int gi = i0 + ii, gk = k0 + kk;
      As[kk][ii] = (gi < M && gk < K) ? (TA ? A[(size_t)gk * lda + gi] : A[(size_t)gi * lda + gk]) : 0.f;
      int kb, jj;
      if (TB) { kb = t & 15; jj = t >> 4; } else { jj = t & 63; kb = t >> 6; }
      const int gj = j0 + jj, gkb = k0 + kb;
      Bs[kb][jj] = (gj < N && gkb < K) ? (TB ? B[(size_t)gj * ldb + gkb] : B[(size_t)gkb * ldb + gj]) : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < 16; kk++) {
      float a[4], b[4];
#pragma unroll
      for (int q = 0; q < 4; q++) {
        a[q] = As[kk][ty + 16 * q];
        b[q] = Bs[kk][tx + 16 * q];
      }
#pragma unroll
      for (int q = 0; q < 4; q++)
#pragma unroll
        for (int s = 0; s < 4; s++) acc[q][s] = fmaf(a[q], b[s], acc[q][s]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int q = 0; q < 4; q++) {
    const int i = i0 + ty + 16 * q;
    if (i >= M) continue;
#pragma unroll
    for (int s = 0; s < 4; s++) {
      const int j = j0 + tx + 16 * s;
      if (j >= N) continue;
      float v = acc[q][s];
      if (beta != 0.f) v += beta * C[(size_t)i * ldc + j];
      C[(size_t)i * ldc + j] = v;
    }
  }
}

// Y = act(Y + b) per row (act: tanh when on)
__global__ void bias_act_kernel(float* __restrict__ Y, int64_t R, int O, const float* __restrict__ b, int act) {
  const int64_t total = R * O;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const float v = Y[t] + b[t % O];
    Y[t] = act ? tanhf(v) : v;
  }
}

// dH *= 1 - H^2 (tanh derivative)
__global__ void dtanh_kernel(float* __restrict__ dH, const float* __restrict__ H, int64_t total) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x)
    dH[t] *= 1.f - H[t] * H[t];
}

// out[o] += sum over rows of Y[r][o]; thread per column, CTA per row range
__global__ void colsum_kernel(const float* __restrict__ Y, int64_t R, int O, int64_t rows_per_block,
                              float* __restrict__ out) {
  const int64_t r0 = blockIdx.x * rows_per_block, r1 = min(R, r0 + rows_per_block);
  for (int o = threadIdx.x; o < O; o += blockDim.x) {
    float s = 0.f;
    for (int64_t r = r0; r < r1; r++) s += Y[r * O + o];
    atomicAdd(out + o, s);
  }
}

__global__ void adam_kernel(int64_t n, float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, float lr, float b1, float b2, float eps, float c1, float c2,
                            float gscale) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    const float gt = g[t] * gscale;
    const float mt = b1 * m[t] + (1.f - b1) * gt;
    const float vt = b2 * v[t] + (1.f - b2) * gt * gt;
    m[t] = mt;
    v[t] = vt;
    p[t] -= lr * (mt / c1) / (sqrtf(vt / c2) + eps);
  }
}

// Projection loss of one Elem patch (one CTA) over S error samples E (n x S row-major, FP64):
//   c_s = (Z^T Z + lam I)^-1 Z^T e_s,  loss_s = (||e_s||^2 - c_s^T Z^T e_s) / ||e_s||^2
// (= (||e_s - Z c_s||^2 + lam ||c_s||^2) / ||e_s||^2), and dZ = scale * sum_s -2 (e_s - Z c_s) c_s^T / ||e_s||^2.
__global__ void __launch_bounds__(256) proj_loss_kernel(const int64_t* __restrict__ pptr,
                                                        const int32_t* __restrict__ rdof, const float* __restrict__ Z,
                                                        int k, const double* __restrict__ E, int S, double lam,
                                                        double scale, float* __restrict__ dZ,
                                                        double* __restrict__ loss_part) {
  const int p = blockIdx.x;
  const int64_t r0 = pptr[p];
  const int np = (int)(pptr[p + 1] - r0);
  __shared__ double G[kMaxK * kMaxK];
  __shared__ double C[kMaxSamples * kMaxK];
  __shared__ double W[kMaxSamples];
  __shared__ double red[256];
  const float* Zp = Z + r0 * k;
  for (int t = threadIdx.x; t < k * k; t += blockDim.x) {
    const int a = t / k, b = t % k;
    double s = 0.0;
    for (int i = 0; i < np; i++) s += (double)Zp[i * k + a] * (double)Zp[i * k + b];
    G[t] = s + (a == b ? lam : 0.0);
  }
  __syncthreads();
  if (threadIdx.x == 0) {   // Cholesky G = L L^T in place (lower triangle)
    for (int j = 0; j < k; j++) {
      double d = G[j * k + j];
      for (int q = 0; q < j; q++) d -= G[j * k + q] * G[j * k + q];
      d = sqrt(fmax(d, 1e-300));
      G[j * k + j] = d;
      for (int i = j + 1; i < k; i++) {
        double s = G[i * k + j];
        for (int q = 0; q < j; q++) s -= G[i * k + q] * G[j * k + q];
        G[i * k + j] = s / d;
      }
    }
  }
  __syncthreads();
  double lsum = 0.0;
  for (int s = threadIdx.x; s < S; s += blockDim.x) {
    double bvec[kMaxK], y[kMaxK];
#pragma unroll
    for (int a = 0; a < kMaxK; a++) bvec[a] = 0.0;
    double ee = 0.0;
    for (int i = 0; i < np; i++) {
      const double e = E[(int64_t)rdof[r0 + i] * S + s];
      ee += e * e;
#pragma unroll
      for (int a = 0; a < kMaxK; a++)
        if (a < k) bvec[a] += (double)Zp[i * k + a] * e;
    }
    // L y = b, L^T c = y
#pragma unroll
    for (int a = 0; a < kMaxK; a++) {
      if (a >= k) break;
      double v = bvec[a];
      for (int q = 0; q < a; q++) v -= G[a * k + q] * y[q];
      y[a] = v / G[a * k + a];
    }
    double cb = 0.0;
    for (int a = k - 1; a >= 0; a--) {
      double v = y[a];
      for (int q = a + 1; q < k; q++) v -= G[q * k + a] * C[s * kMaxK + q];
      v /= G[a * k + a];
      C[s * kMaxK + a] = v;
      cb += v * bvec[a];
    }
    if (ee > 0.0) {
      lsum += (ee - cb) / ee;
      W[s] = -2.0 * scale / ee;
    } else {
      W[s] = 0.0;
    }
  }
  red[threadIdx.x] = lsum;
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st) red[threadIdx.x] += red[threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x == 0) loss_part[p] = red[0];
  for (int i = threadIdx.x; i < np; i += blockDim.x) {
    double zi[kMaxK], acc[kMaxK];
#pragma unroll
    for (int a = 0; a < kMaxK; a++) {
      zi[a] = a < k ? (double)Zp[i * k + a] : 0.0;
      acc[a] = 0.0;
    }
    const int64_t dof = rdof[r0 + i];
    for (int s = 0; s < S; s++) {
      double r = E[dof * S + s];
#pragma unroll
      for (int a = 0; a < kMaxK; a++) r -= zi[a] * C[s * kMaxK + a];
      const double wr = W[s] * r;
#pragma unroll
      for (int a = 0; a < kMaxK; a++) acc[a] += wr * C[s * kMaxK + a];
    }
    for (int a = 0; a < k; a++) dZ[(r0 + i) * k + a] = (float)acc[a];
  }
}

// ------------------------------------------------------------------ PCG kernels
// Block inverse of K restricted to one Elem patch (one CTA): gather from the CSR, Gauss-Jordan
// (K SPD: no pivoting), write the np x np inverse.
__global__ void __launch_bounds__(256) bj_invert_kernel(const int64_t* __restrict__ pptr,
                                                        const int32_t* __restrict__ rdof,
                                                        const int32_t* __restrict__ sdof,
                                                        const int32_t* __restrict__ sloc,
                                                        const int64_t* __restrict__ ioff,
                                                        const int64_t* __restrict__ rp, const int32_t* __restrict__ col,
                                                        const double* __restrict__ va, const double* __restrict__ vb,
                                                        double ca, double cb, double* __restrict__ inv,
                                                        int* __restrict__ flag) {
  extern __shared__ double Ms[];
  const int p = blockIdx.x;
  const int64_t r0 = pptr[p];
  const int np = (int)(pptr[p + 1] - r0);
  for (int t = threadIdx.x; t < np * np; t += blockDim.x) Ms[t] = 0.0;
  __syncthreads();
  const int32_t* sd = sdof + r0;
  const int32_t* sl = sloc + r0;
  for (int i = threadIdx.x; i < np; i += blockDim.x) {
    const int32_t dof = rdof[r0 + i];
    for (int64_t q = rp[dof]; q < rp[dof + 1]; q++) {
      const int32_t j = col[q];
      int lo = 0, hi = np - 1, hit = -1;
      while (lo <= hi) {
        const int mid = (lo + hi) >> 1;
        if (sd[mid] == j) { hit = mid; break; }
        if (sd[mid] < j) lo = mid + 1; else hi = mid - 1;
      }
      if (hit >= 0) Ms[i * np + sl[hit]] = ca * va[q] + cb * vb[q];
    }
  }
  __syncthreads();
  // rows bound to the same DoF twice (a spec listed twice) would make the block singular; K's
  // restriction is SPD otherwise. Gauss-Jordan on [M | I] in place.
  __shared__ double piv_inv;
  for (int q = 0; q < np; q++) {
    if (threadIdx.x == 0) {
      const double d = Ms[q * np + q];
      if (!(d > 0.0)) atomicOr(flag, 1);
      piv_inv = d > 0.0 ? 1.0 / d : 0.0;
    }
    __syncthreads();
    const double pi = piv_inv;
    // scale row q; eliminate column q from the other rows
    for (int j = threadIdx.x; j < np; j += blockDim.x) Ms[q * np + j] = (j == q ? 1.0 : Ms[q * np + j]) * pi;
    __syncthreads();
    for (int t = threadIdx.x; t < np * np; t += blockDim.x) {
      const int i = t / np, j = t % np;
      if (i == q) continue;
      const double f = Ms[i * np + q];
      if (j == q) continue;
      Ms[t] -= f * Ms[q * np + j];
    }
    __syncthreads();
    for (int i = threadIdx.x; i < np; i += blockDim.x)
      if (i != q) Ms[i * np + q] = -Ms[i * np + q] * pi;
    __syncthreads();
  }
  double* out = inv + ioff[p];
  for (int t = threadIdx.x; t < np * np; t += blockDim.x) out[t] = Ms[t];
}

// Z += sum over patches of M_p^-1 r_p (rows of shared DoFs receive several contributions)
__global__ void __launch_bounds__(256) bj_apply_kernel(const int64_t* __restrict__ pptr,
                                                       const int32_t* __restrict__ rdof,
                                                       const int64_t* __restrict__ ioff,
                                                       const double* __restrict__ inv, const double* __restrict__ R,
                                                       int nb, double* __restrict__ Zo) {
  __shared__ double rs[kMaxPatch * kNB];
  const int p = blockIdx.x;
  const int64_t r0 = pptr[p];
  const int np = (int)(pptr[p + 1] - r0);
  for (int t = threadIdx.x; t < np * nb; t += blockDim.x) {
    const int i = t / nb, c = t % nb;
    rs[i * kNB + c] = R[(int64_t)rdof[r0 + i] * kNB + c];
  }
  __syncthreads();
  const double* Mi = inv + ioff[p];
  for (int t = threadIdx.x; t < np * nb; t += blockDim.x) {
    const int i = t / nb, c = t % nb;
    double s = 0.0;
    for (int j = 0; j < np; j++) s += Mi[i * np + j] * rs[j * kNB + c];
    atomicAdd(Zo + (int64_t)rdof[r0 + i] * kNB + c, s);
  }
}

// y[(p k + a) * kNB + c] = sum_i w_i Zn[i][a] R[dof_i][c] over the rows i of patch p
__global__ void coarse_restrict_kernel(const int64_t* __restrict__ pptr, const int32_t* __restrict__ rdof,
                                       const float* __restrict__ Zw, int k, const double* __restrict__ R, int ldr,
                                       int nb, double* __restrict__ y) {
  const int p = blockIdx.x;
  const int64_t r0 = pptr[p];
  const int np = (int)(pptr[p + 1] - r0);
  for (int t = threadIdx.x; t < k * nb; t += blockDim.x) {
    const int a = t / nb, c = t % nb;
    double s = 0.0;
    for (int i = 0; i < np; i++) s += (double)Zw[(r0 + i) * k + a] * R[(int64_t)rdof[r0 + i] * ldr + c];
    y[((int64_t)p * k + a) * kNB + c] = s;
  }
}

// Zo[dof_i][c] += w_i sum_a Zn[i][a] w[(p k + a)][c]
__global__ void coarse_prolong_kernel(const int64_t* __restrict__ pptr, const int32_t* __restrict__ rdof,
                                      const float* __restrict__ Zw, int k, const double* __restrict__ w, int nb,
                                      double* __restrict__ Zo, int ldz) {
  const int p = blockIdx.x;
  const int64_t r0 = pptr[p];
  const int np = (int)(pptr[p + 1] - r0);
  for (int t = threadIdx.x; t < np * nb; t += blockDim.x) {
    const int i = t / nb, c = t % nb;
    double s = 0.0;
    for (int a = 0; a < k; a++) s += (double)Zw[(r0 + i) * k + a] * w[((int64_t)p * k + a) * kNB + c];
    atomicAdd(Zo + (int64_t)rdof[r0 + i] * ldz + c, s);
  }
}

// columns j0 .. j0+31 of the weighted coarse basis, densely (n x kNB)
__global__ void coarse_columns_kernel(const int64_t* __restrict__ pptr, const int32_t* __restrict__ rdof,
                                      const float* __restrict__ Zw, int k, int j0, int p0, int p1,
                                      double* __restrict__ Zc) {
  const int p = p0 + blockIdx.x;
  if (p >= p1) return;
  const int64_t r0 = pptr[p];
  const int np = (int)(pptr[p + 1] - r0);
  for (int t = threadIdx.x; t < np * k; t += blockDim.x) {
    const int i = t / k, a = t % k;
    const int j = p * k + a - j0;
    if (j < 0 || j >= kNB) continue;
    atomicAdd(Zc + (int64_t)rdof[r0 + i] * kNB + j, (double)Zw[(r0 + i) * k + a]);
  }
}

// Kc[(q k + b) * m + j0 + jj] = sum_i w_i Zn[i][b] Y[dof_i][jj] (patch q per CTA)
__global__ void coarse_gram_kernel(const int64_t* __restrict__ pptr, const int32_t* __restrict__ rdof,
                                   const float* __restrict__ Zw, int k, const double* __restrict__ Y, int ncols,
                                   int j0, int m, double* __restrict__ Kc) {
  const int q = blockIdx.x;
  const int64_t r0 = pptr[q];
  const int np = (int)(pptr[q + 1] - r0);
  for (int t = threadIdx.x; t < k * ncols; t += blockDim.x) {
    const int b = t / ncols, jj = t % ncols;
    double s = 0.0;
    for (int i = 0; i < np; i++) s += (double)Zw[(r0 + i) * k + b] * Y[(int64_t)rdof[r0 + i] * kNB + jj];
    Kc[((int64_t)q * k + b) * m + j0 + jj] = s;
  }
}

// one Gauss-Jordan step on an SPD m x m matrix held in place (column q eliminated from every other row):
// after all m steps M holds M^-1. Row q is scaled by 1 / pivot; the rest gets the rank-1 update.
__global__ void gj_step_kernel(int m, int q, double* __restrict__ M) {
  const double piv = M[(int64_t)q * m + q];
  const double inv = 1.0 / piv;
  const int64_t total = (int64_t)m * m;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t / m), j = (int)(t % m);
    if (i == q) continue;
    const double f = M[(int64_t)i * m + q];
    if (j == q) continue;
    M[t] -= f * inv * M[(int64_t)q * m + j];
  }
}
// finishing pass of step q: column q and row q (step q left them intact); the pivot itself is replaced
// by its reciprocal in a separate launch, after every thread here has read it
__global__ void gj_finish_kernel(int m, int q, double* __restrict__ M) {
  const double inv = 1.0 / M[(int64_t)q * m + q];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
    if (i != q) {
      M[(int64_t)i * m + q] = -M[(int64_t)i * m + q] * inv;
      M[(int64_t)q * m + i] = M[(int64_t)q * m + i] * inv;
    }
  }
}
__global__ void gj_pivot_kernel(int m, int q, double* __restrict__ M) {
  if (blockIdx.x == 0 && threadIdx.x == 0) M[(int64_t)q * m + q] = 1.0 / M[(int64_t)q * m + q];
}

// per-column dot products of X and Y (n x nb, ld kNB): partial sums per CTA
__global__ void coldot_kernel(int64_t n, int nb, const double* __restrict__ X, const double* __restrict__ Y,
                              int64_t rows_per_block, double* __restrict__ part) {
  __shared__ double red[256];
  const int c = threadIdx.x % kNB, lane_row = threadIdx.x / kNB;   // 8 row lanes x 32 columns
  const int64_t r0 = blockIdx.x * rows_per_block, r1 = min(n, r0 + rows_per_block);
  double s = 0.0;
  if (c < nb)
    for (int64_t r = r0 + lane_row; r < r1; r += blockDim.x / kNB) s += X[r * kNB + c] * Y[r * kNB + c];
  red[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x < kNB) {
    double t = 0.0;
    for (int q = 0; q < (int)blockDim.x / kNB; q++) t += red[q * kNB + threadIdx.x];
    part[(int64_t)blockIdx.x * kNB + threadIdx.x] = t;
  }
}

// X += a_c P, R -= a_c Q (per column c)
__global__ void cg_update_kernel(int64_t n, int nb, const double* __restrict__ alpha, const double* __restrict__ P,
                                 const double* __restrict__ Q, double* __restrict__ X, double* __restrict__ R) {
  const int64_t total = n * kNB;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(t % kNB);
    if (c >= nb) continue;
    const double a = alpha[c];
    X[t] += a * P[t];
    R[t] -= a * Q[t];
  }
}

// P = Z + b_c P
__global__ void cg_direction_kernel(int64_t n, int nb, const double* __restrict__ beta, const double* __restrict__ Zs,
                                    double* __restrict__ P) {
  const int64_t total = n * kNB;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(t % kNB);
    if (c >= nb) continue;
    P[t] = Zs[t] + beta[c] * P[t];
  }
}

__global__ void to_f32_kernel(int64_t n, const double* __restrict__ x, float* __restrict__ y) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
    y[t] = (float)x[t];
}
__global__ void to_f64_kernel(int64_t n, const float* __restrict__ x, double* __restrict__ y) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
    y[t] = (double)x[t];
}

// Y (ldy) = X (ldx), n x nb
__global__ void strided_copy_kernel(int64_t n, int nb, const double* __restrict__ X, int64_t ldx, double* __restrict__ Y,
                                    int64_t ldy) {
  const int64_t total = n * nb;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = t / nb;
    const int j = (int)(t % nb);
    Y[r * ldy + j] = X[r * ldx + j];
  }
}

// Y = s0_c X0 + s1_c X1 + s2_c X2 per column c (blocks n x kNB; a null X term is skipped; Y may alias X0)
__global__ void lincomb3_kernel(int64_t n, int nb, const double* __restrict__ s, const double* X0, const double* X1,
                                const double* X2, double* Y) {
  const int64_t total = n * kNB;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(t % kNB);
    if (c >= nb) continue;
    double v = s[c] * X0[t];
    if (X1) v += s[kNB + c] * X1[t];
    if (X2) v += s[2 * kNB + c] * X2[t];
    Y[t] = v;
  }
}

// X += a_c P per column
__global__ void axpy_cols_kernel(int64_t n, int nb, const double* __restrict__ a, const double* __restrict__ P,
                                 double* __restrict__ X) {
  const int64_t total = n * kNB;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(t % kNB);
    if (c >= nb) continue;
    X[t] += a[c] * P[t];
  }
}

uint64_t splitmix(uint64_t& s) {
  s += 0x9E3779B97F4A7C15ull;
  uint64_t z = s;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

int grid_for(const Ctx& c, int64_t work, int per_sm = 8) {
  return (int)std::max<int64_t>(1, std::min<int64_t>((work + 255) / 256, (int64_t)c.num_sms * per_sm));
}

template <bool TA, bool TB>
void sgemm(Ctx& c, int M, int N, int K, const float* A, int lda, const float* B, int ldb, float* C, int ldc,
           float beta) {
  if (M <= 0 || N <= 0) return;
  dim3 grid((N + 63) / 64, (M + 63) / 64);
  sgemm_kernel<TA, TB><<<grid, 256, 0, c.stream>>>(M, N, K, A, lda, B, ldb, C, ldc, beta);
  c.launches++;
}

// device buffers of one forward/backward pass over a set of rows
struct NetPass {
  int64_t R = 0;
  DBuf<float> X, H1, H2, Z, dZ, dH2, dH1;
  DBuf<int64_t> pptr;
  DBuf<int32_t> rdof;
  void setup(Ctx& c, const Patches& pt, const PatchNet& net) {
    R = pt.nrows;
    X.upload(pt.feat, c.stream);
    H1.alloc((size_t)R * net.hidden);
    H2.alloc((size_t)R * net.hidden);
    Z.alloc((size_t)R * net.k);
    dZ.alloc((size_t)R * net.k);
    dH2.alloc((size_t)R * net.hidden);
    dH1.alloc((size_t)R * net.hidden);
    pptr.upload(pt.ptr, c.stream);
    rdof.upload(pt.dof, c.stream);
  }
};

struct NetOffsets {
  int64_t W1, b1, W2, b2, W3, b3;
  explicit NetOffsets(const PatchNet& n) {
    W1 = 0;
    b1 = W1 + (int64_t)n.nin * n.hidden;
    W2 = b1 + n.hidden;
    b2 = W2 + (int64_t)n.hidden * n.hidden;
    W3 = b2 + n.hidden;
    b3 = W3 + (int64_t)n.hidden * n.k;
  }
};

void net_forward(Ctx& c, const PatchNet& net, const float* P, NetPass& ps) {
  const NetOffsets o(net);
  const int H = net.hidden, k = net.k, R = (int)ps.R;
  sgemm<false, false>(c, R, H, net.nin, ps.X.p, net.nin, P + o.W1, H, ps.H1.p, H, 0.f);
  bias_act_kernel<<<grid_for(c, (int64_t)R * H), 256, 0, c.stream>>>(ps.H1.p, R, H, P + o.b1, 1);
  sgemm<false, false>(c, R, H, H, ps.H1.p, H, P + o.W2, H, ps.H2.p, H, 0.f);
  bias_act_kernel<<<grid_for(c, (int64_t)R * H), 256, 0, c.stream>>>(ps.H2.p, R, H, P + o.b2, 1);
  sgemm<false, false>(c, R, k, H, ps.H2.p, H, P + o.W3, k, ps.Z.p, k, 0.f);
  bias_act_kernel<<<grid_for(c, (int64_t)R * k), 256, 0, c.stream>>>(ps.Z.p, R, k, P + o.b3, 0);
  c.launches += 3;
}

// gradients of the parameters (added to G) from dZ
void net_backward(Ctx& c, const PatchNet& net, const float* P, NetPass& ps, float* G) {
  const NetOffsets o(net);
  const int H = net.hidden, k = net.k, R = (int)ps.R;
  const int64_t rpb = 64;
  const int nblk = (int)((R + rpb - 1) / rpb);
  // layer 3
  sgemm<true, false>(c, H, k, R, ps.H2.p, H, ps.dZ.p, k, G + o.W3, k, 1.f);
  colsum_kernel<<<nblk, 256, 0, c.stream>>>(ps.dZ.p, R, k, rpb, G + o.b3);
  sgemm<false, true>(c, R, H, k, ps.dZ.p, k, P + o.W3, k, ps.dH2.p, H, 0.f);
  dtanh_kernel<<<grid_for(c, (int64_t)R * H), 256, 0, c.stream>>>(ps.dH2.p, ps.H2.p, (int64_t)R * H);
  // layer 2
  sgemm<true, false>(c, H, H, R, ps.H1.p, H, ps.dH2.p, H, G + o.W2, H, 1.f);
  colsum_kernel<<<nblk, 256, 0, c.stream>>>(ps.dH2.p, R, H, rpb, G + o.b2);
  sgemm<false, true>(c, R, H, H, ps.dH2.p, H, P + o.W2, H, ps.dH1.p, H, 0.f);
  dtanh_kernel<<<grid_for(c, (int64_t)R * H), 256, 0, c.stream>>>(ps.dH1.p, ps.H1.p, (int64_t)R * H);
  // layer 1
  sgemm<true, false>(c, net.nin, H, R, ps.X.p, net.nin, ps.dH1.p, H, G + o.W1, H, 1.f);
  colsum_kernel<<<nblk, 256, 0, c.stream>>>(ps.dH1.p, R, H, rpb, G + o.b1);
  c.launches += 5;
}

// loss on one patch set; dZ into ps.dZ (scaled by `scale`); returns the sum of per-sample losses
double net_loss(Ctx& c, const PatchNet& net, NetPass& ps, const Patches& pt, const double* Ed, int S, double scale) {
  const int P = pt.npatch();
  DBuf<double> lp;
  lp.alloc(std::max(P, 1));
  proj_loss_kernel<<<P, 256, 0, c.stream>>>(ps.pptr.p, ps.rdof.p, ps.Z.p, net.k, Ed, S, 1e-6, scale, ps.dZ.p, lp.p);
  c.launches++;
  FEM2D_CUDA(cudaGetLastError());
  std::vector<double> h(P);
  FEM2D_CUDA(cudaMemcpyAsync(h.data(), lp.p, P * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
  FEM2D_CUDA(cudaStreamSynchronize(c.stream));
  double s = 0.0;
  for (double v : h) s += v;
  return s;
}

void check_net(const PatchNet& net) {
  if (net.k < 1 || net.k > kMaxK) fail(FEM2D_E_INVALID_ARG, "coarse vectors per Elem must be 1..32");
  if (net.hidden < 1 || net.hidden > 1024) fail(FEM2D_E_INVALID_ARG, "hidden width must be 1..1024");
  if ((int64_t)net.params.size() != net.size()) fail(FEM2D_E_INVALID_ARG, "parameter count mismatch");
}

}  // namespace

// ------------------------------------------------------------------ host side
void PatchNet::init(uint64_t seed) {
  params.assign(size(), 0.f);
  const NetOffsets o(*this);
  uint64_t s = seed * 0x9E3779B97F4A7C15ull + 12345;
  auto fill = [&](int64_t off, int fan_in, int fan_out) {
    const double lim = std::sqrt(6.0 / (fan_in + fan_out));
    for (int64_t t = 0; t < (int64_t)fan_in * fan_out; t++) {
      const double u = (splitmix(s) >> 11) * (1.0 / 9007199254740992.0);
      params[off + t] = (float)((2.0 * u - 1.0) * lim);
    }
  };
  fill(o.W1, nin, hidden);
  fill(o.W2, hidden, hidden);
  fill(o.W3, hidden, k);
}

void build_patches(const Domain& d, double shift, Patches& out) {
  const Mesh& m = d.mesh;
  out = Patches();
  out.ptr.push_back(0);
  double bx0 = 1e300, by0 = 1e300, bx1 = -1e300, by1 = -1e300;
  for (const auto& r : m.roots) {
    bx0 = std::min(bx0, std::min(r.x0, r.x3));
    bx1 = std::max(bx1, std::max(r.x0, r.x3));
    by0 = std::min(by0, std::min(r.y0, r.y3));
    by1 = std::max(by1, std::max(r.y0, r.y3));
  }
  const double W = std::max(bx1 - bx0, 1e-300), H = std::max(by1 - by0, 1e-300), L = std::max(W, H);
  std::vector<int> mult(d.ndofs, 0);
  for (const Spec& s : d.specs) mult[s.dof]++;
  for (int64_t e = 0; e < (int64_t)m.elems.size(); e++) {
    if (d.nspecs(e) == 0) continue;
    const MElem& el = m.elems[e];
    const auto pr = m.param_range(e);
    const RootElement& r = m.roots[el.root];
    auto mx = [&](double u) { return r.x0 + (u + 1.0) * 0.5 * (r.x3 - r.x0); };
    auto my = [&](double v) { return r.y0 + (v + 1.0) * 0.5 * (r.y3 - r.y0); };
    const double hu = std::fabs(mx(pr[1]) - mx(pr[0])), hv = std::fabs(my(pr[3]) - my(pr[2]));
    const double xc = 0.5 * (mx(pr[0]) + mx(pr[1])), yc = 0.5 * (my(pr[2]) + my(pr[3]));
    for (int64_t q = d.spec_ptr[e]; q < d.spec_ptr[e + 1]; q++) {
      const Spec& s = d.specs[q];
      float f[kPatchFeatures];
      f[0] = (float)s.dir;
      f[1] = s.i / 8.f;
      f[2] = s.j / 8.f;
      f[3] = s.i == 0;
      f[4] = s.i == 1;
      f[5] = s.j == 0;
      f[6] = s.j == 1;
      f[7] = el.ni / 8.f;
      f[8] = el.nj / 8.f;
      f[9] = (float)(std::log2(hu / L) / 4.0);
      f[10] = (float)(std::log2(hv / L) / 4.0);
      f[11] = (float)el.anc.size() / 4.f;
      f[12] = (float)((xc - bx0) / W);
      f[13] = (float)((yc - by0) / H);
      f[14] = (float)(std::log(std::max(shift * hu * hv, 1e-12)) / 8.0);
      f[15] = mult[s.dof] > 1 ? 1.f : 0.f;
      out.feat.insert(out.feat.end(), f, f + kPatchFeatures);
      out.dof.push_back(s.dof);
      out.weight.push_back(1.f / (float)mult[s.dof]);
    }
    out.ptr.push_back((int64_t)out.dof.size());
  }
  out.nrows = (int64_t)out.dof.size();
}

double patchnet_loss_grad(Ctx& c, const PatchNet& net, const Patches& pt, int64_t n, const double* E, int S,
                          std::vector<float>& grad) {
  check_net(net);
  if (S < 1 || S > kMaxSamples) fail(FEM2D_E_INVALID_ARG, "1..256 error samples per call");
  if ((int64_t)grad.size() != net.size()) grad.assign(net.size(), 0.f);
  DBuf<float> P, G;
  P.upload(net.params, c.stream);
  G.upload(grad, c.stream);
  DBuf<double> Ed;
  Ed.alloc((size_t)n * S);
  FEM2D_CUDA(cudaMemcpyAsync(Ed.p, E, (size_t)n * S * sizeof(double), cudaMemcpyHostToDevice, c.stream));
  NetPass ps;
  ps.setup(c, pt, net);
  net_forward(c, net, P.p, ps);
  const double scale = 1.0 / ((double)pt.npatch() * S);
  const double loss = net_loss(c, net, ps, pt, Ed.p, S, scale) * scale;
  net_backward(c, net, P.p, ps, G.p);
  FEM2D_CUDA(cudaMemcpyAsync(grad.data(), G.p, grad.size() * sizeof(float), cudaMemcpyDeviceToHost, c.stream));
  FEM2D_CUDA(cudaStreamSynchronize(c.stream));
  return loss;
}

std::vector<double> patchnet_train(Ctx& c, PatchNet& net, const std::vector<const Patches*>& pts,
                                   const std::vector<int64_t>& ns, const std::vector<const double*>& Es, int S,
                                   int epochs, double lr) {
  check_net(net);
  if (S < 1 || S > kMaxSamples) fail(FEM2D_E_INVALID_ARG, "1..256 error samples per GEP");
  const int ng = (int)pts.size();
  DBuf<float> P, G, M1, M2;
  P.upload(net.params, c.stream);
  G.alloc(net.size());
  M1.alloc(net.size());
  M2.alloc(net.size());
  FEM2D_CUDA(cudaMemsetAsync(M1.p, 0, net.size() * sizeof(float), c.stream));
  FEM2D_CUDA(cudaMemsetAsync(M2.p, 0, net.size() * sizeof(float), c.stream));
  std::vector<std::unique_ptr<NetPass>> passes(ng);
  std::vector<std::unique_ptr<DBuf<double>>> Ed(ng);
  for (int g = 0; g < ng; g++) {
    passes[g].reset(new NetPass);
    passes[g]->setup(c, *pts[g], net);
    Ed[g].reset(new DBuf<double>);
    Ed[g]->alloc((size_t)ns[g] * S);
    FEM2D_CUDA(cudaMemcpyAsync(Ed[g]->p, Es[g], (size_t)ns[g] * S * sizeof(double), cudaMemcpyHostToDevice,
                               c.stream));
  }
  std::vector<double> hist;
  const float b1 = 0.9f, b2 = 0.999f;
  for (int ep = 1; ep <= epochs; ep++) {
    FEM2D_CUDA(cudaMemsetAsync(G.p, 0, net.size() * sizeof(float), c.stream));
    double loss = 0.0;
    for (int g = 0; g < ng; g++) {
      NetPass& ps = *passes[g];
      net_forward(c, net, P.p, ps);
      const double scale = 1.0 / ((double)pts[g]->npatch() * S);
      loss += net_loss(c, net, ps, *pts[g], Ed[g]->p, S, scale) * scale;
      net_backward(c, net, P.p, ps, G.p);
    }
    hist.push_back(loss / ng);
    const float c1 = 1.f - std::pow(b1, (float)ep), c2 = 1.f - std::pow(b2, (float)ep);
    adam_kernel<<<grid_for(c, net.size()), 256, 0, c.stream>>>(net.size(), P.p, G.p, M1.p, M2.p, (float)lr, b1, b2,
                                                                1e-8f, c1, c2, 1.f / ng);
    c.launches++;
  }
  FEM2D_CUDA(cudaMemcpyAsync(net.params.data(), P.p, net.params.size() * sizeof(float), cudaMemcpyDeviceToHost,
                             c.stream));
  FEM2D_CUDA(cudaStreamSynchronize(c.stream));
  return hist;
}

// ------------------------------------------------------------------ PCG solver
struct PCGSolver::Impl {
  Ctx& c;
  const HostGEP& h;
  const DeviceGEP& d;
  double ca, cb;
  const double* va = nullptr;   // the pencil's A and B values (full CSR order)
  const double* vb = nullptr;
  int64_t n;
  Patches pt;
  // MINRES blocks (n x kNB), allocated on first use
  DBuf<double> Mv[3], Mw[3], Mz, Mz2, Maz;
  DBuf<int64_t> pptr, ioff;
  DBuf<int32_t> rdof;
  DBuf<double> inv;
  // coarse correction
  bool learned = false;
  int k = 0, m = 0;
  DBuf<float> Zw;
  DBuf<double> ycoarse, wcoarse;
  DBuf<float> KinvF, yF, wF;   // the coarse inverse and its operands in FP32 (a preconditioner needs no more)
  // CG blocks (n x kNB)
  DBuf<double> Rb, Zb, Pb, Qb, Xb, part, scal;
  double setup_ms = 0;

  Impl(Ctx& ctx, const HostGEP& hg, const DeviceGEP& dg, double a, double b) : c(ctx), h(hg), d(dg), ca(a), cb(b) {}

  void spmm(double ka, double kb, const double* X, double* Y, int nb) {
    gep_spmm_values(c, h, d, va, vb, ka, kb, X, kNB, nb, Y, kNB);
  }
  void upload_scalars(const std::vector<double>& v) {
    FEM2D_CUDA(cudaMemcpyAsync(scal.p, v.data(), std::min<size_t>(v.size(), 3 * kNB) * sizeof(double),
                               cudaMemcpyHostToDevice, c.stream));
  }
  // preconditioned CG on Rb (overwritten by the residual) into Xb (zeroed first); returns iterations
  int cg_block(int nb, double tol, int max_iter, double& rel, std::vector<double>* snaps, const double* xstar,
               int nrhs, int c0, int every, int max_snaps, int first);

  void precondition(const double* R, double* Zo, int nb, bool coarse = true) {
    FEM2D_CUDA(cudaMemsetAsync(Zo, 0, (size_t)n * kNB * sizeof(double), c.stream));
    const int P = pt.npatch();
    bj_apply_kernel<<<P, 256, 0, c.stream>>>(pptr.p, rdof.p, ioff.p, inv.p, R, nb, Zo);
    c.launches++;
    if (learned && coarse) {
      coarse_restrict_kernel<<<P, 128, 0, c.stream>>>(pptr.p, rdof.p, Zw.p, k, R, kNB, nb, ycoarse.p);
      // w = Kinv y as one FP32 tiled GEMM (m x m times m x nb)
      to_f32_kernel<<<grid_for(c, (int64_t)m * kNB), 256, 0, c.stream>>>((int64_t)m * kNB, ycoarse.p, yF.p);
      dim3 gg((nb + 63) / 64, (m + 63) / 64);
      sgemm_kernel<false, false><<<gg, 256, 0, c.stream>>>(m, nb, m, KinvF.p, m, yF.p, kNB, wF.p, kNB, 0.f);
      to_f64_kernel<<<grid_for(c, (int64_t)m * kNB), 256, 0, c.stream>>>((int64_t)m * kNB, wF.p, wcoarse.p);
      coarse_prolong_kernel<<<P, 128, 0, c.stream>>>(pptr.p, rdof.p, Zw.p, k, wcoarse.p, nb, Zo, kNB);
      c.launches += 5;
    }
  }

  // per-column dot products of two n x kNB blocks
  std::vector<double> dots(const double* X, const double* Y, int nb) {
    const int nblk = std::max(1, std::min<int>(c.num_sms * 2, (int)((n + 255) / 256)));
    const int64_t rpb = (n + nblk - 1) / nblk;
    coldot_kernel<<<nblk, 256, 0, c.stream>>>(n, nb, X, Y, rpb, part.p);
    c.launches++;
    std::vector<double> hp((size_t)nblk * kNB);
    FEM2D_CUDA(cudaMemcpyAsync(hp.data(), part.p, hp.size() * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    FEM2D_CUDA(cudaStreamSynchronize(c.stream));
    std::vector<double> out(nb, 0.0);
    for (int b = 0; b < nblk; b++)
      for (int j = 0; j < nb; j++) out[j] += hp[(size_t)b * kNB + j];
    return out;
  }
};

PCGSolver::PCGSolver(Ctx& c, const Domain& dom, const HostGEP& h, const DeviceGEP& d, double ca, double cb,
                     const PatchNet* net, const float* basis, int basis_k, const double* va, const double* vb)
    : p_(new Impl(c, h, d, ca, cb)) {
  auto t0 = std::chrono::steady_clock::now();
  Impl& I = *p_;
  I.n = h.n;
  I.va = va ? va : d.a.p;
  I.vb = vb ? vb : d.b.p;
  if (!(ca > 0.0) || !(cb > 0.0)) fail(FEM2D_E_INVALID_ARG, "PCG needs an SPD shift: c_a > 0 and c_b > 0");
  build_patches(dom, cb / ca, I.pt);
  const int P = I.pt.npatch();
  if (P == 0) fail(FEM2D_E_EMPTY_DOFS, "no Elem carries basis functions");
  std::vector<int64_t> ioff(P + 1, 0);
  std::vector<int32_t> sdof(I.pt.nrows), sloc(I.pt.nrows);
  for (int p = 0; p < P; p++) {
    const int64_t r0 = I.pt.ptr[p];
    const int np = (int)(I.pt.ptr[p + 1] - r0);
    if (np > kMaxPatch) fail(FEM2D_E_TOO_LARGE, "an Elem carries more than 160 basis functions");
    ioff[p + 1] = ioff[p] + (int64_t)np * np;
    std::vector<std::pair<int32_t, int32_t>> v(np);
    for (int i = 0; i < np; i++) v[i] = {I.pt.dof[r0 + i], i};
    std::sort(v.begin(), v.end());
    for (int i = 0; i < np; i++) {
      if (i > 0 && v[i].first == v[i - 1].first) fail(FEM2D_E_INVALID_ARG, "an Elem lists one DoF twice");
      sdof[r0 + i] = v[i].first;
      sloc[r0 + i] = v[i].second;
    }
  }
  I.pptr.upload(I.pt.ptr, c.stream);
  I.rdof.upload(I.pt.dof, c.stream);
  I.ioff.upload(ioff, c.stream);
  DBuf<int32_t> sd, sl;
  sd.upload(sdof, c.stream);
  sl.upload(sloc, c.stream);
  I.inv.alloc(std::max<int64_t>(ioff[P], 1));
  DBuf<int> flag;
  flag.alloc(1);
  FEM2D_CUDA(cudaMemsetAsync(flag.p, 0, sizeof(int), c.stream));
  static bool attr = false;
  if (!attr) {
    FEM2D_CUDA(cudaFuncSetAttribute(bj_invert_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    kMaxPatch * kMaxPatch * (int)sizeof(double)));
    attr = true;
  }
  int maxnp = 0;
  for (int p = 0; p < P; p++) maxnp = std::max<int>(maxnp, (int)(I.pt.ptr[p + 1] - I.pt.ptr[p]));
  bj_invert_kernel<<<P, 256, (size_t)maxnp * maxnp * sizeof(double), c.stream>>>(
      I.pptr.p, I.rdof.p, sd.p, sl.p, I.ioff.p, d.row_ptr.p, d.col.p, I.va, I.vb, ca, cb, I.inv.p, flag.p);
  c.launches++;
  FEM2D_CUDA(cudaGetLastError());
  int hf = 0;
  FEM2D_CUDA(cudaMemcpyAsync(&hf, flag.p, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
  FEM2D_CUDA(cudaStreamSynchronize(c.stream));
  if (hf) fail(FEM2D_E_B_NOT_SPD, "an Elem block of the shifted matrix is not positive definite");
  for (DBuf<double>* b : {&I.Rb, &I.Zb, &I.Pb, &I.Qb, &I.Xb}) b->alloc((size_t)I.n * kNB);
  I.part.alloc((size_t)c.num_sms * 2 * kNB + kNB);
  I.scal.alloc(3 * kNB);

  std::vector<float> Zh;
  if (net) {
    check_net(*net);
    I.k = net->k;
    // the network's coarse basis on this Domain
    DBuf<float> Pm;
    Pm.upload(net->params, c.stream);
    NetPass ps;
    ps.setup(c, I.pt, *net);
    net_forward(c, *net, Pm.p, ps);
    Zh.resize((size_t)I.pt.nrows * I.k);
    FEM2D_CUDA(cudaMemcpyAsync(Zh.data(), ps.Z.p, Zh.size() * sizeof(float), cudaMemcpyDeviceToHost, c.stream));
    FEM2D_CUDA(cudaStreamSynchronize(c.stream));
  } else if (basis) {
    if (basis_k < 1 || basis_k > kMaxK) fail(FEM2D_E_INVALID_ARG, "coarse vectors per Elem must be 1..32");
    I.k = basis_k;
    Zh.assign(basis, basis + (size_t)I.pt.nrows * I.k);
  }
  if (!Zh.empty()) {
    I.learned = true;
    I.m = P * I.k;
    if (I.m > 20480) fail(FEM2D_E_TOO_LARGE, "coarse space above 20480 vectors (dense coarse inverse)");
    // per Elem: weight rows by the partition of unity of shared functions, then orthonormalise the k
    // vectors (modified Gram-Schmidt, FP64); nearly dependent vectors are zeroed, not kept
    for (int p = 0; p < P; p++) {
      const int64_t r0 = I.pt.ptr[p];
      const int np = (int)(I.pt.ptr[p + 1] - r0);
      std::vector<double> Q((size_t)np * I.k);
      for (int i = 0; i < np; i++)
        for (int a = 0; a < I.k; a++) Q[(size_t)i * I.k + a] = (double)Zh[(size_t)(r0 + i) * I.k + a] * I.pt.weight[r0 + i];
      double scale0 = 0.0;
      for (int a = 0; a < I.k; a++) {
        double nrm0 = 0.0;
        for (int i = 0; i < np; i++) nrm0 += Q[(size_t)i * I.k + a] * Q[(size_t)i * I.k + a];
        scale0 = std::max(scale0, std::sqrt(nrm0));
        for (int pass = 0; pass < 2; pass++)
          for (int b = 0; b < a; b++) {
            double dt = 0.0;
            for (int i = 0; i < np; i++) dt += Q[(size_t)i * I.k + a] * Q[(size_t)i * I.k + b];
            for (int i = 0; i < np; i++) Q[(size_t)i * I.k + a] -= dt * Q[(size_t)i * I.k + b];
          }
        double nrm = 0.0;
        for (int i = 0; i < np; i++) nrm += Q[(size_t)i * I.k + a] * Q[(size_t)i * I.k + a];
        nrm = std::sqrt(nrm);
        const double inv = nrm > 1e-6 * std::max(scale0, 1e-300) ? 1.0 / nrm : 0.0;
        for (int i = 0; i < np; i++) Q[(size_t)i * I.k + a] *= inv;
      }
      for (int i = 0; i < np; i++)
        for (int a = 0; a < I.k; a++) Zh[(size_t)(r0 + i) * I.k + a] = (float)Q[(size_t)i * I.k + a];
    }
    I.Zw.upload(Zh, c.stream);
    // Kc = Zw^T K Zw, 32 coarse columns at a time (dense columns, SpMM, per-patch gram)
    DBuf<double> Kc, Zc, Yc;
    Kc.alloc((size_t)I.m * I.m);
    Zc.alloc((size_t)I.n * kNB);
    Yc.alloc((size_t)I.n * kNB);
    for (int j0 = 0; j0 < I.m; j0 += kNB) {
      const int w = std::min(kNB, I.m - j0);
      FEM2D_CUDA(cudaMemsetAsync(Zc.p, 0, (size_t)I.n * kNB * sizeof(double), c.stream));
      const int p0 = j0 / I.k, p1 = std::min(P, (j0 + w + I.k - 1) / I.k);
      coarse_columns_kernel<<<p1 - p0, 128, 0, c.stream>>>(I.pptr.p, I.rdof.p, I.Zw.p, I.k, j0, p0, p1, Zc.p);
      c.launches++;
      I.spmm(ca, cb, Zc.p, Yc.p, w);
      coarse_gram_kernel<<<P, 128, 0, c.stream>>>(I.pptr.p, I.rdof.p, I.Zw.p, I.k, Yc.p, w, j0, I.m, Kc.p);
      c.launches++;
    }
    // dense inverse of the SPD coarse operator by in-place Gauss-Jordan (no pivoting), after a tiny
    // diagonal shift that keeps Kc definite when the vectors of neighbouring Elems are nearly dependent
    {
      std::vector<double> Kh((size_t)I.m * I.m);
      FEM2D_CUDA(cudaMemcpyAsync(Kh.data(), Kc.p, Kh.size() * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
      FEM2D_CUDA(cudaStreamSynchronize(c.stream));
      double tr = 0.0;
      for (int64_t i = 0; i < I.m; i++) tr += Kh[i * I.m + i];
      const double eps = 1e-10 * tr / I.m;
      for (int64_t i = 0; i < I.m; i++) {
        Kh[i * I.m + i] += eps;
        if (!(Kh[i * I.m + i] > 0.0)) Kh[i * I.m + i] = tr / I.m;   // a zeroed (dependent) vector
      }
      FEM2D_CUDA(cudaMemcpyAsync(Kc.p, Kh.data(), Kh.size() * sizeof(double), cudaMemcpyHostToDevice, c.stream));
    }
    const int ggj = grid_for(c, (int64_t)I.m * I.m);
    for (int q = 0; q < I.m; q++) {
      gj_step_kernel<<<ggj, 256, 0, c.stream>>>(I.m, q, Kc.p);
      gj_finish_kernel<<<(I.m + 255) / 256, 256, 0, c.stream>>>(I.m, q, Kc.p);
      gj_pivot_kernel<<<1, 32, 0, c.stream>>>(I.m, q, Kc.p);
      c.launches += 3;
    }
    FEM2D_CUDA(cudaGetLastError());
    I.KinvF.alloc((size_t)I.m * I.m);
    to_f32_kernel<<<grid_for(c, (int64_t)I.m * I.m), 256, 0, c.stream>>>((int64_t)I.m * I.m, Kc.p, I.KinvF.p);
    c.launches++;
    I.ycoarse.alloc((size_t)I.m * kNB);
    I.wcoarse.alloc((size_t)I.m * kNB);
    I.yF.alloc((size_t)I.m * kNB);
    I.wF.alloc((size_t)I.m * kNB);
    FEM2D_CUDA(cudaMemsetAsync(I.ycoarse.p, 0, (size_t)I.m * kNB * sizeof(double), c.stream));
    FEM2D_CUDA(cudaStreamSynchronize(c.stream));
  }
  I.setup_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

PCGSolver::~PCGSolver() = default;
int PCGSolver::coarse_dim() const { return p_->m; }
double PCGSolver::setup_ms() const { return p_->setup_ms; }

int PCGSolver::Impl::cg_block(int nb, double tol, int max_iter, double& rel, std::vector<double>* snaps,
                               const double* xstar, int nrhs, int c0, int every, int max_snaps, int first) {
  FEM2D_CUDA(cudaMemsetAsync(Xb.p, 0, (size_t)n * kNB * sizeof(double), c.stream));
  const std::vector<double> bb = dots(Rb.p, Rb.p, nb);
  precondition(Rb.p, Zb.p, nb);
  FEM2D_CUDA(cudaMemcpyAsync(Pb.p, Zb.p, (size_t)n * kNB * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
  std::vector<double> rz = dots(Rb.p, Zb.p, nb), alpha(kNB, 0.0), beta(kNB, 0.0);
  std::vector<char> done(nb, 0);
  std::vector<double> hx;
  int it = 0;
  rel = 0.0;
  for (int j = 0; j < nb; j++)
    if (!(bb[j] > 0.0)) done[j] = 1;   // a zero right-hand side: x = 0
  for (; it < max_iter; it++) {
    bool any = false;
    for (int j = 0; j < nb; j++) any = any || !done[j];
    if (!any) break;
    spmm(ca, cb, Pb.p, Qb.p, nb);
    const std::vector<double> pq = dots(Pb.p, Qb.p, nb);
    for (int j = 0; j < nb; j++) alpha[j] = (done[j] || pq[j] <= 0.0) ? 0.0 : rz[j] / pq[j];
    upload_scalars(alpha);
    cg_update_kernel<<<grid_for(c, n * kNB), 256, 0, c.stream>>>(n, nb, scal.p, Pb.p, Qb.p, Xb.p, Rb.p);
    c.launches++;
    if (snaps && xstar && every > 0 && it + 1 >= first && (it + 1) % every == 0 &&
        (int64_t)snaps->size() < (int64_t)max_snaps * n) {
      hx.resize((size_t)n * kNB);
      FEM2D_CUDA(cudaMemcpyAsync(hx.data(), Xb.p, hx.size() * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
      FEM2D_CUDA(cudaStreamSynchronize(c.stream));
      for (int j = 0; j < nb && (int64_t)snaps->size() < (int64_t)max_snaps * n; j++) {
        if (done[j]) continue;
        for (int64_t i = 0; i < n; i++) snaps->push_back(xstar[(size_t)i * nrhs + c0 + j] - hx[(size_t)i * kNB + j]);
      }
    }
    const std::vector<double> rr = dots(Rb.p, Rb.p, nb);
    rel = 0.0;
    bool all = true;
    for (int j = 0; j < nb; j++) {
      const double rj = bb[j] > 0.0 ? std::sqrt(rr[j] / bb[j]) : 0.0;
      if (rj <= tol) done[j] = 1;
      all = all && done[j];
      rel = std::max(rel, rj);
    }
    if (all) {
      it++;
      break;
    }
    precondition(Rb.p, Zb.p, nb);
    const std::vector<double> rz2 = dots(Rb.p, Zb.p, nb);
    for (int j = 0; j < nb; j++) {
      beta[j] = (done[j] || rz[j] == 0.0) ? 0.0 : rz2[j] / rz[j];
      rz[j] = rz2[j];
    }
    upload_scalars(beta);
    cg_direction_kernel<<<grid_for(c, n * kNB), 256, 0, c.stream>>>(n, nb, scal.p, Zb.p, Pb.p);
    c.launches++;
  }
  return it;
}

void PCGSolver::solve(int nrhs, const double* rhs, double* x, double tol, int max_iter, PCGStats* st,
                      std::vector<double>* snaps, const double* xstar, int every, int max_snaps, int first) {
  Impl& I = *p_;
  Ctx& c = I.c;
  const int64_t n = I.n;
  auto t0 = std::chrono::steady_clock::now();
  int total_iters = 0;
  double worst = 0.0;
  std::vector<double> hb((size_t)n * kNB), hx((size_t)n * kNB);
  for (int c0 = 0; c0 < nrhs; c0 += kNB) {
    const int nb = std::min(kNB, nrhs - c0);
    std::fill(hb.begin(), hb.end(), 0.0);
    for (int64_t i = 0; i < n; i++)
      for (int j = 0; j < nb; j++) hb[(size_t)i * kNB + j] = rhs[(size_t)i * nrhs + c0 + j];
    FEM2D_CUDA(cudaMemcpyAsync(I.Rb.p, hb.data(), hb.size() * sizeof(double), cudaMemcpyHostToDevice, c.stream));
    double rel = 0.0;
    const int it = I.cg_block(nb, tol, max_iter, rel, snaps, xstar, nrhs, c0, every, max_snaps, first);
    total_iters = std::max(total_iters, it);
    worst = std::max(worst, rel);
    FEM2D_CUDA(cudaMemcpyAsync(hx.data(), I.Xb.p, hx.size() * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    FEM2D_CUDA(cudaStreamSynchronize(c.stream));
    for (int64_t i = 0; i < n; i++)
      for (int j = 0; j < nb; j++) x[(size_t)i * nrhs + c0 + j] = hx[(size_t)i * kNB + j];
  }
  if (st) {
    st->iters = total_iters;
    st->relres = worst;
    st->ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    st->setup_ms = I.setup_ms;
    st->coarse_dim = I.m;
  }
}

void PCGSolver::cg_device(const double* R, int64_t ldr, double* X, int64_t ldx, int nb, double tol, int max_iter,
                          PCGStats* st) {
  Impl& I = *p_;
  Ctx& c = I.c;
  if (nb < 1 || nb > kNB) fail(FEM2D_E_INVALID_ARG, "cg_device: 1..32 right-hand sides");
  auto t0 = std::chrono::steady_clock::now();
  FEM2D_CUDA(cudaMemsetAsync(I.Rb.p, 0, (size_t)I.n * kNB * sizeof(double), c.stream));
  strided_copy_kernel<<<grid_for(c, I.n * nb), 256, 0, c.stream>>>(I.n, nb, R, ldr, I.Rb.p, kNB);
  c.launches++;
  double rel = 0.0;
  const int it = I.cg_block(nb, tol, max_iter, rel, nullptr, nullptr, 0, 0, 0, 0, 0);
  strided_copy_kernel<<<grid_for(c, I.n * nb), 256, 0, c.stream>>>(I.n, nb, I.Xb.p, kNB, X, ldx);
  c.launches++;
  if (st) {
    st->iters = it;
    st->relres = rel;
    st->ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    st->setup_ms = I.setup_ms;
    st->coarse_dim = I.m;
  }
}

// Preconditioned MINRES (the recurrence of Elman, Silvester and Wathen, "Finite Elements and Fast
// Iterative Solvers", Algorithm 6.1) per column, with this solver's SPD preconditioner; the stopping
// test is on the preconditioned residual norm |eta| <= tol gamma_1.
void PCGSolver::minres_device(double ka, double kb, const double* R, int64_t ldr, double* X, int64_t ldx, int nb,
                              double tol, int max_iter, PCGStats* st, bool coarse) {
  Impl& I = *p_;
  Ctx& c = I.c;
  const int64_t n = I.n;
  if (nb < 1 || nb > kNB) fail(FEM2D_E_INVALID_ARG, "minres_device: 1..32 right-hand sides");
  auto t0 = std::chrono::steady_clock::now();
  for (DBuf<double>* b : {&I.Mv[0], &I.Mv[1], &I.Mv[2], &I.Mw[0], &I.Mw[1], &I.Mw[2], &I.Mz, &I.Mz2, &I.Maz})
    if (b->n != (size_t)n * kNB) b->alloc((size_t)n * kNB);
  const size_t bytes = (size_t)n * kNB * sizeof(double);
  double *v0 = I.Mv[0].p, *v1 = I.Mv[1].p, *v2 = I.Mv[2].p;
  double *w0 = I.Mw[0].p, *w1 = I.Mw[1].p, *w2 = I.Mw[2].p;
  double *z = I.Mz.p, *z2 = I.Mz2.p, *az = I.Maz.p;
  for (double* p : {v0, v1, w0, w1, I.Xb.p}) FEM2D_CUDA(cudaMemsetAsync(p, 0, bytes, c.stream));
  strided_copy_kernel<<<grid_for(c, n * nb), 256, 0, c.stream>>>(n, nb, R, ldr, v1, kNB);   // x0 = 0: v1 = b
  c.launches++;
  I.precondition(v1, z, nb, coarse);
  std::vector<double> g(nb), gprev(nb, 1.0), eta(nb), eta0(nb), cc0(nb, 1.0), cc1(nb, 1.0), ss0(nb, 0.0),
      ss1(nb, 0.0);
  std::vector<char> done(nb, 0);
  {
    const std::vector<double> zv = I.dots(z, v1, nb);
    for (int j = 0; j < nb; j++) {
      g[j] = zv[j] > 0.0 ? std::sqrt(zv[j]) : 0.0;
      eta[j] = eta0[j] = g[j];
      if (!(g[j] > 0.0)) done[j] = 1;
    }
  }
  std::vector<double> sc(3 * kNB, 0.0);
  int it = 0;
  double rel = 0.0;
  for (; it < max_iter; it++) {
    bool any = false;
    for (int j = 0; j < nb; j++) any = any || !done[j];
    if (!any) break;
    // z_j = z_j / gamma_j
    // a finished column gets zero coefficients everywhere: its vectors become and stay exactly zero
    // (frozen recurrences would otherwise grow without bound, and 0 * inf poisons x)
    std::fill(sc.begin(), sc.end(), 0.0);
    for (int j = 0; j < nb; j++) sc[j] = (!done[j] && g[j] > 0.0) ? 1.0 / g[j] : 0.0;
    I.upload_scalars(sc);
    lincomb3_kernel<<<grid_for(c, n * kNB), 256, 0, c.stream>>>(n, nb, I.scal.p, z, nullptr, nullptr, z);
    c.launches++;
    I.spmm(ka, kb, z, az, nb);
    const std::vector<double> delta = I.dots(az, z, nb);
    // v2 = az - (delta / gamma) v1 - (gamma / gamma_prev) v0
    for (int j = 0; j < nb; j++) {
      sc[j] = done[j] ? 0.0 : 1.0;
      sc[kNB + j] = (!done[j] && g[j] > 0.0) ? -delta[j] / g[j] : 0.0;
      sc[2 * kNB + j] = (!done[j] && gprev[j] > 0.0) ? -g[j] / gprev[j] : 0.0;
    }
    I.upload_scalars(sc);
    lincomb3_kernel<<<grid_for(c, n * kNB), 256, 0, c.stream>>>(n, nb, I.scal.p, az, v1, v0, v2);
    c.launches++;
    I.precondition(v2, z2, nb, coarse);
    const std::vector<double> zv = I.dots(z2, v2, nb);
    std::vector<double> a1(nb), a2(nb), a3(nb), cnew(nb), snew(nb), gnew(nb);
    for (int j = 0; j < nb; j++) {
      gnew[j] = zv[j] > 0.0 ? std::sqrt(zv[j]) : 0.0;
      const double al0 = cc1[j] * delta[j] - cc0[j] * ss1[j] * g[j];
      const double al1 = std::sqrt(al0 * al0 + gnew[j] * gnew[j]);
      a2[j] = ss1[j] * delta[j] + cc0[j] * cc1[j] * g[j];
      a3[j] = ss0[j] * g[j];
      a1[j] = al1;
      cnew[j] = al1 > 0.0 ? al0 / al1 : 1.0;
      snew[j] = al1 > 0.0 ? gnew[j] / al1 : 0.0;
    }
    // w2 = (z - a3 w0 - a2 w1) / a1
    for (int j = 0; j < nb; j++) {
      const double inv = (a1[j] > 0.0 && !done[j]) ? 1.0 / a1[j] : 0.0;
      sc[j] = inv;
      sc[kNB + j] = -a3[j] * inv;
      sc[2 * kNB + j] = -a2[j] * inv;
    }
    I.upload_scalars(sc);
    lincomb3_kernel<<<grid_for(c, n * kNB), 256, 0, c.stream>>>(n, nb, I.scal.p, z, w0, w1, w2);
    c.launches++;
    // x += c_new eta w2
    std::vector<double> step(kNB, 0.0);
    for (int j = 0; j < nb; j++) step[j] = done[j] ? 0.0 : cnew[j] * eta[j];
    I.upload_scalars(step);
    axpy_cols_kernel<<<grid_for(c, n * kNB), 256, 0, c.stream>>>(n, nb, I.scal.p, w2, I.Xb.p);
    c.launches++;
    rel = 0.0;
    for (int j = 0; j < nb; j++) {
      if (done[j]) continue;
      eta[j] = -snew[j] * eta[j];
      const double r = std::fabs(eta[j]) / eta0[j];
      if (r <= tol || !(gnew[j] > 0.0)) done[j] = 1;
      rel = std::max(rel, r);
      ss0[j] = ss1[j];
      ss1[j] = snew[j];
      cc0[j] = cc1[j];
      cc1[j] = cnew[j];
      gprev[j] = g[j];
      g[j] = gnew[j];
    }
    // rotate: v0 <- v1 <- v2, w0 <- w1 <- w2, z <- z2
    std::swap(v0, v1);
    std::swap(v1, v2);
    std::swap(w0, w1);
    std::swap(w1, w2);
    std::swap(z, z2);
  }
  strided_copy_kernel<<<grid_for(c, n * nb), 256, 0, c.stream>>>(n, nb, I.Xb.p, kNB, X, ldx);
  c.launches++;
  if (st) {
    st->iters = it;
    st->relres = rel;
    st->ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    st->setup_ms = I.setup_ms;
    st->coarse_dim = I.m;
  }
}

}  // namespace fem2d
