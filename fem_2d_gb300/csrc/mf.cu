// Numeric multifrontal factorization and block solves on the device (plan: mf.h, mf_symbolic.cpp).
//
// Fronts are dense, column-major, processed level by level (all fronts of a level in one launch per
// step). Per level: assemble from the CSR values of c_a*A + c_b*B, extend-add the children's Schur
// complements (one launch per child slot, so no two threads add to one entry), then a blocked
// right-looking LU of the first p columns with partial pivoting restricted to the fully-summed rows
// (or no pivoting in Cholesky mode for SPD shifts): panel (one CTA per front), unit-lower TRSM for
// the U12 rows, FP64 GEMM update of the trailing block. The trailing (f-p)x(f-p) block left in place
// is the update matrix for the parent.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cstring>
#include <mutex>

namespace cg = cooperative_groups;

#include "mfdev.h"

namespace fem2d {

namespace {

constexpr int PANEL = 32;

constexpr int MAXKIDS = 4;   // binary dissection nodes; Elem nodes have 2 (U/V) or 4 (T) children

struct FrontDesc {   // device copy of the per-front scalars
  int32_t f, p, parent;
  int32_t kid[MAXKIDS];
  int64_t off, dptr, aptr, aend, eptr;
  int64_t prow;   // tiled fronts: offset of the front's f + 1 pull-list row pointers
  int64_t aux;    // tiled fronts with p > kSmallP: offset of the p x p scratch copy of the LU square
};

__global__ void mf_assemble_kernel(const int32_t* __restrict__ lf, const FrontDesc* __restrict__ fd,
                                   const int64_t* __restrict__ apos, const int64_t* __restrict__ acsr,
                                   const double* __restrict__ va, const double* __restrict__ vb, double ca, double cb,
                                   double* __restrict__ F) {
  const FrontDesc d = fd[lf[blockIdx.y]];
  for (int64_t k = d.aptr + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < d.aend;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = acsr[k];
    F[d.off + apos[k]] = ca * va[c] + cb * vb[c];
  }
}

// add the child's trailing block (rows/cols >= p_child) into the parent at mapped positions
__global__ void mf_extend_add_kernel(const int32_t* __restrict__ lf, const FrontDesc* __restrict__ fd, int slot,
                                     const int32_t* __restrict__ emap, double* __restrict__ F) {
  const FrontDesc par = fd[lf[blockIdx.y]];
  const int32_t ch = par.kid[slot];
  if (ch < 0) return;
  const FrontDesc c = fd[ch];
  const int s = c.f - c.p;
  const int64_t total = (int64_t)s * s;
  const int32_t* m = emap + c.eptr;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t % s), j = (int)(t / s);   // child (row p+i, col p+j), column-major
    const double v = F[c.off + (int64_t)(c.p + j) * c.f + (c.p + i)];
    F[par.off + (int64_t)m[j] * par.f + m[i]] += v;
  }
}

// columns k0 .. k0+w-1 of every front with p > k0: pivot, swap full rows, scale, update the panel
// A column whose largest fully-summed entry is below kWeakPivot times its largest entry in the rows of
// the front's other (not yet summed) DoFs has no stable pivot here: its DoF is recorded, and the solver
// moves its elimination to the parent front and refactors (delayed pivoting).
constexpr double kWeakPivot = 1e-3;

__global__ void __launch_bounds__(256) mf_panel_kernel(const int32_t* __restrict__ lf,
                                                       const FrontDesc* __restrict__ fd, int k0, int pivoting,
                                                       double* __restrict__ F, int32_t* __restrict__ piv,
                                                       const int64_t* __restrict__ piv_off, int* __restrict__ flags,
                                                       const int32_t* __restrict__ dofs,
                                                       int32_t* __restrict__ weak, int* __restrict__ nweak,
                                                       int weak_cap) {
  const int fr = lf[blockIdx.x];
  const FrontDesc d = fd[fr];
  if (d.p <= k0) return;
  const int w = min(PANEL, d.p - k0);
  const int f = d.f;
  double* A = F + d.off;
  __shared__ double sval[256];
  __shared__ int sidx[256];
  __shared__ int s_piv;
  __shared__ double s_d;
  for (int k = k0; k < k0 + w; k++) {
    double* colk = A + (int64_t)k * f;
    int best = k;
    if (pivoting) {
      double bv = -1.0;
      int bi = k;
      for (int i = k + threadIdx.x; i < d.p; i += blockDim.x) {
        const double a = fabs(colk[i]);
        if (a > bv) { bv = a; bi = i; }
      }
      sval[threadIdx.x] = bv;
      sidx[threadIdx.x] = bi;
      __syncthreads();
      for (int st = blockDim.x / 2; st > 0; st >>= 1) {
        if (threadIdx.x < st) {
          const double o = sval[threadIdx.x + st];
          const int oi = sidx[threadIdx.x + st];
          if (o > sval[threadIdx.x] || (o == sval[threadIdx.x] && oi < sidx[threadIdx.x])) {
            sval[threadIdx.x] = o;
            sidx[threadIdx.x] = oi;
          }
        }
        __syncthreads();
      }
      best = sidx[0];
      const double fully = sval[0];
      __syncthreads();
      // largest entry of column k in the rows of the not-yet-summed DoFs
      double sm = 0.0;
      for (int i = d.p + threadIdx.x; i < f; i += blockDim.x) sm = fmax(sm, fabs(colk[i]));
      sval[threadIdx.x] = sm;
      __syncthreads();
      for (int st = blockDim.x / 2; st > 0; st >>= 1) {
        if (threadIdx.x < st) sval[threadIdx.x] = fmax(sval[threadIdx.x], sval[threadIdx.x + st]);
        __syncthreads();
      }
      if (threadIdx.x == 0 && fully < kWeakPivot * sval[0] && d.parent >= 0) {
        const int slot = atomicAdd(nweak, 1);
        if (slot < weak_cap) weak[slot] = dofs[d.dptr + k];
      }
    }
    if (threadIdx.x == 0) {
      s_piv = best;
      piv[piv_off[fr] + k] = best;
    }
    __syncthreads();
    const int pr = s_piv;
    if (pr != k)
      for (int j = threadIdx.x; j < f; j += blockDim.x) {
        const double t = A[(int64_t)j * f + k];
        A[(int64_t)j * f + k] = A[(int64_t)j * f + pr];
        A[(int64_t)j * f + pr] = t;
      }
    __syncthreads();
    if (threadIdx.x == 0) {
      double dk = colk[k];
      if (!(fabs(dk) > 0.0) || (!pivoting && !(dk > 0.0))) {
        atomicOr(flags, pivoting ? 1 : 2);   // 1: zero pivot (perturbed), 2: not positive definite
        dk = dk == 0.0 ? 1e-300 : dk;
        colk[k] = dk;
      }
      s_d = 1.0 / dk;
    }
    __syncthreads();
    const double inv = s_d;
    for (int i = k + 1 + threadIdx.x; i < f; i += blockDim.x) colk[i] *= inv;
    __syncthreads();
    // rank-1 update of the remaining panel columns
    const int ncols = k0 + w - (k + 1);
    const int nrows = f - (k + 1);
    for (int64_t t = threadIdx.x; t < (int64_t)ncols * nrows; t += blockDim.x) {
      const int jj = k + 1 + (int)(t / nrows);
      const int ii = k + 1 + (int)(t % nrows);
      A[(int64_t)jj * f + ii] -= colk[ii] * A[(int64_t)jj * f + k];
    }
    __syncthreads();
  }
}

// U12 = L11^-1 A12 for rows k0..k0+w-1 and columns k0+w..f-1 (unit lower L11)
__global__ void __launch_bounds__(128) mf_trsm_kernel(const int32_t* __restrict__ lf, const FrontDesc* __restrict__ fd,
                                                      int k0, double* __restrict__ F) {
  const FrontDesc d = fd[lf[blockIdx.y]];
  if (d.p <= k0) return;
  const int w = min(PANEL, d.p - k0);
  const int f = d.f;
  const int j = k0 + w + blockIdx.x * blockDim.x + threadIdx.x;
  __shared__ double L[PANEL][PANEL + 1];
  double* A = F + d.off;
  if (k0 + w + blockIdx.x * blockDim.x >= f) return;
  for (int t = threadIdx.x; t < w * w; t += blockDim.x) {
    const int r = t % w, c = t / w;
    L[r][c] = A[(int64_t)(k0 + c) * f + (k0 + r)];
  }
  __syncthreads();
  if (j >= f) return;
  double x[PANEL];
  double* col = A + (int64_t)j * f + k0;
#pragma unroll
  for (int r = 0; r < PANEL; r++)
    if (r < w) x[r] = col[r];
#pragma unroll
  for (int r = 0; r < PANEL; r++) {
    if (r >= w) break;
    double s = x[r];
#pragma unroll
    for (int c = 0; c < PANEL; c++)
      if (c < r) s -= L[r][c] * x[c];
    x[r] = s;
  }
#pragma unroll
  for (int r = 0; r < PANEL; r++)
    if (r < w) col[r] = x[r];
}

// trailing update: A22 -= L21 * U12, rows/cols k0+w .. f-1; 64x64 tile per CTA, K = w
__global__ void __launch_bounds__(256) mf_gemm_kernel(const int32_t* __restrict__ lf, const FrontDesc* __restrict__ fd,
                                                      int k0, double* __restrict__ F) {
  const FrontDesc d = fd[lf[blockIdx.z]];
  if (d.p <= k0) return;
  const int w = min(PANEL, d.p - k0);
  const int f = d.f;
  const int base = k0 + w;
  const int r0 = base + blockIdx.x * 64, c0 = base + blockIdx.y * 64;
  if (r0 >= f || c0 >= f) return;
  double* A = F + d.off;
  __shared__ double Ls[PANEL][64];
  __shared__ double Us[PANEL][64 + 1];
  for (int t = threadIdx.x; t < PANEL * 64; t += blockDim.x) {
    const int r = t % 64, c = t / 64;
    Ls[c][r] = (c < w && r0 + r < f) ? A[(int64_t)(k0 + c) * f + r0 + r] : 0.0;
    const int uc = t / PANEL, ur = t % PANEL;   // U tile: PANEL rows x 64 cols, coalesced along rows
    Us[ur][uc] = (ur < w && c0 + uc < f) ? A[(int64_t)(c0 + uc) * f + k0 + ur] : 0.0;
  }
  __syncthreads();
  const int tr = threadIdx.x % 16, tc = threadIdx.x / 16;
  double acc[4][4] = {};
  for (int t = 0; t < w; t++) {
    double a[4], b[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
      a[q] = Ls[t][tr + 16 * q];
      b[q] = Us[t][tc + 16 * q];
    }
#pragma unroll
    for (int q = 0; q < 4; q++)
#pragma unroll
      for (int s = 0; s < 4; s++) acc[q][s] += a[q] * b[s];
  }
#pragma unroll
  for (int s = 0; s < 4; s++) {
    const int c = c0 + tc + 16 * s;
    if (c >= f) continue;
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const int r = r0 + tr + 16 * q;
      if (r < f) A[(int64_t)c * f + r] -= acc[q][s];
    }
  }
}

// ------------------------------------------------------------------ cluster block solves
// One 8-CTA thread-block cluster per front. Rows are owned in interleaved 32-row chunks
// (chunk q belongs to CTA q % 8). The triangular factors are walked in 32-column blocks: every CTA
// solves the 32 x nb diagonal block itself (from the rows finalised before the last cluster barrier),
// then updates the rows it owns; cluster.sync() separates the blocks. The solved block is written
// back after the barrier, when no CTA reads those rows any more.
constexpr int CL = 8;

// sequential LAPACK-style row swaps -> gather permutation (v'[i] = v[perm[i]])
__global__ void mf_perm_kernel(int nf, const FrontDesc* __restrict__ fd, const int32_t* __restrict__ piv,
                               const int64_t* __restrict__ piv_off, int32_t* __restrict__ perm,
                               int32_t* __restrict__ iperm) {
  const int fr = blockIdx.x * blockDim.x + threadIdx.x;
  if (fr >= nf) return;
  const int p = fd[fr].p;
  const int32_t* pv = piv + piv_off[fr];
  int32_t* pm = perm + piv_off[fr];
  for (int i = 0; i < p; i++) pm[i] = i;
  for (int k = 0; k < p; k++) {
    const int r = pv[k];
    const int32_t t = pm[k];
    pm[k] = pm[r];
    pm[r] = t;
  }
  int32_t* ip = iperm + piv_off[fr];
  for (int i = 0; i < p; i++) ip[pm[i]] = i;
}

__global__ void __cluster_dims__(CL, 1, 1) __launch_bounds__(256)
    mf_forward_cluster_kernel(const int32_t* __restrict__ lf, const FrontDesc* __restrict__ fd,
                              const int32_t* __restrict__ dofs, const int32_t* __restrict__ emap,
                              const int32_t* __restrict__ perm, const int32_t* __restrict__ iperm,
                              const int64_t* __restrict__ piv_off,
                              const int64_t* __restrict__ woff, const double* __restrict__ F,
                              const double* __restrict__ B, int64_t ldb, int nb, double* __restrict__ W) {
  cg::cluster_group cluster = cg::this_cluster();
  const int r = (int)cluster.block_rank();
  const int fr = lf[blockIdx.x / CL];
  const FrontDesc d = fd[fr];
  const int f = d.f, p = d.p;
  double* v = W + woff[fr];
  const int32_t* D = dofs + d.dptr;
  const int32_t* pm = perm + piv_off[fr];
  const int32_t* ipm = iperm + piv_off[fr];
  const int nchunk = (f + 31) / 32;
  for (int q = r; q < nchunk; q += CL)
    for (int t = threadIdx.x; t < 32 * nb; t += blockDim.x) {
      const int i = q * 32 + (t & 31), c = t >> 5;
      if (i < f) v[(int64_t)c * f + i] = i < p ? B[(int64_t)D[pm[i]] * ldb + c] : 0.0;
    }
  __syncthreads();
  for (int slot = 0; slot < MAXKIDS; slot++) {
    const int ch = d.kid[slot];
    if (ch < 0) continue;
    const FrontDesc cd = fd[ch];
    const int s = cd.f - cd.p;
    const double* cw = W + woff[ch];
    const int32_t* m = emap + cd.eptr;
    for (int t = threadIdx.x; t < s * nb; t += blockDim.x) {
      const int i = t % s, c = t / s;
      const int row = m[i] < p ? ipm[m[i]] : m[i];   // pivot rows are stored permuted
      if (((row >> 5) % CL) == r) v[(int64_t)c * f + row] += cw[(int64_t)c * cd.f + cd.p + i];
    }
    __syncthreads();
  }
  cluster.sync();
  __shared__ double ys[32][33];
  __shared__ double Ld[32][33];
  for (int jb = 0; jb < p; jb += 32) {
    const int bw = min(32, p - jb);
    for (int t = threadIdx.x; t < 32 * nb; t += blockDim.x) {
      const int u = t & 31, c = t >> 5;
      ys[u][c] = u < bw ? v[(int64_t)c * f + jb + u] : 0.0;
    }
    for (int t = threadIdx.x; t < 32 * 32; t += blockDim.x) {
      const int u = t & 31, k = t >> 5;   // row jb+u, col jb+k
      Ld[u][k] = (u < bw && k < bw) ? F[d.off + (int64_t)(jb + k) * f + jb + u] : 0.0;
    }
    __syncthreads();
    if (threadIdx.x < nb) {
      const int c = threadIdx.x;
      for (int u = 0; u < bw; u++) {
        double s = ys[u][c];
        for (int k = 0; k < u; k++) s -= Ld[u][k] * ys[k][c];
        ys[u][c] = s;
      }
    }
    __syncthreads();
    // update owned rows below the block
    const int first = jb + bw;
    for (int q = r; q < nchunk; q += CL) {
      if (q * 32 + 31 < first) continue;
      for (int t = threadIdx.x; t < 32 * nb; t += blockDim.x) {
        const int i = q * 32 + (t & 31), c = t >> 5;
        if (i < first || i >= f) continue;
        double acc = 0.0;
        for (int u = 0; u < bw; u++) acc += F[d.off + (int64_t)(jb + u) * f + i] * ys[u][c];
        v[(int64_t)c * f + i] -= acc;
      }
    }
    cluster.sync();
    // the owner stores the solved block (rows jb.. are read by nobody after the barrier)
    if (((jb >> 5) % CL) == r)
      for (int t = threadIdx.x; t < 32 * nb; t += blockDim.x) {
        const int u = t & 31, c = t >> 5;
        if (u < bw) v[(int64_t)c * f + jb + u] = ys[u][c];
      }
    __syncthreads();
  }
}

__global__ void __cluster_dims__(CL, 1, 1) __launch_bounds__(256)
    mf_backward_cluster_kernel(const int32_t* __restrict__ lf, const FrontDesc* __restrict__ fd,
                               const int32_t* __restrict__ dofs, const int64_t* __restrict__ woff,
                               const double* __restrict__ F, double* __restrict__ W, int nb, double* __restrict__ X,
                               int64_t ldx) {
  cg::cluster_group cluster = cg::this_cluster();
  const int r = (int)cluster.block_rank();
  const int fr = lf[blockIdx.x / CL];
  const FrontDesc d = fd[fr];
  const int f = d.f, p = d.p;
  if (p == 0) return;   // uniform across the cluster
  double* v = W + woff[fr];
  const int32_t* D = dofs + d.dptr;
  const int nchunk = (p + 31) / 32;
  // y -= U12 x_struct on owned rows
  for (int q = r; q < nchunk; q += CL)
    for (int t = threadIdx.x; t < 32 * nb; t += blockDim.x) {
      const int i = q * 32 + (t & 31), c = t >> 5;
      if (i >= p) continue;
      double s = v[(int64_t)c * f + i];
      for (int j = p; j < f; j++) s -= F[d.off + (int64_t)j * f + i] * X[(int64_t)D[j] * ldx + c];
      v[(int64_t)c * f + i] = s;
    }
  cluster.sync();
  __shared__ double xs[32][33];
  __shared__ double Ud[32][33];
  const int last = ((p - 1) / 32) * 32;
  for (int jb = last; jb >= 0; jb -= 32) {
    const int bw = min(32, p - jb);
    for (int t = threadIdx.x; t < 32 * nb; t += blockDim.x) {
      const int u = t & 31, c = t >> 5;
      xs[u][c] = u < bw ? v[(int64_t)c * f + jb + u] : 0.0;
    }
    for (int t = threadIdx.x; t < 32 * 32; t += blockDim.x) {
      const int u = t & 31, k = t >> 5;
      Ud[u][k] = (u < bw && k < bw) ? F[d.off + (int64_t)(jb + k) * f + jb + u] : 0.0;
    }
    __syncthreads();
    if (threadIdx.x < nb) {
      const int c = threadIdx.x;
      for (int u = bw - 1; u >= 0; u--) {
        double s = xs[u][c];
        for (int k = u + 1; k < bw; k++) s -= Ud[u][k] * xs[k][c];
        xs[u][c] = s / Ud[u][u];
      }
    }
    __syncthreads();
    for (int q = r; q * 32 < jb; q += CL)
      for (int t = threadIdx.x; t < 32 * nb; t += blockDim.x) {
        const int i = q * 32 + (t & 31), c = t >> 5;
        if (i >= jb) continue;
        double acc = 0.0;
        for (int u = 0; u < bw; u++) acc += F[d.off + (int64_t)(jb + u) * f + i] * xs[u][c];
        v[(int64_t)c * f + i] -= acc;
      }
    if (((jb >> 5) % CL) == r)
      for (int t = threadIdx.x; t < 32 * nb; t += blockDim.x) {
        const int u = t & 31, c = t >> 5;
        if (u < bw) X[(int64_t)D[jb + u] * ldx + c] = xs[u][c];
      }
    cluster.sync();
  }
}


// ------------------------------------------------------------------ small-front solves
// Fronts with p <= kSmallP and f <= kSmallF (every front of an Elem-level elimination tree at the
// orders this library meets in practice) are solved by one CTA each, with no sequential triangular
// substitution: after the factorization, mf_invdiag_kernel overwrites each such front's p x p
// diagonal LU square by (unit lower L11^-1, upper U11^-1), so both solve directions become dense,
// fully parallel products:
//   forward:  y = L11^-1 P b_p,  b_s -= L21 y          (b_s goes to the parent)
//   backward: x_p = U11^-1 (y - U12 x_s)
constexpr int kSmallP = 160;
constexpr int kSmallF = 512;

// column j of L11^-1 and of U11^-1 per thread, from a shared-memory copy of the LU square
__global__ void __launch_bounds__(256) mf_invdiag_kernel(const int32_t* __restrict__ lf,
                                                         const FrontDesc* __restrict__ fd, double* __restrict__ F) {
  const FrontDesc d = fd[lf[blockIdx.x]];
  const int f = d.f, p = d.p;
  extern __shared__ double S[];   // S[k * p + i] = LU(i, k)
  double* A = F + d.off;
  for (int t = threadIdx.x; t < p * p; t += blockDim.x) {
    const int i = t % p, k = t / p;
    S[t] = A[(int64_t)k * f + i];
  }
  __syncthreads();
  for (int j = threadIdx.x; j < p; j += blockDim.x) {
    double* out = A + (int64_t)j * f;   // column j; only this thread writes it
    // L11 x = e_j (unit diagonal): x_j = 1, x_i = -sum_{k=j}^{i-1} L(i,k) x_k
    for (int i = j + 1; i < p; i++) {
      double acc = -S[j * p + i];
      for (int k = j + 1; k < i; k++) acc -= S[k * p + i] * out[k];
      out[i] = acc;
    }
    // U11 y = e_j: y_j = 1 / U(j,j), y_i = -(sum_{k=i+1}^{j} U(i,k) y_k) / U(i,i)
    out[j] = 1.0 / S[j * p + j];
    for (int i = j - 1; i >= 0; i--) {
      double acc = 0.0;
      for (int k = i + 1; k <= j; k++) acc += S[k * p + i] * out[k];
      out[i] = -acc / S[i * p + i];
    }
  }
}

// sum_{k = k0}^{k1 - 1} A[k * f] * v[k] with four independent accumulators (eight loads in flight per
// thread): the solve loops are latency-bound on the factor reads, not FP64-bound
__device__ __forceinline__ double col_dot(const double* __restrict__ A, int f, const double* __restrict__ v, int k0,
                                          int k1) {
  double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
  int k = k0;
#pragma unroll 2
  for (; k + 4 <= k1; k += 4) {
    a0 += A[(int64_t)k * f] * v[k];
    a1 += A[(int64_t)(k + 1) * f] * v[k + 1];
    a2 += A[(int64_t)(k + 2) * f] * v[k + 2];
    a3 += A[(int64_t)(k + 3) * f] * v[k + 3];
  }
  for (; k < k1; k++) a0 += A[(int64_t)k * f] * v[k];
  return (a0 + a1) + (a2 + a3);
}

struct SolveArgs {
  const FrontDesc* fd;
  const int32_t *dofs, *emap, *perm, *iperm;
  const int64_t *piv_off, *woff;
  const double* F;
  const double* B;
  int64_t ldb;
  double* W;
  double* X;
  int64_t ldx;
  int nb;
};

// the front's gathered right-hand side v[c * f + i] (pivot rows permuted): the pivot rows' entries of
// B, then each child's update vector added in slot order (rows are distinct within one child, so no
// atomics are needed, and the fixed order makes the sums, and the whole solve, reproducible bit for bit)
__device__ __forceinline__ void gather_front_rhs(const FrontDesc& d, const FrontDesc* __restrict__ fd,
                                                 const int32_t* __restrict__ emap, const int32_t* __restrict__ ipm,
                                                 const double* __restrict__ W, const int64_t* __restrict__ woff,
                                                 const double* __restrict__ B, int64_t ldb,
                                                 const int32_t* __restrict__ D, const int32_t* __restrict__ pm, int nb,
                                                 double* v) {
  const int f = d.f, p = d.p;
  for (int t = threadIdx.x; t < f * nb; t += blockDim.x) {
    const int i = t % f, c = t / f;
    v[t] = i < p ? B[(int64_t)D[pm[i]] * ldb + c] : 0.0;
  }
  for (int slot = 0; slot < MAXKIDS; slot++) {
    const int ch = d.kid[slot];
    if (ch < 0) continue;   // uniform across the CTA
    const FrontDesc cd = fd[ch];
    const int sz = cd.f - cd.p;
    const double* cw = W + woff[ch];
    const int32_t* m = emap + cd.eptr;
    __syncthreads();
    for (int t = threadIdx.x; t < sz * nb; t += blockDim.x) {
      const int i = t % sz, c = t / sz;
      const int mi = m[i];
      const int row = mi < p ? ipm[mi] : mi;   // pivot rows are stored permuted
      v[c * f + row] += cw[(int64_t)c * cd.f + cd.p + i];
    }
  }
  __syncthreads();
}

// forward solve of one small front by the calling CTA (sm: (f + p) * nb doubles)
__device__ __forceinline__ void forward_small_front(int fr, const SolveArgs& a, double* sm) {
  const FrontDesc* __restrict__ fd = a.fd;
  const int32_t* __restrict__ dofs = a.dofs;
  const int32_t* __restrict__ emap = a.emap;
  const int32_t* __restrict__ perm = a.perm;
  const int32_t* __restrict__ iperm = a.iperm;
  const int64_t* __restrict__ piv_off = a.piv_off;
  const int64_t* __restrict__ woff = a.woff;
  const double* __restrict__ F = a.F;
  const double* __restrict__ B = a.B;
  const int64_t ldb = a.ldb;
  const int nb = a.nb;
  double* __restrict__ W = a.W;
  const FrontDesc d = fd[fr];
  const int f = d.f, p = d.p;
  double* v = sm;            // v[c * f + i]
  double* y = sm + f * nb;   // y[c * p + i]
  const int32_t* D = dofs + d.dptr;
  const int32_t* pm = perm + piv_off[fr];
  const int32_t* ipm = iperm + piv_off[fr];
  const double* A = F + d.off;
  gather_front_rhs(d, fd, emap, ipm, W, woff, B, ldb, D, pm, nb, v);
  // the unit lower triangle: row i is a dot product of length i, so a thread takes the rows q and
  // p - 1 - q (p - 1 terms together) and the lanes of a warp run equally long
  const int hp = (p + 1) >> 1;
  for (int t = threadIdx.x; t < hp * nb; t += blockDim.x) {
    const int q = t % hp, c = t / hp;
    const double* vc = v + c * f;
    y[c * p + q] = vc[q] + col_dot(A + q, f, vc, 0, q);
    const int i2 = p - 1 - q;
    if (i2 != q) y[c * p + i2] = vc[i2] + col_dot(A + i2, f, vc, 0, i2);
  }
  __syncthreads();
  double* out = W + woff[fr];
  const int s = f - p;
  for (int t = threadIdx.x; t < s * nb; t += blockDim.x) {
    const int i = p + t % s, c = t / s;
    const double* yc = y + c * p;
    out[(int64_t)c * f + i] = v[c * f + i] - col_dot(A + i, f, yc, 0, p);
  }
  for (int t = threadIdx.x; t < p * nb; t += blockDim.x) {
    const int i = t % p, c = t / p;
    out[(int64_t)c * f + i] = y[c * p + i];
  }
}

// NT threads per front: 256 for wide levels, 1024 for the narrow upper levels of the tree, where a
// few fronts occupy the GPU and each front's dependent dot products set the level's latency
template <int NT>
__global__ void __launch_bounds__(NT) mf_forward_small_kernel(const int32_t* __restrict__ lf, SolveArgs a) {
  extern __shared__ double sm[];
  forward_small_front(lf[blockIdx.x], a, sm);
}

// backward solve of one small front by the calling CTA (sm: f * nb doubles)
__device__ __forceinline__ void backward_small_front(int fr, const SolveArgs& a, double* sm) {
  const FrontDesc* __restrict__ fd = a.fd;
  const int32_t* __restrict__ dofs = a.dofs;
  const int64_t* __restrict__ woff = a.woff;
  const double* __restrict__ F = a.F;
  const double* __restrict__ W = a.W;
  const int nb = a.nb;
  double* __restrict__ X = a.X;
  const int64_t ldx = a.ldx;
  const FrontDesc d = fd[fr];
  const int f = d.f, p = d.p;
  if (p == 0) return;
  const int s = f - p;
  double* xs = sm;            // xs[c * s + j]: solved struct unknowns
  double* z = sm + s * nb;    // z[c * p + i]
  const int32_t* D = dofs + d.dptr;
  const double* A = F + d.off;
  const double* v = W + woff[fr];
  for (int t = threadIdx.x; t < s * nb; t += blockDim.x) {
    const int j = t % s, c = t / s;
    xs[t] = X[(int64_t)D[p + j] * ldx + c];
  }
  __syncthreads();
  for (int t = threadIdx.x; t < p * nb; t += blockDim.x) {
    const int i = t % p, c = t / p;
    const double* xc = xs + c * s;
    z[c * p + i] = v[(int64_t)c * f + i] - col_dot(A + (int64_t)p * f + i, f, xc, 0, s);
  }
  __syncthreads();
  // the upper triangle: row i is a dot product of length p - i; rows q and p - 1 - q share a thread
  const int hp = (p + 1) >> 1;
  for (int t = threadIdx.x; t < hp * nb; t += blockDim.x) {
    const int q = t % hp, c = t / hp;
    const double* zc = z + c * p;
    X[(int64_t)D[q] * ldx + c] = col_dot(A + q, f, zc, q, p);
    const int i2 = p - 1 - q;
    if (i2 != q) X[(int64_t)D[i2] * ldx + c] = col_dot(A + i2, f, zc, i2, p);
  }
}

template <int NT>
__global__ void __launch_bounds__(NT) mf_backward_small_kernel(const int32_t* __restrict__ lf, SolveArgs a) {
  extern __shared__ double sm[];
  backward_small_front(lf[blockIdx.x], a, sm);
}

// The narrow upper levels of the tree hold a few fronts each, and GB300's FP64 rate per SM (about two
// FMA per clock) makes one CTA per front the bottleneck there: these variants spread one front over a
// cluster of CL CTAs (CL SMs). Every CTA gathers the front's right-hand side (cheap) and owns a
// contiguous slice of its rows; the block that all rows need (y of the forward pass, z of the backward
// pass) is exchanged through the front's workspace in global memory across one cluster barrier (cluster
// scope orders the global writes before the reads).
__device__ __forceinline__ void row_slice(int rows, int r, int& r0, int& r1) {
  const int per = (rows + CL - 1) / CL;
  r0 = min(rows, r * per);
  r1 = min(rows, r0 + per);
}

__global__ void __cluster_dims__(CL, 1, 1) __launch_bounds__(256)
    mf_forward_small_cluster_kernel(const int32_t* __restrict__ lf, SolveArgs a) {
  extern __shared__ double sm[];
  cg::cluster_group cluster = cg::this_cluster();
  const int r = (int)cluster.block_rank();
  const int fr = lf[blockIdx.x / CL];
  const FrontDesc* __restrict__ fd = a.fd;
  const int32_t* __restrict__ emap = a.emap;
  const int32_t* __restrict__ ipm = a.iperm + a.piv_off[fr];
  const int32_t* __restrict__ pm = a.perm + a.piv_off[fr];
  const int nb = a.nb;
  const FrontDesc d = fd[fr];
  const int f = d.f, p = d.p, s = f - p;
  double* v = sm;            // v[c * f + i]: the whole gathered right-hand side
  double* y = sm + f * nb;   // y[c * p + i]: the whole pivot block after the exchange
  const int32_t* D = a.dofs + d.dptr;
  const double* A = a.F + d.off;
  double* out = a.W + a.woff[fr];
  gather_front_rhs(d, fd, emap, ipm, a.W, a.woff, a.B, a.ldb, D, pm, nb, v);
  // y = L11^-1 v[0:p] for this CTA's slice of pivot rows, straight into the workspace
  int r0, r1;
  row_slice(p, r, r0, r1);
  const int pr = r1 - r0;
  for (int t = threadIdx.x; t < pr * nb; t += blockDim.x) {
    const int i = r0 + t % pr, c = t / pr;
    const double* vc = v + c * f;
    out[(int64_t)c * f + i] = vc[i] + col_dot(A + i, f, vc, 0, i);
  }
  cluster.sync();
  for (int t = threadIdx.x; t < p * nb; t += blockDim.x) {
    const int i = t % p, c = t / p;
    y[c * p + i] = out[(int64_t)c * f + i];
  }
  __syncthreads();
  // out[p:f] = v[p:f] - L21 y for this CTA's slice of the remaining rows
  row_slice(s, r, r0, r1);
  const int sr = r1 - r0;
  for (int t = threadIdx.x; t < sr * nb; t += blockDim.x) {
    const int i = p + r0 + t % sr, c = t / sr;
    const double* yc = y + c * p;
    out[(int64_t)c * f + i] = v[c * f + i] - col_dot(A + i, f, yc, 0, p);
  }
}

__global__ void __cluster_dims__(CL, 1, 1) __launch_bounds__(256)
    mf_backward_small_cluster_kernel(const int32_t* __restrict__ lf, SolveArgs a) {
  extern __shared__ double sm[];
  cg::cluster_group cluster = cg::this_cluster();
  const int r = (int)cluster.block_rank();
  const int fr = lf[blockIdx.x / CL];
  const int nb = a.nb;
  const FrontDesc d = a.fd[fr];
  const int f = d.f, p = d.p;
  if (p == 0) return;   // uniform over the cluster: every CTA of it leaves before any barrier
  const int s = f - p;
  double* xs = sm;            // xs[c * s + j]: solved struct unknowns
  double* z = sm + s * nb;    // z[c * p + i]: the whole pivot block after the exchange
  const int32_t* D = a.dofs + d.dptr;
  const double* A = a.F + d.off;
  double* v = a.W + a.woff[fr];
  for (int t = threadIdx.x; t < s * nb; t += blockDim.x) {
    const int j = t % s, c = t / s;
    xs[t] = a.X[(int64_t)D[p + j] * a.ldx + c];
  }
  __syncthreads();
  // z = y - U12 xs for this CTA's slice of pivot rows, in place over y in the workspace (each row is
  // read and written by its owner only before the barrier)
  int r0, r1;
  row_slice(p, r, r0, r1);
  const int pr = r1 - r0;
  for (int t = threadIdx.x; t < pr * nb; t += blockDim.x) {
    const int i = r0 + t % pr, c = t / pr;
    const double* xc = xs + c * s;
    v[(int64_t)c * f + i] = v[(int64_t)c * f + i] - col_dot(A + (int64_t)p * f + i, f, xc, 0, s);
  }
  cluster.sync();
  for (int t = threadIdx.x; t < p * nb; t += blockDim.x) {
    const int i = t % p, c = t / p;
    z[c * p + i] = v[(int64_t)c * f + i];
  }
  __syncthreads();
  // x = U11^-1 z for the same slice
  for (int t = threadIdx.x; t < pr * nb; t += blockDim.x) {
    const int i = r0 + t % pr, c = t / pr;
    const double* zc = z + c * p;
    a.X[(int64_t)D[i] * a.ldx + c] = col_dot(A + i, f, zc, i, p);
  }
}

// ------------------------------------------------------------------ tiled solves (partitioned inverse)
// The narrow upper levels of the tree hold a few fronts each, some far too large for one CTA, and
// GB300's FP64 rate per SM (under two FMA per clock) makes any solve confined to a few SMs the
// bottleneck. After the factorization, every front of such a level is turned into its partitioned
// inverse:
//   diagonal square: unit lower L11^-1 and upper U11^-1      (mf_invdiag_kernel / _wide_kernel)
//   L21 -> L21' = -L21 L11^-1,  U12 -> U12' = -U11^-1 U12    (mf_partinv_kernel)
// so that each solve direction is one dense product with no dependency between rows:
//   forward:  out[r] = v[r] + sum_{k < min(r, p)} F(r, k) v[k]            every row r < f
//   backward: x[r]   = sum_{k = r}^{f - 1} F(r, k) z[k],  z = [y; x_s]    every pivot row r < p
// (v: the gathered right-hand side in pivot order; out[0:p] = y, out[p:f] the update for the parent).
// A level's rows are cut into tiles of kTileRows (one warp per row, lane c owns right-hand side c),
// so a level of a few large fronts spreads over hundreds of CTAs. v is pulled without atomics from
// the B rows and the children's update vectors through a per-front source list, chunk by chunk, into
// shared memory by every CTA of the front.
constexpr int kTileRows = 8;
constexpr int kChunkK = 128;
constexpr int kTiledMaxP = 768;   // the wide inversion keeps one column per thread in shared memory

struct TiledArgs {
  const FrontDesc* fd;
  const int32_t* dofs;
  const int32_t* perm;
  const int64_t* piv_off;
  const int64_t* woff;
  const int64_t* prow;      // per tiled front (at FrontDesc::prow): f + 1 offsets into the sources
  const int64_t* src_off;   // source: W[src_off + c * src_str] (a child's update row)
  const int32_t* src_str;
  const double* F;
  const double* B;
  int64_t ldb;
  double* W;
  double* X;
  int64_t ldx;
  int nb;
};

// row k (pivot order) of front d's gathered right-hand side, column c
__device__ __forceinline__ double pull_row(const TiledArgs& a, const FrontDesc& d, const int32_t* D, const int32_t* pm,
                                           int k, int c) {
  const int u = k < d.p ? pm[k] : k;
  double s = k < d.p ? a.B[(int64_t)D[u] * a.ldb + c] : 0.0;
  const int64_t* pr = a.prow + d.prow;
  const int64_t q1 = pr[u + 1];
  for (int64_t q = pr[u]; q < q1; q++) s += a.W[a.src_off[q] + (int64_t)c * a.src_str[q]];
  return s;
}

// items: (front, first row) pairs
__global__ void __launch_bounds__(256) mf_forward_tiled_kernel(const int2* __restrict__ items, TiledArgs a) {
  __shared__ double vs[kChunkK * 33];   // vs[kk * 33 + c]: row k0 + kk of v
  const int2 it = items[blockIdx.x];
  const FrontDesc d = a.fd[it.x];
  const int f = d.f, p = d.p, nb = a.nb;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int r = it.y + warp;
  const bool live = r < f && lane < nb;
  const int32_t* D = a.dofs + d.dptr;
  const int32_t* pm = a.perm + a.piv_off[it.x];
  const double* Ar = a.F + d.off + r;
  const int kend = min(p, it.y + kTileRows);   // rows r < p need k < r, rows r >= p need k < p
  const int klim = min(r, p);
  double acc0 = 0.0, acc1 = 0.0;
  for (int k0 = 0; k0 < kend; k0 += kChunkK) {
    const int kc = min(kChunkK, kend - k0);
    __syncthreads();
    for (int t = threadIdx.x; t < kc * nb; t += blockDim.x) {
      const int kk = t % kc, c = t / kc;
      vs[kk * 33 + c] = pull_row(a, d, D, pm, k0 + kk, c);
    }
    __syncthreads();
    if (live) {
      const int k1 = min(k0 + kc, klim);
      int k = k0;
      for (; k + 2 <= k1; k += 2) {
        acc0 += Ar[(int64_t)k * f] * vs[(k - k0) * 33 + lane];
        acc1 += Ar[(int64_t)(k + 1) * f] * vs[(k + 1 - k0) * 33 + lane];
      }
      if (k < k1) acc0 += Ar[(int64_t)k * f] * vs[(k - k0) * 33 + lane];
    }
  }
  if (live) a.W[a.woff[it.x] + (int64_t)lane * f + r] = pull_row(a, d, D, pm, r, lane) + (acc0 + acc1);
}

__global__ void __launch_bounds__(256) mf_backward_tiled_kernel(const int2* __restrict__ items, TiledArgs a) {
  __shared__ double zs[kChunkK * 33];   // zs[kk * 33 + c]: row k0 + kk of z = [y; x_s]
  const int2 it = items[blockIdx.x];
  const FrontDesc d = a.fd[it.x];
  const int f = d.f, p = d.p, nb = a.nb;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int r = it.y + warp;
  const bool live = r < p && lane < nb;
  const int32_t* D = a.dofs + d.dptr;
  const double* Ar = a.F + d.off + r;
  const double* y = a.W + a.woff[it.x];
  double acc0 = 0.0, acc1 = 0.0;
  for (int k0 = it.y; k0 < f; k0 += kChunkK) {
    const int kc = min(kChunkK, f - k0);
    __syncthreads();
    for (int t = threadIdx.x; t < kc * nb; t += blockDim.x) {
      const int kk = t % kc, c = t / kc, k = k0 + kk;
      zs[kk * 33 + c] = k < p ? y[(int64_t)c * f + k] : a.X[(int64_t)D[k] * a.ldx + c];
    }
    __syncthreads();
    if (live) {
      const int k1 = k0 + kc;
      int k = max(k0, r);
      for (; k + 2 <= k1; k += 2) {
        acc0 += Ar[(int64_t)k * f] * zs[(k - k0) * 33 + lane];
        acc1 += Ar[(int64_t)(k + 1) * f] * zs[(k + 1 - k0) * 33 + lane];
      }
      if (k < k1) acc0 += Ar[(int64_t)k * f] * zs[(k - k0) * 33 + lane];
    }
  }
  if (live) a.X[(int64_t)D[r] * a.ldx + lane] = acc0 + acc1;
}

// the p x p LU square of each listed front, copied (column-major) to scratch at FrontDesc::aux
__global__ void mf_square_copy_kernel(const int32_t* __restrict__ lf, const FrontDesc* __restrict__ fd,
                                      const double* __restrict__ F, double* __restrict__ S) {
  const FrontDesc d = fd[lf[blockIdx.y]];
  const int64_t pp = (int64_t)d.p * d.p;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < pp; t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t % d.p), k = (int)(t / d.p);
    S[d.aux + t] = F[d.off + (int64_t)k * d.f + i];
  }
}

// columns j0 .. j0 + 31 of (L11^-1, U11^-1) of a front with p > kSmallP, one thread per column, from
// the scratch copy of its LU square; the column being built stays in shared memory (o[i * 32])
__global__ void __launch_bounds__(32) mf_invdiag_wide_kernel(const int2* __restrict__ items,
                                                             const FrontDesc* __restrict__ fd,
                                                             const double* __restrict__ S, double* __restrict__ F) {
  extern __shared__ double ob[];
  const int2 it = items[blockIdx.x];
  const FrontDesc d = fd[it.x];
  const int p = d.p, f = d.f;
  const int lane = threadIdx.x, j = it.y + lane;
  if (j >= p) return;
  const double* Sp = S + d.aux;   // Sp[k * p + i] = LU(i, k)
  double* o = ob + lane;
  // L11 x = e_j (unit diagonal): x_i = -L(i, j) - sum_{k = j+1}^{i-1} L(i, k) x_k for i > j
  for (int i = j + 1; i < p; i++) {
    double a0 = -Sp[(int64_t)j * p + i], a1 = 0.0;
    int k = j + 1;
    for (; k + 2 <= i; k += 2) {
      a0 -= Sp[(int64_t)k * p + i] * o[k * 32];
      a1 -= Sp[(int64_t)(k + 1) * p + i] * o[(k + 1) * 32];
    }
    if (k < i) a0 -= Sp[(int64_t)k * p + i] * o[k * 32];
    o[i * 32] = a0 + a1;
  }
  // U11 y = e_j: y_j = 1 / U(j, j), y_i = -(sum_{k = i+1}^{j} U(i, k) y_k) / U(i, i) for i < j
  o[j * 32] = 1.0 / Sp[(int64_t)j * p + j];
  for (int i = j - 1; i >= 0; i--) {
    double a0 = 0.0, a1 = 0.0;
    int k = i + 1;
    for (; k + 2 <= j + 1; k += 2) {
      a0 += Sp[(int64_t)k * p + i] * o[k * 32];
      a1 += Sp[(int64_t)(k + 1) * p + i] * o[(k + 1) * 32];
    }
    if (k <= j) a0 += Sp[(int64_t)k * p + i] * o[k * 32];
    o[i * 32] = -(a0 + a1) / Sp[(int64_t)i * p + i];
  }
  double* out = F + d.off + (int64_t)j * f;
  for (int i = 0; i < p; i++) out[i] = o[i * 32];
}

// L21' = -L21 L11^-1 (kind 0: rows t0 .. t0 + 7 of L21) and U12' = -U11^-1 U12 (kind 1: columns
// t0 .. t0 + 7 of U12), one warp per row / column, from the inverted diagonal square; items are
// (front, kind, t0, 0). Each warp reads only the square and writes only its own row / column.
__global__ void __launch_bounds__(256) mf_partinv_kernel(const int4* __restrict__ items,
                                                         const FrontDesc* __restrict__ fd, double* __restrict__ F) {
  extern __shared__ double pb[];   // kTileRows x p: the warp's original row / column
  const int4 it = items[blockIdx.x];
  const FrontDesc d = fd[it.x];
  const int f = d.f, p = d.p;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int q = p + it.z + warp;   // row (kind 0) or column (kind 1) of the front
  double* A = F + d.off;
  double* b = pb + (size_t)warp * p;
  if (q >= f) return;   // no block-wide barrier below
  if (it.y == 0) {
    for (int i = lane; i < p; i += 32) b[i] = A[(int64_t)i * f + q];
    __syncwarp();
    for (int k = 0; k < p; k++) {
      double s = 0.0;
      for (int i = k + 1 + lane; i < p; i += 32) s += b[i] * A[(int64_t)k * f + i];
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
      if (lane == 0) A[(int64_t)k * f + q] = -(b[k] + s);
    }
  } else {
    for (int k = lane; k < p; k += 32) b[k] = A[(int64_t)q * f + k];
    __syncwarp();
    for (int i = lane; i < p; i += 32) {
      double s0 = 0.0, s1 = 0.0;
      int k = i;
      for (; k + 2 <= p; k += 2) {
        s0 += A[(int64_t)k * f + i] * b[k];
        s1 += A[(int64_t)(k + 1) * f + i] * b[k + 1];
      }
      if (k < p) s0 += A[(int64_t)k * f + i] * b[k];
      A[(int64_t)q * f + i] = -(s0 + s1);
    }
  }
}

// X = Kinv B for a dense inverse (n x n, row-major): one warp per row, lane c owns right-hand side c;
// four accumulators keep the inverse-row and B-row loads in flight
__global__ void __launch_bounds__(256) dense_inverse_apply_kernel(int64_t n, const double* __restrict__ Kinv,
                                                                  const double* __restrict__ B, int64_t ldb, int nb,
                                                                  double* __restrict__ X, int64_t ldx) {
  const int lane = threadIdx.x & 31;
  for (int64_t i = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; i < n;
       i += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const double* row = Kinv + i * n;
    const bool live = lane < nb;
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
    int64_t j = 0;
    for (; j + 4 <= n; j += 4) {
      if (live) {
        s0 += row[j] * B[j * ldb + lane];
        s1 += row[j + 1] * B[(j + 1) * ldb + lane];
        s2 += row[j + 2] * B[(j + 2) * ldb + lane];
        s3 += row[j + 3] * B[(j + 3) * ldb + lane];
      }
    }
    for (; j < n; j++)
      if (live) s0 += row[j] * B[j * ldb + lane];
    if (live) X[i * ldx + lane] = (s0 + s1) + (s2 + s3);
  }
}

// Gauss-Jordan inversion of a dense n x n matrix in place (n <= 4096), one pivot per step:
//   gjp_pivot_kernel   (1 CTA)  partial pivoting: the largest |M[i][q]|, i >= q, row q <-> row p, recorded
//   gjp_update_kernel           M[i][j] -= M[i][q] M[q][j] / M[q][q] for i, j != q
//   gjp_finish_kernel           column q and row q scaled, then (one thread, next launch) the pivot inverted
// and after the last step the row interchanges are undone as column interchanges in reverse order.
// Without pivoting (SPD shifts) a non-positive pivot sets flag 2; a zero pivot sets flag 1 and is
// perturbed.
__global__ void __launch_bounds__(1024) gjp_pivot_kernel(int n, int q, int pivoting, double* __restrict__ M,
                                                         int32_t* __restrict__ piv, int* __restrict__ flags) {
  __shared__ double bv[1024];
  __shared__ int bi[1024];
  double best = -1.0;
  int bidx = q;
  if (pivoting)
    for (int i = q + threadIdx.x; i < n; i += blockDim.x) {
      const double a = fabs(M[(int64_t)i * n + q]);
      if (a > best) { best = a; bidx = i; }
    }
  bv[threadIdx.x] = best;
  bi[threadIdx.x] = bidx;
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st) {
      const double o = bv[threadIdx.x + st];
      const int oi = bi[threadIdx.x + st];
      if (o > bv[threadIdx.x] || (o == bv[threadIdx.x] && oi < bi[threadIdx.x])) {
        bv[threadIdx.x] = o;
        bi[threadIdx.x] = oi;
      }
    }
    __syncthreads();
  }
  const int p = pivoting ? bi[0] : q;
  if (threadIdx.x == 0) piv[q] = p;
  if (p != q)
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
      const double t = M[(int64_t)q * n + j];
      M[(int64_t)q * n + j] = M[(int64_t)p * n + j];
      M[(int64_t)p * n + j] = t;
    }
  __syncthreads();
  if (threadIdx.x == 0) {
    const double d = M[(int64_t)q * n + q];
    if (!(fabs(d) > 0.0) || (!pivoting && !(d > 0.0))) {
      atomicOr(flags, pivoting ? 1 : 2);
      if (d == 0.0) M[(int64_t)q * n + q] = 1e-300;
    }
  }
}

__global__ void gjp_update_kernel(int n, int q, double* __restrict__ M) {
  const double inv = 1.0 / M[(int64_t)q * n + q];
  const int64_t total = (int64_t)n * n;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t / n), j = (int)(t % n);
    if (i == q || j == q) continue;
    M[t] -= M[(int64_t)i * n + q] * inv * M[(int64_t)q * n + j];
  }
}

__global__ void gjp_finish_kernel(int n, int q, double* __restrict__ M) {
  const double inv = 1.0 / M[(int64_t)q * n + q];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    if (i != q) {
      M[(int64_t)i * n + q] = -M[(int64_t)i * n + q] * inv;
      M[(int64_t)q * n + i] = M[(int64_t)q * n + i] * inv;
    }
}

__global__ void gjp_recip_kernel(int n, int q, double* __restrict__ M) {
  if (blockIdx.x == 0 && threadIdx.x == 0) M[(int64_t)q * n + q] = 1.0 / M[(int64_t)q * n + q];
}

// undo the row interchanges as column interchanges, last pivot first; one thread per row
__global__ void gjp_unscramble_kernel(int n, const int32_t* __restrict__ piv, double* __restrict__ M) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double* row = M + (int64_t)i * n;
    for (int k = n - 1; k >= 0; k--) {
      const int p = piv[k];
      if (p != k) {
        const double t = row[k];
        row[k] = row[p];
        row[p] = t;
      }
    }
  }
}

}  // namespace

void MFDevice::setup(Ctx& c, const MFSymbolic& s, int nb_max) {
  cudaStream_t st = c.stream;
  nf = s.nfronts;
  nlevels = s.nlevels;
  level_ptr = s.level_ptr;
  max_f = s.max_f;
  max_p = s.max_p;
  nb_cap = nb_max;
  factor_flops = s.flops;
  // fronts laid out level by level so each level's storage is contiguous
  std::vector<int64_t> off(nf, 0), poff(nf, 0), woff_h(nf, 0);
  std::vector<std::array<int32_t, MAXKIDS>> kids(nf);
  for (auto& k : kids) k.fill(-1);
  std::vector<int> nk(nf, 0);
  for (int f = 0; f < nf; f++) {
    int pa = s.parent[f];
    if (pa >= 0) {
      if (nk[pa] >= MAXKIDS) fail(FEM2D_E_INVALID_ARG, "elimination tree node with more than 4 children");
      kids[pa][nk[pa]++] = f;
    }
  }
  int64_t o = 0, po = 0, wo = 0;
  level_off.assign(nlevels + 1, 0);
  for (int l = 0; l < nlevels; l++) {
    level_off[l] = o;
    for (int k = s.level_ptr[l]; k < s.level_ptr[l + 1]; k++) {
      int f = s.level_fronts[k];
      off[f] = o;
      o += (int64_t)s.f[f] * s.f[f];
      poff[f] = po;
      po += s.p[f];
      woff_h[f] = wo;
      wo += (int64_t)s.f[f] * nb_max;
    }
  }
  level_off[nlevels] = o;
  mat_total = o;
  std::vector<FrontDesc> fdh(nf);
  for (int f = 0; f < nf; f++) {
    FrontDesc& x = fdh[f];
    x.f = s.f[f];
    x.p = s.p[f];
    x.parent = s.parent[f];
    for (int k = 0; k < MAXKIDS; k++) x.kid[k] = kids[f][k];
    x.off = off[f];
    x.dptr = s.dof_ptr[f];
    x.aptr = s.asm_ptr[f];
    x.aend = s.asm_ptr[f + 1];
    x.eptr = s.ea_ptr[f];
  }
  for (FrontDesc& x : fdh) x.prow = x.aux = 0;
  // Tiled levels: the narrow upper levels (at most 2 * num_sms / CL small fronts, or any front too
  // large for one CTA) whose fronts all have p <= kTiledMaxP. Their fronts get pull lists (for each
  // front row, the children's update rows that add into it) and factor-time work items.
  level_tiled.assign(nlevels, 0);
  tf_ptr.assign(nlevels + 1, 0);
  tb_ptr.assign(nlevels + 1, 0);
  std::vector<int32_t> tf_h, tb_h, mid_h, wide_h, wi_h, pi_h, sstr_h;
  std::vector<int64_t> prow_h, soff_h;
  nmid = nwide = npinv = 0;
  max_mid_p = max_wide_p = max_tiled_p = 0;
  int64_t sq_total = 0;
  const bool single_dense = nf == 1 && max_p == max_f && max_f <= 4096;   // factor() inverts it whole
  for (int l = 0; l < nlevels; l++) {
    tf_ptr[l] = (int32_t)(tf_h.size() / 2);
    tb_ptr[l] = (int32_t)(tb_h.size() / 2);
    int ns = 0, nl = 0;
    bool fits = true;
    for (int k = s.level_ptr[l]; k < s.level_ptr[l + 1]; k++) {
      const int fr = s.level_fronts[k];
      if (s.p[fr] <= kSmallP && s.f[fr] <= kSmallF) ns++;
      else nl++;
      if (s.p[fr] > kTiledMaxP) fits = false;
    }
    if (single_dense || !fits || !(nl > 0 || ns * CL <= 2 * c.num_sms)) continue;
    level_tiled[l] = 1;
    for (int k = s.level_ptr[l]; k < s.level_ptr[l + 1]; k++) {
      const int fr = s.level_fronts[k];
      const int F = s.f[fr], P = s.p[fr];
      max_tiled_p = std::max(max_tiled_p, P);
      for (int r0 = 0; r0 < F; r0 += kTileRows) tf_h.insert(tf_h.end(), {fr, r0});
      for (int r0 = 0; r0 < P; r0 += kTileRows) tb_h.insert(tb_h.end(), {fr, r0});
      const bool small = P <= kSmallP && F <= kSmallF;
      if (!small && P > 0 && P <= kSmallP) {
        mid_h.push_back(fr);
        max_mid_p = std::max(max_mid_p, P);
      }
      if (P > kSmallP) {
        wide_h.push_back(fr);
        fdh[fr].aux = sq_total;
        sq_total += (int64_t)P * P;
        max_wide_p = std::max(max_wide_p, P);
        for (int j0 = 0; j0 < P; j0 += 32) wi_h.insert(wi_h.end(), {fr, j0});
      }
      if (P > 0)
        for (int t0 = 0; t0 < F - P; t0 += kTileRows) pi_h.insert(pi_h.end(), {fr, 0, t0, 0, fr, 1, t0, 0});
      // pull lists: row u of the front (before pivoting) receives row i of child ch's update block
      std::vector<std::vector<std::pair<int64_t, int32_t>>> rows(F);
      for (int slot = 0; slot < MAXKIDS; slot++) {
        const int ch = kids[fr][slot];
        if (ch < 0) continue;
        const int sc = s.f[ch] - s.p[ch];
        for (int i = 0; i < sc; i++) {
          const int u = s.ea_map[s.ea_ptr[ch] + i];
          if (u < 0 || u >= F) fail(FEM2D_E_INVALID_ARG, "extend-add map outside the parent front");
          rows[u].push_back({woff_h[ch] + s.p[ch] + i, s.f[ch]});
        }
      }
      fdh[fr].prow = (int64_t)prow_h.size();
      for (int u = 0; u < F; u++) {
        prow_h.push_back((int64_t)soff_h.size());
        for (const auto& e : rows[u]) {
          soff_h.push_back(e.first);
          sstr_h.push_back(e.second);
        }
      }
      prow_h.push_back((int64_t)soff_h.size());
    }
  }
  tf_ptr[nlevels] = (int32_t)(tf_h.size() / 2);
  tb_ptr[nlevels] = (int32_t)(tb_h.size() / 2);
  nmid = (int)mid_h.size();
  nwide = (int)wide_h.size();
  nwide_items = (int)(wi_h.size() / 2);
  npinv = (int)(pi_h.size() / 4);
  tf_items.upload(tf_h, st);
  tb_items.upload(tb_h, st);
  prow.upload(prow_h, st);
  src_off.upload(soff_h, st);
  src_str.upload(sstr_h, st);
  lmid.upload(mid_h, st);
  lwide.upload(wide_h, st);
  wide_items.upload(wi_h, st);
  pinv_items.upload(pi_h, st);
  sq.alloc(std::max<int64_t>(sq_total, 1));
  std::vector<uint8_t> raw(fdh.size() * sizeof(FrontDesc));
  std::memcpy(raw.data(), fdh.data(), raw.size());
  desc.upload(raw, st);
  lfronts.upload(s.level_fronts, st);
  dofs.upload(s.dofs, st);
  asm_pos.upload(s.asm_pos, st);
  asm_csr.upload(s.asm_csr, st);
  ea_map.upload(s.ea_map, st);
  piv_off.upload(poff, st);
  woff.upload(woff_h, st);
  piv_total = po;
  work.alloc(std::max<int64_t>(wo, 1));
  flags.alloc(1);
  weak_list.alloc(std::max<int64_t>(s.n, 1));
  weak_count.alloc(1);
  level_max_f.assign(nlevels, 0);
  level_max_p.assign(nlevels, 0);
  level_factor_bytes.assign(nlevels, 0.0);
  for (int l = 0; l < nlevels; l++)
    for (int k = s.level_ptr[l]; k < s.level_ptr[l + 1]; k++) {
      const double F = s.f[s.level_fronts[k]], P = s.p[s.level_fronts[k]];
      level_max_f[l] = std::max(level_max_f[l], s.f[s.level_fronts[k]]);
      level_max_p[l] = std::max(level_max_p[l], s.p[s.level_fronts[k]]);
      level_factor_bytes[l] += 8.0 * (0.5 * P * P + P * (F - P));
    }
  std::vector<int32_t> ls, ll;
  small_ptr.assign(nlevels + 1, 0);
  large_ptr.assign(nlevels + 1, 0);
  level_small_f.assign(nlevels, 0);
  level_small_p.assign(nlevels, 0);
  max_small_p = 0;
  for (int l = 0; l < nlevels; l++) {
    small_ptr[l] = (int32_t)ls.size();
    large_ptr[l] = (int32_t)ll.size();
    for (int k = s.level_ptr[l]; k < s.level_ptr[l + 1]; k++) {
      const int fr = s.level_fronts[k];
      if (s.p[fr] <= kSmallP && s.f[fr] <= kSmallF) {
        ls.push_back(fr);
        level_small_f[l] = std::max(level_small_f[l], s.f[fr]);
        level_small_p[l] = std::max(level_small_p[l], s.p[fr]);
        max_small_p = std::max(max_small_p, s.p[fr]);
      } else {
        ll.push_back(fr);
      }
    }
  }
  small_ptr[nlevels] = (int32_t)ls.size();
  large_ptr[nlevels] = (int32_t)ll.size();
  nsmall = (int)ls.size();
  lsmall.upload(ls, st);
  llarge.upload(ll, st);
  // dynamic shared memory limits are set once per device (a function attribute of the device's context)
  static std::mutex attr_mu;
  static bool attr_done[256] = {};
  std::lock_guard<std::mutex> lk(attr_mu);
  if (c.device >= 0 && c.device < 256 && !attr_done[c.device]) {
    FEM2D_CUDA(cudaFuncSetAttribute(mf_invdiag_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    kSmallP * kSmallP * (int)sizeof(double)));
    FEM2D_CUDA(cudaFuncSetAttribute(mf_forward_small_kernel<256>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (kSmallF + kSmallP) * 32 * (int)sizeof(double)));
    FEM2D_CUDA(cudaFuncSetAttribute(mf_forward_small_kernel<512>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (kSmallF + kSmallP) * 32 * (int)sizeof(double)));
    FEM2D_CUDA(cudaFuncSetAttribute(mf_forward_small_kernel<1024>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (kSmallF + kSmallP) * 32 * (int)sizeof(double)));
    FEM2D_CUDA(cudaFuncSetAttribute(mf_backward_small_kernel<256>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    kSmallF * 32 * (int)sizeof(double)));
    FEM2D_CUDA(cudaFuncSetAttribute(mf_backward_small_kernel<512>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    kSmallF * 32 * (int)sizeof(double)));
    FEM2D_CUDA(cudaFuncSetAttribute(mf_backward_small_kernel<1024>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    kSmallF * 32 * (int)sizeof(double)));
    FEM2D_CUDA(cudaFuncSetAttribute(mf_forward_small_cluster_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (kSmallF + kSmallP) * 32 * (int)sizeof(double)));
    FEM2D_CUDA(cudaFuncSetAttribute(mf_backward_small_cluster_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    kSmallF * 32 * (int)sizeof(double)));
    FEM2D_CUDA(cudaFuncSetAttribute(mf_invdiag_wide_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    kTiledMaxP * 32 * (int)sizeof(double)));
    FEM2D_CUDA(cudaFuncSetAttribute(mf_partinv_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    kTileRows * kTiledMaxP * (int)sizeof(double)));
    attr_done[c.device] = true;
  }
}

void MFDevice::factor(Ctx& c, const double* va, const double* vb, double ca, double cb, bool cholesky,
                      MFFactor& out) {
  cudaStream_t st = c.stream;
  DBuf<double>& Fbuf = out.F;
  enable_stream_pool(c.device);
  if (Fbuf.n != (size_t)std::max<int64_t>(mat_total, 1)) Fbuf.alloc_on(std::max<int64_t>(mat_total, 1), st);
  if (out.piv.n != (size_t)std::max<int64_t>(piv_total, 1)) out.piv.alloc_on(std::max<int64_t>(piv_total, 1), st);
  FEM2D_CUDA(cudaMemsetAsync(flags.p, 0, sizeof(int), st));
  FEM2D_CUDA(cudaMemsetAsync(weak_count.p, 0, sizeof(int), st));
  out.weak.clear();
  const FrontDesc* fd = reinterpret_cast<const FrontDesc*>(desc.p);
  ProfScope ps(c, "mf_factor", 8.0 * (double)mat_total, cholesky ? 0.5 * factor_flops : factor_flops);
  out.inv_n = 0;
  if (nf == 1 && max_p == max_f && max_f <= 4096) {
    // one dense front (a small GEP): its explicit inverse by Gauss-Jordan, kept in F; solves are then
    // one dense product
    const int n = max_f;
    FEM2D_CUDA(cudaMemsetAsync(Fbuf.p, 0, (size_t)n * n * sizeof(double), st));
    mf_assemble_kernel<<<dim3(8, 1), 256, 0, st>>>(lfronts.p, fd, asm_pos.p, asm_csr.p, va, vb, ca, cb, Fbuf.p);
    c.launches++;
    const int gu = (int)std::min<int64_t>(((int64_t)n * n + 255) / 256, (int64_t)c.num_sms * 8);
    const int pivoting = cholesky ? 0 : 1;
    for (int q = 0; q < n; q++) {
      gjp_pivot_kernel<<<1, 1024, 0, st>>>(n, q, pivoting, Fbuf.p, out.piv.p, flags.p);
      gjp_update_kernel<<<gu, 256, 0, st>>>(n, q, Fbuf.p);
      gjp_finish_kernel<<<(n + 255) / 256, 256, 0, st>>>(n, q, Fbuf.p);
      gjp_recip_kernel<<<1, 32, 0, st>>>(n, q, Fbuf.p);
      c.launches += 4;
    }
    if (pivoting) {
      gjp_unscramble_kernel<<<(n + 127) / 128, 128, 0, st>>>(n, out.piv.p, Fbuf.p);
      c.launches++;
    }
    FEM2D_CUDA(cudaGetLastError());
    out.inv_n = n;
    out.flags = read_flags(c);
    return;
  }
  for (int l = 0; l < nlevels; l++) {
    const int nfl = level_ptr[l + 1] - level_ptr[l];
    const int32_t* lf = lfronts.p + level_ptr[l];
    FEM2D_CUDA(cudaMemsetAsync(Fbuf.p + level_off[l], 0, (level_off[l + 1] - level_off[l]) * sizeof(double), st));
    mf_assemble_kernel<<<dim3(8, nfl), 256, 0, st>>>(lf, fd, asm_pos.p, asm_csr.p, va, vb, ca, cb, Fbuf.p);
    c.launches++;
    if (l > 0) {
      for (int slot = 0; slot < MAXKIDS; slot++) {
        mf_extend_add_kernel<<<dim3(16, nfl), 256, 0, st>>>(lf, fd, slot, ea_map.p, Fbuf.p);
        c.launches++;
      }
    }
    const int mf = level_max_f[l], mp = level_max_p[l];
    for (int k0 = 0; k0 < mp; k0 += PANEL) {
      mf_panel_kernel<<<nfl, 256, 0, st>>>(lf, fd, k0, cholesky ? 0 : 1, Fbuf.p, out.piv.p, piv_off.p, flags.p,
                                           dofs.p, weak_list.p, weak_count.p, (int)weak_list.n);
      const int rest = mf - k0;   // upper bound of remaining columns
      if (rest > 0) {
        dim3 gt((rest + 127) / 128, nfl);
        mf_trsm_kernel<<<gt, 128, 0, st>>>(lf, fd, k0, Fbuf.p);
        dim3 gg((rest + 63) / 64, (rest + 63) / 64, nfl);
        mf_gemm_kernel<<<gg, 256, 0, st>>>(lf, fd, k0, Fbuf.p);
        c.launches += 2;
      }
      c.launches++;
    }
  }
  if (out.perm.n != out.piv.n) out.perm.alloc_on(out.piv.n, st);
  if (out.iperm.n != out.piv.n) out.iperm.alloc_on(out.piv.n, st);
  mf_perm_kernel<<<(nf + 127) / 128, 128, 0, st>>>(nf, fd, out.piv.p, piv_off.p, out.perm.p, out.iperm.p);
  c.launches++;
  if (nsmall > 0) {
    mf_invdiag_kernel<<<nsmall, 256, (size_t)max_small_p * max_small_p * sizeof(double), st>>>(lsmall.p, fd,
                                                                                              Fbuf.p);
    c.launches++;
  }
  // the tiled levels' fronts: inverted diagonal squares, then L21' = -L21 L11^-1 and U12' = -U11^-1 U12
  if (nmid > 0) {
    mf_invdiag_kernel<<<nmid, 256, (size_t)max_mid_p * max_mid_p * sizeof(double), st>>>(lmid.p, fd, Fbuf.p);
    c.launches++;
  }
  if (nwide > 0) {
    mf_square_copy_kernel<<<dim3(64, nwide), 256, 0, st>>>(lwide.p, fd, Fbuf.p, sq.p);
    mf_invdiag_wide_kernel<<<nwide_items, 32, (size_t)max_wide_p * 32 * sizeof(double), st>>>(
        reinterpret_cast<const int2*>(wide_items.p), fd, sq.p, Fbuf.p);
    c.launches += 2;
  }
  if (npinv > 0) {
    mf_partinv_kernel<<<npinv, 256, (size_t)kTileRows * max_tiled_p * sizeof(double), st>>>(
        reinterpret_cast<const int4*>(pinv_items.p), fd, Fbuf.p);
    c.launches++;
  }

  FEM2D_CUDA(cudaGetLastError());
  out.flags = read_flags(c);
  if (!cholesky) {
    int nw = 0;
    FEM2D_CUDA(cudaMemcpyAsync(&nw, weak_count.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    FEM2D_CUDA(cudaStreamSynchronize(st));
    nw = std::min<int>(nw, (int)weak_list.n);
    if (nw > 0) {
      out.weak.resize(nw);
      FEM2D_CUDA(cudaMemcpyAsync(out.weak.data(), weak_list.p, nw * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
      FEM2D_CUDA(cudaStreamSynchronize(st));
    }
  }
}

// Threads per front for a level of ns small fronts solved one CTA per front: a level that fits one
// front per SM takes 1024 threads (one CTA per SM at 40 registers a thread), one that fits two fronts per
// SM takes 512 (two CTAs per SM when their shared memory fits twice), wider levels 256. Narrow levels are
// latency-bound within each front, so the threads a front gets set their time.
static int small_threads(int ns, size_t smem, int num_sms) {
  if (ns <= num_sms) return 1024;
  if (ns <= 2 * num_sms && smem <= 100 * 1024) return 512;
  return 256;
}

void MFDevice::solve(Ctx& c, const MFFactor& fac, const double* B, int64_t ldb, double* X, int64_t ldx, int nb) {
  const DBuf<double>& Fbuf = fac.F;
  cudaStream_t st = c.stream;
  if (nb > nb_cap) fail(FEM2D_E_INVALID_ARG, "solve block wider than the workspace");
  if (fac.inv_n > 0) {
    ProfScope ps(c, "mf_solve", 8.0 * fac.inv_n * fac.inv_n, 2.0 * fac.inv_n * fac.inv_n * nb);
    const int64_t blocks = std::min<int64_t>((fac.inv_n * 32 + 255) / 256, (int64_t)c.num_sms * 8);
    dense_inverse_apply_kernel<<<(int)std::max<int64_t>(blocks, 1), 256, 0, st>>>(fac.inv_n, Fbuf.p, B, ldb, nb, X,
                                                                                 ldx);
    c.launches++;
    FEM2D_CUDA(cudaGetLastError());
    return;
  }
  const FrontDesc* fd = reinterpret_cast<const FrontDesc*>(desc.p);
  double fbytes = 0.0;
  for (double b : level_factor_bytes) fbytes += b;
  // the whole solve is one profiled region: per-level events would dominate the short level launches
  ProfScope ps(c, "mf_solve", 2.0 * fbytes, 2.0 * 2.0 * (fbytes / 8.0) * nb);
  SolveArgs a{fd, dofs.p, ea_map.p, fac.perm.p, fac.iperm.p, piv_off.p, woff.p, Fbuf.p, B, ldb, work.p, X, ldx, nb};
  TiledArgs ta{fd,     dofs.p, fac.perm.p, piv_off.p, woff.p, prow.p, src_off.p, src_str.p,
               Fbuf.p, B,      ldb,        work.p,    X,      ldx,    nb};
  const int2* tfi = reinterpret_cast<const int2*>(tf_items.p);
  const int2* tbi = reinterpret_cast<const int2*>(tb_items.p);
  for (int l = 0; l < nlevels; l++) {
    if (level_tiled[l]) {
      const int ni = tf_ptr[l + 1] - tf_ptr[l];
      if (ni > 0) {
        mf_forward_tiled_kernel<<<ni, 256, 0, st>>>(tfi + tf_ptr[l], ta);
        c.launches++;
      }
      continue;
    }
    const int ns = small_ptr[l + 1] - small_ptr[l], nl = large_ptr[l + 1] - large_ptr[l];
    if (ns > 0) {
      const size_t smem = (size_t)(level_small_f[l] + level_small_p[l]) * nb * sizeof(double);
      const int nt = small_threads(ns, smem, c.num_sms);
      if (ns * CL <= 2 * c.num_sms)
        mf_forward_small_cluster_kernel<<<ns * CL, 256, smem, st>>>(lsmall.p + small_ptr[l], a);
      else if (nt == 1024)
        mf_forward_small_kernel<1024><<<ns, 1024, smem, st>>>(lsmall.p + small_ptr[l], a);
      else if (nt == 512)
        mf_forward_small_kernel<512><<<ns, 512, smem, st>>>(lsmall.p + small_ptr[l], a);
      else
        mf_forward_small_kernel<256><<<ns, 256, smem, st>>>(lsmall.p + small_ptr[l], a);
      c.launches++;
    }
    if (nl > 0) {
      mf_forward_cluster_kernel<<<nl * CL, 256, 0, st>>>(llarge.p + large_ptr[l], fd, dofs.p, ea_map.p, fac.perm.p,
                                                         fac.iperm.p, piv_off.p, woff.p, Fbuf.p, B, ldb, nb,
                                                         work.p);
      c.launches++;
    }
  }
  for (int l = nlevels - 1; l >= 0; l--) {
    if (level_tiled[l]) {
      const int ni = tb_ptr[l + 1] - tb_ptr[l];
      if (ni > 0) {
        mf_backward_tiled_kernel<<<ni, 256, 0, st>>>(tbi + tb_ptr[l], ta);
        c.launches++;
      }
      continue;
    }
    const int ns = small_ptr[l + 1] - small_ptr[l], nl = large_ptr[l + 1] - large_ptr[l];
    if (ns > 0) {
      const size_t smem = (size_t)level_small_f[l] * nb * sizeof(double);
      const int nt = small_threads(ns, smem, c.num_sms);
      if (ns * CL <= 2 * c.num_sms)
        mf_backward_small_cluster_kernel<<<ns * CL, 256, smem, st>>>(lsmall.p + small_ptr[l], a);
      else if (nt == 1024)
        mf_backward_small_kernel<1024><<<ns, 1024, smem, st>>>(lsmall.p + small_ptr[l], a);
      else if (nt == 512)
        mf_backward_small_kernel<512><<<ns, 512, smem, st>>>(lsmall.p + small_ptr[l], a);
      else
        mf_backward_small_kernel<256><<<ns, 256, smem, st>>>(lsmall.p + small_ptr[l], a);
      c.launches++;
    }
    if (nl > 0) {
      mf_backward_cluster_kernel<<<nl * CL, 256, 0, st>>>(llarge.p + large_ptr[l], fd, dofs.p, woff.p, Fbuf.p,
                                                          work.p, nb, X, ldx);
      c.launches++;
    }
  }
  FEM2D_CUDA(cudaGetLastError());
}

int MFDevice::read_flags(Ctx& c) {
  int h = 0;
  FEM2D_CUDA(cudaMemcpyAsync(&h, flags.p, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
  FEM2D_CUDA(cudaStreamSynchronize(c.stream));
  return h;
}

}  // namespace fem2d
