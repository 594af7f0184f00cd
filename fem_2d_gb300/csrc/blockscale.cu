// Block congruence scaling of the pencil over row runs.
//
// The rows of one run (consecutive DoFs with one column list: an Elem's interior functions) keep a
// common pattern, and by symmetry so do their columns. With S = blockdiag(L_g^-1), B_gg = L_g L_g^T
// the Cholesky factor of B's diagonal block of run g, the pencil (S A S^T, S B S^T) has exactly the
// sparsity pattern of (A, B), the same eigenvalues, eigenvectors x = S^T x~, and identity diagonal
// blocks in S B S^T. For high-order monomial (HierPoly) bases this lowers cond(B) by three or more
// orders of magnitude where the diagonal (Jacobi) scaling only normalises the diagonal, and with it
// the digits the shifted factorizations lose. It costs (|g| + |h|) |g| |h| FP64 FMAs per coupled
// block pair, so the solver applies it only when the Jacobi-scaled factorizations are inaccurate.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <vector>

#include "blockscale.h"

namespace fem2d {

namespace {

constexpr int kRun = 64;   // rows per run (the runs of device_upload are at most 64 long)

// per run: Cholesky of B_gg in shared memory, then S_g = L^-1 (row-major, lower) to global
__global__ void __launch_bounds__(256) run_cholinv_kernel(const int32_t* __restrict__ grp,
                                                          const int64_t* __restrict__ rp,
                                                          const int32_t* __restrict__ col,
                                                          const double* __restrict__ vb,
                                                          const int64_t* __restrict__ soff,
                                                          double* __restrict__ S, int* __restrict__ flag) {
  extern __shared__ double csm[];
  double* M = csm;                 // kRun x kRun
  double* Li = csm + kRun * kRun;  // kRun x kRun
  __shared__ int s_off;
  const int g = blockIdx.x;
  const int g0 = grp[g], R = grp[g + 1] - g0;
  if (threadIdx.x == 0) {   // position of column g0 in row g0 (every row of the run has the same list)
    int lo = 0, hi = (int)(rp[g0 + 1] - rp[g0]) - 1, at = -1;
    const int32_t* cl = col + rp[g0];
    while (lo <= hi) {
      const int mid = (lo + hi) >> 1;
      if (cl[mid] == g0) { at = mid; break; }
      if (cl[mid] < g0) lo = mid + 1; else hi = mid - 1;
    }
    s_off = at;
    if (at < 0) atomicOr(flag, 2);
  }
  __syncthreads();
  if (s_off < 0) return;
  for (int t = threadIdx.x; t < R * R; t += blockDim.x) {
    const int r = t / R, q = t % R;
    M[r * kRun + q] = vb[rp[g0 + r] + s_off + q];
  }
  __syncthreads();
  for (int j = 0; j < R; j++) {   // right-looking Cholesky, lower triangle
    if (threadIdx.x == 0) {
      const double d = M[j * kRun + j];
      if (!(d > 0.0)) atomicOr(flag, 1);
      M[j * kRun + j] = d > 0.0 ? sqrt(d) : 1.0;
    }
    __syncthreads();
    const double dj = M[j * kRun + j];
    for (int i = j + 1 + threadIdx.x; i < R; i += blockDim.x) M[i * kRun + j] /= dj;
    __syncthreads();
    for (int t = threadIdx.x; t < (R - j - 1) * (R - j - 1); t += blockDim.x) {
      const int i = j + 1 + t / (R - j - 1), k = j + 1 + t % (R - j - 1);
      if (k <= i) M[i * kRun + k] -= M[i * kRun + j] * M[k * kRun + j];
    }
    __syncthreads();
  }
  // column q of L^-1 per thread: L x = e_q
  for (int q = threadIdx.x; q < R; q += blockDim.x) {
    for (int i = 0; i < q; i++) Li[i * kRun + q] = 0.0;
    Li[q * kRun + q] = 1.0 / M[q * kRun + q];
    for (int i = q + 1; i < R; i++) {
      double s = 0.0;
      for (int k = q; k < i; k++) s += M[i * kRun + k] * Li[k * kRun + q];
      Li[i * kRun + q] = -s / M[i * kRun + i];
    }
  }
  __syncthreads();
  double* out = S + soff[g];
  for (int t = threadIdx.x; t < R * R; t += blockDim.x) out[t] = Li[(t / R) * kRun + t % R];
}

// per run g and each column run h of its pattern: block <- S_g block S_h^T, for A and B (256 threads)
constexpr int kTransformThreads = 256;
constexpr int kT1Regs = kRun * kRun / kTransformThreads;
__global__ void __launch_bounds__(kTransformThreads) run_transform_kernel(const int32_t* __restrict__ grp,
                                                            const int64_t* __restrict__ rp,
                                                            const int64_t* __restrict__ seg_ptr,
                                                            const int2* __restrict__ seg,
                                                            const int64_t* __restrict__ soff,
                                                            const double* __restrict__ S,
                                                            const double* __restrict__ va,
                                                            const double* __restrict__ vb, double* __restrict__ sa,
                                                            double* __restrict__ sb) {
  extern __shared__ double smem[];
  double* Sg = smem;                    // R x R
  double* ShT = Sg + kRun * kRun;       // H x H, transposed: ShT[k H + q] = S_h[q][k]
  double* Blk = ShT + kRun * kRun;      // R x H: the block, then T1 = S_g Blk in its place
  const int g = blockIdx.x;
  const int g0 = grp[g], R = grp[g + 1] - g0;
  for (int t = threadIdx.x; t < R * R; t += blockDim.x) Sg[t] = S[soff[g] + t];
  for (int64_t sgi = seg_ptr[g]; sgi < seg_ptr[g + 1]; sgi++) {
    const int2 sh = seg[sgi];   // (column run h, offset of its first column in the rows of g)
    const int h0 = grp[sh.x], H = grp[sh.x + 1] - h0;
    __syncthreads();
    // S_h is stored transposed so that the lanes of the second product (consecutive q) read consecutive
    // doubles (row-major S_h would put all 32 lanes of a warp in one bank for H = 64)
    for (int t = threadIdx.x; t < H * H; t += blockDim.x) ShT[(t % H) * H + t / H] = S[soff[sh.x] + t];
    for (int m = 0; m < 2; m++) {
      const double* src = m == 0 ? va : vb;
      double* dst = m == 0 ? sa : sb;
      __syncthreads();
      for (int t = threadIdx.x; t < R * H; t += blockDim.x) {
        const int r = t / H, q = t % H;
        Blk[t] = src[rp[g0 + r] + sh.y + q];
      }
      __syncthreads();
      // T1 = S_g Blk (S_g lower), held in registers (at most 16 entries a thread: 64 x 64 over 256
      // threads) and written over Blk once every thread has read it: two CTAs fit an SM
      double t1[kT1Regs];
#pragma unroll
      for (int i = 0; i < kT1Regs; i++) {
        const int t = threadIdx.x + kTransformThreads * i;
        t1[i] = 0.0;
        if (t < R * H) {
          const int r = t / H, q = t % H;
          double s = 0.0;
          for (int k = 0; k <= r; k++) s += Sg[r * R + k] * Blk[k * H + q];
          t1[i] = s;
        }
      }
      __syncthreads();
#pragma unroll
      for (int i = 0; i < kT1Regs; i++) {
        const int t = threadIdx.x + kTransformThreads * i;
        if (t < R * H) Blk[t] = t1[i];
      }
      __syncthreads();
      for (int t = threadIdx.x; t < R * H; t += blockDim.x) {   // out = T1 S_h^T (S_h lower)
        const int r = t / H, q = t % H;
        double s = 0.0;
        for (int k = 0; k <= q; k++) s += Blk[r * H + k] * ShT[k * H + q];
        dst[rp[g0 + r] + sh.y + q] = s;
      }
    }
  }
}

// X_g <- S_g^T X_g per run (back to the original basis)
__global__ void __launch_bounds__(256) run_back_kernel(const int32_t* __restrict__ grp,
                                                       const int64_t* __restrict__ soff,
                                                       const double* __restrict__ S, double* __restrict__ X,
                                                       int64_t ldx, int nb) {
  __shared__ double xs[kRun * 32];
  const int g = blockIdx.x;
  const int g0 = grp[g], R = grp[g + 1] - g0;
  for (int t = threadIdx.x; t < R * nb; t += blockDim.x) xs[t] = X[(int64_t)(g0 + t / nb) * ldx + t % nb];
  __syncthreads();
  const double* Sg = S + soff[g];
  for (int t = threadIdx.x; t < R * nb; t += blockDim.x) {
    const int r = t / nb, c = t % nb;
    double s = 0.0;
    for (int k = r; k < R; k++) s += Sg[k * R + r] * xs[k * nb + c];   // (S_g^T)[r][k] = S_g[k][r]
    X[(int64_t)(g0 + r) * ldx + c] = s;
  }
}

}  // namespace

void BlockScale::build(Ctx& c, const HostGEP& h, const DeviceGEP& d, double* sa, double* sb) {
  if (!ready) {
    const int64_t n = h.n;
    // runs exactly as device_upload forms them, their column-run segments, block offsets
    const std::vector<int32_t>& grp = d.grp_h;
    ngrp = (int)grp.size() - 1;
    std::vector<int32_t> run_of(n);
    for (int g = 0; g < ngrp; g++)
      for (int32_t i = grp[g]; i < grp[g + 1]; i++) run_of[i] = g;
    std::vector<int64_t> so(ngrp + 1, 0), sp(ngrp + 1, 0);
    std::vector<int2> sg;
    for (int g = 0; g < ngrp; g++) {
      const int R = grp[g + 1] - grp[g];
      so[g + 1] = so[g] + (int64_t)R * R;
      alg_flops += (double)R * R * R;        // Cholesky (R^3 / 3 FMA) and inverse (R^3 / 6 FMA)
      alg_bytes += 8.0 * 3.0 * R * R;        // B's diagonal block read, S_g written and read back
      const int64_t b = h.row_ptr[grp[g]], e = h.row_ptr[grp[g] + 1];
      int64_t q = b;
      while (q < e) {
        const int32_t hr = run_of[h.col[q]];
        const int H = grp[hr + 1] - grp[hr];
        // a column run appears whole and in order (its columns are consecutive DoFs)
        if (h.col[q] != grp[hr] || q + H > e || h.col[q + H - 1] != grp[hr] + H - 1)
          fail(FEM2D_E_INVALID_ARG, "block scaling: a column run is split in a row pattern");
        sg.push_back(make_int2(hr, (int)(q - b)));
        alg_flops += 2.0 * 2.0 * ((double)R * (R + 1) / 2.0 * H + (double)R * H * (H + 1) / 2.0);
        alg_bytes += 8.0 * (double)H * H;   // S_h read for this block
        q += H;
      }
      sp[g + 1] = (int64_t)sg.size();
    }
    // kept in the GEP's plan across solves: plain (not stream-ordered) allocations
    grp_d.upload(grp, c.stream);
    soff.upload(so, c.stream);
    seg_ptr.upload(sp, c.stream);
    seg.upload(sg, c.stream);
    S.alloc(std::max<int64_t>(so[ngrp], 1));
    alg_bytes += 32.0 * (double)h.nnz_full;
    ready = true;
  }
  DBuf<int> flag;
  flag.alloc_on(1, c.stream);
  FEM2D_CUDA(cudaMemsetAsync(flag.p, 0, sizeof(int), c.stream));
  static std::mutex mu;
  static bool attr[256] = {};
  {
    std::lock_guard<std::mutex> lk(mu);
    if (c.device >= 0 && c.device < 256 && !attr[c.device]) {
      FEM2D_CUDA(cudaFuncSetAttribute(run_cholinv_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      2 * kRun * kRun * (int)sizeof(double)));
      FEM2D_CUDA(cudaFuncSetAttribute(run_transform_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      3 * kRun * kRun * (int)sizeof(double)));
      attr[c.device] = true;
    }
  }
  run_cholinv_kernel<<<ngrp, 256, 2 * kRun * kRun * sizeof(double), c.stream>>>(grp_d.p, d.row_ptr.p, d.col.p, d.b.p,
                                                                                soff.p, S.p, flag.p);
  c.launches++;
  run_transform_kernel<<<ngrp, kTransformThreads, 3 * kRun * kRun * sizeof(double), c.stream>>>(
      grp_d.p, d.row_ptr.p, seg_ptr.p, seg.p, soff.p, S.p, d.a.p, d.b.p, sa, sb);
  c.launches++;
  FEM2D_CUDA(cudaGetLastError());
  int hf = 0;
  FEM2D_CUDA(cudaMemcpyAsync(&hf, flag.p, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
  FEM2D_CUDA(cudaStreamSynchronize(c.stream));
  if (hf & 2) fail(FEM2D_E_INVALID_ARG, "block scaling: a run's diagonal block is missing from the pattern");
  if (hf & 1) fail(FEM2D_E_B_NOT_SPD, "a diagonal block of B is not positive definite");
}

void BlockScale::unscale(Ctx& c, double* X, int64_t ldx, int nb) const {
  if (nb > 32) fail(FEM2D_E_INVALID_ARG, "block unscaling of more than 32 columns");
  run_back_kernel<<<ngrp, 256, 0, c.stream>>>(grp_d.p, soff.p, S.p, X, ldx, nb);
  c.launches++;
  FEM2D_CUDA(cudaGetLastError());
}

}  // namespace fem2d
