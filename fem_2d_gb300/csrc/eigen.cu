// Eigensolvers on the device.
//
// gpu_solve_gep (stands beside slepc_solve_gep, slepc_solve.rs:14-68): the n_pairs eigenpairs of
// (A, B) nearest the target sigma among the non-spurious spectrum. The curl-curl operator has a large
// null space (gradients, lambda = 0) which sits at distance |sigma| from the target; the reference
// treats such modes as spurious (nalgebra_solve.rs:24-26). The search space is generated with
//     T = (A - sigma B)^-1 A (A + c B)^-1 B
// with c = 0.05 |sigma|: eigenvalue lambda / ((lambda - sigma)(lambda + c)), close to the plain
// shift-invert 1 / (lambda - sigma) for every physical mode, zero on the null space (A kills it
// whatever the accuracy of the SPD solve) and small for high-frequency modes; exact multifrontal
// solves (mf.cu). Each cycle builds a block Krylov basis [X, TX, T^2 X] B-orthonormalised by CGS2
// in FP64, then a Rayleigh-Ritz step on the pencil (A, B) itself (FP64); Ritz pairs with a relative
// residual above 1 (mixtures of null-space and high-frequency directions that land near sigma) are
// not selected. Residuals ||A x - lambda B x|| / (|lambda| ||B x||) are computed in FP64.
//
// nalgebra_solve_gep (nalgebra_solve.rs:14-50) on the device: B is factored (Cholesky mode; a
// non-positive pivot is FailedToInvertB), Z = B^-1 A is formed column block by column block, and
// the eigen-decomposition of the symmetric matrix built from the lower triangle of Z (the triangle
// nalgebra's SymmetricEigen reads) gives the pair nearest the target.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <numeric>

#include "eigen.h"
#include "mf.h"
#include "mfdev.h"
#include "symeig.h"

namespace fem2d {

void mf_symbolic(const Domain& d, const HostGEP& g, MFSymbolic& s);

namespace {

// ---------------------------------------------------------------- dense block kernels
// Y = ca*A*X + cb*B*X; X, Y row-major (ldx, ldy), nb <= 32 columns. One warp per row; the warp's
// lanes split into (32 / G) groups of G >= nb lanes, each group walking a slice of the row's entries.
__global__ void __launch_bounds__(256) spmm_kernel(int64_t n, const int64_t* __restrict__ rp,
                                                   const int32_t* __restrict__ col, const double* __restrict__ va,
                                                   const double* __restrict__ vb, double ca, double cb,
                                                   const double* __restrict__ X, int64_t ldx, int nb, int G,
                                                   double* __restrict__ Y, int64_t ldy) {
  const int lane = threadIdx.x & 31;
  const int groups = 32 / G;
  const int c = lane % G, sub = lane / G;
  for (int64_t row = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; row < n;
       row += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    double acc = 0.0;
    const int64_t k1 = rp[row + 1];
    for (int64_t k = rp[row] + sub; k < k1; k += groups) {
      double v = 0.0;
      if (ca != 0.0) v += ca * __ldg(va + k);
      if (cb != 0.0) v += cb * __ldg(vb + k);
      if (c < nb) acc += v * __ldg(X + (int64_t)__ldg(col + k) * ldx + c);
    }
    for (int off = G; off < 32; off <<= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
    if (sub == 0 && c < nb) Y[row * ldy + c] = acc;
  }
}

// partial Gram: P[blk][i*b + j] = sum over the block's rows of X[r][i] * Y[r][j]
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
                                                      const double* __restrict__ C, int b, double beta,
                                                      double* __restrict__ Z, int64_t ldz) {
  extern __shared__ double cs[];
  for (int t = threadIdx.x; t < a * b; t += blockDim.x) cs[t] = C[t];
  __syncthreads();
  const int64_t total = n * b;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = t / b;
    const int j = (int)(t % b);
    double s = 0.0;
    const double* xr = X + r * ldx;
    for (int i = 0; i < a; i++) s += xr[i] * cs[i * b + j];
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

// R = AX - BX * diag(theta) column by column, accumulating column sums of squares of R and of BX
__global__ void __launch_bounds__(256) resid_partial_kernel(int64_t n, const double* __restrict__ AX,
                                                            const double* __restrict__ BX, int64_t ld, int b,
                                                            const double* __restrict__ theta, int64_t rows_per_block,
                                                            double* __restrict__ P) {
  __shared__ double sr[256], sb[256];
  const int64_t r0 = blockIdx.x * rows_per_block, r1 = min(n, r0 + rows_per_block);
  for (int j = 0; j < b; j++) {
    double a1 = 0.0, a2 = 0.0;
    const double th = theta[j];
    for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
      const double bx = BX[r * ld + j];
      const double res = AX[r * ld + j] - th * bx;
      a1 += res * res;
      a2 += bx * bx;
    }
    sr[threadIdx.x] = a1;
    sb[threadIdx.x] = a2;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
      if (threadIdx.x < s) {
        sr[threadIdx.x] += sr[threadIdx.x + s];
        sb[threadIdx.x] += sb[threadIdx.x + s];
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      P[(int64_t)blockIdx.x * 2 * b + j] = sr[0];
      P[(int64_t)blockIdx.x * 2 * b + b + j] = sb[0];
    }
    __syncthreads();
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
struct Dev {
  Ctx& c;
  const HostGEP& h;
  const DeviceGEP& d;
  DBuf<double> part;
  DBuf<double> small;
  int grid_rows() const { return std::max(1, c.num_sms * 2); }

  void spmm(double ca, double cb, const double* X, int64_t ldx, int nb, double* Y, int64_t ldy) {
    const double nv = (ca != 0.0) + (cb != 0.0);
    ProfScope ps(c, "spmm", (double)h.nnz_full * (4.0 + 8.0 * nv) + 8.0 * (h.n + 1) + 16.0 * h.n * nb);
    for (int c0 = 0; c0 < nb; c0 += 32) {
      const int w = std::min(32, nb - c0);
      int G = 1;
      while (G < w) G <<= 1;
      const int64_t warps = h.n;
      const int64_t blocks = std::min<int64_t>((warps * 32 + 255) / 256, (int64_t)c.num_sms * 16);
      spmm_kernel<<<(int)std::max<int64_t>(blocks, 1), 256, 0, c.stream>>>(h.n, d.row_ptr.p, d.col.p, d.a.p, d.b.p, ca,
                                                                           cb, X + c0, ldx, w, G, Y + c0, ldy);
      c.launches++;
    }
  }
  // C (a x b, host row-major) = X^T Y
  void gram(const double* X, int64_t ldx, int a, const double* Y, int64_t ldy, int b, std::vector<double>& C) {
    const int nblk = std::min<int64_t>(grid_rows(), std::max<int64_t>(1, (h.n + 255) / 256));
    const int64_t rpb = (h.n + nblk - 1) / nblk;
    const int ab = a * b;
    if (part.n < (size_t)nblk * ab) part.alloc((size_t)nblk * ab);
    if (small.n < (size_t)ab) small.alloc(std::max<size_t>(ab, 16384));
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
  // Z = beta Z + X * C (C host a x b)
  void gemm(const double* X, int64_t ldx, int a, const std::vector<double>& C, int b, double beta, double* Z,
            int64_t ldz) {
    if (small.n < (size_t)a * b) small.alloc(std::max<size_t>((size_t)a * b, 16384));
    FEM2D_CUDA(cudaMemcpyAsync(small.p, C.data(), (size_t)a * b * sizeof(double), cudaMemcpyHostToDevice, c.stream));
    const size_t smem = (size_t)a * b * sizeof(double);
    if (smem > 96 * 1024) fail(FEM2D_E_INVALID_ARG, "GEMM block too large");
    const int64_t blocks = std::min<int64_t>((h.n * b + 255) / 256, (int64_t)c.num_sms * 8);
    gemm_nn_kernel<<<(int)std::max<int64_t>(blocks, 1), 256, smem, c.stream>>>(h.n, X, ldx, a, small.p, b, beta, Z,
                                                                              ldz);
    c.launches++;
  }
  void copy(const double* X, int64_t ldx, int b, double* Y, int64_t ldy) {
    const int64_t blocks = std::min<int64_t>((h.n * b + 255) / 256, (int64_t)c.num_sms * 8);
    copy_block_kernel<<<(int)std::max<int64_t>(blocks, 1), 256, 0, c.stream>>>(h.n, b, X, ldx, Y, ldy);
    c.launches++;
  }
};

void setup_gemm_smem() {
  static bool done = false;
  if (done) return;
  cudaFuncSetAttribute(gemm_nn_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024);
  cudaFuncSetAttribute(gram_partial_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024);
  done = true;
}

// splitmix64 -> standard normal (Box-Muller), deterministic start blocks
void random_block(int64_t n, int b, uint64_t seed, std::vector<double>& out) {
  out.resize((size_t)n * b);
  uint64_t s = seed * 0x9E3779B97F4A7C15ull + 0x2545F4914F6CDD1Dull;
  auto next = [&]() {
    s += 0x9E3779B97F4A7C15ull;
    uint64_t z = s;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  };
  for (size_t k = 0; k < out.size(); k += 2) {
    double u1 = ((next() >> 11) + 0.5) / 9007199254740992.0, u2 = ((next() >> 11) + 0.5) / 9007199254740992.0;
    double r = std::sqrt(-2.0 * std::log(u1));
    out[k] = r * std::cos(2.0 * M_PI * u2);
    if (k + 1 < out.size()) out[k + 1] = r * std::sin(2.0 * M_PI * u2);
  }
}

}  // namespace

// ================================================================ sparse shift-invert eigensolver
void sparse_solve(Ctx& c, const Domain& dom, const HostGEP& h, const DeviceGEP& d, double sigma, int k,
                  const fem2d_solve_opts& o, double* values, double* vectors, double* residuals,
                  fem2d_solve_stats* st) {
  auto t0 = std::chrono::steady_clock::now();
  setup_gemm_smem();
  const int64_t n = h.n;
  const int guard = std::max(4, k / 2);
  int b = o.block > 0 ? o.block : std::min<int64_t>(k + guard, n);
  if (b < k) b = k;
  if (b > 32) fail(FEM2D_E_INVALID_ARG, "block size above 32 (n_pairs too large for one block)");
  const int steps = 2;
  const int mmax = b * (steps + 1);
  const double tol = o.tol > 0 ? o.tol : 1e-10;
  const int max_cycles = o.max_outer > 0 ? o.max_outer : 40;
  const double spur = 1e-6 * std::max(1.0, std::fabs(sigma));
  if (sigma == 0.0) fail(FEM2D_E_INVALID_ARG, "target 0 is the null space of the curl-curl operator");

  MFSymbolic sym;
  mf_symbolic(dom, h, sym);
  MFDevice mf;
  mf.setup(c, sym, 32);
  MFFactor fm, fp;
  mf.factor(c, d.a.p, d.b.p, 1.0, -sigma, false, fm);
  // A + c B (c > 0) is SPD: factored without pivoting
  const double cshift = 0.05 * std::fabs(sigma);
  mf.factor(c, d.a.p, d.b.p, 1.0, cshift, true, fp);
  if (fp.flags & 2) fail(FEM2D_E_B_NOT_SPD, "A + c B is not positive definite; B is likely ill-conditioned");
  FEM2D_CUDA(cudaStreamSynchronize(c.stream));
  auto t1 = std::chrono::steady_clock::now();

  Dev D{c, h, d};
  DBuf<double> V, AV, BV, X, W1, W2, W3;
  V.alloc((size_t)n * mmax);
  AV.alloc((size_t)n * mmax);
  BV.alloc((size_t)n * mmax);
  X.alloc((size_t)n * 32);
  W1.alloc((size_t)n * 32);
  W2.alloc((size_t)n * 32);
  W3.alloc((size_t)n * 32);
  int64_t spmv = 0, napply = 0;

  // Out (ld lo) = T In (ld li), nb columns; In and Out may not alias W1..W3
  auto apply_T = [&](const double* In, int64_t li, double* Out, int64_t lo, int nb) {
    D.spmm(0.0, 1.0, In, li, nb, W1.p, 32);
    mf.solve(c, fp, W1.p, 32, W2.p, 32, nb);
    D.spmm(1.0, 0.0, W2.p, 32, nb, W3.p, 32);
    mf.solve(c, fm, W3.p, 32, Out, lo, nb);
    spmv += 2 * nb;
    napply += nb;
  };
  // B-orthonormalise columns [m0, m0+r) of V against [0, m0) and among themselves; returns kept count
  auto borth = [&](int m0, int r) -> int {
    double* Wb = V.p + m0;
    std::vector<double> C, G, w, z;
    for (int pass = 0; pass < 2; pass++) {
      if (m0 > 0) {
        D.spmm(0.0, 1.0, Wb, mmax, r, W1.p, 32);
        D.gram(V.p, mmax, m0, W1.p, 32, r, C);
        for (auto& x : C) x = -x;
        D.gemm(V.p, mmax, m0, C, r, 1.0, Wb, mmax);
      }
    }
    int keep = r;
    for (int pass = 0; pass < 2; pass++) {
      D.spmm(0.0, 1.0, Wb, mmax, keep, W1.p, 32);
      D.gram(Wb, mmax, keep, W1.p, 32, keep, G);
      if (!symeig(keep, G, w, z)) fail(FEM2D_E_NOT_CONVERGED, "Gram eigen-decomposition failed");
      const double wmax = *std::max_element(w.begin(), w.end());
      std::vector<int> kept;
      for (int q = 0; q < keep; q++)
        if (w[q] > (pass == 0 ? 1e-8 : 1e-14) * wmax && w[q] > 0) kept.push_back(q);
      const int nk = (int)kept.size();
      std::vector<double> T((size_t)keep * nk);
      for (int i = 0; i < keep; i++)
        for (int q = 0; q < nk; q++) T[(size_t)i * nk + q] = z[(size_t)i * keep + kept[q]] / std::sqrt(w[kept[q]]);
      if (nk == 0) return 0;
      D.gemm(Wb, mmax, keep, T, nk, 0.0, W2.p, 32);
      D.copy(W2.p, 32, nk, Wb, mmax);
      keep = nk;
      if (m0 > 0) {
        D.spmm(0.0, 1.0, Wb, mmax, keep, W1.p, 32);
        D.gram(V.p, mmax, m0, W1.p, 32, keep, C);
        for (auto& x : C) x = -x;
        D.gemm(V.p, mmax, m0, C, keep, 1.0, Wb, mmax);
      }
    }
    return keep;
  };

  // start block: T applied to a fixed pseudo-random block
  {
    std::vector<double> R0;
    random_block(n, b, 12345, R0);
    DBuf<double> R;
    R.alloc((size_t)n * b);
    FEM2D_CUDA(cudaMemcpyAsync(R.p, R0.data(), R0.size() * sizeof(double), cudaMemcpyHostToDevice, c.stream));
    apply_T(R.p, b, X.p, 32, b);
  }
  std::vector<double> theta_sel, rel_sel;
  std::vector<int> sel;
  int cycles = 0;
  bool converged = false;
  int bx = b;
  for (; cycles < max_cycles; cycles++) {
    D.copy(X.p, 32, bx, V.p, mmax);
    int m = borth(0, bx);
    int last0 = 0, lastn = m;
    for (int s = 0; s < steps && m + lastn <= mmax; s++) {
      apply_T(V.p + last0, mmax, V.p + m, mmax, lastn);
      int r = borth(m, lastn);
      if (r == 0) break;
      last0 = m;
      lastn = r;
      m += r;
    }
    D.spmm(1.0, 0.0, V.p, mmax, m, AV.p, mmax);
    D.spmm(0.0, 1.0, V.p, mmax, m, BV.p, mmax);
    spmv += 2 * m;
    std::vector<double> GA, th, Y;
    D.gram(V.p, mmax, m, AV.p, mmax, m, GA);
    for (int i = 0; i < m; i++)
      for (int j = 0; j < i; j++) GA[(size_t)i * m + j] = GA[(size_t)j * m + i] = 0.5 * (GA[(size_t)i * m + j] + GA[(size_t)j * m + i]);
    if (!symeig(m, GA, th, Y)) fail(FEM2D_E_NOT_CONVERGED, "Rayleigh-Ritz eigen-decomposition failed");
    // Ritz residuals of all m pairs: AV*Y - BV*Y*theta
    const int m2 = m;
    DBuf<double> AY, BY;
    AY.alloc((size_t)n * m2);
    BY.alloc((size_t)n * m2);
    D.gemm(AV.p, mmax, m, Y, m2, 0.0, AY.p, m2);
    D.gemm(BV.p, mmax, m, Y, m2, 0.0, BY.p, m2);
    DBuf<double> th_d, P;
    std::vector<double> thv(th);
    th_d.upload(thv, c.stream);
    const int nblk = std::min<int64_t>(D.grid_rows(), std::max<int64_t>(1, (n + 255) / 256));
    const int64_t rpb = (n + nblk - 1) / nblk;
    P.alloc((size_t)nblk * 2 * m2);
    resid_partial_kernel<<<nblk, 256, 0, c.stream>>>(n, AY.p, BY.p, m2, m2, th_d.p, rpb, P.p);
    c.launches++;
    std::vector<double> Ph((size_t)nblk * 2 * m2);
    FEM2D_CUDA(cudaMemcpyAsync(Ph.data(), P.p, Ph.size() * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    FEM2D_CUDA(cudaStreamSynchronize(c.stream));
    std::vector<double> rel(m2);
    for (int j = 0; j < m2; j++) {
      double sr = 0, sb = 0;
      for (int q = 0; q < nblk; q++) {
        sr += Ph[(size_t)q * 2 * m2 + j];
        sb += Ph[(size_t)q * 2 * m2 + m2 + j];
      }
      rel[j] = std::sqrt(sr) / (std::fabs(th[j]) * std::sqrt(sb) + 1e-300);
    }
    std::vector<int> cand;
    for (int j = 0; j < m2; j++)
      if (std::fabs(th[j]) > spur && rel[j] < 1.0) cand.push_back(j);
    std::stable_sort(cand.begin(), cand.end(),
                     [&](int x, int y) { return std::fabs(th[x] - sigma) < std::fabs(th[y] - sigma); });
    if ((int)cand.size() < k) {
      // not enough credible Ritz pairs yet: keep the nearest non-spurious ones regardless of residual
      cand.clear();
      for (int j = 0; j < m2; j++)
        if (std::fabs(th[j]) > spur) cand.push_back(j);
      std::stable_sort(cand.begin(), cand.end(),
                       [&](int x, int y) { return std::fabs(th[x] - sigma) < std::fabs(th[y] - sigma); });
    }
    sel.assign(cand.begin(), cand.begin() + std::min<size_t>(cand.size(), (size_t)b));
    if ((int)sel.size() < k) fail(FEM2D_E_SPURIOUS, "only spurious (null-space) Ritz values were found");
    bx = (int)sel.size();
    std::vector<double> Ysel((size_t)m * bx);
    for (int i = 0; i < m; i++)
      for (int q = 0; q < bx; q++) Ysel[(size_t)i * bx + q] = Y[(size_t)i * m + sel[q]];
    D.gemm(V.p, mmax, m, Ysel, bx, 0.0, X.p, 32);
    theta_sel.resize(bx);
    rel_sel.resize(bx);
    for (int q = 0; q < bx; q++) {
      theta_sel[q] = th[sel[q]];
      rel_sel[q] = rel[sel[q]];
    }
    double worst = 0;
    for (int q = 0; q < k; q++) worst = std::max(worst, rel_sel[q]);
    if (o.verbose)
      fprintf(stderr, "[gpu_solve_gep] cycle %d basis %d worst residual %.3e  theta0 %.12f\n", cycles, m, worst,
              theta_sel[0]);
    if (worst < tol) {
      converged = true;
      cycles++;
      break;
    }
  }
  FEM2D_CUDA(cudaStreamSynchronize(c.stream));
  auto t2 = std::chrono::steady_clock::now();
  if (st) {
    st->outer_iters = cycles;
    st->inner_iters_total = (int)napply;
    st->converged = converged ? 1 : 0;
    st->t_setup_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
    st->t_solve_ms = std::chrono::duration<double, std::milli>(t2 - t1).count();
    double w = 0;
    for (int q = 0; q < k; q++) w = std::max(w, rel_sel[q]);
    st->max_rel_residual = w;
    st->spmv_count = spmv;
  }
  // outputs: B-normalised (the Ritz vectors are B-orthonormal), sign fixed by the largest entry
  std::vector<double> Xh((size_t)n * 32);
  FEM2D_CUDA(cudaMemcpyAsync(Xh.data(), X.p, Xh.size() * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
  FEM2D_CUDA(cudaStreamSynchronize(c.stream));
  for (int q = 0; q < k; q++) {
    if (values) values[q] = theta_sel[q];
    if (residuals) residuals[q] = rel_sel[q];
    if (vectors) {
      int64_t imax = 0;
      for (int64_t i = 0; i < n; i++)
        if (std::fabs(Xh[(size_t)i * 32 + q]) > std::fabs(Xh[(size_t)imax * 32 + q])) imax = i;
      const double sgn = Xh[(size_t)imax * 32 + q] < 0 ? -1.0 : 1.0;
      for (int64_t i = 0; i < n; i++) vectors[(size_t)q * n + i] = sgn * Xh[(size_t)i * 32 + q];
    }
  }
  if (!converged)
    fail(FEM2D_E_NOT_CONVERGED, "gpu_solve_gep did not reach the residual tolerance (outputs hold the last iterate)");
}

// ================================================================ dense solve (nalgebra_solve_gep)
void dense_solve(Ctx& c, const Domain& dom, const HostGEP& h, const DeviceGEP& d, double target, double* value,
                 double* vector) {
  const int64_t n = h.n;
  if (n > 1000) fail(FEM2D_E_TOO_LARGE, "Matrices Exceeded Maximum Size (1000x1000); Cannot Solve!");
  MFSymbolic sym;
  mf_symbolic(dom, h, sym);
  MFDevice mf;
  mf.setup(c, sym, 32);
  MFFactor fb;
  mf.factor(c, d.a.p, d.b.p, 0.0, 1.0, true, fb);
  if (fb.flags & 2) fail(FEM2D_E_B_NOT_SPD, "Failed to invert B-matrix (via cholesky); likely ill-conditioned!");
  DBuf<double> Ad, Z;
  Ad.alloc((size_t)n * n);
  Z.alloc((size_t)n * n);
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

void shifted_solve(Ctx& c, const Domain& dom, const HostGEP& h, const DeviceGEP& d, double ca, double cb, bool spd,
                   int nrhs, const double* rhs, double* x) {
  const int64_t n = h.n;
  MFSymbolic sym;
  mf_symbolic(dom, h, sym);
  MFDevice mf;
  mf.setup(c, sym, 32);
  MFFactor fac;
  mf.factor(c, d.a.p, d.b.p, ca, cb, spd, fac);
  if (spd && (fac.flags & 2)) fail(FEM2D_E_B_NOT_SPD, "the shifted matrix is not positive definite");
  DBuf<double> R, X;
  R.alloc((size_t)n * 32);
  X.alloc((size_t)n * 32);
  std::vector<double> hr((size_t)n * 32), hx((size_t)n * 32);
  for (int c0 = 0; c0 < nrhs; c0 += 32) {
    const int w = std::min(32, nrhs - c0);
    for (int64_t i = 0; i < n; i++)
      for (int k = 0; k < w; k++) hr[(size_t)i * 32 + k] = rhs[(size_t)i * nrhs + c0 + k];
    FEM2D_CUDA(cudaMemcpyAsync(R.p, hr.data(), hr.size() * sizeof(double), cudaMemcpyHostToDevice, c.stream));
    mf.solve(c, fac, R.p, 32, X.p, 32, w);
    FEM2D_CUDA(cudaMemcpyAsync(hx.data(), X.p, hx.size() * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    FEM2D_CUDA(cudaStreamSynchronize(c.stream));
    for (int64_t i = 0; i < n; i++)
      for (int k = 0; k < w; k++) x[(size_t)i * nrhs + c0 + k] = hx[(size_t)i * 32 + k];
  }
}

}  // namespace fem2d
