// Device numeric phase of galerkin_sample_gep_hcurl.
//
// K1 fem2d_contract1d_kernel: the 1-D quadrature contractions (basis x quad-point x basis) between
//    the shape-function families of an outer Elem sampled over a dyadic sub-interval and of the inner
//    Elem (glq.rs:19-32 restricted to one axis; shape functions hierarchical_basis_fns.rs).
// K2 fem2d_values_kernel: one thread per entry of the full symmetric CSR; sums its visits, each the
//    product C * Gu * Gv that equals the reference's 2-D sum (integrals.rs:26-92, 292-354) for affine
//    Elems. FP64 throughout, deterministic (fixed summation order, no atomics). HBM-bound: the
//    traffic is the contribution list read and the two FP64 value arrays written.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>

#include "device.h"
#include "contract.cuh"

namespace fem2d {

namespace {

__global__ void fem2d_contract1d_kernel(int basis, int P, int nivl, const double* __restrict__ ivl,
                                        const double* __restrict__ glq, int nq_u, int nq_v,
                                        double* __restrict__ tables) {
  contract1d_table(basis, P, nivl, blockIdx.x, blockIdx.y, blockIdx.z, ivl, glq, nq_u, nq_v, tables);
}

__global__ void __launch_bounds__(256) fem2d_values_kernel(int64_t nnz, const int32_t* __restrict__ fsrc,
                                                           const int64_t* __restrict__ vptr,
                                                           const uint64_t* __restrict__ codes,
                                                           const GBlock* __restrict__ blocks,
                                                           const uint32_t* __restrict__ specs,
                                                           const double* __restrict__ tables, int P, int nivl,
                                                           double* __restrict__ A, double* __restrict__ B) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nnz; e += (int64_t)gridDim.x * blockDim.x) {
    double sa, sb;
    const int64_t u = __ldg(fsrc + e);   // the upper entry whose visits this entry sums
    entry_values(__ldg(vptr + u), __ldg(vptr + u + 1), codes, blocks, specs, tables, P, nivl, sa, sb);
    A[e] = sa;
    B[e] = sb;
  }
}

}  // namespace

std::vector<int32_t> row_runs(const HostGEP& g) {
  std::vector<int32_t> grp{0};
  for (int64_t i = 1; i <= g.n; i++) {
    const int64_t h = grp.back();
    bool brk = i == g.n || i - h >= 64;
    if (!brk) {
      const int64_t li = g.row_ptr[i + 1] - g.row_ptr[i], lh = g.row_ptr[h + 1] - g.row_ptr[h];
      brk = li != lh || std::memcmp(g.col.data() + g.row_ptr[i], g.col.data() + g.row_ptr[h], li * sizeof(int32_t)) != 0;
    }
    if (brk) grp.push_back((int32_t)i);
  }
  if (g.n == 0) grp.assign(1, 0);
  return grp;
}

void device_upload(Ctx& c, const HostGEP& g, DeviceGEP& d) {
  cudaStream_t s = c.stream;
  d.row_ptr.upload(g.row_ptr, s);
  d.col.upload(g.col, s);
  d.vptr.upload(g.vptr, s);
  d.fsrc.upload(g.fsrc, s);
  d.codes.upload(g.codes, s);
  d.blocks.upload(g.blocks, s);
  d.specs.upload(g.specs, s);
  std::vector<double> iv(2 * g.ivl_s.size());
  for (size_t k = 0; k < g.ivl_s.size(); k++) {
    iv[2 * k] = g.ivl_s[k];
    iv[2 * k + 1] = g.ivl_o[k];
  }
  d.ivl.upload(iv, s);
  d.nivl = (int)g.ivl_s.size();
  std::vector<double> q;
  q.insert(q.end(), g.glq_u_x.begin(), g.glq_u_x.end());
  q.insert(q.end(), g.glq_u_w.begin(), g.glq_u_w.end());
  q.insert(q.end(), g.glq_v_x.begin(), g.glq_v_x.end());
  q.insert(q.end(), g.glq_v_w.begin(), g.glq_v_w.end());
  d.glq.upload(q, s);
  const int P = g.pmax + 1;
  d.tables.alloc((size_t)2 * d.nivl * 5 * P * P);
  d.a.alloc(g.nnz_full);
  d.b.alloc(g.nnz_full);
  // rows of one Elem's interior functions share their column list; the operator products stage each
  // run's gathered X rows once (eigen.cu spmm_group_kernel, ozaki.cu spmm_tc_kernel)
  std::vector<int32_t> grp = row_runs(g);
  std::vector<int2> work;
  for (size_t q = 0; q + 1 < grp.size(); q++) {
    const int64_t len = g.row_ptr[grp[q] + 1] - g.row_ptr[grp[q]];
    for (int64_t c0 = 0; c0 < std::max<int64_t>(len, 1); c0 += 256) work.push_back(make_int2((int)q, (int)c0));
  }
  d.grp.upload(grp, s);
  d.grp_h = grp;
  d.gwork.upload(work, s);
  d.ngrp = (int)grp.size() - 1;
  d.nwork = (int)work.size();
  d.h2d_bytes = (int64_t)(grp.size() * 4 + work.size() * 8 + g.row_ptr.size() * 8 + g.col.size() * 4 + g.vptr.size() * 8 + g.fsrc.size() * 4 + g.codes.size() * 8 +
                          g.blocks.size() * sizeof(GBlock) + g.specs.size() * 4 + iv.size() * 8 + q.size() * 8);
}

void device_assemble(Ctx& c, const HostGEP& g, DeviceGEP& d, float* ms_tables, float* ms_values) {
  cudaStream_t s = c.stream;
  cudaEvent_t e0, e1, e2;
  FEM2D_CUDA(cudaEventCreate(&e0));
  FEM2D_CUDA(cudaEventCreate(&e1));
  FEM2D_CUDA(cudaEventCreate(&e2));
  const int P = g.pmax + 1;
  FEM2D_CUDA(cudaEventRecord(e0, s));
  dim3 grid1(d.nivl, 2, 5);
  fem2d_contract1d_kernel<<<grid1, 128, 0, s>>>(g.basis, P, d.nivl, d.ivl.p, d.glq.p, g.nq_u, g.nq_v, d.tables.p);
  FEM2D_CUDA(cudaGetLastError());
  c.launches++;
  FEM2D_CUDA(cudaEventRecord(e1, s));
  if (g.nnz_full > 0) {
    ProfScope ps(c, "assembly_values", 20.0 * g.nnz_full + 8.0 * (g.nnz_upper + 1) + 8.0 * g.codes.size());
    const int threads = 256;
    int64_t want = (g.nnz_full + threads - 1) / threads;
    int64_t cap = (int64_t)c.num_sms * 8 * 4;   // persistent-ish grid: 8 blocks/SM x 4 waves
    int grid = (int)std::max<int64_t>(1, std::min(want, cap));
    fem2d_values_kernel<<<grid, threads, 0, s>>>(g.nnz_full, d.fsrc.p, d.vptr.p, d.codes.p, d.blocks.p, d.specs.p,
                                                 d.tables.p, P, d.nivl, d.a.p, d.b.p);
    FEM2D_CUDA(cudaGetLastError());
    c.launches++;
  }
  FEM2D_CUDA(cudaEventRecord(e2, s));
  FEM2D_CUDA(cudaEventSynchronize(e2));
  float t1 = 0, t2 = 0;
  cudaEventElapsedTime(&t1, e0, e1);
  cudaEventElapsedTime(&t2, e1, e2);
  if (ms_tables) *ms_tables = t1;
  if (ms_values) *ms_values = t2;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaEventDestroy(e2);
}

}  // namespace fem2d

// ---------------------------------------------------------------------------------------------------
// Assembly values without any device allocation.
//
// For hosts that own every byte of device memory themselves (an application that hands the library
// pointers from its own pool or arena and forbids allocations behind its back) or that cannot pay for
// cudaMalloc/cudaFree on their critical path (cudaFree synchronises the device). The 1-D contraction
// tables that the two assembly kernels exchange live in this file-scope array instead of a buffer
// allocated per GEP. Every GPU that loads the library holds the array until the process exits.
// ---------------------------------------------------------------------------------------------------
namespace fem2d {

namespace {
constexpr size_t kNoAllocTableDoubles = 524288;   // 4 MiB of FP64 contraction tables
__device__ __align__(256) double g_noalloc_tables[kNoAllocTableDoubles];

// device address of g_noalloc_tables per device ordinal, looked up once per device
std::mutex g_noalloc_mu;
double* g_noalloc_addr[256] = {};
}  // namespace

size_t noalloc_table_capacity() { return kNoAllocTableDoubles; }

void device_values_noalloc(Ctx& c, const HostGEP& g, const DeviceGEP& d, double* out_a, double* out_b) {
  const int P = g.pmax + 1;
  const size_t need = (size_t)2 * d.nivl * 5 * P * P;
  if (need > kNoAllocTableDoubles)
    fail(FEM2D_E_TOO_LARGE, "the contraction tables need " + std::to_string(need) +
                                " doubles; the allocation-free path holds at most " +
                                std::to_string(kNoAllocTableDoubles) + " (2 x intervals x 5 x (max order + 1)^2)");
  if (c.device < 0 || c.device >= 256) fail(FEM2D_E_INVALID_ARG, "device ordinal out of range");
  double* tables = nullptr;
  {
    // The array's device address, taken on this device (the caller made it current). It is looked up
    // again on every call made outside a stream capture, so a context rebuilt after cudaDeviceReset
    // (which reloads the module at a new address) is picked up; inside a capture the address from the
    // last call outside one is used, which is why the first call on a device must precede any capture.
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    FEM2D_CUDA(cudaStreamIsCapturing(c.stream, &cap));
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (cap == cudaStreamCaptureStatusNone || !g_noalloc_addr[c.device]) {
      if (cap != cudaStreamCaptureStatusNone)
        fail(FEM2D_E_INVALID_ARG, "first allocation-free call on a device inside a stream capture");
      void* p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_tables);
      if (e != cudaSuccess) fail(FEM2D_E_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      g_noalloc_addr[c.device] = static_cast<double*>(p);
    }
    tables = g_noalloc_addr[c.device];
  }
  // every table entry the values kernel reads is written by the contraction kernel first, so the
  // previous call's contents never leak into this one
  dim3 grid1(d.nivl, 2, 5);
  fem2d_contract1d_kernel<<<grid1, 128, 0, c.stream>>>(g.basis, P, d.nivl, d.ivl.p, d.glq.p, g.nq_u, g.nq_v, tables);
  FEM2D_CUDA(cudaGetLastError());
  c.launches++;
  if (g.nnz_full > 0) {
    const int threads = 256;
    int64_t want = (g.nnz_full + threads - 1) / threads;
    int64_t cap = (int64_t)c.num_sms * 8 * 4;
    int grid = (int)std::max<int64_t>(1, std::min(want, cap));
    fem2d_values_kernel<<<grid, threads, 0, c.stream>>>(g.nnz_full, d.fsrc.p, d.vptr.p, d.codes.p, d.blocks.p,
                                                        d.specs.p, tables, P, d.nivl, out_a, out_b);
    FEM2D_CUDA(cudaGetLastError());
    c.launches++;
  }
}

}  // namespace fem2d
