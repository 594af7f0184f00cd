// Batched assembly: the numeric phase of many GEPs (independent meshes, each with its own orders,
// intervals and GLQ) in two launches in total, instead of two per GEP.
//
//  * fem2d_contract1d_batch_kernel: one CTA per (interval of any GEP, axis, kind); a CTA finds its GEP
//    by binary search over the interval prefix sums and writes that GEP's 1-D contraction table.
//  * fem2d_values_batch_kernel: a persistent grid (a whole number of CTAs per SM) strides over the
//    concatenated index space of all full CSR entries of all GEPs; each entry finds its GEP by
//    binary search over the entry prefix sums and sums its visits into that GEP's own A and B arrays.
//
// Entries of uneven expansion orders (short and long contribution lists) share one launch, so the
// tail of one GEP overlaps the head of the next. The launch shape (threads per CTA, CTAs per SM) is
// picked by timing a fixed candidate list on the batch itself and cached per (device, table stride,
// size class); the cache can be exported and imported as text.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "batch.h"
#include "contract.cuh"

namespace fem2d {

namespace {

struct BatchItem {
  const int32_t* fsrc;
  const int64_t* vptr;
  const uint64_t* codes;
  const GBlock* blocks;
  const uint32_t* specs;
  const double* ivl;
  const double* glq;
  double* tables;
  double* A;
  double* B;
  int32_t P, nivl, basis, nq_u, nq_v, pad;
};

// largest i in [0, count) with pref[i] <= x (pref ascending, pref[0] = 0)
__device__ __forceinline__ int find_item(const int64_t* __restrict__ pref, int count, int64_t x) {
  int lo = 0, hi = count - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(pref + mid) <= x) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

__global__ void fem2d_contract1d_batch_kernel(const BatchItem* __restrict__ items, const int64_t* __restrict__ ivl_pref,
                                              int count) {
  const int it = find_item(ivl_pref, count, blockIdx.x);
  const BatchItem b = items[it];
  const int iv = (int)(blockIdx.x - ivl_pref[it]);
  contract1d_table(b.basis, b.P, b.nivl, iv, blockIdx.y, blockIdx.z, b.ivl, b.glq, b.nq_u, b.nq_v, b.tables);
}

__global__ void fem2d_values_batch_kernel(const BatchItem* __restrict__ items, const int64_t* __restrict__ nnz_pref,
                                          int count, int64_t total) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int it = find_item(nnz_pref, count, e);
    const BatchItem& b = items[it];
    const int64_t local = e - __ldg(nnz_pref + it);
    const int64_t u = __ldg(b.fsrc + local);
    double sa, sb;
    entry_values(__ldg(b.vptr + u), __ldg(b.vptr + u + 1), b.codes, b.blocks, b.specs, b.tables, b.P, b.nivl, sa, sb);
    b.A[local] = sa;
    b.B[local] = sb;
  }
}

std::mutex g_tune_mu;
std::map<std::string, LaunchShape> g_tune;

const LaunchShape kCandidates[] = {{128, 4}, {128, 8}, {128, 16}, {256, 2}, {256, 4}, {256, 8},
                                   {512, 1}, {512, 2}, {512, 4},  {1024, 1}, {1024, 2}};

std::string tune_key(int device, int P, int64_t total) {
  cudaDeviceProp prop;
  std::string name = "device" + std::to_string(device);
  if (cudaGetDeviceProperties(&prop, device) == cudaSuccess) name = prop.name;
  for (auto& ch : name)
    if (ch == ' ' || ch == '|') ch = '_';
  const int cls = total > 0 ? (int)std::floor(std::log2((double)total)) : 0;
  return name + "|values|P" + std::to_string(P) + "|nnz2^" + std::to_string(cls);
}

void launch_values(Ctx& c, const LaunchShape& s, const BatchItem* items, const int64_t* pref, int count,
                   int64_t total) {
  const int64_t want = (total + s.threads - 1) / s.threads;
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)c.num_sms * s.ctas_per_sm));
  fem2d_values_batch_kernel<<<grid, s.threads, 0, c.stream>>>(items, pref, count, total);
  c.launches++;
}

}  // namespace

void batch_assemble(Ctx& c, const std::vector<BatchMember>& members, bool autotune, BatchReport* rep) {
  const int count = (int)members.size();
  if (count == 0) return;
  std::vector<BatchItem> items(count);
  std::vector<int64_t> nnz_pref(count + 1, 0), ivl_pref(count + 1, 0);
  int Pmax = 0;
  for (int i = 0; i < count; i++) {
    const HostGEP& h = *members[i].h;
    DeviceGEP& d = *members[i].d;
    BatchItem& b = items[i];
    b.fsrc = d.fsrc.p;
    b.vptr = d.vptr.p;
    b.codes = d.codes.p;
    b.blocks = d.blocks.p;
    b.specs = d.specs.p;
    b.ivl = d.ivl.p;
    b.glq = d.glq.p;
    b.tables = d.tables.p;
    b.A = d.a.p;
    b.B = d.b.p;
    b.P = h.pmax + 1;
    b.nivl = d.nivl;
    b.basis = h.basis;
    b.nq_u = h.nq_u;
    b.nq_v = h.nq_v;
    b.pad = 0;
    nnz_pref[i + 1] = nnz_pref[i] + h.nnz_full;
    ivl_pref[i + 1] = ivl_pref[i] + d.nivl;
    Pmax = std::max(Pmax, b.P);
  }
  const int64_t total = nnz_pref[count];
  const int64_t total_ivl = ivl_pref[count];
  if (total_ivl > 0x7fffffff) fail(FEM2D_E_TOO_LARGE, "too many intervals in one batch");
  DBuf<uint8_t> raw;
  std::vector<uint8_t> bytes(sizeof(BatchItem) * count);
  std::memcpy(bytes.data(), items.data(), bytes.size());
  raw.upload(bytes, c.stream);
  DBuf<int64_t> np, ip;
  np.upload(nnz_pref, c.stream);
  ip.upload(ivl_pref, c.stream);
  const BatchItem* di = reinterpret_cast<const BatchItem*>(raw.p);

  cudaEvent_t e0, e1, f0, e2;
  FEM2D_CUDA(cudaEventCreate(&e0));
  FEM2D_CUDA(cudaEventCreate(&e1));
  FEM2D_CUDA(cudaEventCreate(&f0));
  FEM2D_CUDA(cudaEventCreate(&e2));
  FEM2D_CUDA(cudaEventRecord(e0, c.stream));
  if (total_ivl > 0) {
    fem2d_contract1d_batch_kernel<<<dim3((unsigned)total_ivl, 2, 5), 128, 0, c.stream>>>(di, ip.p, count);
    c.launches++;
    FEM2D_CUDA(cudaGetLastError());
  }
  FEM2D_CUDA(cudaEventRecord(e1, c.stream));

  LaunchShape shape{256, 8};
  bool tuned = false;
  const std::string key = tune_key(c.device, Pmax, total);
  if (autotune && total > 0) {
    {
      std::lock_guard<std::mutex> lk(g_tune_mu);
      auto it = g_tune.find(key);
      if (it != g_tune.end()) {
        shape = it->second;
        tuned = true;
      }
    }
    if (!tuned) {
      // time every candidate on this batch (the outputs are rewritten with identical values)
      cudaEvent_t a, b;
      FEM2D_CUDA(cudaEventCreate(&a));
      FEM2D_CUDA(cudaEventCreate(&b));
      float best = 1e30f;
      for (const LaunchShape& s : kCandidates) {
        launch_values(c, s, di, np.p, count, total);   // warm-up
        FEM2D_CUDA(cudaEventRecord(a, c.stream));
        for (int r = 0; r < 3; r++) launch_values(c, s, di, np.p, count, total);
        FEM2D_CUDA(cudaEventRecord(b, c.stream));
        FEM2D_CUDA(cudaEventSynchronize(b));
        FEM2D_CUDA(cudaGetLastError());
        float ms = 0;
        cudaEventElapsedTime(&ms, a, b);
        if (ms < best) {
          best = ms;
          shape = s;
        }
      }
      cudaEventDestroy(a);
      cudaEventDestroy(b);
      std::lock_guard<std::mutex> lk(g_tune_mu);
      g_tune[key] = shape;
      tuned = true;
    }
  }
  FEM2D_CUDA(cudaEventRecord(f0, c.stream));   // the final launch is timed alone
  if (total > 0) {
    launch_values(c, shape, di, np.p, count, total);
    FEM2D_CUDA(cudaGetLastError());
  }
  FEM2D_CUDA(cudaEventRecord(e2, c.stream));
  FEM2D_CUDA(cudaEventSynchronize(e2));
  float t1 = 0, t2 = 0;
  cudaEventElapsedTime(&t1, e0, e1);
  cudaEventElapsedTime(&t2, f0, e2);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaEventDestroy(f0);
  cudaEventDestroy(e2);
  if (rep) {
    rep->ms_tables = t1;
    rep->ms_values = t2;
    rep->shape = shape;
    rep->total_entries = total;
    int64_t codes = 0;
    for (const auto& m : members) codes += (int64_t)m.h->codes.size();
    rep->total_codes = codes;
    rep->key = key;
  }
}

std::string tune_export() {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  std::ostringstream os;
  for (const auto& kv : g_tune) os << kv.first << ' ' << kv.second.threads << ' ' << kv.second.ctas_per_sm << '\n';
  return os.str();
}

int tune_import(const std::string& text) {
  std::istringstream is(text);
  std::string key;
  int t, k, n = 0;
  std::map<std::string, LaunchShape> add;
  while (is >> key >> t >> k) {
    bool ok = false;
    for (const LaunchShape& s : kCandidates) ok = ok || (s.threads == t && s.ctas_per_sm == k);
    if (!ok) fail(FEM2D_E_INVALID_ARG, "launch shape " + std::to_string(t) + "x" + std::to_string(k) +
                                           " is not one of the autotuner's candidates");
    add[key] = LaunchShape{t, k};
    n++;
  }
  std::lock_guard<std::mutex> lk(g_tune_mu);
  for (auto& kv : add) g_tune[kv.first] = kv.second;
  return n;
}

void tune_clear() {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune.clear();
}

}  // namespace fem2d
