// Device context and device-resident GEP.
#pragma once
#include <cuda_runtime.h>

#include <chrono>
#include <cstdint>
#include <map>
#include <string>
#include <vector>

#include "common.h"
#include "gep.h"

namespace fem2d {

#define FEM2D_CUDA(call)                                                                          \
  do {                                                                                            \
    cudaError_t _e = (call);                                                                      \
    if (_e != cudaSuccess)                                                                        \
      ::fem2d::fail(FEM2D_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e));            \
  } while (0)

struct ProfRec {
  double ms = 0, bytes = 0, flops = 0;
  int64_t count = 0;
};

struct Ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  int64_t launches = 0;        // kernels launched by this library on this context
  void* flush_buf = nullptr;   // 256 MiB, for L2 flushes between timed repetitions
  int num_sms = 0;
  bool profile = false;        // time named regions with events (synchronising) when set
  std::map<std::string, ProfRec> prof;
  cudaEvent_t t0 = nullptr, t1 = nullptr;
};

// Times a region on the context's stream with CUDA events when profiling is enabled.
struct ProfScope {
  Ctx& c;
  const char* name;
  double bytes, flops;
  cudaEvent_t a = nullptr, b = nullptr;
  ProfScope(Ctx& ctx, const char* n, double by, double fl = 0.0) : c(ctx), name(n), bytes(by), flops(fl) {
    if (!c.profile) return;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    cudaEventRecord(a, c.stream);
  }
  ~ProfScope() {
    if (!c.profile) return;
    cudaEventRecord(b, c.stream);
    cudaEventSynchronize(b);
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    ProfRec& r = c.prof[name];
    r.ms += ms;
    r.bytes += bytes;
    r.flops += flops;
    r.count++;
    cudaEventDestroy(a);
    cudaEventDestroy(b);
  }
};

// Times host work (wall clock, after draining the stream) when profiling is enabled, under a region name.
struct HostScope {
  Ctx& c;
  const char* name;
  double flops = 0.0;   // algorithmic FLOPs of the region, set by its owner before the scope ends
  std::chrono::steady_clock::time_point t0;
  HostScope(Ctx& ctx, const char* n) : c(ctx), name(n) {
    if (!c.profile) return;
    cudaStreamSynchronize(c.stream);
    t0 = std::chrono::steady_clock::now();
  }
  ~HostScope() {
    if (!c.profile) return;
    ProfRec& r = c.prof[name];
    r.ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    r.flops += flops;
    r.count++;
  }
};

// A device buffer owned by this library.
// Buffers that live for one call on one stream (solver temporaries, numeric factors) use the
// stream-ordered allocator (alloc_on): their release does not synchronise the device, so concurrent
// solves on other streams keep running. Buffers that outlive the call use alloc.
void enable_stream_pool(int device);   // once per device: freed stream-ordered memory stays cached

template <class T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  cudaStream_t st = nullptr;   // set when the buffer came from the stream-ordered allocator
  DBuf() = default;
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  ~DBuf() { release(); }
  void release() {
    if (p) {
      if (st) cudaFreeAsync(p, st);
      else cudaFree(p);
    }
    p = nullptr;
    n = 0;
    st = nullptr;
  }
  void alloc(size_t count) {
    release();
    if (count == 0) return;
    FEM2D_CUDA(cudaMalloc(&p, count * sizeof(T)));
    n = count;
  }
  void alloc_on(size_t count, cudaStream_t s) {
    release();
    if (count == 0) return;
    FEM2D_CUDA(cudaMallocAsync(&p, count * sizeof(T), s));
    n = count;
    st = s;
  }
  template <class Alloc>
  void upload_on(const std::vector<T, Alloc>& v, cudaStream_t s) {
    alloc_on(v.size(), s);
    if (!v.empty()) FEM2D_CUDA(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s));
  }
  template <class Alloc>
  void upload(const std::vector<T, Alloc>& v, cudaStream_t s) {
    alloc(v.size());
    if (!v.empty()) FEM2D_CUDA(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s));
  }
};

struct DeviceGEP {
  DBuf<int64_t> row_ptr, vptr;
  DBuf<int32_t> col, fsrc;
  DBuf<uint64_t> codes;
  DBuf<GBlock> blocks;
  DBuf<uint32_t> specs;
  DBuf<double> ivl, glq, tables;   // ivl: (s, o) pairs; glq: u x, u w, v x, v w
  DBuf<double> a, b;               // values, full symmetric CSR order
  // runs of consecutive rows with identical column lists (at most 64 rows each): row starts, ngrp + 1;
  // work items (run, first column of a <= 256-column segment) for the operator products
  DBuf<int32_t> grp;
  std::vector<int32_t> grp_h;   // the same run starts on the host
  DBuf<int2> gwork;
  int ngrp = 0, nwork = 0;
  int nivl = 0;
  int64_t h2d_bytes = 0;
};

// assemble.cu
// runs of at most 64 consecutive rows with one column list: run starts, then n (the GEP's pattern)
std::vector<int32_t> row_runs(const HostGEP& g);
void device_upload(Ctx& c, const HostGEP& g, DeviceGEP& d);
// launches the table kernel and the value kernel; returns device times in ms (tables, values)
void device_assemble(Ctx& c, const HostGEP& g, DeviceGEP& d, float* ms_tables, float* ms_values);
// the same two kernels with the tables in a file-scope device array; writes caller-owned A and B
void device_values_noalloc(Ctx& c, const HostGEP& g, const DeviceGEP& d, double* out_a, double* out_b);
size_t noalloc_table_capacity();
// peaks.cu: measured FP64 FMA throughput (TFLOP/s) on the context's device
double measure_fp64_peak(Ctx& c);

}  // namespace fem2d
