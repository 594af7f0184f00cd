// extern "C" boundary of fem2d_gb300 (declared in include/fem2d_gb300.h).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <fstream>
#include <memory>
#include <mutex>
#include <sstream>

#include "byparts.h"
#include "common.h"
#include "device.h"
#include "domain.h"
#include "eigen.h"
#include "fields.h"
#include "gep.h"
#include "mesh.h"
#include "batch.h"
#include "mf.h"
#include "petsc_io.h"
#include "precond.h"

namespace fem2d {
static thread_local std::string g_last_error;
void set_last_error(const std::string& msg) { g_last_error = msg; }
void build_symbolic(const Domain& d, int basis, int nq_u, int nq_v, HostGEP& g);
}  // namespace fem2d

using namespace fem2d;

struct fem2d_mesh { Mesh m; };
struct fem2d_domain { Domain d; };
struct fem2d_ctx { Ctx c; };
struct fem2d_fields { FieldSpace f; };
struct fem2d_patchnet { PatchNet net; };
struct fem2d_pcg {
  std::unique_ptr<PCGSolver> s;
  int64_t n = 0;
  int device = 0;
};
struct fem2d_gep {
  Domain dom;   // the Domain the GEP was sampled from (its Elem trees drive the factorization)
  HostGEP h;
  DeviceGEP d;
  Ctx* ctx = nullptr;
  int device = 0;   // kept apart from ctx: freeing must not read a context that may already be gone
  double t_symbolic_ms = 0, t_tables_ms = 0, t_values_ms = 0, t_upload_ms = 0;
  mutable MFPlan plan;   // factorization plan, built by the first solve and reused (pattern-only)
};

#define API_BEGIN try {
#define API_END                      \
  }                                  \
  catch (const Error& e) {           \
    set_last_error(e.what());        \
    return e.code;                   \
  }                                  \
  catch (const std::bad_alloc&) {    \
    set_last_error("out of memory"); \
    return FEM2D_E_INVALID_ARG;      \
  }                                  \
  catch (const std::exception& e) {  \
    set_last_error(e.what());        \
    return FEM2D_E_INVALID_ARG;      \
  }                                  \
  return FEM2D_OK;

static std::vector<int64_t> id_list(const int64_t* ids, int64_t n) {
  if (n < 0) fail(FEM2D_E_INVALID_ARG, "negative id count");
  if (n > 0 && !ids) fail(FEM2D_E_INVALID_ARG, "null id list");
  return std::vector<int64_t>(ids, ids + n);
}

extern "C" {

const char* fem2d_last_error(void) { return g_last_error.c_str(); }
const char* fem2d_version(void) { return "fem2d_gb300 0.1 (sm_103a)"; }

// ------------------------------------------------------------------ mesh
int fem2d_mesh_from_json(const char* json_text, fem2d_mesh** out) {
  API_BEGIN
  if (!json_text || !out) fail(FEM2D_E_INVALID_ARG, "null argument");
  auto* m = new fem2d_mesh{Mesh::from_json(json_text)};
  *out = m;
  API_END
}

int fem2d_mesh_from_file(const char* path, fem2d_mesh** out) {
  API_BEGIN
  if (!path || !out) fail(FEM2D_E_INVALID_ARG, "null argument");
  std::ifstream f(path);
  if (!f) fail(FEM2D_E_IO, std::string("cannot open mesh file ") + path);
  std::stringstream ss;
  ss << f.rdbuf();
  *out = new fem2d_mesh{Mesh::from_json(ss.str())};
  API_END
}

int fem2d_mesh_unit(fem2d_mesh** out) {
  API_BEGIN
  if (!out) fail(FEM2D_E_INVALID_ARG, "null argument");
  *out = new fem2d_mesh{Mesh::unit()};
  API_END
}

int fem2d_mesh_clone(const fem2d_mesh* m, fem2d_mesh** out) {
  API_BEGIN
  if (!m || !out) fail(FEM2D_E_INVALID_ARG, "null argument");
  *out = new fem2d_mesh{m->m};
  API_END
}

void fem2d_mesh_free(fem2d_mesh* m) { delete m; }

int fem2d_mesh_set_expansion_orders(fem2d_mesh* m, const int64_t* ids, int64_t n, int i, int j) {
  API_BEGIN
  if (!m) fail(FEM2D_E_INVALID_ARG, "null mesh");
  std::vector<int64_t> v;
  if (!ids)
    for (size_t e = 0; e < m->m.elems.size(); e++) v.push_back((int64_t)e);
  else
    v = id_list(ids, n);
  m->m.set_expansion(v, i, j);
  API_END
}

int fem2d_mesh_p_refine(fem2d_mesh* m, const int64_t* ids, int64_t n, int di, int dj) {
  API_BEGIN
  if (!m) fail(FEM2D_E_INVALID_ARG, "null mesh");
  if (!ids) {
    std::vector<int64_t> v;
    for (size_t e = 0; e < m->m.elems.size(); e++) v.push_back((int64_t)e);
    m->m.p_refine(v, di, dj, true);
  } else {
    m->m.p_refine(id_list(ids, n), di, dj, false);
  }
  API_END
}

int fem2d_mesh_h_refine(fem2d_mesh* m, const int64_t* ids, int64_t n, int kind, int ext) {
  API_BEGIN
  if (!m) fail(FEM2D_E_INVALID_ARG, "null mesh");
  if (kind < 0 || kind > 2 || ext < -1 || ext > 1 || (kind == 0 && ext != -1))
    fail(FEM2D_E_HREF, "invalid h-refinement kind");
  if (!ids) m->m.global_h_refinement(kind, ext);
  else m->m.h_refine_elems(id_list(ids, n), kind, ext);
  API_END
}

int fem2d_mesh_execute_h_refinements(fem2d_mesh* m, const int64_t* ids, const int32_t* kinds, int64_t n) {
  API_BEGIN
  if (!m || (n > 0 && (!ids || !kinds))) fail(FEM2D_E_INVALID_ARG, "null argument");
  std::vector<int64_t> v = id_list(ids, n);
  std::vector<int> k(kinds, kinds + n);
  for (int x : k)
    if (x < 0 || x > 2) fail(FEM2D_E_HREF, "invalid h-refinement kind");
  m->m.execute_h_refinements(v, k, std::vector<int>(n, -1));
  API_END
}

int64_t fem2d_mesh_num_elems(const fem2d_mesh* m) { return m ? (int64_t)m->m.elems.size() : -1; }
int64_t fem2d_mesh_num_edges(const fem2d_mesh* m) { return m ? (int64_t)m->m.edges.size() : -1; }
int64_t fem2d_mesh_num_nodes(const fem2d_mesh* m) { return m ? (int64_t)m->m.nodes.size() : -1; }

int fem2d_mesh_elem_info(const fem2d_mesh* m, int64_t* out) {
  API_BEGIN
  if (!m || !out) fail(FEM2D_E_INVALID_ARG, "null argument");
  for (size_t e = 0; e < m->m.elems.size(); e++) {
    const MElem& el = m->m.elems[e];
    int64_t* o = out + 14 * e;
    o[0] = el.leaf() ? 1 : 0;
    o[1] = el.ni;
    o[2] = el.nj;
    o[3] = el.anc.empty() ? -1 : el.anc.back();
    for (int k = 0; k < 4; k++) o[4 + k] = el.nodes[k];
    for (int k = 0; k < 4; k++) o[8 + k] = el.edges[k];
    o[12] = el.hu;
    o[13] = el.hv;
  }
  API_END
}

int fem2d_mesh_elem_bounds(const fem2d_mesh* m, double* out) {
  API_BEGIN
  if (!m || !out) fail(FEM2D_E_INVALID_ARG, "null argument");
  for (size_t e = 0; e < m->m.elems.size(); e++) {
    auto pr = m->m.param_range((int64_t)e);
    const RootElement& r = m->m.roots[m->m.elems[e].root];
    auto mr = [](double v, double lo, double hi) { return (v + 1.0) * (hi - lo) / 2.0 + lo; };
    out[4 * e + 0] = mr(pr[0], r.x0, r.x3);
    out[4 * e + 1] = mr(pr[2], r.y0, r.y3);
    out[4 * e + 2] = mr(pr[1], r.x0, r.x3);
    out[4 * e + 3] = mr(pr[3], r.y0, r.y3);
  }
  API_END
}

// ------------------------------------------------------------------ domain
int fem2d_domain_from_mesh(const fem2d_mesh* m, int cc, fem2d_domain** out) {
  API_BEGIN
  if (!m || !out) fail(FEM2D_E_INVALID_ARG, "null argument");
  if (cc < 0 || cc > 2) fail(FEM2D_E_INVALID_ARG, "unknown continuity condition");
  *out = new fem2d_domain{Domain::from_mesh(m->m, cc)};
  API_END
}
void fem2d_domain_free(fem2d_domain* d) { delete d; }
int64_t fem2d_domain_num_dofs(const fem2d_domain* d) { return d ? d->d.ndofs : -1; }
int64_t fem2d_domain_num_specs(const fem2d_domain* d) { return d ? (int64_t)d->d.specs.size() : -1; }
int fem2d_domain_basis_specs(const fem2d_domain* d, int64_t* out) {
  API_BEGIN
  if (!d || !out) fail(FEM2D_E_INVALID_ARG, "null argument");
  size_t k = 0;
  for (size_t e = 0; e + 1 < d->d.spec_ptr.size(); e++)
    for (int64_t s = d->d.spec_ptr[e]; s < d->d.spec_ptr[e + 1]; s++, k++) {
      const Spec& sp = d->d.specs[s];
      int64_t* o = out + 6 * k;
      o[0] = (int64_t)e;
      o[1] = s - d->d.spec_ptr[e];
      o[2] = sp.i;
      o[3] = sp.j;
      o[4] = sp.dir;
      o[5] = sp.dof;
    }
  API_END
}

int fem2d_domain_pattern(const fem2d_domain* d, int64_t* nnz_upper, int32_t* rows, int32_t* cols) {
  API_BEGIN
  if (!d || !nnz_upper) fail(FEM2D_E_INVALID_ARG, "null argument");
  if (d->d.cc != FEM2D_CC_HCURL) fail(FEM2D_E_WRONG_CC, "Wrong Continuity Condition on Domain (required: H(Curl))");
  if (d->d.ndofs == 0) fail(FEM2D_E_EMPTY_DOFS, "No Degrees-of-Freedom Defined over Domain");
  HostGEP g;
  build_symbolic(d->d, 0, 4, 4, g);
  *nnz_upper = g.nnz_upper;
  if (rows || cols) {
    int64_t k = 0;
    for (int64_t r = 0; r < g.n; r++)
      for (int64_t e = g.row_ptr[r]; e < g.row_ptr[r + 1]; e++)
        if (g.col[e] >= r) {
          if (rows) rows[k] = (int32_t)r;
          if (cols) cols[k] = g.col[e];
          k++;
        }
  }
  API_END
}

int fem2d_domain_factor_plan(const fem2d_domain* d, int64_t* sizes, int32_t* fronts, int64_t* dof_ptr,
                             int32_t* dofs, int64_t* asm_ptr, int64_t* asm_pos, int64_t* asm_csr, int64_t* ea_ptr,
                             int32_t* ea_map) {
  API_BEGIN
  if (!d || !sizes) fail(FEM2D_E_INVALID_ARG, "null argument");
  if (d->d.ndofs == 0) fail(FEM2D_E_EMPTY_DOFS, "No Degrees-of-Freedom Defined over Domain");
  HostGEP g;
  build_symbolic(d->d, 0, 4, 4, g);
  MFSymbolic s;
  mf_symbolic(d->d, g, s);
  sizes[0] = s.nfronts;
  sizes[1] = (int64_t)s.dofs.size();
  sizes[2] = (int64_t)s.asm_pos.size();
  sizes[3] = (int64_t)s.ea_map.size();
  sizes[4] = s.nlevels;
  sizes[5] = s.max_f;
  sizes[6] = s.max_p;
  sizes[7] = s.mat_total;
  if (fronts)
    for (int f = 0; f < s.nfronts; f++) {
      fronts[4 * f] = s.parent[f];
      fronts[4 * f + 1] = s.level[f];
      fronts[4 * f + 2] = s.f[f];
      fronts[4 * f + 3] = s.p[f];
    }
  if (dof_ptr) std::copy(s.dof_ptr.begin(), s.dof_ptr.end(), dof_ptr);
  if (dofs) std::copy(s.dofs.begin(), s.dofs.end(), dofs);
  if (asm_ptr) std::copy(s.asm_ptr.begin(), s.asm_ptr.end(), asm_ptr);
  if (asm_pos) std::copy(s.asm_pos.begin(), s.asm_pos.end(), asm_pos);
  if (asm_csr) std::copy(s.asm_csr.begin(), s.asm_csr.end(), asm_csr);
  if (ea_ptr) std::copy(s.ea_ptr.begin(), s.ea_ptr.end(), ea_ptr);
  if (ea_map) std::copy(s.ea_map.begin(), s.ea_map.end(), ea_map);
  API_END
}

// ------------------------------------------------------------------ context
int fem2d_ctx_create(int device, fem2d_ctx** out) {
  API_BEGIN
  if (!out) fail(FEM2D_E_INVALID_ARG, "null argument");
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    cudaGetLastError();
    fail(FEM2D_E_NO_DEVICE, "no CUDA device is visible");
  }
  if (device < 0 || device >= n) fail(FEM2D_E_INVALID_ARG, "device index out of range");
  std::unique_ptr<fem2d_ctx> c(new fem2d_ctx);
  c->c.device = device;
  FEM2D_CUDA(cudaSetDevice(device));
  FEM2D_CUDA(cudaStreamCreateWithFlags(&c->c.stream, cudaStreamNonBlocking));
  FEM2D_CUDA(cudaDeviceGetAttribute(&c->c.num_sms, cudaDevAttrMultiProcessorCount, device));
  *out = c.release();
  API_END
}

void fem2d_ctx_destroy(fem2d_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->c.device);
  if (c->c.t0) cudaEventDestroy(c->c.t0);
  if (c->c.t1) cudaEventDestroy(c->c.t1);
  if (c->c.flush_buf) cudaFree(c->c.flush_buf);
  if (c->c.stream) cudaStreamDestroy(c->c.stream);
  delete c;
  cudaGetLastError();
}

int fem2d_ctx_synchronize(fem2d_ctx* c) {
  API_BEGIN
  if (!c) fail(FEM2D_E_INVALID_ARG, "null context");
  FEM2D_CUDA(cudaSetDevice(c->c.device));
  FEM2D_CUDA(cudaStreamSynchronize(c->c.stream));
  API_END
}

int fem2d_ctx_flush_l2(fem2d_ctx* c) {
  API_BEGIN
  if (!c) fail(FEM2D_E_INVALID_ARG, "null context");
  FEM2D_CUDA(cudaSetDevice(c->c.device));
  const size_t bytes = 256ull << 20;
  if (!c->c.flush_buf) FEM2D_CUDA(cudaMalloc(&c->c.flush_buf, bytes));
  FEM2D_CUDA(cudaMemsetAsync(c->c.flush_buf, c->c.launches & 0xff, bytes, c->c.stream));
  API_END
}

int64_t fem2d_ctx_kernel_launches(const fem2d_ctx* c) { return c ? c->c.launches : -1; }

int fem2d_ctx_timer_start(fem2d_ctx* c) {
  API_BEGIN
  if (!c) fail(FEM2D_E_INVALID_ARG, "null context");
  FEM2D_CUDA(cudaSetDevice(c->c.device));
  if (!c->c.t0) FEM2D_CUDA(cudaEventCreate(&c->c.t0));
  if (!c->c.t1) FEM2D_CUDA(cudaEventCreate(&c->c.t1));
  FEM2D_CUDA(cudaEventRecord(c->c.t0, c->c.stream));
  API_END
}

int fem2d_ctx_timer_stop(fem2d_ctx* c, double* ms) {
  API_BEGIN
  if (!c || !ms || !c->c.t0) fail(FEM2D_E_INVALID_ARG, "timer not started");
  FEM2D_CUDA(cudaSetDevice(c->c.device));
  FEM2D_CUDA(cudaEventRecord(c->c.t1, c->c.stream));
  FEM2D_CUDA(cudaEventSynchronize(c->c.t1));
  float f = 0;
  FEM2D_CUDA(cudaEventElapsedTime(&f, c->c.t0, c->c.t1));
  *ms = f;
  API_END
}

int fem2d_ctx_set_profiling(fem2d_ctx* c, int on) {
  API_BEGIN
  if (!c) fail(FEM2D_E_INVALID_ARG, "null context");
  c->c.profile = on != 0;
  API_END
}

int fem2d_ctx_profile_reset(fem2d_ctx* c) {
  API_BEGIN
  if (!c) fail(FEM2D_E_INVALID_ARG, "null context");
  c->c.prof.clear();
  API_END
}

int fem2d_ctx_profile_query(const fem2d_ctx* c, const char* region, double* ms, int64_t* count, double* bytes) {
  API_BEGIN
  if (!c || !region) fail(FEM2D_E_INVALID_ARG, "null argument");
  auto it = c->c.prof.find(region);
  ProfRec r = it == c->c.prof.end() ? ProfRec() : it->second;
  if (ms) *ms = r.ms;
  if (count) *count = r.count;
  if (bytes) *bytes = r.bytes;
  API_END
}

int fem2d_ctx_profile_flops(const fem2d_ctx* c, const char* region, double* flops) {
  API_BEGIN
  if (!c || !region || !flops) fail(FEM2D_E_INVALID_ARG, "null argument");
  auto it = c->c.prof.find(region);
  *flops = it == c->c.prof.end() ? 0.0 : it->second.flops;
  API_END
}

int fem2d_ctx_mma_ns(fem2d_ctx* c, int n, double* ns) {
  API_BEGIN
  if (!c || !ns) fail(FEM2D_E_INVALID_ARG, "null argument");
  FEM2D_CUDA(cudaSetDevice(c->c.device));
  *ns = measure_mma_ns(c->c, n);
  API_END
}

int fem2d_ctx_fp64_peak(fem2d_ctx* c, double* tflops) {
  API_BEGIN
  if (!c || !tflops) fail(FEM2D_E_INVALID_ARG, "null argument");
  FEM2D_CUDA(cudaSetDevice(c->c.device));
  *tflops = measure_fp64_peak(c->c);
  API_END
}

// ------------------------------------------------------------------ galerkin
int fem2d_galerkin_sample_gep_hcurl(fem2d_ctx* c, const fem2d_domain* d, int basis, int nq_u, int nq_v,
                                    fem2d_gep** out) {
  API_BEGIN
  if (!c || !d || !out) fail(FEM2D_E_INVALID_ARG, "null argument");
  // galerkin.rs:42-59
  if (d->d.cc != FEM2D_CC_HCURL)
    fail(FEM2D_E_WRONG_CC, "Wrong Continuity Condition on Domain (required: H(Curl)); Cannot execute Galerkin Sampling!");
  if (d->d.ndofs == 0)
    fail(FEM2D_E_EMPTY_DOFS, "No Degrees-of-Freedom Defined over Domain; Cannot execute Galerkin Sampling!");
  if ((nq_u != 0 || nq_v != 0) && (nq_u < 4 || nq_v < 4))
    fail(FEM2D_E_INVALID_GLQ, "Invalid GLQ Settings (the number of GLQ points must be at least 4); Cannot execute Galerkin Sampling!");
  if (basis != FEM2D_BASIS_HIERPOLY && basis != FEM2D_BASIS_KOLEG) fail(FEM2D_E_INVALID_ARG, "unknown basis space");
  auto mo = d->d.mesh.max_orders();
  if (basis == FEM2D_BASIS_KOLEG && std::max(mo[0], mo[1]) > 12)
    fail(FEM2D_E_INVALID_ARG, "KOLeg is tabulated for expansion orders up to 12");
  if (d->d.ndofs >= (1ll << 31)) fail(FEM2D_E_INVALID_ARG, "more than 2^31 DoFs");
  FEM2D_CUDA(cudaSetDevice(c->c.device));
  std::unique_ptr<fem2d_gep> g(new fem2d_gep);
  g->ctx = &c->c;
  g->device = c->c.device;
  g->dom = d->d;
  auto t0 = std::chrono::steady_clock::now();
  build_symbolic(d->d, basis, nq_u == 0 ? 0 : nq_u, nq_v == 0 ? 0 : nq_v, g->h);
  auto t1 = std::chrono::steady_clock::now();
  device_upload(c->c, g->h, g->d);
  FEM2D_CUDA(cudaStreamSynchronize(c->c.stream));
  auto t2 = std::chrono::steady_clock::now();
  float mt = 0, mv = 0;
  device_assemble(c->c, g->h, g->d, &mt, &mv);
  g->t_symbolic_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
  g->t_upload_ms = std::chrono::duration<double, std::milli>(t2 - t1).count();
  g->t_tables_ms = mt;
  g->t_values_ms = mv;
  *out = g.release();
  API_END
}

int fem2d_gep_recompute(fem2d_ctx* c, fem2d_gep* g) {
  API_BEGIN
  if (!c || !g) fail(FEM2D_E_INVALID_ARG, "null argument");
  FEM2D_CUDA(cudaSetDevice(c->c.device));
  float mt = 0, mv = 0;
  device_assemble(c->c, g->h, g->d, &mt, &mv);
  g->t_tables_ms = mt;
  g->t_values_ms = mv;
  API_END
}

int fem2d_gep_values_noalloc(fem2d_ctx* c, const fem2d_gep* g, double* d_a, double* d_b) {
  int prev = -1;
  API_BEGIN
  if (!c || !g || !d_a || !d_b) fail(FEM2D_E_INVALID_ARG, "null argument");
  if (g->ctx != &c->c) fail(FEM2D_E_INVALID_ARG, "the GEP was built on another context");
  // the caller's current device is put back on every return (its own later launches go there)
  FEM2D_CUDA(cudaGetDevice(&prev));
  struct Restore {
    int dev;
    ~Restore() {
      if (dev >= 0) cudaSetDevice(dev);
    }
  } restore{prev};
  FEM2D_CUDA(cudaSetDevice(c->c.device));
  // both arrays must be device (or managed) memory of the context's device: a host pointer or another
  // GPU's array would otherwise fault inside the kernels (cudaPointerGetAttributes allocates nothing)
  for (const double* p : {d_a, d_b}) {
    cudaPointerAttributes at{};
    cudaError_t e = cudaPointerGetAttributes(&at, p);
    if (e != cudaSuccess) {
      cudaGetLastError();
      fail(FEM2D_E_INVALID_ARG, "output array is not CUDA memory");
    }
    if (at.type != cudaMemoryTypeDevice && at.type != cudaMemoryTypeManaged)
      fail(FEM2D_E_INVALID_ARG, "output array is not device or managed memory");
    if (at.type == cudaMemoryTypeDevice && at.device != c->c.device)
      fail(FEM2D_E_INVALID_ARG, "output array lives on device " + std::to_string(at.device) + ", the context on " +
                                    std::to_string(c->c.device));
  }
  device_values_noalloc(c->c, g->h, g->d, d_a, d_b);
  API_END
}

static void check_galerkin_args(const fem2d_domain* d, int basis, int nq_u, int nq_v) {
  // galerkin.rs:42-59
  if (d->d.cc != FEM2D_CC_HCURL)
    fail(FEM2D_E_WRONG_CC, "Wrong Continuity Condition on Domain (required: H(Curl)); Cannot execute Galerkin Sampling!");
  if (d->d.ndofs == 0)
    fail(FEM2D_E_EMPTY_DOFS, "No Degrees-of-Freedom Defined over Domain; Cannot execute Galerkin Sampling!");
  if ((nq_u != 0 || nq_v != 0) && (nq_u < 4 || nq_v < 4))
    fail(FEM2D_E_INVALID_GLQ, "Invalid GLQ Settings (the number of GLQ points must be at least 4); Cannot execute Galerkin Sampling!");
  if (basis != FEM2D_BASIS_HIERPOLY && basis != FEM2D_BASIS_KOLEG) fail(FEM2D_E_INVALID_ARG, "unknown basis space");
  auto mo = d->d.mesh.max_orders();
  if (basis == FEM2D_BASIS_KOLEG && std::max(mo[0], mo[1]) > 12)
    fail(FEM2D_E_INVALID_ARG, "KOLeg is tabulated for expansion orders up to 12");
  if (d->d.ndofs >= (1ll << 31)) fail(FEM2D_E_INVALID_ARG, "more than 2^31 DoFs");
}

int fem2d_domain_table_doubles(const fem2d_domain* d, int basis, int nq_u, int nq_v, int64_t* doubles) {
  API_BEGIN
  if (!d || !doubles) fail(FEM2D_E_INVALID_ARG, "null argument");
  check_galerkin_args(d, basis, nq_u, nq_v);
  HostGEP h;
  build_symbolic(d->d, basis, nq_u, nq_v, h);
  const int64_t P = h.pmax + 1;
  *doubles = 2 * (int64_t)h.ivl_s.size() * 5 * P * P;
  API_END
}


static void batch_report_out(const BatchReport& r, double* report) {
  if (!report) return;
  report[0] = r.ms_tables;
  report[1] = r.ms_values;
  report[2] = r.shape.threads;
  report[3] = r.shape.ctas_per_sm;
  report[4] = (double)r.total_entries;
  report[5] = (double)r.total_codes;
}

int fem2d_galerkin_sample_gep_hcurl_batch(fem2d_ctx* c, const fem2d_domain* const* domains, int64_t count, int basis,
                                          int nq_u, int nq_v, int autotune, fem2d_gep** out, double* report) {
  API_BEGIN
  if (!c || !out || (count > 0 && !domains)) fail(FEM2D_E_INVALID_ARG, "null argument");
  if (count < 0 || count > (1 << 24)) fail(FEM2D_E_INVALID_ARG, "batch size out of range");
  for (int64_t i = 0; i < count; i++) {
    if (!domains[i]) fail(FEM2D_E_INVALID_ARG, "null domain in the batch");
    check_galerkin_args(domains[i], basis, nq_u, nq_v);
  }
  FEM2D_CUDA(cudaSetDevice(c->c.device));
  std::vector<std::unique_ptr<fem2d_gep>> gs;
  std::vector<BatchMember> members;
  for (int64_t i = 0; i < count; i++) {
    std::unique_ptr<fem2d_gep> g(new fem2d_gep);
    g->ctx = &c->c;
    g->device = c->c.device;
  g->device = c->c.device;
    g->dom = domains[i]->d;
    auto t0 = std::chrono::steady_clock::now();
    build_symbolic(domains[i]->d, basis, nq_u, nq_v, g->h);
    auto t1 = std::chrono::steady_clock::now();
    device_upload(c->c, g->h, g->d);
    g->t_symbolic_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
    gs.push_back(std::move(g));
  }
  for (auto& g : gs) members.push_back(BatchMember{&g->h, &g->d});
  FEM2D_CUDA(cudaStreamSynchronize(c->c.stream));
  BatchReport rep;
  batch_assemble(c->c, members, autotune != 0, &rep);
  batch_report_out(rep, report);
  for (int64_t i = 0; i < count; i++) {
    gs[i]->t_tables_ms = rep.ms_tables;   // shared by the whole batch
    gs[i]->t_values_ms = rep.ms_values;
    out[i] = gs[i].release();
  }
  API_END
}

int fem2d_gep_batch_recompute(fem2d_ctx* c, fem2d_gep* const* geps, int64_t count, int autotune, double* report) {
  API_BEGIN
  if (!c || (count > 0 && !geps)) fail(FEM2D_E_INVALID_ARG, "null argument");
  std::vector<BatchMember> members;
  for (int64_t i = 0; i < count; i++) {
    if (!geps[i]) fail(FEM2D_E_INVALID_ARG, "null GEP in the batch");
    if (geps[i]->ctx->device != c->c.device) fail(FEM2D_E_INVALID_ARG, "the batch spans devices");
    members.push_back(BatchMember{&geps[i]->h, &geps[i]->d});
  }
  FEM2D_CUDA(cudaSetDevice(c->c.device));
  BatchReport rep;
  batch_assemble(c->c, members, autotune != 0, &rep);
  batch_report_out(rep, report);
  API_END
}

int fem2d_autotune_export(char* buf, int64_t capacity, int64_t* length) {
  API_BEGIN
  const std::string t = tune_export();
  if (length) *length = (int64_t)t.size();
  if (buf) {
    if (capacity < (int64_t)t.size() + 1) fail(FEM2D_E_INVALID_ARG, "buffer too small for the autotuner cache");
    std::memcpy(buf, t.c_str(), t.size() + 1);
  }
  API_END
}

int fem2d_autotune_import(const char* text, int64_t* entries) {
  API_BEGIN
  if (!text) fail(FEM2D_E_INVALID_ARG, "null argument");
  const int n = tune_import(text);
  if (entries) *entries = n;
  API_END
}

int fem2d_autotune_clear(void) {
  API_BEGIN
  tune_clear();
  API_END
}

void fem2d_gep_free(fem2d_gep* g) {
  if (!g) return;
  cudaSetDevice(g->device);
  delete g;
  cudaGetLastError();   // a failed release must not surface in a later, unrelated call
}

int fem2d_gep_dims(const fem2d_gep* g, int64_t* ndofs, int64_t* nnz_upper, int64_t* nnz_full) {
  API_BEGIN
  if (!g) fail(FEM2D_E_INVALID_ARG, "null gep");
  if (ndofs) *ndofs = g->h.n;
  if (nnz_upper) *nnz_upper = g->h.nnz_upper;
  if (nnz_full) *nnz_full = g->h.nnz_full;
  API_END
}

int64_t fem2d_gep_num_visits(const fem2d_gep* g) { return g ? g->h.visits : -1; }
int64_t fem2d_gep_h2d_bytes(const fem2d_gep* g) { return g ? g->d.h2d_bytes : -1; }

int fem2d_gep_timings(const fem2d_gep* g, double* out) {
  API_BEGIN
  if (!g || !out) fail(FEM2D_E_INVALID_ARG, "null argument");
  out[0] = g->t_tables_ms;
  out[1] = g->t_values_ms;
  out[2] = g->t_tables_ms + g->t_values_ms;
  out[3] = g->t_symbolic_ms;
  out[4] = g->t_upload_ms;
  API_END
}

static void fetch_values(const fem2d_gep* g, std::vector<double>& a, std::vector<double>& b) {
  FEM2D_CUDA(cudaSetDevice(g->ctx->device));
  a.resize(g->h.nnz_full);
  b.resize(g->h.nnz_full);
  if (g->h.nnz_full) {
    FEM2D_CUDA(cudaMemcpyAsync(a.data(), g->d.a.p, a.size() * 8, cudaMemcpyDeviceToHost, g->ctx->stream));
    FEM2D_CUDA(cudaMemcpyAsync(b.data(), g->d.b.p, b.size() * 8, cudaMemcpyDeviceToHost, g->ctx->stream));
  }
  FEM2D_CUDA(cudaStreamSynchronize(g->ctx->stream));
}

int fem2d_gep_export_upper(const fem2d_gep* g, int32_t* rows, int32_t* cols, double* a, double* b) {
  API_BEGIN
  if (!g) fail(FEM2D_E_INVALID_ARG, "null gep");
  std::vector<double> va, vb;
  fetch_values(g, va, vb);
  int64_t k = 0;
  for (int64_t r = 0; r < g->h.n; r++)
    for (int64_t e = g->h.row_ptr[r]; e < g->h.row_ptr[r + 1]; e++) {
      if (g->h.col[e] < r) continue;
      if (rows) rows[k] = (int32_t)r;
      if (cols) cols[k] = g->h.col[e];
      if (a) a[k] = va[e];
      if (b) b[k] = vb[e];
      k++;
    }
  API_END
}

int fem2d_gep_set_upper_values(fem2d_gep* g, const double* a, const double* b) {
  API_BEGIN
  if (!g || !a || !b) fail(FEM2D_E_INVALID_ARG, "null argument");
  const HostGEP& h = g->h;
  for (int64_t k = 0; k < h.nnz_upper; k++)
    if (!std::isfinite(a[k]) || !std::isfinite(b[k]))
      fail(FEM2D_E_INVALID_ARG, "A or B has a non-finite entry (upper-triangle index " + std::to_string(k) + ")");
  std::vector<double> va(h.nnz_full), vb(h.nnz_full);
  int64_t k = 0;
  for (int64_t r = 0; r < h.n; r++)
    for (int64_t e = h.row_ptr[r]; e < h.row_ptr[r + 1]; e++) {
      const int32_t cc = h.col[e];
      if (cc < r) continue;
      va[e] = a[k];
      vb[e] = b[k];
      if (cc != r) {   // the mirrored entry (cc, r) in row cc
        const int32_t* c0 = h.col.data() + h.row_ptr[cc];
        const int32_t* c1 = h.col.data() + h.row_ptr[cc + 1];
        const int32_t* it = std::lower_bound(c0, c1, (int32_t)r);
        if (it == c1 || *it != r) fail(FEM2D_E_INVALID_ARG, "GEP pattern is not symmetric");
        va[it - h.col.data()] = a[k];
        vb[it - h.col.data()] = b[k];
      }
      k++;
    }
  FEM2D_CUDA(cudaSetDevice(g->ctx->device));
  if (h.nnz_full) {
    FEM2D_CUDA(cudaMemcpyAsync(g->d.a.p, va.data(), h.nnz_full * 8, cudaMemcpyHostToDevice, g->ctx->stream));
    FEM2D_CUDA(cudaMemcpyAsync(g->d.b.p, vb.data(), h.nnz_full * 8, cudaMemcpyHostToDevice, g->ctx->stream));
    FEM2D_CUDA(cudaStreamSynchronize(g->ctx->stream));
  }
  API_END
}

int fem2d_gep_by_parts(fem2d_ctx* c, const fem2d_gep* g, double* vals6) {
  API_BEGIN
  if (!c || !g || !vals6) fail(FEM2D_E_INVALID_ARG, "null argument");
  FEM2D_CUDA(cudaSetDevice(c->c.device));
  gep_by_parts(c->c, g->h, g->d, vals6);
  API_END
}

int fem2d_gep_export_csr(const fem2d_gep* g, int which, int64_t* row_ptr, int32_t* col, double* val) {
  API_BEGIN
  if (!g) fail(FEM2D_E_INVALID_ARG, "null gep");
  if (which != FEM2D_MAT_A && which != FEM2D_MAT_B) fail(FEM2D_E_INVALID_ARG, "which must be A or B");
  if (row_ptr) std::memcpy(row_ptr, g->h.row_ptr.data(), g->h.row_ptr.size() * 8);
  if (col) std::memcpy(col, g->h.col.data(), g->h.col.size() * 4);
  if (val && g->h.nnz_full) {
    FEM2D_CUDA(cudaSetDevice(g->ctx->device));
    const double* src = which == FEM2D_MAT_A ? g->d.a.p : g->d.b.p;
    FEM2D_CUDA(cudaMemcpyAsync(val, src, g->h.nnz_full * 8, cudaMemcpyDeviceToHost, g->ctx->stream));
    FEM2D_CUDA(cudaStreamSynchronize(g->ctx->stream));
  }
  API_END
}

// ------------------------------------------------------------------ PETSc-style files
int fem2d_gep_print_to_petsc_binary_files(const fem2d_gep* g, const char* dir, const char* prefix) {
  API_BEGIN
  if (!g || !dir || !prefix) fail(FEM2D_E_INVALID_ARG, "null argument");
  std::vector<double> v(g->h.nnz_full);
  const std::string base = std::string(dir) + "/tmp/" + prefix;
  for (int which = 0; which < 2; which++) {
    if (g->h.nnz_full) {
      FEM2D_CUDA(cudaSetDevice(g->ctx->device));
      const double* src = which == 0 ? g->d.a.p : g->d.b.p;
      FEM2D_CUDA(cudaMemcpyAsync(v.data(), src, g->h.nnz_full * 8, cudaMemcpyDeviceToHost, g->ctx->stream));
      FEM2D_CUDA(cudaStreamSynchronize(g->ctx->stream));
    }
    aij_write(base + (which == 0 ? "_a.dat" : "_b.dat"), g->h.n, g->h.row_ptr.data(), g->h.col.data(), v.data());
  }
  API_END
}

int fem2d_aij_write(const char* path, int64_t n, const int64_t* row_ptr, const int32_t* col, const double* val) {
  API_BEGIN
  if (!path || !row_ptr || (n > 0 && row_ptr[n] > 0 && (!col || !val))) fail(FEM2D_E_INVALID_ARG, "null argument");
  aij_write(path, n, row_ptr, col, val);
  API_END
}

int fem2d_aij_read(const char* path, int64_t* n, int64_t* nnz, int64_t* row_ptr, int32_t* col, double* val) {
  API_BEGIN
  if (!path || !n || !nnz) fail(FEM2D_E_INVALID_ARG, "null argument");
  AIJ m;
  aij_read(path, m);
  *n = m.n;
  *nnz = (int64_t)m.col.size();
  if (row_ptr) std::copy(m.row_ptr.begin(), m.row_ptr.end(), row_ptr);
  if (col) std::copy(m.col.begin(), m.col.end(), col);
  if (val) std::copy(m.val.begin(), m.val.end(), val);
  API_END
}

int fem2d_petsc_vec_write(const char* path, const double* v, int64_t n) {
  API_BEGIN
  if (!path || (n > 0 && !v)) fail(FEM2D_E_INVALID_ARG, "null argument");
  vec_write(path, v, n);
  API_END
}

int fem2d_petsc_vec_read(const char* path, double* out, int64_t capacity, int64_t* n) {
  API_BEGIN
  if (!path || !n) fail(FEM2D_E_INVALID_ARG, "null argument");
  std::vector<double> v;
  vec_read(path, v);
  *n = (int64_t)v.size();
  if (out) {
    if (capacity < (int64_t)v.size()) fail(FEM2D_E_INVALID_ARG, "output buffer too small");
    std::copy(v.begin(), v.end(), out);
  }
  API_END
}

int fem2d_petsc_scalar_write(const char* path, double x) {
  API_BEGIN
  if (!path) fail(FEM2D_E_INVALID_ARG, "null argument");
  scalar_write(path, x);
  API_END
}

int fem2d_petsc_scalar_read(const char* path, double* x) {
  API_BEGIN
  if (!path || !x) fail(FEM2D_E_INVALID_ARG, "null argument");
  *x = scalar_read(path);
  API_END
}

// ------------------------------------------------------------------ eigensolvers
int fem2d_dense_solve_gep(fem2d_ctx* c, const fem2d_gep* g, double target, double* value, double* vector) {
  API_BEGIN
  if (!c || !g) fail(FEM2D_E_INVALID_ARG, "null argument");
  FEM2D_CUDA(cudaSetDevice(c->c.device));
  std::lock_guard<std::mutex> lk(g->plan.mu);
  dense_solve(c->c, g->dom, g->h, g->d, g->plan, target, value, vector);
  API_END
}

int fem2d_gep_shifted_solve(fem2d_ctx* c, const fem2d_gep* g, double c_a, double c_b, int spd, int nrhs,
                            const double* rhs, double* x) {
  API_BEGIN
  if (!c || !g || !rhs || !x || nrhs <= 0) fail(FEM2D_E_INVALID_ARG, "invalid argument");
  FEM2D_CUDA(cudaSetDevice(c->c.device));
  std::lock_guard<std::mutex> lk(g->plan.mu);
  shifted_solve(c->c, g->dom, g->h, g->d, g->plan, c_a, c_b, spd != 0, nrhs, rhs, x);
  API_END
}

int fem2d_gep_spmm_device(fem2d_ctx* c, const fem2d_gep* g, double c_a, double c_b, const double* d_x, int64_t ldx,
                          int nb, double* d_y, int64_t ldy) {
  API_BEGIN
  if (!c || !g || !d_x || !d_y) fail(FEM2D_E_INVALID_ARG, "null argument");
  if (nb < 1 || nb > 32 || ldx < nb || ldy < nb) fail(FEM2D_E_INVALID_ARG, "block width must be 1..32 and fit both leading dimensions");
  if (g->ctx->device != c->c.device) fail(FEM2D_E_INVALID_ARG, "the GEP lives on another device");
  FEM2D_CUDA(cudaSetDevice(c->c.device));
  gep_spmm(c->c, g->h, g->d, c_a, c_b, d_x, ldx, nb, d_y, ldy);
  API_END
}

int fem2d_gep_spmm_tensor_device(fem2d_ctx* c, const fem2d_gep* g, int which, double coef, const double* d_x,
                                 int64_t ldx, int nb, double* d_y, int64_t ldy) {
  API_BEGIN
  if (!c || !g || !d_x || !d_y) fail(FEM2D_E_INVALID_ARG, "null argument");
  if (nb < 1 || nb > 32 || ldx < nb || ldy < nb) fail(FEM2D_E_INVALID_ARG, "block width must be 1..32 and fit both leading dimensions");
  if (g->ctx->device != c->c.device) fail(FEM2D_E_INVALID_ARG, "the GEP lives on another device");
  FEM2D_CUDA(cudaSetDevice(c->c.device));
  gep_spmm_tensor(c->c, g->h, g->d, which, coef, d_x, ldx, nb, d_y, ldy);
  API_END
}

int fem2d_block_gram_device(fem2d_ctx* c, int method, int64_t n, const double* d_x, int64_t ldx, int a,
                            const double* d_y, int64_t ldy, int b, double* d_c) {
  API_BEGIN
  if (!c || !d_x || !d_y || !d_c) fail(FEM2D_E_INVALID_ARG, "null argument");
  if (n < 0 || a < 1 || b < 1 || ldx < a || ldy < b) fail(FEM2D_E_INVALID_ARG, "bad block sizes");
  if (method != 0 && method != 1) fail(FEM2D_E_INVALID_ARG, "method must be 0 (tensor) or 1 (FP64)");
  FEM2D_CUDA(cudaSetDevice(c->c.device));
  block_gram(c->c, method, n, d_x, ldx, a, d_y, ldy, b, d_c);
  API_END
}

int fem2d_block_gemm_device(fem2d_ctx* c, int method, int64_t n, const double* d_x, int64_t ldx, int a,
                            const double* d_c, int b, double alpha, double beta, double* d_z, int64_t ldz) {
  API_BEGIN
  if (!c || !d_x || !d_c || !d_z) fail(FEM2D_E_INVALID_ARG, "null argument");
  if (n < 0 || a < 1 || b < 1 || ldx < a || ldz < b) fail(FEM2D_E_INVALID_ARG, "bad block sizes");
  if (method != 0 && method != 1) fail(FEM2D_E_INVALID_ARG, "method must be 0 (tensor) or 1 (FP64)");
  FEM2D_CUDA(cudaSetDevice(c->c.device));
  block_gemm(c->c, method, n, d_x, ldx, a, d_c, b, alpha, beta, d_z, ldz);
  API_END
}

int fem2d_gpu_solve_gep(fem2d_ctx* c, const fem2d_gep* g, double target, int n_pairs, const fem2d_solve_opts* opts,
                        double* values, double* vectors, double* residuals, fem2d_solve_stats* stats) {
  API_BEGIN
  if (!c || !g) fail(FEM2D_E_INVALID_ARG, "null argument");
  if (n_pairs <= 0 || n_pairs > g->h.n) fail(FEM2D_E_INVALID_ARG, "n_pairs out of range");
  FEM2D_CUDA(cudaSetDevice(c->c.device));
  fem2d_solve_opts o{};
  if (opts) o = *opts;
  fem2d_solve_stats st{};
  try {
    std::lock_guard<std::mutex> lk(g->plan.mu);
    sparse_solve(c->c, g->dom, g->h, g->d, g->plan, target, n_pairs, o, values, vectors, residuals, &st,
                 o.net ? &o.net->net : nullptr);
  } catch (...) {
    if (stats) *stats = st;
    throw;
  }
  if (stats) *stats = st;
  API_END
}

// ------------------------------------------------------------------ field evaluation
int fem2d_fields_create(fem2d_ctx* c, const fem2d_domain* d, int basis, int d0, int d1, fem2d_fields** out) {
  API_BEGIN
  if (!c || !d || !out) fail(FEM2D_E_INVALID_ARG, "null argument");
  auto f = std::make_unique<fem2d_fields>();
  fields_plan(c->c, d->d, basis, d0, d1, f->f);
  *out = f.release();
  API_END
}

void fem2d_fields_free(fem2d_fields* f) {
  if (!f) return;
  cudaSetDevice(f->f.device);
  delete f;
  cudaGetLastError();
}

int64_t fem2d_fields_num_leaves(const fem2d_fields* f) { return f ? (int64_t)f->f.leaves.size() : -1; }

int fem2d_fields_leaves(const fem2d_fields* f, int64_t* ids) {
  API_BEGIN
  if (!f || !ids) fail(FEM2D_E_INVALID_ARG, "null argument");
  std::copy(f->f.leaves.begin(), f->f.leaves.end(), ids);
  API_END
}

int fem2d_fields_leaf_bounds(const fem2d_fields* f, double* out) {
  API_BEGIN
  if (!f || !out) fail(FEM2D_E_INVALID_ARG, "null argument");
  std::copy(f->f.leaf_bounds.begin(), f->f.leaf_bounds.end(), out);
  API_END
}

static void check_solution_size(const FieldSpace& f, int64_t n) {
  // fields.rs:68-72 MismatchedSolutionSize
  if (n != f.ndofs)
    fail(FEM2D_E_INVALID_ARG, "Domain size (" + std::to_string(f.ndofs) + ") does not match solution size (" +
                                  std::to_string(n) + ")!");
}

int fem2d_fields_xy(fem2d_fields* f, const double* solution, int64_t n_solution, double* x_out, double* y_out) {
  API_BEGIN
  if (!f || !solution || !x_out || !y_out) fail(FEM2D_E_INVALID_ARG, "null argument");
  check_solution_size(f->f, n_solution);
  FieldSpace& F = f->f;
  Ctx& c = *F.ctx;
  FEM2D_CUDA(cudaSetDevice(c.device));
  const size_t pts = F.leaves.size() * (size_t)F.d0 * F.d1;
  if (F.sol.n < (size_t)F.ndofs) F.sol.alloc((size_t)F.ndofs);
  if (F.out.n < 2 * pts) F.out.alloc(2 * pts);
  if (F.ndofs > 0)
    FEM2D_CUDA(cudaMemcpyAsync(F.sol.p, solution, F.ndofs * sizeof(double), cudaMemcpyHostToDevice, c.stream));
  fields_eval(F, F.sol.p, F.out.p, F.out.p + pts);
  if (pts > 0) {
    FEM2D_CUDA(cudaMemcpyAsync(x_out, F.out.p, pts * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    FEM2D_CUDA(cudaMemcpyAsync(y_out, F.out.p + pts, pts * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
  }
  FEM2D_CUDA(cudaStreamSynchronize(c.stream));
  API_END
}

int fem2d_fields_xy_device(fem2d_fields* f, const double* d_solution, int64_t n_solution, double* d_x, double* d_y) {
  API_BEGIN
  if (!f || !d_x || !d_y || (!d_solution && n_solution > 0)) fail(FEM2D_E_INVALID_ARG, "null argument");
  check_solution_size(f->f, n_solution);
  FEM2D_CUDA(cudaSetDevice(f->f.ctx->device));
  fields_eval(f->f, d_solution, d_x, d_y);
  API_END
}

}  // extern "C"

// ---------------------------------------------------------------------------------------------------
// Inner PCG solver and the learned per-Elem-patch coarse-space network (precond.h)
int fem2d_patchnet_create(int k, int hidden, uint64_t seed, fem2d_patchnet** out) {
  API_BEGIN
  if (!out) fail(FEM2D_E_INVALID_ARG, "null argument");
  if (k < 1 || k > 32 || hidden < 1 || hidden > 1024) fail(FEM2D_E_INVALID_ARG, "k must be 1..32, hidden 1..1024");
  std::unique_ptr<fem2d_patchnet> p(new fem2d_patchnet);
  p->net.k = k;
  p->net.hidden = hidden;
  p->net.init(seed);
  *out = p.release();
  API_END
}

void fem2d_patchnet_free(fem2d_patchnet* p) { delete p; }

int64_t fem2d_patchnet_num_params(const fem2d_patchnet* p) { return p ? p->net.size() : -1; }

int fem2d_patchnet_get_params(const fem2d_patchnet* p, float* out) {
  API_BEGIN
  if (!p || !out) fail(FEM2D_E_INVALID_ARG, "null argument");
  std::memcpy(out, p->net.params.data(), p->net.params.size() * sizeof(float));
  API_END
}

int fem2d_patchnet_set_params(fem2d_patchnet* p, const float* in) {
  API_BEGIN
  if (!p || !in) fail(FEM2D_E_INVALID_ARG, "null argument");
  std::memcpy(p->net.params.data(), in, p->net.params.size() * sizeof(float));
  API_END
}

int fem2d_patchnet_features(const fem2d_domain* d, double shift, int64_t* sizes, int64_t* patch_ptr, int32_t* dof,
                            float* feat, float* weight) {
  API_BEGIN
  if (!d || !sizes) fail(FEM2D_E_INVALID_ARG, "null argument");
  Patches pt;
  build_patches(d->d, shift, pt);
  sizes[0] = pt.npatch();
  sizes[1] = pt.nrows;
  if (patch_ptr) std::memcpy(patch_ptr, pt.ptr.data(), pt.ptr.size() * sizeof(int64_t));
  if (dof) std::memcpy(dof, pt.dof.data(), pt.dof.size() * sizeof(int32_t));
  if (feat) std::memcpy(feat, pt.feat.data(), pt.feat.size() * sizeof(float));
  if (weight) std::memcpy(weight, pt.weight.data(), pt.weight.size() * sizeof(float));
  API_END
}

static std::vector<double> to_row_major(const double* samples, int S, int64_t n) {
  std::vector<double> E((size_t)n * S);
  for (int s = 0; s < S; s++)
    for (int64_t i = 0; i < n; i++) E[(size_t)i * S + s] = samples[(size_t)s * n + i];
  return E;
}

int fem2d_patchnet_loss_grad(fem2d_ctx* c, const fem2d_patchnet* p, const fem2d_gep* g, double shift,
                             const double* samples, int S, double* loss, float* grad) {
  API_BEGIN
  if (!c || !p || !g || !samples || !loss) fail(FEM2D_E_INVALID_ARG, "null argument");
  FEM2D_CUDA(cudaSetDevice(c->c.device));
  Patches pt;
  build_patches(g->dom, shift, pt);
  const std::vector<double> E = to_row_major(samples, S, g->h.n);
  std::vector<float> gr(p->net.size(), 0.f);
  *loss = patchnet_loss_grad(c->c, p->net, pt, g->h.n, E.data(), S, gr);
  if (grad) std::memcpy(grad, gr.data(), gr.size() * sizeof(float));
  API_END
}

int fem2d_patchnet_train(fem2d_ctx* c, fem2d_patchnet* p, const fem2d_gep* const* geps, int count, double shift,
                         const double* const* samples, int S, int epochs, double lr, double* loss_history) {
  API_BEGIN
  if (!c || !p || !geps || !samples || count < 1 || epochs < 1) fail(FEM2D_E_INVALID_ARG, "invalid argument");
  FEM2D_CUDA(cudaSetDevice(c->c.device));
  std::vector<Patches> pts(count);
  std::vector<std::vector<double>> Es(count);
  std::vector<const Patches*> pp;
  std::vector<int64_t> ns;
  std::vector<const double*> ep;
  for (int i = 0; i < count; i++) {
    if (!geps[i] || !samples[i]) fail(FEM2D_E_INVALID_ARG, "null GEP or sample set");
    build_patches(geps[i]->dom, shift, pts[i]);
    Es[i] = to_row_major(samples[i], S, geps[i]->h.n);
    pp.push_back(&pts[i]);
    ns.push_back(geps[i]->h.n);
    ep.push_back(Es[i].data());
  }
  const std::vector<double> h = patchnet_train(c->c, p->net, pp, ns, ep, S, epochs, lr);
  if (loss_history) std::memcpy(loss_history, h.data(), h.size() * sizeof(double));
  API_END
}

int fem2d_pcg_create(fem2d_ctx* c, const fem2d_gep* g, double c_a, double c_b, const fem2d_patchnet* net,
                     fem2d_pcg** out) {
  API_BEGIN
  if (!c || !g || !out) fail(FEM2D_E_INVALID_ARG, "null argument");
  if (g->ctx->device != c->c.device) fail(FEM2D_E_INVALID_ARG, "the GEP lives on another device");
  FEM2D_CUDA(cudaSetDevice(c->c.device));
  std::unique_ptr<fem2d_pcg> p(new fem2d_pcg);
  p->s.reset(new PCGSolver(c->c, g->dom, g->h, g->d, c_a, c_b, net ? &net->net : nullptr));
  p->n = g->h.n;
  p->device = c->c.device;
  *out = p.release();
  API_END
}

int fem2d_pcg_solve(fem2d_pcg* p, int nrhs, const double* rhs, double* x, double tol, int max_iter, double* stats) {
  API_BEGIN
  if (!p || !rhs || !x || nrhs < 1 || max_iter < 1) fail(FEM2D_E_INVALID_ARG, "invalid argument");
  PCGStats st;
  p->s->solve(nrhs, rhs, x, tol, max_iter, &st);
  if (stats) {
    stats[0] = st.iters;
    stats[1] = st.relres;
    stats[2] = st.ms;
    stats[3] = st.setup_ms;
    stats[4] = st.coarse_dim;
  }
  if (!(st.relres <= tol)) fail(FEM2D_E_NOT_CONVERGED, "PCG did not reach the tolerance (x holds the last iterate)");
  API_END
}

int fem2d_pcg_harvest(fem2d_pcg* p, int nrhs, const double* rhs, const double* xstar, double tol, int max_iter,
                      int first, int every, int max_samples, double* samples, int* nsamples) {
  API_BEGIN
  if (!p || !rhs || !xstar || !samples || !nsamples || every < 1 || max_samples < 1)
    fail(FEM2D_E_INVALID_ARG, "invalid argument");
  std::vector<double> x((size_t)p->n * nrhs), snaps;
  PCGStats st;
  p->s->solve(nrhs, rhs, x.data(), tol, max_iter, &st, &snaps, xstar, every, max_samples, first);
  const int S = (int)(snaps.size() / std::max<int64_t>(p->n, 1));
  std::memcpy(samples, snaps.data(), snaps.size() * sizeof(double));
  *nsamples = S;
  API_END
}

int fem2d_pcg_create_with_basis(fem2d_ctx* c, const fem2d_gep* g, double c_a, double c_b, int k, const float* basis,
                                fem2d_pcg** out) {
  API_BEGIN
  if (!c || !g || !out || !basis) fail(FEM2D_E_INVALID_ARG, "null argument");
  if (g->ctx->device != c->c.device) fail(FEM2D_E_INVALID_ARG, "the GEP lives on another device");
  FEM2D_CUDA(cudaSetDevice(c->c.device));
  std::unique_ptr<fem2d_pcg> p(new fem2d_pcg);
  p->s.reset(new PCGSolver(c->c, g->dom, g->h, g->d, c_a, c_b, nullptr, basis, k));
  p->n = g->h.n;
  p->device = c->c.device;
  *out = p.release();
  API_END
}

void fem2d_pcg_free(fem2d_pcg* p) {
  if (!p) return;
  cudaSetDevice(p->device);
  delete p;
  cudaGetLastError();
}
