// UniformFieldSpace::xy_fields (fields.rs:63-122) on the device.
//
// One CTA per leaf Elem (grid-stride). For each (leaf, ancestor) pair, leaf first then up to the root
// (mesh.rs:520-541), the CTA tabulates N and T of the ancestor's shape space at the leaf grid mapped
// into the ancestor's parametric square (basis.rs:186-211 with glq.rs:238-249 scaling), stages the
// ancestor's specs and their solution coefficients in shared memory, and every thread accumulates
// its grid points in registers in the reference's order (ancestors, then specs). The products are
// formed as the reference writes them, ((jac_inv * N) * T) * coefficient, with separate rounded
// multiplies and adds.
#include <algorithm>

#include "fields.h"
#include "shape.cuh"

namespace fem2d {

namespace {

constexpr int kFieldThreads = 128;
constexpr int kFieldPts = 2;        // grid points per thread per pass
constexpr int kSpecChunk = 256;     // specs staged per shared-memory pass

__global__ void __launch_bounds__(kFieldThreads)
fem2d_xy_fields_kernel(const FieldItem* __restrict__ items, const int32_t* __restrict__ item_ptr,
                       const uint32_t* __restrict__ codes, const int32_t* __restrict__ dofs,
                       const double* __restrict__ sol, int basis, int d0, int d1, int imax, int jmax,
                       int64_t nleaves, double* __restrict__ ox, double* __restrict__ oy) {
  extern __shared__ double sm[];
  const int P = d0 * d1;
  const int tu = (imax + 1) * d0, tv = (jmax + 1) * d1;
  double* Nu = sm;
  double* Tu = Nu + tu;
  double* Nv = Tu + tu;
  double* Tv = Nv + tv;
  double* sval = Tv + tv;
  uint32_t* scode = reinterpret_cast<uint32_t*>(sval + kSpecChunk);
  const int tid = threadIdx.x;
  // fields.rs:386-389 uniform_range(-1, 1, n)
  const double stepu = (1.0 - -1.0) / (double)(d0 - 1);
  const double stepv = (1.0 - -1.0) / (double)(d1 - 1);

  for (int64_t leaf = blockIdx.x; leaf < nleaves; leaf += gridDim.x) {
    const int it0 = item_ptr[leaf], it1 = item_ptr[leaf + 1];
    for (int pass = 0; pass < P; pass += kFieldThreads * kFieldPts) {
      int pm[kFieldPts], pn[kFieldPts];
      double ax[kFieldPts], ay[kFieldPts];
#pragma unroll
      for (int k = 0; k < kFieldPts; k++) {
        const int p = pass + k * kFieldThreads + tid;
        const int q = p < P ? p : 0;
        pm[k] = q / d1;
        pn[k] = q % d1;
        ax[k] = 0.0;
        ay[k] = 0.0;
      }
      for (int it = it0; it < it1; it++) {
        const FieldItem I = items[it];
        __syncthreads();   // the previous item's tables and specs are consumed
        for (int k = tid; k < tu; k += kFieldThreads) {
          const int a = k / d0, m = k % d0;
          const double u = __dadd_rn(__dmul_rn(__dadd_rn(__dmul_rn((double)m, stepu), -1.0), I.su), I.ou);
          Nu[k] = shape(basis, 0, a, u);
          Tu[k] = shape(basis, 2, a, u);
        }
        for (int k = tid; k < tv; k += kFieldThreads) {
          const int b = k / d1, n = k % d1;
          const double v = __dadd_rn(__dmul_rn(__dadd_rn(__dmul_rn((double)n, stepv), -1.0), I.sv), I.ov);
          Nv[k] = shape(basis, 0, b, v);
          Tv[k] = shape(basis, 2, b, v);
        }
        for (int c0 = I.sp0; c0 < I.sp1; c0 += kSpecChunk) {
          const int nc = min(kSpecChunk, I.sp1 - c0);
          if (c0 != I.sp0) __syncthreads();
          for (int k = tid; k < nc; k += kFieldThreads) {
            scode[k] = codes[c0 + k];
            sval[k] = sol[dofs[c0 + k]];
          }
          __syncthreads();
          for (int k = 0; k < nc; k++) {
            const uint32_t code = scode[k];
            const int i = code & 0xff, j = (code >> 8) & 0xff, dir = code >> 16;
            const double s = sval[k];
            if (dir == 0) {   // f_u: jac_inv.u * N_i(u) * T_j(v)   (basis.rs:225-228)
#pragma unroll
              for (int q = 0; q < kFieldPts; q++) {
                const double f = __dmul_rn(__dmul_rn(I.jiu, Nu[i * d0 + pm[q]]), Tv[j * d1 + pn[q]]);
                ax[q] = __dadd_rn(ax[q], __dmul_rn(f, s));
              }
            } else if (dir == 1) {   // f_v: jac_inv.v * T_i(u) * N_j(v)   (basis.rs:230-233)
#pragma unroll
              for (int q = 0; q < kFieldPts; q++) {
                const double f = __dmul_rn(__dmul_rn(I.jiv, Tu[i * d0 + pm[q]]), Nv[j * d1 + pn[q]]);
                ay[q] = __dadd_rn(ay[q], __dmul_rn(f, s));
              }
            }
          }
        }
      }
#pragma unroll
      for (int k = 0; k < kFieldPts; k++) {
        const int p = pass + k * kFieldThreads + tid;
        if (p < P) {
          ox[leaf * P + p] = ax[k];
          oy[leaf * P + p] = ay[k];
        }
      }
    }
    __syncthreads();
  }
}

}  // namespace

void fields_plan(Ctx& c, const Domain& d, int basis, int d0, int d1, FieldSpace& f) {
  if (basis != FEM2D_BASIS_HIERPOLY && basis != FEM2D_BASIS_KOLEG) fail(FEM2D_E_INVALID_ARG, "unknown basis space");
  if (d.cc != FEM2D_CC_HCURL) fail(FEM2D_E_WRONG_CC, "xy fields need an H(curl) Domain");
  // uniform_range divides by n - 1 (fields.rs:386-389): two points per axis at least
  if (d0 < 2 || d1 < 2 || d0 > 1024 || d1 > 1024) fail(FEM2D_E_INVALID_ARG, "field densities must lie in [2, 1024]");
  const Mesh& m = d.mesh;
  auto mo = m.max_orders();
  if (basis == FEM2D_BASIS_KOLEG && std::max(mo[0], mo[1]) > 12)
    fail(FEM2D_E_INVALID_ARG, "KOLeg is tabulated for expansion orders up to 12");
  f.ctx = &c;
  f.device = c.device;
  f.basis = basis;
  f.d0 = d0;
  f.d1 = d1;
  f.imax = mo[0];
  f.jmax = mo[1];
  f.ndofs = d.ndofs;
  f.leaves.clear();
  f.leaf_bounds.clear();
  f.h_items.clear();
  f.h_item_ptr.assign(1, 0);
  const int64_t ne = (int64_t)m.elems.size();
  std::vector<ElemJac> jac(ne);
  for (int64_t e = 0; e < ne; e++) jac[e] = elem_jacobian(m, e);
  for (int64_t e = 0; e < ne; e++) {
    if (!m.elems[e].leaf()) continue;
    f.leaves.push_back(e);
    {   // elem_diag_points (mesh.rs): real-space nodes[0] and nodes[3] of the leaf
      const MElem& el = m.elems[e];
      f.leaf_bounds.push_back(m.nodes[el.nodes[0]].p.x);
      f.leaf_bounds.push_back(m.nodes[el.nodes[0]].p.y);
      f.leaf_bounds.push_back(m.nodes[el.nodes[3]].p.x);
      f.leaf_bounds.push_back(m.nodes[el.nodes[3]].p.y);
    }
    // ancestor_elems(leaf, true): the leaf, its parent, ..., the root Elem (mesh.rs:520-541)
    std::vector<int64_t> chain{e};
    const auto& anc = m.elems[e].anc;
    for (auto it = anc.rbegin(); it != anc.rend(); ++it) chain.push_back(*it);
    for (int64_t a : chain) {
      FieldItem I;
      I.su = 1.0; I.ou = 0.0; I.sv = 1.0; I.ov = 0.0;
      if (a != e) {   // basis.rs:186-211: sampled over the descendant leaf, points scaled into a
        auto r = m.relative_range(e, a);
        I.su = (r[1] - r[0]) / 2.0;
        I.ou = (r[1] + r[0]) / 2.0;
        I.sv = (r[3] - r[2]) / 2.0;
        I.ov = (r[3] + r[2]) / 2.0;
      }
      I.jiu = jac[a].ji_u0;
      I.jiv = jac[a].ji_v1;
      I.sp0 = (int32_t)d.spec_ptr[a];
      I.sp1 = (int32_t)d.spec_ptr[a + 1];
      f.h_items.push_back(I);
    }
    f.h_item_ptr.push_back((int32_t)f.h_items.size());
  }
  std::vector<uint32_t> codes(d.specs.size());
  std::vector<int32_t> dofs(d.specs.size());
  for (size_t k = 0; k < d.specs.size(); k++) {
    codes[k] = (uint32_t)d.specs[k].i | ((uint32_t)d.specs[k].j << 8) | ((uint32_t)d.specs[k].dir << 16);
    dofs[k] = d.specs[k].dof;
  }
  const size_t tu = (size_t)(f.imax + 1) * d0, tv = (size_t)(f.jmax + 1) * d1;
  f.smem = (2 * tu + 2 * tv + kSpecChunk) * sizeof(double) + kSpecChunk * sizeof(uint32_t);
  if (f.smem > 200 * 1024) fail(FEM2D_E_TOO_LARGE, "field grid too dense for the shape tables");
  FEM2D_CUDA(cudaSetDevice(c.device));
  f.items.upload(f.h_items, c.stream);
  f.item_ptr.upload(f.h_item_ptr, c.stream);
  f.codes.upload(codes, c.stream);
  f.dofs.upload(dofs, c.stream);
  f.h2d_bytes = (int64_t)(f.h_items.size() * sizeof(FieldItem) + f.h_item_ptr.size() * 4 + codes.size() * 8);
  FEM2D_CUDA(cudaFuncSetAttribute(fem2d_xy_fields_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)std::max<size_t>(f.smem, 48 * 1024)));
  FEM2D_CUDA(cudaStreamSynchronize(c.stream));
}

void fields_eval(FieldSpace& f, const double* d_solution, double* d_x, double* d_y) {
  Ctx& c = *f.ctx;
  const int64_t nl = (int64_t)f.leaves.size();
  if (nl == 0) return;
  const double P = (double)f.d0 * f.d1;
  // algorithmic bytes: the two grids written once, plan and specs read, one coefficient per spec visit
  double spec_visits = 0;
  for (const FieldItem& I : f.h_items) spec_visits += I.sp1 - I.sp0;
  const double bytes = 16.0 * P * nl + sizeof(FieldItem) * f.h_items.size() + 16.0 * spec_visits;
  ProfScope ps(c, "xy_fields", bytes);
  const int64_t grid = std::min<int64_t>(nl, (int64_t)std::max(c.num_sms, 1) * 16);
  fem2d_xy_fields_kernel<<<(unsigned)grid, kFieldThreads, f.smem, c.stream>>>(
      f.items.p, f.item_ptr.p, f.codes.p, f.dofs.p, d_solution, f.basis, f.d0, f.d1, f.imax, f.jmax, nl, d_x, d_y);
  FEM2D_CUDA(cudaGetLastError());
  c.launches++;
}

}  // namespace fem2d
