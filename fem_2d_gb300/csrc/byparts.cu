// integrate_by_parts over the Galerkin visit set, on the device.
//
// CurlCurl::integrate_by_parts (integrals.rs:94-237) splits each curl-curl integral into a face term
// (second derivatives of p against q over the interior quadrature points) and four edge terms (curl
// of p against the tangential trace of q at the edge points); L2Inner::integrate_by_parts
// (integrals.rs:356-418) is the full L2 integral over the interior points. The samplers hold second
// derivatives and GLQ points with the endpoints -1 and +1 appended (glq.rs:179-222, basis.rs:76-103);
// the face sum skips the endpoints (real_gauss_quad_inner glq.rs:53-77) and each edge sum runs over one
// endpoint row or column (real_gauss_quad_edge glq.rs:101-156). Visits are the pairs of
// galerkin_sample_gep_hcurl (galerkin.rs:73-184), p the spec of the outer Elem sampled over the inner
// one, q the inner spec; per upper-triangle key the six results are summed. The reference has no
// driver for the by-parts form; this is the Galerkin loop with the by-parts integrals.
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "../../include/fem2d_gb300.h"
#include "byparts.h"
#include "common.h"
#include "device.h"
#include "gep.h"

namespace fem2d {

namespace {

constexpr int kFam = 6;   // 0 N, 1 N', 2 N'', 3 T, 4 T', 5 T''

double q_num_host(int idx, int k) {   // Q_WEIGHTS numerators (hierarchical_basis_fns.rs:210-223)
  const int dim = idx + 3;
  static const int tops[12] = {1, 3, 6, 10, 15, 21, 28, 36, 40, 55, 66, 72};
  if (k == dim - 1) return (double)tops[idx];
  if ((idx & 1) == 0) return (k & 1) ? 0.0 : -(double)(2 * k + 1);
  return (k & 1) ? -(double)(2 * k + 1) : 0.0;
}
const double kEuc[12] = {0.968246, 2.561738, 0.838525, 4.248161, 0.816397, 5.882766,
                         0.808509, 1.0, 1.0, 1.0, 1.0, 1.0};
const int kQden[12] = {1, 3, 6, 10, 15, 21, 28, 36, 40, 55, 66, 72};

// all families of orders 0..P-1 at one point, in the reference's construction order
void shapes_at(int basis, int P, double x, double* out /* kFam x P */) {
  auto at = [&](int fam, int a) -> double& { return out[fam * P + a]; };
  if (basis == FEM2D_BASIS_HIERPOLY) {   // HierPoly::new_with_d2 (hierarchical_basis_fns.rs:24-100)
    std::vector<double> pw(P), pwd(P), pwd2(P);
    for (int n = 0; n < P; n++) {
      const double nf = (double)n;
      if (n == 0) {
        pw[0] = 1.0; pwd[0] = 0.0; pwd2[0] = 0.0;
        at(3, 0) = 1.0 - x; at(4, 0) = -1.0;
      } else if (n == 1) {
        pw[1] = x; pwd[1] = 1.0; pwd2[1] = 0.0;
        at(3, 1) = 1.0 + x; at(4, 1) = 1.0;
      } else {
        pw[n] = pw[n - 1] * x;
        pwd[n] = nf * pw[n - 1];
        pwd2[n] = n == 2 ? 2.0 : (n == 3 ? 6.0 * x : nf * (nf - 1.0) * pw[n - 2]);
        if (n % 2 == 0) {
          at(3, n) = pw[n] - 1.0;
          at(4, n) = pwd[n];
        } else {
          at(3, n) = pw[n] - x;
          at(4, n) = pwd[n] - 1.0;
        }
      }
      at(0, n) = pw[n];
      at(1, n) = pwd[n];
      at(2, n) = pwd2[n];
      at(5, n) = pwd2[n];   // tang_d2 returns the same table (hierarchical_basis_fns.rs:194-197)
    }
    return;
  }
  // KOLeg: Legendre values, first and second derivatives (LegendrePoly 466-590; the denominator 1 - x^2
  // is replaced by 1 at the endpoints +-1), Q functions as weighted Legendre sums (356-395)
  std::vector<double> L(P), L1(P), L2(P);
  const double den = std::fabs(std::fabs(x) - 1.0) < 1e-15 ? 1.0 : 1.0 - std::pow(x, 2);
  for (int i = 0; i < P; i++) {
    const double f = (double)i;
    if (i == 0) { L[0] = 1.0; L1[0] = 0.0; L2[0] = 0.0; }
    else if (i == 1) { L[1] = x; L1[1] = 1.0; L2[1] = 0.0; }
    else {
      L[i] = ((2.0 * f - 1.0) * x * L[i - 1] - (f - 1.0) * L[i - 2]) / f;
      L1[i] = f * L[i - 1] + x * L1[i - 1];
      L2[i] = i == 2 ? 3.0 : (2.0 * x * L1[i] - (f * (f + 1.0)) * L[i]) / den;
    }
    at(0, i) = L[i];
    at(1, i) = L1[i];
    at(2, i) = L2[i];
  }
  for (int i = 0; i < P; i++) {
    if (i == 0) { at(3, 0) = 1.0 - x; at(4, 0) = -1.0; at(5, 0) = 0.0; continue; }
    if (i == 1) { at(3, 1) = 1.0 + x; at(4, 1) = 1.0; at(5, 1) = 0.0; continue; }
    const int idx = i - 2;
    double v = 0.0, d1 = 0.0, d2 = 0.0;
    for (int k = 0; k < i + 1; k++) {
      const double w = q_num_host(idx, k) / (double)kQden[idx];
      v += w * L[k];
      d1 += w * L1[k];
      d2 += w * L2[k];
    }
    at(3, i) = v * kEuc[idx];
    at(4, i) = d1 * kEuc[idx];
    at(5, i) = d2 * kEuc[idx];
  }
}

struct V2 { double x, y; };
__device__ __forceinline__ double dot2(V2 a, V2 b) { return a.x * b.x + a.y * b.y; }
__device__ __forceinline__ double curl2(V2 a) { return a.x * -1.0 + a.y * 1.0; }

struct BPArgs {
  int64_t nu;
  const int64_t* vptr;
  const uint64_t* codes;
  const GBlock* blocks;
  const double* braw;
  const uint32_t* specs;
  const double* ivl_s;
  const double* tab_u;   // [ivl][fam][order][point], Mu points
  const double* tab_v;   // [ivl][fam][order][point], Mv points
  const double* wu;      // Mu weights (endpoints first and last)
  const double* wv;
  int Mu, Mv, P;
  double* out;           // 6 per upper entry
};

// one (p, q) visit: out[0] face, out[1..4] edges, out[5] the L2 value
__device__ void visit(const BPArgs& A, uint64_t code, double* out) {
  const int64_t b = (int64_t)(code >> 32);
  const int i = (int)((code >> 16) & 0xffff), k = (int)(code & 0xffff);
  const GBlock blk = A.blocks[b];
  const double* rw = A.braw + 12 * b;
  const double pa = rw[0], pb = rw[1], pdet = rw[2];
  const double qa = rw[5], qb = rw[6], qdet = rw[7];
  const double mu = rw[10], eps = rw[11];
  // jac_inv of an axis-aligned rectangle, as space.rs:142-147 forms it (zero off-diagonal entries -0/det)
  const double pji_u0 = rw[3], pji_u1 = (-1.0 * 0.0) / pdet, pji_v0 = (-1.0 * 0.0) / pdet, pji_v1 = rw[4];
  const double qji_u0 = rw[8], qji_u1 = (-1.0 * 0.0) / qdet, qji_v0 = (-1.0 * 0.0) / qdet, qji_v1 = rw[9];
  const double pps0 = A.ivl_s[blk.iu], pps1 = A.ivl_s[blk.iv];   // p sampled over q's Elem
  const double qps0 = 1.0, qps1 = 1.0;                             // q over itself
  const uint32_t sp = A.specs[blk.sp_p + i], sq = A.specs[blk.sp_q + k];
  const int pi = (int)(sp & 0xff), pj = (int)((sp >> 8) & 0xff), pd = (int)((sp >> 16) & 0xff);
  const int qi = (int)(sq & 0xff), qj = (int)((sq >> 8) & 0xff), qd = (int)((sq >> 16) & 0xff);
  const int Mu = A.Mu, Mv = A.Mv, P = A.P;
  // table entries: u-shapes of p over interval iu, v-shapes over iv; q over interval 0 (identity)
  auto tu = [&](int ivl, int fam, int ord, int m) { return A.tab_u[(((int64_t)ivl * kFam + fam) * P + ord) * Mu + m]; };
  auto tv = [&](int ivl, int fam, int ord, int n) { return A.tab_v[(((int64_t)ivl * kFam + fam) * P + ord) * Mv + n]; };
  const int iu = blk.iu, iv = blk.iv;
  // max_uv_ratios / max_vu_ratios (integrals.rs:249-271)
  const double ruv = (double)(pdet >= qdet) * (pa / pb) + (double)(pdet < qdet) * (qa / qb);
  const double rvu = (double)(pdet >= qdet) * (pb / pa) + (double)(pdet < qdet) * (qb / qa);
  // basis.rs:225-292 for p (sampled at (m, n), derivative scale = q's) and q
  auto q_f = [&](int m, int n) -> V2 {
    if (qd == 0) return {(qji_u0 * tu(0, 0, qi, m)) * tv(0, 3, qj, n), (qji_u1 * tu(0, 0, qi, m)) * tv(0, 3, qj, n)};
    return {(qji_v0 * tu(0, 3, qi, m)) * tv(0, 0, qj, n), (qji_v1 * tu(0, 3, qi, m)) * tv(0, 0, qj, n)};
  };
  auto p_d1 = [&](int m, int n) -> V2 {
    V2 a;
    if (pd == 0)
      a = {pji_u0 * (tu(iu, 0, pi, m) * tv(iv, 4, pj, n)), pji_u1 * (tu(iu, 1, pi, m) * tv(iv, 3, pj, n))};
    else
      a = {pji_v0 * (tu(iu, 3, pi, m) * tv(iv, 1, pj, n)), pji_v1 * (tu(iu, 4, pi, m) * tv(iv, 0, pj, n))};
    return {a.x * qps0, a.y * qps1};
  };
  auto p_face = [&](int m, int n) -> V2 {   // [dd.y + d2.x, d2.y + dd.x]
    V2 d2, dd;
    if (pd == 0) {
      V2 a = {pji_u0 * (tu(iu, 0, pi, m) * tv(iv, 5, pj, n)), pji_u1 * (tu(iu, 2, pi, m) * tv(iv, 3, pj, n))};
      d2 = {a.x * qps0 * qps0, a.y * qps1 * qps1};
      const double nt = tu(iu, 1, pi, m), td = tv(iv, 4, pj, n);
      dd = {pji_u0 * nt * td * qps0 * qps1, pji_u1 * nt * td * qps0 * qps1};
    } else {
      V2 a = {pji_v0 * (tu(iu, 3, pi, m) * tv(iv, 2, pj, n)), pji_v1 * (tu(iu, 5, pi, m) * tv(iv, 0, pj, n))};
      d2 = {a.x * qps0 * qps0, a.y * qps1 * qps1};
      const double td = tu(iu, 4, pi, m), nd = tv(iv, 1, pj, n);
      dd = {pji_v0 * td * nd * qps0 * qps1, pji_v1 * td * nd * qps0 * qps1};
    }
    return {dd.y + d2.x, d2.y + dd.x};
  };
  auto p_f = [&](int m, int n) -> V2 {
    if (pd == 0) return {(pji_u0 * tu(iu, 0, pi, m)) * tv(iv, 3, pj, n), (pji_u1 * tu(iu, 0, pi, m)) * tv(iv, 3, pj, n)};
    return {(pji_v0 * tu(iu, 3, pi, m)) * tv(iv, 0, pj, n), (pji_v1 * tu(iu, 3, pi, m)) * tv(iv, 0, pj, n)};
  };
  const double gp = pps0 * pps1, gq = qps0 * qps1;
  const double gq2 = gq * gq;
  // face term and L2 value over the interior points (real_gauss_quad_inner)
  double face = 0.0, l2 = 0.0;
  const double pm = fmax(pdet, qdet);
  for (int m = 1; m < Mu - 1; m++) {
    double inner = 0.0, inner2 = 0.0;
    for (int n = 1; n < Mv - 1; n++) {
      const V2 qv = q_f(m, n);
      double fv = dot2(p_face(m, n), qv) / gq2;
      if (pd == 0 && qd == 0) fv = fv * ruv;
      if (pd == 1 && qd == 1) fv = fv * rvu;
      inner += fv * A.wv[n];
      inner2 += dot2(p_f(m, n), qv) * pm * A.wv[n];
    }
    face += inner * A.wu[m];
    l2 += inner2 * A.wu[m];
  }
  if (pd == qd) face = face * -1.0;
  out[0] = (1.0 / mu) * gp * gq * face;
  out[5] = eps * (pps0 * pps1) * (qps0 * qps1) * l2;
  // edge terms (real_gauss_quad_edge): U-q on edges 0, 1 (u runs); V-q on edges 2, 3 (v runs)
  const V2 unit[4] = {{-1.0, 0.0}, {1.0, 0.0}, {0.0, -1.0}, {0.0, 1.0}};
  for (int e = 0; e < 4; e++) {
    const bool active = (qd == 0 && e < 2) || (qd == 1 && e >= 2);
    double v = 0.0;
    if (active) {
      auto g = [&](int m, int n) {
        double r = curl2(p_d1(m, n)) * dot2(q_f(m, n), unit[e]) / gq;
        if (pd == 0 && qd == 0) r = r * ruv;
        if (pd == 1 && qd == 1) r = r * rvu;
        return r;
      };
      if (e == 0)
        for (int m = 1; m < Mu - 1; m++) v += g(m, 0) * A.wu[m];
      else if (e == 1)
        for (int m = Mu - 2; m >= 1; m--) v += g(m, Mv - 1) * A.wu[m];
      else if (e == 2)
        for (int n = Mv - 2; n >= 1; n--) v += g(0, n) * A.wv[n];
      else
        for (int n = 1; n < Mv - 1; n++) v += g(Mu - 1, n) * A.wv[n];
      if (qd == 1) v = v * -1.0;
    }
    const double pe = e < 2 ? pps0 : pps1, qe = e < 2 ? qps0 : qps1;
    out[1 + e] = -1.0 * (1.0 / mu) * pe * qe * v;
  }
}

__global__ void __launch_bounds__(128) byparts_kernel(BPArgs A) {
  const int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (u >= A.nu) return;
  double acc[6] = {0, 0, 0, 0, 0, 0};
  const int64_t c0 = A.vptr[u], c1 = A.vptr[u + 1];
  for (int64_t c = c0; c < c1; c++) {
    double v[6];
    visit(A, A.codes[c], v);
    for (int t = 0; t < 6; t++) acc[t] = c == c0 ? v[t] : acc[t] + v[t];
  }
  for (int t = 0; t < 6; t++) A.out[u * 6 + t] = acc[t];
}

}  // namespace

void gep_by_parts(Ctx& c, const HostGEP& h, const DeviceGEP& d, double* out6) {
  if ((int64_t)h.braw.size() != 12 * (int64_t)h.blocks.size())
    fail(FEM2D_E_INVALID_ARG, "by-parts integrals need the GEP's block geometry");
  // GLQ points with the endpoints appended (weight 1.0), as the second-derivative samplers hold them
  std::vector<double> xu, wu, xv, wv;
  glq_points(h.nq_u, xu, wu);
  glq_points(h.nq_v, xv, wv);
  xu.insert(xu.begin(), -1.0); xu.push_back(1.0); wu.insert(wu.begin(), 1.0); wu.push_back(1.0);
  xv.insert(xv.begin(), -1.0); xv.push_back(1.0); wv.insert(wv.begin(), 1.0); wv.push_back(1.0);
  const int Mu = (int)xu.size(), Mv = (int)xv.size(), P = h.pmax + 1;
  const int nivl = (int)h.ivl_s.size();
  // shape tables per interval: points x * s + o (glq.rs:238-249 as defined_over applies it)
  std::vector<double> tu((size_t)nivl * kFam * P * Mu), tv((size_t)nivl * kFam * P * Mv), buf(kFam * P);
  for (int iv = 0; iv < nivl; iv++) {
    const double s = h.ivl_s[iv], o = h.ivl_o[iv];
    for (int m = 0; m < Mu; m++) {
      const double x = iv == 0 ? xu[m] : xu[m] * s + o;
      shapes_at(h.basis, P, x, buf.data());
      for (int f = 0; f < kFam; f++)
        for (int a = 0; a < P; a++) tu[(((size_t)iv * kFam + f) * P + a) * Mu + m] = buf[f * P + a];
    }
    for (int n = 0; n < Mv; n++) {
      const double x = iv == 0 ? xv[n] : xv[n] * s + o;
      shapes_at(h.basis, P, x, buf.data());
      for (int f = 0; f < kFam; f++)
        for (int a = 0; a < P; a++) tv[(((size_t)iv * kFam + f) * P + a) * Mv + n] = buf[f * P + a];
    }
  }
  // one result per upper-triangle entry, in (row, col) order: the GEP's visit lists are grouped by it
  const int64_t nu = h.nnz_upper;
  DBuf<double> braw, tab_u, tab_v, wud, wvd, ivs, out;
  braw.upload_on(h.braw, c.stream);
  tab_u.upload_on(tu, c.stream);
  tab_v.upload_on(tv, c.stream);
  wud.upload_on(wu, c.stream);
  wvd.upload_on(wv, c.stream);
  ivs.upload_on(h.ivl_s, c.stream);
  out.alloc_on((size_t)std::max<int64_t>(nu, 1) * 6, c.stream);
  BPArgs a{nu, d.vptr.p, d.codes.p, d.blocks.p, braw.p, d.specs.p, ivs.p, tab_u.p, tab_v.p, wud.p, wvd.p,
           Mu, Mv, P, out.p};
  if (nu > 0) {
    byparts_kernel<<<(unsigned)((nu + 127) / 128), 128, 0, c.stream>>>(a);
    c.launches++;
    FEM2D_CUDA(cudaGetLastError());
    FEM2D_CUDA(cudaMemcpyAsync(out6, out.p, (size_t)nu * 6 * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
  }
  FEM2D_CUDA(cudaStreamSynchronize(c.stream));
}

}  // namespace fem2d
