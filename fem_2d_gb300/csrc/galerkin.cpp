// Host symbolic phase of galerkin_sample_gep_hcurl (src/fem_problem/galerkin.rs:33-187).
//
// Visit set (galerkin.rs:73-184): for every Elem E (leaves and ancestors), the upper triangle of
// its own spec list (local-local, diagonal included) and every (spec of E) x (spec of D) for each
// descendant D of E in depth-first order. Each visit lands on the key (min dof, max dof) of the
// upper triangle (sparse_matrix.rs:68-98) and collisions are summed. Here the visits are bucketed
// by key row, sorted, and turned into a full symmetric CSR pattern plus, per key (upper-triangle
// entry), the list of visits that sum into it; each full entry names the key it mirrors. The pattern
// is integer work and bit-exact with the reference's BTreeMap.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <thread>

#include "common.h"
#include "domain.h"
#include "gep.h"

namespace fem2d {

int num_host_threads() {
  unsigned h = std::thread::hardware_concurrency();
  return h == 0 ? 4 : (int)std::min(h, 64u);
}

template <class F>
static void parallel_for(int64_t n, F f) {
  int nt = num_host_threads();
  if (n < 4096 || nt <= 1) {
    f(0, n);
    return;
  }
  std::vector<std::thread> th;
  int64_t chunk = (n + nt - 1) / nt;
  for (int t = 0; t < nt; t++) {
    int64_t a = t * chunk, b = std::min(n, a + chunk);
    if (a >= b) break;
    th.emplace_back([=]() { f(a, b); });
  }
  for (auto& x : th) x.join();
}

// f(t) on nt threads (t = 0..nt-1), inline when nt == 1
template <class F>
static void run_threads(int nt, F f) {
  if (nt <= 1) {
    f(0);
    return;
  }
  std::vector<std::thread> th;
  for (int t = 0; t < nt; t++) th.emplace_back([=]() { f(t); });
  for (auto& x : th) x.join();
}

// out[0] = 0, out[r + 1] = out[r] + term(r) for r < n: the terms in parallel, then a two-pass prefix
// sum over contiguous chunks (the same integers as the serial loop)
template <class F>
static void parallel_prefix(int64_t n, int64_t* out, F term) {
  out[0] = 0;
  const int nt = (n < 65536 || num_host_threads() <= 1) ? 1 : num_host_threads();
  const int64_t chunk = (n + nt - 1) / nt;
  std::vector<int64_t> part(nt + 1, 0);
  run_threads(nt, [&](int t) {
    const int64_t r0 = std::min(n, t * chunk), r1 = std::min(n, r0 + chunk);
    int64_t acc = 0;
    for (int64_t r = r0; r < r1; r++) {
      acc += term(r);
      out[r + 1] = acc;
    }
    part[t + 1] = acc;
  });
  for (int t = 0; t < nt; t++) part[t + 1] += part[t];
  run_threads(nt, [&](int t) {
    const int64_t r0 = std::min(n, t * chunk), r1 = std::min(n, r0 + chunk);
    for (int64_t r = r0; r < r1; r++) out[r + 1] += part[t];
  });
}

// Gauss-Legendre nodes and weights on (-1, 1) by Newton iteration on P_n (the points the reference
// obtains from the Golub-Welsch eigenproblem, glq.rs:179-222), sorted ascending.
void glq_points(int n, std::vector<double>& x, std::vector<double>& w) {
  x.assign(n, 0.0);
  w.assign(n, 0.0);
  for (int k = 0; k < n; k++) {
    double z = std::cos(M_PI * (k + 0.75) / (n + 0.5));
    double dp = 1.0;
    for (int it = 0; it < 100; it++) {
      double p0 = 1.0, p1 = z;
      for (int m = 2; m <= n; m++) {
        double p2 = ((2.0 * m - 1.0) * z * p1 - (m - 1.0) * p0) / m;
        p0 = p1;
        p1 = p2;
      }
      double pn = n == 0 ? 1.0 : p1, pm1 = n == 1 ? 1.0 : p0;
      if (n == 1) { pn = z; pm1 = 1.0; }
      dp = n * (z * pn - pm1) / (z * z - 1.0);
      double dz = pn / dp;
      z -= dz;
      if (std::fabs(dz) < 1e-16) break;
    }
    x[k] = z;
    w[k] = 2.0 / ((1.0 - z * z) * dp * dp);
  }
  std::vector<int> idx(n);
  for (int k = 0; k < n; k++) idx[k] = k;
  std::sort(idx.begin(), idx.end(), [&](int a, int b) { return x[a] < x[b]; });
  std::vector<double> xs(n), ws(n);
  for (int k = 0; k < n; k++) { xs[k] = x[idx[k]]; ws[k] = w[idx[k]]; }
  x.swap(xs);
  w.swap(ws);
}

int default_ngq(int max_order) {   // basis.rs:172-177 (computed in f32 like the reference)
  float conv = (float)(max_order * 4);
  int p2 = (int)std::ceil(std::log2(conv));
  return (int)std::lround(std::pow(2.0f, (float)p2));
}

namespace {
struct IvlKey {
  uint64_t s, o;
  bool operator<(const IvlKey& k) const { return s != k.s ? s < k.s : o < k.o; }
};
}  // namespace

void build_symbolic(const Domain& d, int basis, int nq_u, int nq_v, HostGEP& g) {
  const Mesh& m = d.mesh;
  const int64_t ne = (int64_t)m.elems.size();
  auto mo = m.max_orders();
  g.n = d.ndofs;
  g.basis = basis;
  g.nq_u = nq_u > 0 ? nq_u : default_ngq(mo[0]);
  g.nq_v = nq_v > 0 ? nq_v : default_ngq(mo[1]);
  g.pmax = std::max(mo[0], mo[1]);
  glq_points(g.nq_u, g.glq_u_x, g.glq_u_w);
  glq_points(g.nq_v, g.glq_v_x, g.glq_v_w);
  g.specs.resize(d.specs.size());
  for (size_t k = 0; k < d.specs.size(); k++)
    g.specs[k] = (uint32_t)d.specs[k].i | ((uint32_t)d.specs[k].j << 8) | ((uint32_t)d.specs[k].dir << 16);

  // ---- visit blocks with their constants (integrals.rs:26-92, 249-271, 292-354, 421-423)
  std::map<IvlKey, int32_t> ivl;
  g.ivl_s.assign(1, 1.0);
  g.ivl_o.assign(1, 0.0);
  auto ivl_id = [&](double s, double o) {
    if (s == 1.0 && o == 0.0) return 0;
    IvlKey k;
    std::memcpy(&k.s, &s, 8);
    std::memcpy(&k.o, &o, 8);
    auto it = ivl.find(k);
    if (it != ivl.end()) return it->second;
    int32_t id = (int32_t)g.ivl_s.size();
    ivl[k] = id;
    g.ivl_s.push_back(s);
    g.ivl_o.push_back(o);
    return id;
  };
  std::vector<ElemJac> jac(ne);
  for (int64_t e = 0; e < ne; e++) jac[e] = elem_jacobian(m, e);
  struct BInfo { int64_t p, q; int64_t nvis; bool local; };
  std::vector<BInfo> binfo;
  std::vector<int64_t> desc;
  g.blocks.clear();
  g.braw.clear();
  for (int64_t e = 0; e < ne; e++) {
    int64_t np = d.nspecs(e);
    if (np == 0) continue;
    const RootElement& root = m.roots[m.elems[e].root];
    auto add_block = [&](int64_t q, bool local) {
      const ElemJac& P = jac[e];
      const ElemJac& Q = jac[q];
      double su = 1.0, sv = 1.0, ou = 0.0, ov = 0.0;
      if (!local) {
        auto r = m.relative_range(q, e);
        su = (r[1] - r[0]) / 2.0;
        ou = (r[1] + r[0]) / 2.0;
        sv = (r[3] - r[2]) / 2.0;
        ov = (r[3] + r[2]) / 2.0;
      }
      GBlock b;
      b.sp_p = (int32_t)d.spec_ptr[e];
      b.sp_q = (int32_t)d.spec_ptr[q];
      b.iu = ivl_id(su, ou);
      b.iv = ivl_id(sv, ov);
      // para scales: P sampled over Q carries (su, sv); Q sampled over itself carries (1, 1)
      const double psP0 = su, psP1 = sv, psQ0 = 1.0, psQ1 = 1.0;
      const bool p_big = P.det >= Q.det;
      const double r_uv = p_big ? P.a / P.b : Q.a / Q.b;
      const double r_vu = p_big ? P.b / P.a : Q.b / Q.a;
      const double inv_mu = 1.0 / root.mu_re;
      b.ca[0] = inv_mu * (P.ji_u0 * psQ0) * (Q.ji_u0 * psP0) * r_uv;
      b.ca[1] = -inv_mu * (P.ji_u0 * psQ0) * (Q.ji_v1 * psP1);
      b.ca[2] = -inv_mu * (P.ji_v1 * psQ1) * (Q.ji_u0 * psP0);
      b.ca[3] = inv_mu * (P.ji_v1 * psQ1) * (Q.ji_v1 * psP1) * r_vu;
      const double wB = root.eps_re * (su * sv) * (1.0 * 1.0) * std::max(P.det, Q.det);
      b.cb[0] = wB * P.ji_u0 * Q.ji_u0;
      b.cb[1] = wB * P.ji_v1 * Q.ji_v1;
      g.blocks.push_back(b);
      // the raw geometry of the pair for integrate_by_parts: P (a, b, det, ji_u0, ji_v1), Q (same),
      // the material of P's root element (mu_re, eps_re)
      const double raw[12] = {P.a, P.b, P.det, P.ji_u0, P.ji_v1, Q.a, Q.b, Q.det, Q.ji_u0, Q.ji_v1,
                              root.mu_re, root.eps_re};
      g.braw.insert(g.braw.end(), raw, raw + 12);
      int64_t nq = d.nspecs(q);
      binfo.push_back({e, q, local ? np * (np + 1) / 2 : np * nq, local});
    };
    add_block(e, true);
    desc.clear();
    m.descendants(e, desc);
    for (int64_t q : desc)
      if (d.nspecs(q) > 0) add_block(q, false);
  }
  if (g.blocks.size() >= (1ull << 32)) fail(FEM2D_E_INVALID_ARG, "too many visit blocks");
  const int64_t nb = (int64_t)g.blocks.size();
  std::vector<int64_t> voff(nb + 1, 0);
  for (int64_t b = 0; b < nb; b++) voff[b + 1] = voff[b] + binfo[b].nvis;
  const int64_t V = voff[nb];
  g.visits = V;

  // ---- bucket visits by key row: each thread counts the rows of a contiguous range of blocks (ranges
  // balanced by visit count), per-row offsets are laid out thread by thread, then each thread writes
  // its own positions (no atomics; the per-row sort below makes the order canonical)
  const int64_t n = d.ndofs;
  auto visit_block = [&](int64_t b, auto&& emit) {
    const BInfo& bi = binfo[b];
    const Spec* P = &d.specs[d.spec_ptr[bi.p]];
    const Spec* Q = &d.specs[d.spec_ptr[bi.q]];
    int64_t np = d.nspecs(bi.p), nq = d.nspecs(bi.q);
    if (bi.local) {
      for (int64_t i = 0; i < np; i++)
        for (int64_t k = i; k < np; k++) emit(P[i].dof, P[k].dof, (uint32_t)i, (uint32_t)k);
    } else {
      for (int64_t i = 0; i < np; i++)
        for (int64_t k = 0; k < nq; k++) emit(P[i].dof, Q[k].dof, (uint32_t)i, (uint32_t)k);
    }
  };
  const int nt = (V < 65536 || num_host_threads() <= 1) ? 1 : num_host_threads();
  std::vector<int64_t> brange(nt + 1, 0);
  for (int t = 1; t < nt; t++) {
    const int64_t target = V / nt * t;
    brange[t] = std::lower_bound(voff.begin(), voff.end(), target) - voff.begin();
  }
  brange[nt] = nb;
  std::vector<std::vector<int64_t>> tcnt(nt);
  run_threads(nt, [&](int t) {
    std::vector<int64_t>& c = tcnt[t];
    c.assign(n, 0);
    for (int64_t b = brange[t]; b < brange[t + 1]; b++)
      visit_block(b, [&](int32_t dp, int32_t dq, uint32_t, uint32_t) { c[std::min(dp, dq)]++; });
  });
  std::vector<int64_t> bptr(n + 1, 0);
  parallel_prefix(n, bptr.data(), [&](int64_t r) {
    int64_t s = 0;
    for (int t = 0; t < nt; t++) s += tcnt[t][r];
    return s;
  });
  parallel_for(n, [&](int64_t r0, int64_t r1) {
    for (int64_t r = r0; r < r1; r++) {
      int64_t o = bptr[r];
      for (int t = 0; t < nt; t++) {
        const int64_t c = tcnt[t][r];
        tcnt[t][r] = o;
        o += c;
      }
    }
  });
  struct Item { int32_t col; uint64_t code; };
  // scratch arrays are left uninitialised (every element is written before it is read): zeroing them
  // would add a full serial pass over hundreds of MB at 1M DoFs
  HostVec<Item> items_buf;   // huge-page backed above 64 MB (fewer first-touch faults)
  items_buf.resize(V);
  Item* items = items_buf.data();
  run_threads(nt, [&](int t) {
    std::vector<int64_t>& pos = tcnt[t];
    for (int64_t b = brange[t]; b < brange[t + 1]; b++)
      visit_block(b, [&](int32_t dp, int32_t dq, uint32_t i, uint32_t k) {
        const int32_t r = std::min(dp, dq), c = std::max(dp, dq);
        items[pos[r]++] = {c, make_code((uint32_t)b, i, k)};
      });
  });

  // ---- per row: sort by (col, code), unique columns = upper pattern. A row's items arrive in ascending
  // code order (thread ranges, blocks and each block's (p, q) loops all ascend), so the sort is by
  // (col, arrival index): one 64-bit key per item and a gather. A row that does not arrive ordered (the
  // check is one pass) takes the two-key sort instead; both give the same order.
  std::vector<int64_t> ucnt(n, 0);
  parallel_for(n, [&](int64_t r0, int64_t r1) {
    std::vector<uint64_t> key;
    std::vector<Item> tmp;
    for (int64_t r = r0; r < r1; r++) {
      Item* a = items + bptr[r];
      Item* z = items + bptr[r + 1];
      const int64_t len = z - a;
      bool ordered = true;
      for (int64_t q = 1; q < len && ordered; q++) ordered = a[q - 1].code < a[q].code;
      if (!ordered) {
        std::sort(a, z, [](const Item& x, const Item& y) { return x.col != y.col ? x.col < y.col : x.code < y.code; });
      } else if (len > 1) {
        key.resize(len);
        tmp.assign(a, z);
        for (int64_t q = 0; q < len; q++) key[q] = ((uint64_t)(uint32_t)a[q].col << 32) | (uint64_t)q;
        std::sort(key.begin(), key.end());
        for (int64_t q = 0; q < len; q++) a[q] = tmp[key[q] & 0xffffffffu];
      }
      int64_t u = 0;
      for (Item* it = a; it < z; it++)
        if (it == a || it->col != (it - 1)->col) u++;
      ucnt[r] = u;
    }
  });
  std::vector<int64_t> uptr(n + 1, 0);
  parallel_prefix(n, uptr.data(), [&](int64_t r) { return ucnt[r]; });
  const int64_t nu = uptr[n];
  g.nnz_upper = nu;
  if (nu >= (int64_t)INT32_MAX) fail(FEM2D_E_TOO_LARGE, "more than 2^31 - 1 upper-triangle entries");
  HostVec<int32_t> ucol_buf;
  ucol_buf.resize(nu);
  int32_t* ucol = ucol_buf.data();
  g.vptr.resize(nu + 1);
  int64_t* uc0 = g.vptr.data();   // start of each upper entry's items (grouped by entry)
  parallel_for(n, [&](int64_t r0, int64_t r1) {
    for (int64_t r = r0; r < r1; r++) {
      int64_t u = uptr[r];
      for (int64_t k = bptr[r]; k < bptr[r + 1]; k++)
        if (k == bptr[r] || items[k].col != items[k - 1].col) {
          ucol[u] = items[k].col;
          uc0[u] = k;
          u++;
        }
    }
  });
  uc0[nu] = V;

  // ---- full symmetric CSR: row r = (entries (c, r) of upper rows c < r, ascending c) + upper row r.
  // The transposed (lower) entries are counted and placed per thread over contiguous, ascending ranges
  // of upper rows (balanced by entry count), which keeps each lower row sorted without atomics.
  std::vector<int64_t> rrange(nt + 1, 0);
  for (int t = 1; t < nt; t++) {
    const int64_t target = nu / nt * t;
    rrange[t] = std::lower_bound(uptr.begin(), uptr.end(), target) - uptr.begin();
  }
  rrange[nt] = n;
  run_threads(nt, [&](int t) {
    std::vector<int64_t>& c = tcnt[t];
    std::fill(c.begin(), c.end(), 0);
    for (int64_t r = rrange[t]; r < rrange[t + 1]; r++)
      for (int64_t u = uptr[r]; u < uptr[r + 1]; u++)
        if (ucol[u] != r) c[ucol[u]]++;
  });
  g.row_ptr.assign(n + 1, 0);
  std::vector<int64_t> lcnt(n, 0);
  parallel_prefix(n, g.row_ptr.data(), [&](int64_t r) {
    int64_t l = 0;
    for (int t = 0; t < nt; t++) l += tcnt[t][r];
    lcnt[r] = l;
    return l + (uptr[r + 1] - uptr[r]);
  });
  const int64_t nf = g.row_ptr[n];
  g.nnz_full = nf;
  g.col.resize(nf);
  g.fsrc.resize(nf);
  int32_t* src = g.fsrc.data();   // the upper entry of each full entry
  parallel_for(n, [&](int64_t r0, int64_t r1) {
    for (int64_t r = r0; r < r1; r++) {
      int64_t o = g.row_ptr[r];
      for (int t = 0; t < nt; t++) {
        const int64_t c = tcnt[t][r];
        tcnt[t][r] = o;
        o += c;
      }
    }
  });
  run_threads(nt, [&](int t) {
    std::vector<int64_t>& pos = tcnt[t];
    for (int64_t r = rrange[t]; r < rrange[t + 1]; r++)
      for (int64_t u = uptr[r]; u < uptr[r + 1]; u++)
        if (ucol[u] != r) {
          const int64_t p = pos[ucol[u]]++;
          g.col[p] = (int32_t)r;
          src[p] = (int32_t)u;
        }
  });
  parallel_for(n, [&](int64_t r0, int64_t r1) {
    for (int64_t r = r0; r < r1; r++) {
      int64_t pos = g.row_ptr[r] + lcnt[r];
      for (int64_t u = uptr[r]; u < uptr[r + 1]; u++, pos++) {
        g.col[pos] = ucol[u];
        src[pos] = (int32_t)u;
      }
    }
  });
  // the visit codes in upper-entry order: the items of upper entry u are items[uc0[u] .. uc0[u + 1]),
  // already grouped and sorted, so the codes are a straight copy
  g.codes.resize(V);
  parallel_for(V, [&](int64_t k0, int64_t k1) {
    for (int64_t k = k0; k < k1; k++) g.codes[k] = items[k].code;
  });
}

}  // namespace fem2d
