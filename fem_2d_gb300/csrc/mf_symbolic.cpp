// Symbolic phase of the multifrontal factorization (see mf.h).
//
// Elimination tree: a nested dissection of the base Elems by coordinate bisection (binary nodes);
// below each base Elem its own refinement tree (an Elem node per Elem, with its 2 or 4 children).
// A DoF is eliminated at the lowest common ancestor of the Elems it is attached to. Every Elem whose
// functions couple with the DoF is an ancestor or a descendant of one of those Elems, so all its
// couplings lie on root paths through that node: the tree is a valid elimination tree, and leaf
// fronts are single leaf Elems (tens to ~150 DoFs) instead of whole refined trees.
#include <algorithm>
#include <array>
#include <cmath>
#include <functional>

#include <atomic>
#include <thread>

#include "common.h"
#include "domain.h"
#include "gep.h"
#include "mf.h"

namespace fem2d {

int num_host_threads();

namespace {
// f(t, i0, i1) on up to nt threads over [0, n) in contiguous chunks (inline for small n)
template <class F>
void chunked(int64_t n, F f) {
  const int nt = n < 64 ? 1 : num_host_threads();
  if (nt <= 1) {
    f(0, (int64_t)0, n);
    return;
  }
  std::vector<std::thread> th;
  const int64_t chunk = (n + nt - 1) / nt;
  for (int t = 0; t < nt; t++) {
    const int64_t a = t * chunk, b = std::min(n, a + chunk);
    if (a >= b) break;
    th.emplace_back([=]() { f(t, a, b); });
  }
  for (auto& x : th) x.join();
}
}  // namespace

void mf_symbolic(const Domain& d, const HostGEP& g, MFSymbolic& s, const std::vector<uint8_t>* lift) {
  const Mesh& m = d.mesh;
  const int64_t n = g.n;
  const int R = (int)m.roots.size();
  s = MFSymbolic();
  s.n = n;
  if (n == 0) return;

  // ---- build the tree in postorder: ND over base Elems, Elem refinement trees below
  std::vector<double> cx(R), cy(R);
  for (int r = 0; r < R; r++) {
    cx[r] = 0.5 * (m.roots[r].x0 + m.roots[r].x3);
    cy[r] = 0.5 * (m.roots[r].y0 + m.roots[r].y3);
  }
  std::vector<int32_t> parent, first_desc;
  std::vector<std::vector<int32_t>> kids;
  std::vector<int32_t> elem_node(m.elems.size(), -1);
  auto new_node = [&](int32_t first, const std::vector<int32_t>& ch) {
    int32_t id = (int32_t)parent.size();
    parent.push_back(-1);
    first_desc.push_back(first);
    kids.push_back(ch);
    for (int32_t c : ch) parent[c] = id;
    return id;
  };
  std::function<int32_t(int64_t)> build_elem = [&](int64_t e) -> int32_t {
    int32_t first = (int32_t)parent.size();
    std::vector<int32_t> ch;
    const MElem& el = m.elems[e];
    for (int k = 0; k < el.nchild; k++) ch.push_back(build_elem(el.child[k]));
    int32_t id = new_node(first, ch);
    elem_node[e] = id;
    return id;
  };
  std::function<int32_t(std::vector<int>&)> build = [&](std::vector<int>& roots) -> int32_t {
    if (roots.size() == 1) return build_elem(roots[0]);   // base Elem r is Elem r
    int32_t first = (int32_t)parent.size();
    double x0 = 1e300, x1 = -1e300, y0 = 1e300, y1 = -1e300;
    for (int r : roots) {
      x0 = std::min(x0, cx[r]); x1 = std::max(x1, cx[r]);
      y0 = std::min(y0, cy[r]); y1 = std::max(y1, cy[r]);
    }
    bool by_x = (x1 - x0) >= (y1 - y0);
    std::stable_sort(roots.begin(), roots.end(), [&](int a, int b) {
      double ka = by_x ? cx[a] : cy[a], kb = by_x ? cx[b] : cy[b];
      if (ka != kb) return ka < kb;
      double la = by_x ? cy[a] : cx[a], lb = by_x ? cy[b] : cx[b];
      return la != lb ? la < lb : a < b;
    });
    size_t half = roots.size() / 2;
    std::vector<int> lo(roots.begin(), roots.begin() + half), hi(roots.begin() + half, roots.end());
    int32_t a = build(lo);
    int32_t b = build(hi);
    return new_node(first, {a, b});
  };
  std::vector<int> all(R);
  for (int r = 0; r < R; r++) all[r] = r;
  build(all);
  const int NF = (int)parent.size();
  std::vector<int32_t> depth(NF, 0);
  for (int f = NF - 1; f >= 0; f--)
    if (parent[f] >= 0) depth[f] = depth[parent[f]] + 1;
  auto is_proper_anc = [&](int32_t a, int32_t x) { return a > x && first_desc[a] <= x; };
  auto lca = [&](int32_t a, int32_t b) {
    while (a != b) {
      if (depth[a] > depth[b]) a = parent[a];
      else if (depth[b] > depth[a]) b = parent[b];
      else { a = parent[a]; b = parent[b]; }
    }
    return a;
  };

  // ---- DoF -> node: the lowest common ancestor of the Elems the DoF is attached to
  std::vector<int32_t> node(n, -1);
  for (size_t e = 0; e + 1 < d.spec_ptr.size(); e++) {
    int32_t en = elem_node[e];
    for (int64_t k = d.spec_ptr[e]; k < d.spec_ptr[e + 1]; k++) {
      int32_t dof = d.specs[k].dof;
      node[dof] = node[dof] < 0 ? en : lca(node[dof], en);
    }
  }
  // delayed pivots: a DoF whose column could not be pivoted stably in its front is eliminated that many
  // levels higher (every coupling of the DoF stays on one root path, so the tree remains valid)
  if (lift && (int64_t)lift->size() == n)
    for (int64_t x = 0; x < n; x++)
      for (int l = 0; l < (*lift)[x] && node[x] >= 0 && parent[node[x]] >= 0; l++) node[x] = parent[node[x]];
  std::vector<std::vector<int32_t>> piv(NF);
  for (int64_t x = 0; x < n; x++) {
    if (node[x] < 0) fail(FEM2D_E_INVALID_ARG, "a DoF has no basis spec");
    piv[node[x]].push_back((int32_t)x);
  }
  std::vector<int64_t> order(n);
  {
    int64_t k = 0;
    for (int f = 0; f < NF; f++)
      for (int32_t x : piv[f]) order[x] = k++;
  }

  // ---- struct sets (bottom-up): fronts numbered in post-order, so a level's fronts depend only on
  // lower levels; the fronts of one level are processed in parallel, one mark array per thread
  std::vector<int32_t> lev(NF, 0);
  int nlev = 0;
  for (int f = 0; f < NF; f++) {
    for (int32_t c : kids[f]) lev[f] = std::max(lev[f], 1 + lev[c]);
    nlev = std::max(nlev, lev[f] + 1);
  }
  std::vector<std::vector<int32_t>> by_level(nlev);
  for (int f = 0; f < NF; f++) by_level[lev[f]].push_back(f);
  std::vector<std::vector<int32_t>> st(NF);
  const int nthr = std::max(1, num_host_threads());
  std::vector<std::vector<int32_t>> marks(nthr);
  for (int l = 0; l < nlev; l++) {
    const std::vector<int32_t>& fl = by_level[l];
    chunked((int64_t)fl.size(), [&](int t, int64_t i0, int64_t i1) {
      std::vector<int32_t>& mark = marks[t];
      if ((int64_t)mark.size() != n) mark.assign(n, -1);
      for (int64_t i = i0; i < i1; i++) {
        const int f = fl[i];
        std::vector<int32_t> cand;
        auto add = [&](int32_t y) {
          if (mark[y] == f) return;
          if (!is_proper_anc(node[y], f)) return;
          mark[y] = f;
          cand.push_back(y);
        };
        for (int32_t x : piv[f])
          for (int64_t k = g.row_ptr[x]; k < g.row_ptr[x + 1]; k++) add(g.col[k]);
        for (int32_t c : kids[f])
          for (int32_t y : st[c]) add(y);
        std::sort(cand.begin(), cand.end(), [&](int32_t a, int32_t b) { return order[a] < order[b]; });
        st[f] = std::move(cand);
      }
    });
  }

  // ---- fronts, maps, levels
  s.nfronts = NF;
  s.parent = parent;
  s.f.resize(NF);
  s.p.resize(NF);
  s.level.assign(NF, 0);
  s.dof_ptr.assign(NF + 1, 0);
  for (int f = 0; f < NF; f++) {
    s.p[f] = (int32_t)piv[f].size();
    s.f[f] = (int32_t)(piv[f].size() + st[f].size());
    s.dof_ptr[f + 1] = s.dof_ptr[f] + s.f[f];
    for (int32_t c : kids[f]) s.level[f] = std::max(s.level[f], 1 + s.level[c]);
    s.max_f = std::max(s.max_f, s.f[f]);
    s.max_p = std::max(s.max_p, s.p[f]);
    double F = s.f[f], P = s.p[f];
    s.flops += 2.0 * (F * F * F - (F - P) * (F - P) * (F - P)) / 3.0;
  }
  s.dofs.resize(s.dof_ptr[NF]);
  s.mat_off.resize(NF + 1);
  s.mat_off[0] = 0;
  for (int f = 0; f < NF; f++) {
    std::copy(piv[f].begin(), piv[f].end(), s.dofs.begin() + s.dof_ptr[f]);
    std::copy(st[f].begin(), st[f].end(), s.dofs.begin() + s.dof_ptr[f] + piv[f].size());
    s.mat_off[f + 1] = s.mat_off[f] + (int64_t)s.f[f] * s.f[f];
  }
  s.mat_total = s.mat_off[NF];
  // assembly maps: per front, the positions of its pivot rows' CSR entries (and their mirrors) in the
  // dense front, and the positions of each child's update rows in it. Counted and filled front by
  // front in parallel (one position array per thread), laid out in front order.
  std::vector<int64_t> acount(NF, 0);
  std::vector<std::vector<int32_t>> ea(NF);
  std::vector<std::vector<int32_t>> posv(nthr);
  std::atomic<int> bad_coupling{0}, bad_update{0};
  for (int pass = 0; pass < 2; pass++) {
    chunked((int64_t)NF, [&](int t, int64_t f0, int64_t f1) {
      std::vector<int32_t>& pos = posv[t];
      if ((int64_t)pos.size() != n) pos.assign(n, -1);
      for (int64_t f = f0; f < f1; f++) {
        const int32_t* D = s.dofs.data() + s.dof_ptr[f];
        const int F = s.f[f], P = s.p[f];
        for (int i = 0; i < F; i++) pos[D[i]] = i;
        int64_t w = pass == 0 ? 0 : s.asm_ptr[f];
        for (int i = 0; i < P; i++) {
          int32_t x = D[i];
          for (int64_t k = g.row_ptr[x]; k < g.row_ptr[x + 1]; k++) {
            // entries whose column was eliminated in a descendant front were assembled there
            const int32_t nc = node[g.col[k]];
            if (nc < f && nc >= first_desc[f]) continue;
            int32_t pc = pos[g.col[k]];
            if (pc < 0) {   // (reported after the threads join: no exception may leave a worker)
              bad_coupling = 1;
              continue;
            }
            if (pass == 0) {
              w += pc >= P ? 2 : 1;
              continue;
            }
            s.asm_pos[w] = (int64_t)i * F + pc;
            s.asm_csr[w++] = k;
            if (pc >= P) {
              s.asm_pos[w] = (int64_t)pc * F + i;
              s.asm_csr[w++] = k;
            }
          }
        }
        if (pass == 0) {
          acount[f] = w;
          for (int32_t ch : kids[f]) {
            std::vector<int32_t>& m = ea[ch];
            m.resize(st[ch].size());
            for (size_t q = 0; q < st[ch].size(); q++) {
              const int32_t y = st[ch][q];
              if (pos[y] < 0) bad_update = 1;
              m[q] = pos[y];
            }
          }
        }
        for (int i = 0; i < F; i++) pos[D[i]] = -1;
      }
    });
    if (bad_coupling) fail(FEM2D_E_INVALID_ARG, "multifrontal symbolic: coupling outside the front");
    if (bad_update) fail(FEM2D_E_INVALID_ARG, "multifrontal symbolic: child update outside the parent front");
    if (pass == 0) {
      s.asm_ptr.assign(NF + 1, 0);
      for (int f = 0; f < NF; f++) s.asm_ptr[f + 1] = s.asm_ptr[f] + acount[f];
      s.asm_pos.resize(s.asm_ptr[NF]);
      s.asm_csr.resize(s.asm_ptr[NF]);
    }
  }
  s.ea_ptr.assign(NF + 1, 0);
  for (int f = 0; f < NF; f++) s.ea_ptr[f + 1] = s.ea_ptr[f] + (int64_t)ea[f].size();
  s.ea_map.reserve(s.ea_ptr[NF]);
  for (int f = 0; f < NF; f++) s.ea_map.insert(s.ea_map.end(), ea[f].begin(), ea[f].end());
  s.nlevels = 0;
  for (int f = 0; f < NF; f++) s.nlevels = std::max(s.nlevels, s.level[f] + 1);
  s.level_ptr.assign(s.nlevels + 1, 0);
  for (int f = 0; f < NF; f++) s.level_ptr[s.level[f] + 1]++;
  for (int l = 0; l < s.nlevels; l++) s.level_ptr[l + 1] += s.level_ptr[l];
  s.level_fronts.resize(NF);
  std::vector<int32_t> cur(s.level_ptr.begin(), s.level_ptr.end() - 1);
  for (int f = 0; f < NF; f++) s.level_fronts[cur[s.level[f]]++] = f;
}

// One dense front holding every DoF: LU with partial pivoting over all rows (no restriction to a
// front's fully-summed rows). Used for small GEPs whose sparse factorization loses too many digits.
void mf_symbolic_dense(const HostGEP& g, MFSymbolic& s) {
  const int64_t n = g.n;
  s = MFSymbolic();
  s.n = n;
  if (n == 0) return;
  if (n > 46340) fail(FEM2D_E_TOO_LARGE, "dense factorization plan above 46340 DoFs");
  s.nfronts = 1;
  s.parent = {-1};
  s.level = {0};
  s.f = {(int32_t)n};
  s.p = {(int32_t)n};
  s.dof_ptr = {0, n};
  s.dofs.resize(n);
  for (int64_t i = 0; i < n; i++) s.dofs[i] = (int32_t)i;
  s.mat_off = {0, n * n};
  s.mat_total = n * n;
  s.asm_ptr = {0, (int64_t)g.col.size()};
  s.asm_pos.resize(g.col.size());
  s.asm_csr.resize(g.col.size());
  for (int64_t x = 0; x < n; x++)
    for (int64_t k = g.row_ptr[x]; k < g.row_ptr[x + 1]; k++) {
      s.asm_pos[k] = x * n + g.col[k];
      s.asm_csr[k] = k;
    }
  s.ea_ptr = {0, 0};
  s.nlevels = 1;
  s.level_ptr = {0, 1};
  s.level_fronts = {0};
  s.max_f = s.max_p = (int)n;
  s.flops = 2.0 * (double)n * n * n / 3.0;
}

}  // namespace fem2d
