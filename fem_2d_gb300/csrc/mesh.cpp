// RBS mesh: JSON import, h-/p-refinement and Edge activation.
// Reference: src/fem_domain/domain/mesh.rs (+ edge.rs, elem.rs, node.rs, element.rs,
// h_refinement.rs, p_refinement.rs, space.rs).
#include "mesh.h"

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstring>
#include <map>

#include "common.h"

namespace fem2d {

// ------------------------------------------------------------------ coordinates
QKey QKey::of(double v) {   // space.rs:364-376
  double mag = std::fabs(v);
  double ip = std::trunc(mag);
  double fr = std::round((mag - ip) / 1e-12) * 1e-12;
  double t = ip + fr;
  QKey k;
  k.pos = !std::signbit(v);
  std::memcpy(&k.bits, &t, sizeof t);
  return k;
}
int QKey::cmp(const QKey& o) const {   // space.rs:368-382
  if (pos != o.pos) return pos ? 1 : -1;
  if (bits == o.bits) return 0;
  bool lt = bits < o.bits;
  return pos ? (lt ? -1 : 1) : (lt ? 1 : -1);
}

static Axis axis_between(const Pt& a, const Pt& b) {   // space.rs:243-259
  if (a.same(b)) fail(FEM2D_E_MESH, "cannot orient an edge between two points at the same location");
  double dx = std::fabs(b.x - a.x), dy = std::fabs(b.y - a.y);
  return std::atan(dy / dx) < 0.78539816339744830962 ? AX_U : AX_V;
}
static double distance(const Pt& a, const Pt& b) {
  double dx = std::fabs(b.x - a.x), dy = std::fabs(b.y - a.y);
  return std::sqrt(dx * dx + dy * dy);
}

// ------------------------------------------------------------------ minimal JSON reader
namespace {
struct JVal {
  enum T { NUL, NUM, STR, ARR, OBJ, BOOL } t = NUL;
  double num = 0;
  std::string str;
  std::vector<JVal> arr;
  std::vector<std::pair<std::string, JVal>> obj;
  const JVal* get(const char* k) const {
    for (auto& kv : obj)
      if (kv.first == k) return &kv.second;
    return nullptr;
  }
};
struct JParser {
  const char* s;
  size_t i = 0, n;
  explicit JParser(const std::string& t) : s(t.c_str()), n(t.size()) {}
  void ws() {
    while (i < n && std::isspace((unsigned char)s[i])) i++;
  }
  [[noreturn]] void bad(const char* what) {
    fail(FEM2D_E_MESH, std::string("unable to parse mesh file as JSON: ") + what + " at offset " + std::to_string(i));
  }
  JVal value() {
    ws();
    if (i >= n) bad("unexpected end");
    char c = s[i];
    JVal v;
    if (c == '{') {
      v.t = JVal::OBJ;
      i++;
      ws();
      if (i < n && s[i] == '}') { i++; return v; }
      for (;;) {
        ws();
        if (i >= n || s[i] != '"') bad("expected key");
        std::string k = string_lit();
        ws();
        if (i >= n || s[i] != ':') bad("expected ':'");
        i++;
        v.obj.emplace_back(k, value());
        ws();
        if (i < n && s[i] == ',') { i++; continue; }
        if (i < n && s[i] == '}') { i++; return v; }
        bad("expected ',' or '}'");
      }
    }
    if (c == '[') {
      v.t = JVal::ARR;
      i++;
      ws();
      if (i < n && s[i] == ']') { i++; return v; }
      for (;;) {
        v.arr.push_back(value());
        ws();
        if (i < n && s[i] == ',') { i++; continue; }
        if (i < n && s[i] == ']') { i++; return v; }
        bad("expected ',' or ']'");
      }
    }
    if (c == '"') {
      v.t = JVal::STR;
      v.str = string_lit();
      return v;
    }
    if (!std::strncmp(s + i, "true", 4)) { i += 4; v.t = JVal::BOOL; v.num = 1; return v; }
    if (!std::strncmp(s + i, "false", 5)) { i += 5; v.t = JVal::BOOL; return v; }
    if (!std::strncmp(s + i, "null", 4)) { i += 4; return v; }
    char* end = nullptr;
    v.num = std::strtod(s + i, &end);
    if (end == s + i) bad("unexpected token");
    i = (size_t)(end - s);
    v.t = JVal::NUM;
    return v;
  }
  std::string string_lit() {
    std::string out;
    i++;
    while (i < n && s[i] != '"') {
      if (s[i] == '\\' && i + 1 < n) i++;
      out.push_back(s[i++]);
    }
    if (i >= n) bad("unterminated string");
    i++;
    return out;
  }
};
}  // namespace

// ------------------------------------------------------------------ construction
static const int kEdgeDefs[4][3] = {{0, 1, 1}, {2, 3, 0}, {0, 2, 1}, {1, 3, 0}};   // mesh.rs:1522-1531

Mesh Mesh::from_json(const std::string& text) {   // mesh.rs:142-327
  JParser p(text);
  JVal root = p.value();
  const JVal* jel = root.get("Elements");
  const JVal* jno = root.get("Nodes");
  if (!jel || jel->t != JVal::ARR) fail(FEM2D_E_MESH, "Elements must be an Array!");
  if (!jno || jno->t != JVal::ARR) fail(FEM2D_E_MESH, "Nodes must be an Array!");
  Mesh m;
  std::vector<Pt> pts;
  for (auto& jn : jno->arr) {
    if (jn.t != JVal::ARR || jn.arr.size() != 2) fail(FEM2D_E_MESH, "nodes must be arrays of length 2!");
    if (jn.arr[0].t != JVal::NUM || jn.arr[1].t != JVal::NUM)
      fail(FEM2D_E_MESH, "nodes must be composed of numerical values!");
    pts.emplace_back(jn.arr[0].num, jn.arr[1].num);
  }
  for (size_t a = 0; a < pts.size(); a++)
    for (size_t b = a + 1; b < pts.size(); b++)
      if (pts[a].same(pts[b])) fail(FEM2D_E_MESH, "All Nodes must be at unique locations!");
  std::vector<std::array<int64_t, 4>> ids;
  for (auto& je : jel->arr) {
    const JVal* ni = je.get("node_ids");
    const JVal* ma = je.get("materials");
    if (!ni || ni->t != JVal::ARR || ni->arr.size() != 4)
      fail(FEM2D_E_MESH, "Elements Array of node_ids must have a length of 4!");
    if (!ma || ma->t != JVal::ARR || ma->arr.size() != 4)
      fail(FEM2D_E_MESH, "Elements Array of materials must have a length of 4!");
    std::array<int64_t, 4> q;
    for (int k = 0; k < 4; k++) {
      const JVal& v = ni->arr[k];
      if (v.t != JVal::NUM || v.num < 0 || v.num != std::floor(v.num))
        fail(FEM2D_E_MESH, "node_ids must be positive integers!");
      q[k] = (int64_t)v.num;
      if ((size_t)q[k] >= pts.size()) fail(FEM2D_E_MESH, "node_ids must be smaller than the total number of nodes!");
    }
    for (int a = 0; a < 4; a++)
      for (int b = a + 1; b < 4; b++)
        if (q[a] == q[b]) fail(FEM2D_E_MESH, "Element's node_ids should have 4 unique values!");
    RootElement r;
    double mv[4];
    for (int k = 0; k < 4; k++) {
      if (ma->arr[k].t != JVal::NUM) fail(FEM2D_E_MESH, "Element materials must be numerical values");
      mv[k] = ma->arr[k].num;
    }
    r.x0 = pts[q[0]].x;
    r.y0 = pts[q[0]].y;
    r.x3 = pts[q[3]].x;
    r.y3 = pts[q[3]].y;
    r.eps_re = mv[0];
    r.eps_im = mv[1];
    r.mu_re = mv[2];
    r.mu_im = mv[3];
    m.roots.push_back(r);
    ids.push_back(q);
  }
  std::vector<int> uses(pts.size(), 0);
  for (auto& q : ids)
    for (int k = 0; k < 4; k++) uses[q[k]]++;
  for (size_t k = 0; k < pts.size(); k++) {
    if (uses[k] > 4) fail(FEM2D_E_MESH, "Nodes can only be shared by a maximum of 4 Elements");
    m.nodes.push_back({pts[k], uses[k] < 4});
  }
  // edge records keyed by their ordered node pair, in key order (BTreeMap iteration, mesh.rs:222-251)
  struct Rec { int64_t a, b; int side; int64_t el; };
  std::vector<Rec> recs;
  for (size_t e = 0; e < ids.size(); e++)
    for (auto& d : kEdgeDefs) recs.push_back({ids[e][d[0]], ids[e][d[1]], d[2], (int64_t)e});
  std::stable_sort(recs.begin(), recs.end(), [](const Rec& x, const Rec& y) {
    return x.a != y.a ? x.a < y.a : x.b < y.b;
  });
  std::vector<std::array<int64_t, 4>> el_edges(ids.size(), {-1, -1, -1, -1});
  for (size_t k = 0; k < recs.size();) {
    size_t j = k;
    int64_t sides[2] = {-1, -1};
    while (j < recs.size() && recs[j].a == recs[k].a && recs[j].b == recs[k].b) {
      if (sides[recs[j].side] >= 0) fail(FEM2D_E_MESH, "an Edge side is claimed by two Elements");
      sides[recs[j].side] = recs[j].el;
      j++;
    }
    MEdge ed;
    ed.n0 = recs[k].a;
    ed.n1 = recs[k].b;
    ed.boundary = (sides[0] < 0) != (sides[1] < 0);
    ed.dir = axis_between(m.nodes[ed.n0].p, m.nodes[ed.n1].p);
    ed.length = distance(m.nodes[ed.n0].p, m.nodes[ed.n1].p);
    int64_t id = (int64_t)m.edges.size();
    for (int s = 0; s < 2; s++) {
      if (sides[s] < 0) continue;
      int idx = ed.dir == AX_U ? (s == 0 ? 1 : 0) : (s == 0 ? 3 : 2);
      if (el_edges[sides[s]][idx] >= 0) fail(FEM2D_E_MESH, "an Elem edge slot is claimed twice");
      el_edges[sides[s]][idx] = id;
    }
    m.edges.push_back(ed);
    k = j;
  }
  for (size_t e = 0; e < ids.size(); e++) {
    MElem el;
    for (int k = 0; k < 4; k++) {
      el.nodes[k] = ids[e][k];
      if (el_edges[e][k] < 0) fail(FEM2D_E_MESH, "an Elem is missing an Edge");
      el.edges[k] = el_edges[e][k];
    }
    el.root = (int64_t)e;
    m.elems.push_back(el);
  }
  for (size_t e = 0; e < m.elems.size(); e++)
    for (int k = 0; k < 4; k++) m.attach(m.elems[e].edges[k], (int64_t)e);
  m.set_edge_activation();
  return m;
}

Mesh Mesh::unit() {   // mesh.rs:58-91 (its Edges are not connected to the Elem)
  Mesh m;
  m.roots.push_back({-1.0, -1.0, 1.0, 1.0, 1.0, 0.0, 1.0, 0.0});
  const double c[4][2] = {{-1, -1}, {1, -1}, {-1, 1}, {1, 1}};
  for (auto& q : c) m.nodes.push_back({Pt(q[0], q[1]), true});
  const int en[4][2] = {{0, 1}, {2, 3}, {0, 2}, {1, 3}};
  for (auto& q : en) {
    MEdge ed;
    ed.n0 = q[0];
    ed.n1 = q[1];
    ed.boundary = true;
    ed.dir = axis_between(m.nodes[q[0]].p, m.nodes[q[1]].p);
    ed.length = distance(m.nodes[q[0]].p, m.nodes[q[1]].p);
    m.edges.push_back(ed);
  }
  MElem el;
  for (int k = 0; k < 4; k++) { el.nodes[k] = k; el.edges[k] = k; }
  el.root = 0;
  m.elems.push_back(el);
  return m;
}

// edge.rs:36-62: the Elem lies on side 1 of its edges 0 and 2 and on side 0 of edges 1 and 3
void Mesh::attach(int64_t e, int64_t elem) {
  MEdge& ed = edges[e];
  const MElem& el = elems[elem];
  int idx = -1;
  for (int k = 0; k < 4; k++)
    if (el.edges[k] == e) idx = k;
  if (idx < 0) fail(FEM2D_E_MESH, "Elem is not connected to this Edge");
  uint16_t rank = ed.dir == AX_U ? (uint16_t)((el.hv << 8) | el.hu) : (uint16_t)((el.hu << 8) | el.hv);
  auto& side = ed.side[(idx == 0 || idx == 2) ? 1 : 0];
  for (auto& r : side)
    if (r.first == rank) {
      if (r.second != elem) fail(FEM2D_E_MESH, "two Elems connect to one Edge at the same level");
      return;
    }
  side.emplace_back(rank, elem);
}

// ------------------------------------------------------------------ activation (mesh.rs:1180-1215)
bool Mesh::activate_tree(int64_t e) {
  MEdge& ed = edges[e];
  if (ed.side[0].empty() || ed.side[1].empty()) {
    ed.active = false;
    return false;
  }
  for (int s = 0; s < 2; s++) {
    auto best = ed.side[s][0];
    for (auto& r : ed.side[s])
      if (r.first > best.first) best = r;
    ed.act[s] = best.second;
  }
  ed.active = true;
  if (ed.child[0] >= 0) {
    bool a = activate_tree(ed.child[0]);
    bool b = activate_tree(ed.child[1]);
    if (a && b) edges[e].active = false;
    else if (a != b) fail(FEM2D_E_MESH, "children of an Edge do not have consistent support for basis functions");
  }
  return true;
}

void Mesh::set_edge_activation() {
  for (auto& ed : edges) ed.active = false;
  for (size_t e = 0; e < edges.size(); e++)
    if (edges[e].parent < 0 && !edges[e].boundary && !activate_tree((int64_t)e))
      fail(FEM2D_E_MESH, "unable to find an active Edge pair over Edge " + std::to_string(e));
}

// ------------------------------------------------------------------ queries
bool Mesh::refineable(int64_t e) const {   // mesh.rs:649-662
  const MElem& el = elems[e];
  if (!el.leaf()) return false;
  for (int k = 0; k < 4; k++)
    if (!(edges[el.edges[k]].length > 3.0518e-5)) return false;
  return true;
}

std::array<int, 2> Mesh::max_orders() const {
  std::array<int, 2> r = {0, 0};
  for (auto& el : elems) {
    r[0] = std::max(r[0], (int)el.ni);
    r[1] = std::max(r[1], (int)el.nj);
  }
  return r;
}

static void shrink(uint8_t loc, double& a, double& b, bool u_axis) {   // h_refinement.rs:247-279
  double mid = (a + b) / 2.0;
  bool low, high;
  if (u_axis) {
    low = loc == L_SW || loc == L_NW || loc == L_W;
    high = loc == L_SE || loc == L_NE || loc == L_E;
  } else {
    low = loc == L_SW || loc == L_SE || loc == L_S;
    high = loc == L_NW || loc == L_NE || loc == L_N;
  }
  if (low) b = mid;
  else if (high) a = mid;
}

std::array<double, 4> Mesh::relative_range(int64_t e, int64_t a) const {
  const MElem& el = elems[e];
  size_t start = el.anc.size();
  for (size_t k = 0; k < el.anc.size(); k++)
    if (el.anc[k] == a) { start = k; break; }
  if (a >= 0 && start == el.anc.size()) fail(FEM2D_E_INVALID_ARG, "not an ancestor");
  if (a < 0) start = 0;
  std::array<double, 4> r = {-1.0, 1.0, -1.0, 1.0};
  for (size_t k = start; k < el.anc.size(); k++) {
    shrink(el.locs[k], r[0], r[1], true);
    shrink(el.locs[k], r[2], r[3], false);
  }
  return r;
}

std::array<double, 4> Mesh::param_range(int64_t e) const { return relative_range(e, -1); }

ElemJac elem_jacobian(const Mesh& m, int64_t e) {
  auto pr = m.param_range(e);
  const RootElement& r = m.roots[m.elems[e].root];
  auto mr = [](double v, double lo, double hi) { return (v - -1.0) * (hi - lo) / (1.0 - -1.0) + lo; };
  double xmin = mr(pr[0], r.x0, r.x3), xmax = mr(pr[1], r.x0, r.x3);
  double ymin = mr(pr[2], r.y0, r.y3), ymax = mr(pr[3], r.y0, r.y3);
  ElemJac j;
  j.a = (xmax - xmin) / 2.0;
  j.b = (ymax - ymin) / 2.0;
  j.det = j.a * j.b - 0.0 * 0.0;
  j.ji_u0 = j.b / j.det;
  j.ji_v1 = j.a / j.det;
  return j;
}

void Mesh::descendants(int64_t e, std::vector<int64_t>& out) const {
  const MElem& el = elems[e];
  for (int k = 0; k < el.nchild; k++) {
    out.push_back(el.child[k]);
    descendants(el.child[k], out);
  }
}

// ------------------------------------------------------------------ p-refinement
void Mesh::set_expansion(const std::vector<int64_t>& ids, int i, int j) {   // mesh.rs:1446-1468
  if (i < 1 || j < 1 || i > 20 || j > 20)
    fail(FEM2D_E_PREF, "Invalid expansion orders: (" + std::to_string(i) + ", " + std::to_string(j) + ")");
  for (size_t a = 0; a < ids.size(); a++) {
    if (ids[a] < 0 || (size_t)ids[a] >= elems.size()) fail(FEM2D_E_PREF, "Elem does not exist");
    for (size_t b = a + 1; b < ids.size(); b++)
      if (ids[a] == ids[b]) fail(FEM2D_E_PREF, "Duplicate element ids in p-Refinement");
  }
  for (int64_t id : ids) {
    elems[id].ni = (uint8_t)i;
    elems[id].nj = (uint8_t)j;
  }
}

void Mesh::p_refine(const std::vector<int64_t>& ids, int di, int dj, bool clamp_to_window) {
  // mesh.rs:1236-1424, p_refinement.rs:86-188: deltas per Elem summed, window [1-n, 20-n] checked
  if (!clamp_to_window)
    for (size_t a = 0; a < ids.size(); a++)
      for (size_t b = a + 1; b < ids.size(); b++)
        if (ids[a] == ids[b]) fail(FEM2D_E_PREF, "Duplicate element ids in p-Refinement");
  std::map<int64_t, std::array<int, 2>> acc;
  for (int64_t id : ids) {
    if (id < 0 || (size_t)id >= elems.size()) fail(FEM2D_E_PREF, "Elem does not exist");
    int a = di, b = dj;
    if (clamp_to_window) {
      a = std::min(std::max(a, 1 - (int)elems[id].ni), 20 - (int)elems[id].ni);
      b = std::min(std::max(b, 1 - (int)elems[id].nj), 20 - (int)elems[id].nj);
    }
    auto& s = acc[id];
    s[0] += a;
    s[1] += b;
  }
  for (auto& kv : acc) {
    const MElem& el = elems[kv.first];
    if (kv.second[0] < 1 - el.ni || kv.second[0] > 20 - el.ni || kv.second[1] < 1 - el.nj ||
        kv.second[1] > 20 - el.nj)
      fail(FEM2D_E_PREF, "Refinement out of bounds for Elem " + std::to_string(kv.first));
  }
  for (auto& kv : acc) {
    elems[kv.first].ni = (uint8_t)(elems[kv.first].ni + kv.second[0]);
    elems[kv.first].nj = (uint8_t)(elems[kv.first].nj + kv.second[1]);
  }
}

// ------------------------------------------------------------------ h-refinement
// Split an Edge (or reuse its children): two edge ids, then one node id (mesh.rs:1091-1122).
int64_t Mesh::split_edge(int64_t pe, int64_t& next_node, int64_t& next_edge, int64_t ch[2]) {
  if (edges[pe].child[0] >= 0) {
    ch[0] = edges[pe].child[0];
    ch[1] = edges[pe].child[1];
    return edges[pe].mid_node;
  }
  int64_t e0 = next_edge, e1 = next_edge + 1;
  next_edge += 2;
  int64_t nn = next_node++;
  double half = edges[pe].length / 2.0;
  if (half < 3.0518e-5) fail(FEM2D_E_HREF, "h-refinement would make an Edge shorter than the minimum length");
  if ((int64_t)edges.size() != e0 || (int64_t)nodes.size() != nn) fail(FEM2D_E_HREF, "id allocation out of order");
  edges[pe].child[0] = e0;
  edges[pe].child[1] = e1;
  edges[pe].mid_node = nn;
  MEdge a, b;
  a.n0 = edges[pe].n0;
  a.n1 = nn;
  b.n0 = nn;
  b.n1 = edges[pe].n1;
  for (MEdge* c : {&a, &b}) {
    c->boundary = edges[pe].boundary;
    c->dir = edges[pe].dir;
    c->length = half;
    c->parent = pe;
  }
  const Pt& p0 = nodes[edges[pe].n0].p;
  const Pt& p1 = nodes[edges[pe].n1].p;
  bool bnd = edges[pe].boundary;
  edges.push_back(a);
  edges.push_back(b);
  nodes.push_back({Pt((p0.x + p1.x) / 2.0, (p0.y + p1.y) / 2.0), bnd});
  ch[0] = e0;
  ch[1] = e1;
  return nn;
}

// New interior Edge with its nodes ordered along its axis (mesh.rs:1124-1152, element.rs:52-57).
int64_t Mesh::join_nodes(int64_t a, int64_t b, int64_t& next_edge) {
  if (a == b) fail(FEM2D_E_HREF, "an Edge cannot join a Node to itself");
  int64_t id = next_edge++;
  const Pt& pa = nodes[a].p;
  const Pt& pb = nodes[b].p;
  Axis ax = axis_between(pa, pb);
  int c = ax == AX_U ? pa.kx.cmp(pb.kx) : pa.ky.cmp(pb.ky);
  if (c == 0) fail(FEM2D_E_HREF, "attempt to generate a child Edge between two identical points");
  MEdge ed;
  ed.n0 = c < 0 ? a : b;
  ed.n1 = c < 0 ? b : a;
  ed.boundary = false;
  ed.dir = ax;
  ed.length = distance(pa, pb);
  if ((int64_t)edges.size() != id) fail(FEM2D_E_HREF, "id allocation out of order");
  edges.push_back(ed);
  return id;
}

void Mesh::execute_h_refinements(const std::vector<int64_t>& ids, const std::vector<int>& kinds,
                                 const std::vector<int>& exts) {
  // mesh.rs:844-914: one refinement per Elem (duplicates merged by HRef +=, h_refinement.rs:159-195)
  std::map<int64_t, std::pair<int, int>> plan;
  for (size_t k = 0; k < ids.size(); k++) {
    int64_t id = ids[k];
    if (id < 0 || (size_t)id >= elems.size()) fail(FEM2D_E_HREF, "Elem " + std::to_string(id) + " does not exist");
    if (!refineable(id)) fail(FEM2D_E_HREF, "Elem " + std::to_string(id) + " cannot be h-refined");
    int kind = kinds[k], ext = exts[k];
    auto it = plan.find(id);
    if (it == plan.end()) { plan[id] = {kind, ext}; continue; }
    auto& cur = it->second;
    if (cur.first == 0) continue;
    bool other_axis = (cur.first == 1 && kind == 2) || (cur.first == 2 && kind == 1);
    if (kind == 0 || other_axis) cur = {0, -1};
    else if (cur.second >= 0 && ext >= 0 && ext != cur.second) cur = {0, -1};
  }
  std::vector<int64_t> x_ids;
  std::vector<int> x_kinds, x_exts;
  int64_t next_elem = (int64_t)elems.size();
  int64_t next_node = (int64_t)nodes.size(), next_edge = (int64_t)edges.size();
  for (auto& kv : plan) {
    int64_t pid = kv.first;
    int kind = kv.second.first, ext = kv.second.second;
    int nch = kind == 0 ? 4 : 2;
    MElem par = elems[pid];
    std::vector<MElem> kids(nch);
    for (int k = 0; k < nch; k++) {
      MElem& c = kids[k];
      std::fill(c.nodes, c.nodes + 4, -1);
      std::fill(c.edges, c.edges + 4, -1);
      c.root = par.root;
      c.anc = par.anc;
      c.anc.push_back(pid);
      c.locs = par.locs;
      c.locs.push_back((uint8_t)(kind == 0 ? L_SW + k : (kind == 1 ? L_W + k : L_S + k)));
      c.hu = (uint8_t)(par.hu + (kind != 2));
      c.hv = (uint8_t)(par.hv + (kind != 1));
      c.ni = par.ni;
      c.nj = par.nj;
      elems[pid].child[k] = next_elem + k;
    }
    elems[pid].nchild = (int8_t)nch;
    auto set_node = [&](int c, int slot, int64_t id) {
      if (kids[c].nodes[slot] >= 0 && kids[c].nodes[slot] != id) fail(FEM2D_E_HREF, "Node slot set twice");
      kids[c].nodes[slot] = id;
    };
    auto set_edge = [&](int c, int slot, int64_t id) {
      if (kids[c].edges[slot] >= 0) fail(FEM2D_E_HREF, "Edge slot set twice");
      kids[c].edges[slot] = id;
    };
    if (kind == 0) {   // mesh.rs:915-983
      const Pt& a = nodes[par.nodes[0]].p;
      const Pt& b = nodes[par.nodes[3]].p;
      int64_t center = next_node++;
      if ((int64_t)nodes.size() != center) fail(FEM2D_E_HREF, "id allocation out of order");
      nodes.push_back({Pt((a.x + b.x) / 2.0, (a.y + b.y) / 2.0), false});
      for (int k = 0; k < 4; k++) {
        set_node(k, 3 - k, center);
        set_node(k, k, par.nodes[k]);
      }
      // (parent edge, children on it, their slot for the shared node, their slot for the new edge)
      const int plan_t[4][7] = {{0, 0, 1, 1, 0, 3, 2}, {1, 2, 3, 3, 2, 3, 2}, {2, 0, 2, 2, 0, 1, 0}, {3, 1, 3, 3, 1, 1, 0}};
      for (auto& r : plan_t) {
        int64_t ch[2];
        int64_t mid = split_edge(par.edges[r[0]], next_node, next_edge, ch);
        set_edge(r[1], r[0], ch[0]);
        set_edge(r[2], r[0], ch[1]);
        set_node(r[1], r[3], mid);
        set_node(r[2], r[4], mid);
        int64_t ne = join_nodes(mid, center, next_edge);
        set_edge(r[1], r[5], ne);
        set_edge(r[2], r[6], ne);
      }
    } else {   // mesh.rs:985-1089
      bool u = kind == 1;
      const int plan_u[2][5] = {{0, 1, 0, 0, 1}, {1, 3, 2, 2, 3}};
      const int plan_v[2][5] = {{2, 2, 0, 0, 2}, {3, 3, 1, 1, 3}};
      int64_t mids[2];
      for (int t = 0; t < 2; t++) {
        const int* r = u ? plan_u[t] : plan_v[t];
        int64_t ch[2];
        mids[t] = split_edge(par.edges[r[0]], next_node, next_edge, ch);
        set_edge(0, r[0], ch[0]);
        set_edge(1, r[0], ch[1]);
        set_node(0, r[1], mids[t]);
        set_node(1, r[2], mids[t]);
        set_node(0, r[3], par.nodes[r[3]]);
        set_node(1, r[4], par.nodes[r[4]]);
      }
      int64_t ne = join_nodes(mids[0], mids[1], next_edge);
      if (u) {
        set_edge(0, 3, ne);
        set_edge(1, 2, ne);
        set_edge(0, 2, par.edges[2]);
        set_edge(1, 3, par.edges[3]);
      } else {
        set_edge(0, 1, ne);
        set_edge(1, 0, ne);
        set_edge(0, 0, par.edges[0]);
        set_edge(1, 1, par.edges[1]);
      }
    }
    for (int k = 0; k < nch; k++)
      for (int s = 0; s < 4; s++)
        if (kids[k].nodes[s] < 0 || kids[k].edges[s] < 0) fail(FEM2D_E_HREF, "child Elem left uninitialized");
    for (int k = 0; k < nch; k++) elems.push_back(kids[k]);
    for (int k = 0; k < nch; k++)
      for (int s = 0; s < 4; s++) attach(elems[next_elem + k].edges[s], next_elem + k);
    if (kind != 0 && ext >= 0) {
      x_ids.push_back(next_elem + ext);
      x_kinds.push_back(kind == 1 ? 2 : 1);
      x_exts.push_back(-1);
    }
    next_elem += nch;
  }
  if (!x_ids.empty()) execute_h_refinements(x_ids, x_kinds, x_exts);
  set_edge_activation();
}

void Mesh::global_h_refinement(int kind, int ext) {
  std::vector<int64_t> ids;
  for (size_t e = 0; e < elems.size(); e++)
    if (refineable((int64_t)e)) ids.push_back((int64_t)e);
  execute_h_refinements(ids, std::vector<int>(ids.size(), kind), std::vector<int>(ids.size(), ext));
}

void Mesh::h_refine_elems(const std::vector<int64_t>& ids, int kind, int ext) {
  for (size_t a = 0; a < ids.size(); a++)
    for (size_t b = a + 1; b < ids.size(); b++)
      if (ids[a] == ids[b]) fail(FEM2D_E_HREF, "Duplicate element ids in h-Refinement");
  execute_h_refinements(ids, std::vector<int>(ids.size(), kind), std::vector<int>(ids.size(), ext));
}

}  // namespace fem2d
