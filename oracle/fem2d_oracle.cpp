// fem2d oracle: a literal CPU restatement of fem_2d's Galerkin GEP path.
//
// TEST INFRASTRUCTURE ONLY. This file is the checker for the GPU product in
// fem_2d_gb300/. Only tests/, __graft_entry__.smoke() and bench.py's CPU
// baseline leg may load the library built from it. The product never links it.
//
// Every function follows the reference (jeremiah-corrado/fem_2d, Rust) step by
// step, including its iteration orders, so that DoF numbering and the sparsity
// pattern are bit-exact and the values agree to rounding. Citations are
// path:line within the reference project.
//
// Pinned by: the reference's known-answer tests (src/lib.rs:46-120),
// test_input/test_eval.dat, test_input/test_evec.dat, and the GLQ tables in
// src/fem_problem/integration/glq.rs:255-375 (see tests/test_oracle_golden.py).
#include <algorithm>
#include <atomic>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

namespace oracle {

// ---------------------------------------------------------------------------
// space.rs: Point, FloatRep (src/fem_domain/domain/mesh/space.rs:222-382)
// ---------------------------------------------------------------------------
static const double POINT_UNIQUENESS_ACCURACY = 1e-12;   // space.rs:218

struct FloatRep {   // space.rs:349-382
  bool sign;
  uint64_t bits;
  static FloatRep from(double value) {
    double ip = std::trunc(std::fabs(value));
    double fr = std::fabs(value) - ip;
    double fr_r = std::round(fr / POINT_UNIQUENESS_ACCURACY) * POINT_UNIQUENESS_ACCURACY;
    double tot = ip + fr_r;
    FloatRep r;
    r.sign = !std::signbit(value);
    std::memcpy(&r.bits, &tot, 8);
    return r;
  }
  int cmp(const FloatRep& o) const {
    if (sign && o.sign) return bits < o.bits ? -1 : (bits > o.bits ? 1 : 0);
    if (!sign && o.sign) return -1;
    if (sign && !o.sign) return 1;
    return bits < o.bits ? 1 : (bits > o.bits ? -1 : 0);
  }
  bool operator==(const FloatRep& o) const { return sign == o.sign && bits == o.bits; }
};

enum ParaDir { DIR_U = 0, DIR_V = 1 };

struct Point {
  double x, y;
  FloatRep xc, yc;
  Point() : x(0), y(0), xc(FloatRep::from(0.0)), yc(FloatRep::from(0.0)) {}
  Point(double x_, double y_) : x(x_), y(y_), xc(FloatRep::from(x_)), yc(FloatRep::from(y_)) {}
  static Point between(const Point& a, const Point& b) {   // space.rs:230-232
    return Point((a.x + b.x) / 2.0, (a.y + b.y) / 2.0);
  }
  ParaDir orientation_with(const Point& o) const {   // space.rs:243-259
    if (xc == o.xc && yc == o.yc) throw std::runtime_error("orientation between equal points");
    double dx = std::fabs(o.x - x), dy = std::fabs(o.y - y);
    double theta = std::atan(dy / dx);
    return theta < M_PI / 4.0 ? DIR_U : DIR_V;
  }
  double dist(const Point& o) const {   // space.rs:261-266
    double dx = std::fabs(o.x - x), dy = std::fabs(o.y - y);
    return std::sqrt(dx * dx + dy * dy);
  }
  bool operator==(const Point& o) const { return xc == o.xc && yc == o.yc; }
};

// ---------------------------------------------------------------------------
// h_refinement.rs (src/fem_domain/domain/mesh/h_refinement.rs)
// ---------------------------------------------------------------------------
struct HLevels { uint8_t u = 0, v = 0; };
enum HRefKind { HREF_T = 0, HREF_U = 1, HREF_V = 2 };
struct HRef { int kind; int ext; };   // ext = -1 for None, else child index
enum HRefLoc { SW = 0, SE, NW, NE, W, E, S, N };

static HLevels refined(HLevels h, HRef r) {   // h_refinement.rs:22-28
  if (r.kind == HREF_T) return {uint8_t(h.u + 1), uint8_t(h.v + 1)};
  if (r.kind == HREF_U) return {uint8_t(h.u + 1), h.v};
  return {h.u, uint8_t(h.v + 1)};
}
static std::array<uint8_t, 2> edge_ranking(HLevels h, ParaDir d) {   // h_refinement.rs:31-36
  if (d == DIR_U) return {h.v, h.u};
  return {h.u, h.v};
}
static HRefLoc href_loc(HRef r, int idx) {   // h_refinement.rs:119-140
  if (r.kind == HREF_T) return (HRefLoc)(SW + idx);
  if (r.kind == HREF_U) return idx == 0 ? W : E;
  return idx == 0 ? S : N;
}
static void href_add_assign(HRef& self, HRef rhs) {   // h_refinement.rs:159-195
  if (self.kind == HREF_T) return;
  if (self.kind == HREF_U && self.ext < 0) {
    if (rhs.kind == HREF_V || rhs.kind == HREF_T) self = {HREF_T, -1};
  } else if (self.kind == HREF_V && self.ext < 0) {
    if (rhs.kind == HREF_U || rhs.kind == HREF_T) self = {HREF_T, -1};
  } else if (self.kind == HREF_U) {
    if (rhs.kind == HREF_U && rhs.ext >= 0) { if (rhs.ext != self.ext) self = {HREF_T, -1}; }
    else if (rhs.kind == HREF_V || rhs.kind == HREF_T) self = {HREF_T, -1};
  } else {
    if (rhs.kind == HREF_V && rhs.ext >= 0) { if (rhs.ext != self.ext) self = {HREF_T, -1}; }
    else if (rhs.kind == HREF_U || rhs.kind == HREF_T) self = {HREF_T, -1};
  }
}
typedef std::array<std::array<double, 2>, 2> Range2;
static std::array<double, 2> sub_u(HRefLoc l, std::array<double, 2> r) {   // h_refinement.rs:252-265
  double mid = (r[0] + r[1]) / 2.0;
  switch (l) {
    case SW: case NW: case W: return {r[0], mid};
    case SE: case NE: case E: return {mid, r[1]};
    default: return r;
  }
}
static std::array<double, 2> sub_v(HRefLoc l, std::array<double, 2> r) {   // h_refinement.rs:267-279
  double mid = (r[0] + r[1]) / 2.0;
  switch (l) {
    case SW: case SE: case S: return {r[0], mid};
    case NW: case NE: case N: return {mid, r[1]};
    default: return r;
  }
}
static Range2 sub_range(HRefLoc l, Range2 r) { return {sub_u(l, r[0]), sub_v(l, r[1])}; }

// ---------------------------------------------------------------------------
// mesh entities (node.rs, edge.rs, elem.rs, element.rs)
// ---------------------------------------------------------------------------
static const double MIN_EDGE_LENGTH = 3.0518e-5;   // mesh.rs:36
static const int MAX_POLYNOMIAL_ORDER = 20;         // mesh.rs:42

struct Element {   // element.rs:7-60
  size_t id;
  Point points[4];
  double eps_re, eps_im, mu_re, mu_im;
};

typedef std::map<std::array<uint8_t, 2>, size_t> RankMap;

struct Node {
  size_t id;
  Point coords;
  bool boundary;
  RankMap elems[4];
};

struct Edge {   // edge.rs:7-36
  size_t id;
  size_t nodes[2];
  bool boundary;
  ParaDir dir;
  double length;
  bool has_children = false;
  size_t children[2] = {0, 0};
  long parent = -1;
  RankMap elems[2];
  bool active = false;
  size_t active_elems[2] = {0, 0};
  size_t child_node = 0;
};

struct Elem {   // elem.rs:12-36
  size_t id;
  size_t nodes[4];
  size_t edges[4];
  size_t element;
  HLevels h_levels;
  uint8_t ni = 1, nj = 1;   // PolyOrders::default p_refinement.rs:74-78
  bool has_children = false;
  std::vector<size_t> children;
  std::vector<std::pair<size_t, HRefLoc>> ancestors;
};

struct ElemUninit {   // elem.rs:200-330
  size_t id;
  long nodes[4] = {-1, -1, -1, -1};
  long edges[4] = {-1, -1, -1, -1};
  size_t element;
  std::vector<std::pair<size_t, HRefLoc>> ancestors;
  HLevels h_levels;
  uint8_t ni, nj;
  void set_node(int idx, size_t id_) {
    if (nodes[idx] >= 0 && (size_t)nodes[idx] != id_) throw std::runtime_error("node already set");
    nodes[idx] = (long)id_;
  }
  void set_edge(int idx, size_t id_) {
    if (edges[idx] >= 0) throw std::runtime_error("edge already set");
    edges[idx] = (long)id_;
  }
};

struct Mesh {
  std::vector<Element> elements;
  std::vector<Elem> elems;
  std::vector<Node> nodes;
  std::vector<Edge> edges;

  // edge.rs:36-62
  void edge_connect_elem(Edge& e, const Elem& el) {
    int idx = -1;
    for (int k = 0; k < 4; k++)
      if (el.edges[k] == e.id) { idx = k; break; }
    if (idx < 0) throw std::runtime_error("elem not connected to edge");
    auto addr = edge_ranking(el.h_levels, e.dir);
    int side = (idx == 0 || idx == 2) ? 1 : 0;
    auto it = e.elems[side].find(addr);
    if (it != e.elems[side].end()) {
      if (it->second != el.id) throw std::runtime_error("edge already connected at rank");
    } else {
      e.elems[side][addr] = el.id;
    }
  }
  // node.rs:31-52
  void node_connect_elem(Node& n, const Elem& el) {
    int idx = -1;
    for (int k = 0; k < 4; k++)
      if (el.nodes[k] == n.id) { idx = k; break; }
    if (idx < 0) throw std::runtime_error("elem not connected to node");
    std::array<uint8_t, 2> addr = {el.h_levels.u, el.h_levels.v};
    auto it = n.elems[idx].find(addr);
    if (it != n.elems[idx].end()) {
      if (it->second != el.id) throw std::runtime_error("node already connected");
    } else {
      n.elems[idx][addr] = el.id;
    }
  }

  Edge new_edge(size_t id, size_t n0, size_t n1, bool boundary) {   // edge.rs:21-35
    Edge e;
    e.id = id;
    e.nodes[0] = n0;
    e.nodes[1] = n1;
    e.boundary = boundary;
    e.dir = nodes[n0].coords.orientation_with(nodes[n1].coords);
    e.length = nodes[n0].coords.dist(nodes[n1].coords);
    return e;
  }

  // mesh.rs:142-327 (Mesh::from_file, after JSON parsing)
  void from_arrays(size_t n_nodes, const double* xy, size_t n_el, const int64_t* node_ids,
                   const double* mats) {
    std::vector<Point> points(n_nodes);
    for (size_t i = 0; i < n_nodes; i++) points[i] = Point(xy[2 * i], xy[2 * i + 1]);
    for (size_t i = 0; i < n_nodes; i++)
      for (size_t j = i + 1; j < n_nodes; j++)
        if (points[i] == points[j]) throw std::runtime_error("duplicate nodes");
    for (size_t e = 0; e < n_el; e++) {
      Element el;
      el.id = e;
      for (int k = 0; k < 4; k++) {
        int64_t nid = node_ids[4 * e + k];
        if (nid < 0 || (size_t)nid >= n_nodes) throw std::runtime_error("bad node id");
        el.points[k] = points[nid];
      }
      el.eps_re = mats[4 * e + 0];
      el.eps_im = mats[4 * e + 1];
      el.mu_re = mats[4 * e + 2];
      el.mu_im = mats[4 * e + 3];
      elements.push_back(el);
    }
    std::vector<int> counts(n_nodes, 0);
    for (size_t e = 0; e < n_el; e++)
      for (int k = 0; k < 4; k++) counts[node_ids[4 * e + k]]++;
    for (size_t i = 0; i < n_nodes; i++) {
      if (counts[i] > 4) throw std::runtime_error("node shared by more than 4 elements");
      Node n;
      n.id = i;
      n.coords = points[i];
      n.boundary = counts[i] < 4;
      nodes.push_back(n);
    }
    // EDGE_IDX_DEFS mesh.rs:1530-1531
    const int defs[4][3] = {{0, 1, 1}, {2, 3, 0}, {0, 2, 1}, {1, 3, 0}};
    std::map<std::array<size_t, 2>, std::array<long, 2>> edge_node_pairs;
    for (size_t e = 0; e < n_el; e++) {
      for (int d = 0; d < 4; d++) {
        std::array<size_t, 2> key = {(size_t)node_ids[4 * e + defs[d][0]], (size_t)node_ids[4 * e + defs[d][1]]};
        int side = defs[d][2];
        auto it = edge_node_pairs.find(key);
        if (it != edge_node_pairs.end()) {
          if (it->second[side] >= 0) throw std::runtime_error("edge side already set");
          it->second[side] = (long)e;
        } else {
          std::array<long, 2> v = {-1, -1};
          v[side] = (long)e;
          edge_node_pairs[key] = v;
        }
      }
    }
    size_t eid = 0;
    std::vector<std::array<long, 2>> adj;
    for (auto& kv : edge_node_pairs) {
      int cnt = (kv.second[0] >= 0) + (kv.second[1] >= 0);
      edges.push_back(new_edge(eid, kv.first[0], kv.first[1], cnt == 1));
      adj.push_back(kv.second);
      eid++;
    }
    std::vector<std::array<long, 4>> elem_edges(n_el, {-1, -1, -1, -1});
    for (size_t ed = 0; ed < edges.size(); ed++) {
      for (int side = 0; side < 2; side++) {
        if (adj[ed][side] < 0) continue;
        size_t el = (size_t)adj[ed][side];
        int idx;
        if (side == 0 && edges[ed].dir == DIR_U) idx = 1;
        else if (side == 1 && edges[ed].dir == DIR_U) idx = 0;
        else if (side == 0) idx = 3;
        else idx = 2;
        if (elem_edges[el][idx] >= 0) throw std::runtime_error("elem edge already set");
        elem_edges[el][idx] = (long)ed;
      }
    }
    for (size_t e = 0; e < n_el; e++) {
      Elem el;
      el.id = e;
      for (int k = 0; k < 4; k++) {
        el.nodes[k] = (size_t)node_ids[4 * e + k];
        if (elem_edges[e][k] < 0) throw std::runtime_error("elem missing an edge");
        el.edges[k] = (size_t)elem_edges[e][k];
      }
      el.element = e;
      for (int k = 0; k < 4; k++) edge_connect_elem(edges[el.edges[k]], el);
      for (int k = 0; k < 4; k++) node_connect_elem(nodes[el.nodes[k]], el);
      elems.push_back(el);
    }
    set_edge_activation();
  }

  // mesh.rs:58-91 Mesh::unit: one Elem on [-1,1]^2, edges built explicitly and not connected
  void unit() {
    Point pts[4] = {Point(-1.0, -1.0), Point(1.0, -1.0), Point(-1.0, 1.0), Point(1.0, 1.0)};
    Element el;
    el.id = 0;
    for (int k = 0; k < 4; k++) el.points[k] = pts[k];
    el.eps_re = 1.0;
    el.eps_im = 0.0;
    el.mu_re = 1.0;
    el.mu_im = 0.0;
    elements.push_back(el);
    for (int k = 0; k < 4; k++) {
      Node n;
      n.id = (size_t)k;
      n.coords = pts[k];
      n.boundary = true;
      nodes.push_back(n);
    }
    const size_t en[4][2] = {{0, 1}, {2, 3}, {0, 2}, {1, 3}};
    for (size_t k = 0; k < 4; k++) edges.push_back(new_edge(k, en[k][0], en[k][1], true));
    Elem e;
    e.id = 0;
    for (int k = 0; k < 4; k++) { e.nodes[k] = (size_t)k; e.edges[k] = (size_t)k; }
    e.element = 0;
    elems.push_back(e);
  }

  Range2 parametric_range(const Elem& el) const {   // elem.rs:191-197
    Range2 r = {{{-1.0, 1.0}, {-1.0, 1.0}}};
    for (auto& a : el.ancestors) r = sub_range(a.second, r);
    return r;
  }
  Range2 relative_parametric_range(const Elem& el, size_t from_ancestor) const {   // elem.rs:170-188
    size_t start = el.ancestors.size();
    for (size_t k = 0; k < el.ancestors.size(); k++)
      if (el.ancestors[k].first == from_ancestor) { start = k; break; }
    if (start == el.ancestors.size()) throw std::runtime_error("not an ancestor");
    Range2 r = {{{-1.0, 1.0}, {-1.0, 1.0}}};
    for (size_t k = start; k < el.ancestors.size(); k++) r = sub_range(el.ancestors[k].second, r);
    return r;
  }

  void rec_desc(size_t id, bool include, std::vector<size_t>& out) const {   // mesh.rs:484-493
    if (include) out.push_back(id);
    if (elems[id].has_children)
      for (size_t c : elems[id].children) rec_desc(c, true, out);
  }
  std::vector<size_t> descendant_elems(size_t id) const {
    std::vector<size_t> out;
    rec_desc(id, false, out);
    return out;
  }

  std::array<uint8_t, 2> max_expansion_orders() const {   // mesh.rs:626-630
    std::array<uint8_t, 2> acc = {0, 0};
    for (auto& e : elems) {
      acc[0] = std::max(acc[0], e.ni);
      acc[1] = std::max(acc[1], e.nj);
    }
    return acc;
  }

  bool elem_is_h_refineable(size_t id) const {   // mesh.rs:649-662
    const Elem& el = elems[id];
    if (el.has_children) return false;
    for (int k = 0; k < 4; k++)
      if (!(edges[el.edges[k]].length > MIN_EDGE_LENGTH)) return false;
    return true;
  }

  // edge.rs:205-222
  bool edge_set_activation(Edge& e) {
    if (!e.elems[0].empty() && !e.elems[1].empty()) {
      e.active = true;
      e.active_elems[0] = e.elems[0].rbegin()->second;
      e.active_elems[1] = e.elems[1].rbegin()->second;
      return true;
    }
    e.active = false;
    return false;
  }
  // mesh.rs:1180-1215
  void set_edge_activation() {
    for (auto& e : edges) e.active = false;
    std::vector<size_t> base;
    for (auto& e : edges)
      if (e.parent < 0 && !e.boundary) base.push_back(e.id);
    for (size_t b : base)
      if (!rec_activation(b)) throw std::runtime_error("unable to find active edge pair");
  }
  bool rec_activation(size_t eid) {
    if (edge_set_activation(edges[eid])) {
      if (edges[eid].has_children) {
        size_t c0 = edges[eid].children[0], c1 = edges[eid].children[1];
        bool r0 = rec_activation(c0);
        bool r1 = rec_activation(c1);
        if (r0 && r1) edges[eid].active = false;
        else if (r0 != r1) throw std::runtime_error("inconsistent child edge support");
      }
      return true;
    }
    return false;
  }

  // mesh.rs:1091-1122 (h_refine_edge_if_needed); ids: two edges then one node
  void h_refine_edge_if_needed(size_t pe, size_t& next_node, size_t& next_edge, size_t out_children[2],
                               size_t& out_node) {
    if (edges[pe].has_children) {
      out_children[0] = edges[pe].children[0];
      out_children[1] = edges[pe].children[1];
      out_node = edges[pe].child_node;
      return;
    }
    size_t ids[2] = {next_edge, next_edge + 1};
    next_edge += 2;
    size_t nn = next_node++;
    double child_len = edges[pe].length / 2.0;   // edge.rs:71-107
    if (child_len < MIN_EDGE_LENGTH) throw std::runtime_error("min edge length");
    edges[pe].has_children = true;
    edges[pe].children[0] = ids[0];
    edges[pe].children[1] = ids[1];
    edges[pe].child_node = nn;
    Edge c0, c1;
    c0.id = ids[0];
    c0.nodes[0] = edges[pe].nodes[0];
    c0.nodes[1] = nn;
    c1.id = ids[1];
    c1.nodes[0] = nn;
    c1.nodes[1] = edges[pe].nodes[1];
    for (Edge* c : {&c0, &c1}) {
      c->boundary = edges[pe].boundary;
      c->dir = edges[pe].dir;
      c->length = child_len;
      c->parent = (long)pe;
    }
    if (edges.size() != ids[0]) throw std::runtime_error("edge id mismatch");
    edges.push_back(c0);
    edges.push_back(c1);
    Point p = Point::between(nodes[edges[pe].nodes[0]].coords, nodes[edges[pe].nodes[1]].coords);
    if (nn != nodes.size()) throw std::runtime_error("node id mismatch");
    Node n;
    n.id = nn;
    n.coords = p;
    n.boundary = edges[pe].boundary;
    nodes.push_back(n);
    out_children[0] = ids[0];
    out_children[1] = ids[1];
    out_node = nn;
  }

  // mesh.rs:1124-1152
  size_t new_edge_between_nodes(size_t n0, size_t n1, size_t& next_edge, size_t parent_elem) {
    if (n0 == n1) throw std::runtime_error("edge on equal nodes");
    size_t id = next_edge++;
    const Point& p0 = nodes[n0].coords;
    const Point& p1 = nodes[n1].coords;
    (void)parent_elem;
    // element.rs:52-57 order_points
    int ord = (p0.orientation_with(p1) == DIR_U) ? p0.xc.cmp(p1.xc) : p0.yc.cmp(p1.yc);
    if (ord == 0) throw std::runtime_error("edge on equal points");
    size_t a = ord < 0 ? n0 : n1, b = ord < 0 ? n1 : n0;
    if (edges.size() != id) throw std::runtime_error("edge id mismatch");
    edges.push_back(new_edge(id, a, b, false));
    return id;
  }

  std::vector<Elem> upgrade(std::vector<ElemUninit>& us) {   // mesh.rs:1154-1176
    std::vector<Elem> out;
    for (auto& u : us) {
      Elem el;
      el.id = u.id;
      for (int k = 0; k < 4; k++) {
        if (u.nodes[k] < 0 || u.edges[k] < 0) throw std::runtime_error("uninitialized elem");
        el.nodes[k] = (size_t)u.nodes[k];
        el.edges[k] = (size_t)u.edges[k];
      }
      el.element = u.element;
      el.h_levels = u.h_levels;
      el.ni = u.ni;
      el.nj = u.nj;
      el.ancestors = u.ancestors;
      out.push_back(el);
    }
    for (auto& el : out) {
      for (int k = 0; k < 4; k++) edge_connect_elem(edges[el.edges[k]], el);
      for (int k = 0; k < 4; k++) node_connect_elem(nodes[el.nodes[k]], el);
    }
    return out;
  }

  // mesh.rs:915-983
  std::vector<Elem> t_refine(std::vector<ElemUninit>& ne, size_t pid, size_t& nn, size_t& ned) {
    const Point& p0 = nodes[elems[pid].nodes[0]].coords;
    const Point& p3 = nodes[elems[pid].nodes[3]].coords;
    size_t center = nn++;
    Point cp = Point::between(p0, p3);
    if (center != nodes.size()) throw std::runtime_error("node id mismatch");
    Node cn;
    cn.id = center;
    cn.coords = cp;
    cn.boundary = false;
    nodes.push_back(cn);
    for (int k = 0; k < 4; k++) {
      ne[k].set_node(3 - k, center);
      ne[k].set_node(k, elems[pid].nodes[k]);
    }
    const int tab[4][7] = {{0, 0, 1, 1, 0, 3, 2}, {1, 2, 3, 3, 2, 3, 2}, {2, 0, 2, 2, 0, 1, 0}, {3, 1, 3, 3, 1, 1, 0}};
    for (int t = 0; t < 4; t++) {
      int edge_index = tab[t][0];
      int a0 = tab[t][1], a1 = tab[t][2];
      int s0 = tab[t][3], s1 = tab[t][4];
      int i0 = tab[t][5], i1 = tab[t][6];
      size_t ch[2], shared;
      h_refine_edge_if_needed(elems[pid].edges[edge_index], nn, ned, ch, shared);
      ne[a0].set_edge(edge_index, ch[0]);
      ne[a1].set_edge(edge_index, ch[1]);
      ne[a0].set_node(s0, shared);
      ne[a1].set_node(s1, shared);
      size_t nid = new_edge_between_nodes(shared, center, ned, pid);
      ne[a0].set_edge(i0, nid);
      ne[a1].set_edge(i1, nid);
    }
    return upgrade(ne);
  }

  // mesh.rs:985-1038 and 1040-1089
  std::vector<Elem> uv_refine(std::vector<ElemUninit>& ne, size_t pid, size_t& nn, size_t& ned, bool is_u) {
    size_t outer[2] = {0, 0};
    const int tu[2][5] = {{0, 1, 0, 0, 1}, {1, 3, 2, 2, 3}};
    const int tv[2][5] = {{2, 2, 0, 0, 2}, {3, 3, 1, 1, 3}};
    for (int t = 0; t < 2; t++) {
      const int* r = is_u ? tu[t] : tv[t];
      int edge_index = r[0];
      size_t ch[2], shared;
      h_refine_edge_if_needed(elems[pid].edges[edge_index], nn, ned, ch, shared);
      outer[is_u ? edge_index : edge_index - 2] = shared;
      ne[0].set_edge(edge_index, ch[0]);
      ne[1].set_edge(edge_index, ch[1]);
      ne[0].set_node(r[1], shared);
      ne[1].set_node(r[2], shared);
      ne[0].set_node(r[3], elems[pid].nodes[r[3]]);
      ne[1].set_node(r[4], elems[pid].nodes[r[4]]);
    }
    size_t nid = new_edge_between_nodes(outer[0], outer[1], ned, pid);
    if (is_u) {
      ne[0].set_edge(3, nid);
      ne[1].set_edge(2, nid);
      ne[0].set_edge(2, elems[pid].edges[2]);
      ne[1].set_edge(3, elems[pid].edges[3]);
    } else {
      ne[0].set_edge(1, nid);
      ne[1].set_edge(0, nid);
      ne[0].set_edge(0, elems[pid].edges[0]);
      ne[1].set_edge(1, elems[pid].edges[1]);
    }
    return upgrade(ne);
  }

  // mesh.rs:844-914
  void execute_h_refinements(const std::vector<std::pair<size_t, HRef>>& refs) {
    std::map<size_t, HRef> rmap;
    for (auto& r : refs) {
      if (r.first >= elems.size()) throw std::runtime_error("ElemDoesNotExist");
      if (!elem_is_h_refineable(r.first)) throw std::runtime_error("ElemNotRefineable");
      auto it = rmap.find(r.first);
      if (it != rmap.end()) href_add_assign(it->second, r.second);
      else rmap[r.first] = r.second;
    }
    std::vector<std::pair<size_t, HRef>> ext;
    size_t next_elem = elems.size();
    size_t nn = nodes.size(), ned = edges.size();
    for (auto& kv : rmap) {
      size_t pid = kv.first;
      HRef r = kv.second;
      // elem.rs:40-64 h_refine
      if (elems[pid].has_children) throw std::runtime_error("ElemHasChildren");
      int nch = r.kind == HREF_T ? 4 : 2;
      std::vector<ElemUninit> ne(nch);
      elems[pid].has_children = true;
      elems[pid].children.clear();
      for (int k = 0; k < nch; k++) {
        ne[k].id = next_elem + k;
        ne[k].element = elems[pid].element;
        ne[k].ancestors = elems[pid].ancestors;
        ne[k].ancestors.push_back({pid, href_loc(r, k)});
        ne[k].h_levels = refined(elems[pid].h_levels, r);
        ne[k].ni = elems[pid].ni;
        ne[k].nj = elems[pid].nj;
        elems[pid].children.push_back(next_elem + k);
      }
      next_elem += nch;
      std::vector<Elem> made;
      if (r.kind == HREF_T) made = t_refine(ne, pid, nn, ned);
      else made = uv_refine(ne, pid, nn, ned, r.kind == HREF_U);
      if (r.kind == HREF_U && r.ext >= 0) ext.push_back({made[r.ext].id, HRef{HREF_V, -1}});
      if (r.kind == HREF_V && r.ext >= 0) ext.push_back({made[r.ext].id, HRef{HREF_U, -1}});
      for (auto& m : made) elems.push_back(m);
    }
    if (!ext.empty()) execute_h_refinements(ext);
    set_edge_activation();
  }

  void global_h_refinement(HRef r) {   // mesh.rs:681-696
    std::vector<std::pair<size_t, HRef>> refs;
    for (auto& e : elems)
      if (elem_is_h_refineable(e.id)) refs.push_back({e.id, r});
    execute_h_refinements(refs);
  }
  void h_refine_elems(const std::vector<size_t>& ids, HRef r) {   // mesh.rs:716-726
    for (size_t i = 0; i < ids.size(); i++)
      for (size_t j = i + 1; j < ids.size(); j++)
        if (ids[i] == ids[j]) throw std::runtime_error("DuplicateElemIds");
    std::vector<std::pair<size_t, HRef>> refs;
    for (size_t id : ids) refs.push_back({id, r});
    execute_h_refinements(refs);
  }

  // p-refinement (mesh.rs:1217-1468, p_refinement.rs)
  void set_expansion_orders(const std::vector<size_t>& ids, int i, int j) {
    if (i > MAX_POLYNOMIAL_ORDER || j > MAX_POLYNOMIAL_ORDER || i < 1 || j < 1)
      throw std::runtime_error("InvalidExpansionOrders");
    for (size_t id : ids) {
      if (id >= elems.size()) throw std::runtime_error("ElemDoesNotExist");
      elems[id].ni = (uint8_t)i;
      elems[id].nj = (uint8_t)j;
    }
  }
  static int clamp_delta(int d, int lo, int hi) {   // p_refinement.rs:133-141
    if (d < lo) return lo;
    if (d > hi) return hi;
    return d;
  }
  void p_refine(const std::vector<size_t>& ids, int di, int dj, bool constrain) {
    // merge duplicates by += (p_refinement.rs:145-170), check window, apply
    std::map<size_t, std::array<int, 2>> rmap;
    for (size_t id : ids) {
      if (id >= elems.size()) throw std::runtime_error("ElemDoesNotExist");
      const Elem& e = elems[id];
      int a = di, b = dj;
      if (constrain) {
        a = clamp_delta(a, -(e.ni - 1), MAX_POLYNOMIAL_ORDER - e.ni);
        b = clamp_delta(b, -(e.nj - 1), MAX_POLYNOMIAL_ORDER - e.nj);
      }
      auto it = rmap.find(id);
      if (it != rmap.end()) { it->second[0] += a; it->second[1] += b; }
      else rmap[id] = {a, b};
    }
    for (auto& kv : rmap) {
      const Elem& e = elems[kv.first];
      int lo_u = -(e.ni - 1), hi_u = MAX_POLYNOMIAL_ORDER - e.ni;
      int lo_v = -(e.nj - 1), hi_v = MAX_POLYNOMIAL_ORDER - e.nj;
      if (kv.second[0] < lo_u || kv.second[0] > hi_u || kv.second[1] < lo_v || kv.second[1] > hi_v)
        throw std::runtime_error("RefinementOutOfBounds");
    }
    for (auto& kv : rmap) {
      elems[kv.first].ni = (uint8_t)(elems[kv.first].ni + kv.second[0]);
      elems[kv.first].nj = (uint8_t)(elems[kv.first].nj + kv.second[1]);
    }
  }
};

// ---------------------------------------------------------------------------
// domain.rs + basis_spec.rs + dof.rs
// ---------------------------------------------------------------------------
enum BasisDir { BD_U = 0, BD_V = 1, BD_W = 2 };
enum LocKind { LOC_ELEM = 0, LOC_EDGE = 1, LOC_NODE = 2 };

struct BasisSpec {   // basis_spec.rs:8-27
  size_t id;
  uint8_t i, j;
  BasisDir dir;
  size_t elem_id;
  long elem_idx = -1;
  long dof_id = -1;
  LocKind loc;
  uint8_t loc_idx = 0;
  size_t loc_id = 0;
};

// basis_spec.rs:41-75 (HCurl branch)
static BasisSpec make_spec(size_t id, uint8_t i, uint8_t j, BasisDir dir, const Elem& el) {
  BasisSpec bs;
  bs.id = id;
  bs.i = i;
  bs.j = j;
  bs.dir = dir;
  bs.elem_id = el.id;
  auto edge = [&](uint8_t idx) { bs.loc = LOC_EDGE; bs.loc_idx = idx; bs.loc_id = el.edges[idx]; };
  auto node = [&](uint8_t idx) { bs.loc = LOC_NODE; bs.loc_idx = idx; bs.loc_id = el.nodes[idx]; };
  if (i >= 2 && j >= 2) bs.loc = LOC_ELEM;
  else if (dir == BD_U && j <= 1) edge(j);
  else if (dir == BD_V && i <= 1) edge((uint8_t)(i + 2));
  else if (dir == BD_W) {
    bool a = i < 2, b = j < 2;
    if (a && !b) edge((uint8_t)(i + 2));
    else if (!a && b) edge(j);
    else if (a && b) node((uint8_t)(i + 2 * j));
    else bs.loc = LOC_ELEM;
  } else bs.loc = LOC_ELEM;
  return bs;
}

// basis_spec.rs:80-110
static bool matches_with_edge(const BasisSpec& a, const BasisSpec& b) {
  if (a.loc != LOC_EDGE || b.loc != LOC_EDGE) throw std::runtime_error("non edge-type match");
  if (a.loc_id != b.loc_id) throw std::runtime_error("different edges");
  int idx = a.loc_idx + b.loc_idx;
  if (a.dir == BD_U && b.dir == BD_U) return a.i == b.i && a.j + b.j == 1 && idx == 1;
  if (a.dir == BD_V && b.dir == BD_V) return a.j == b.j && a.i + b.i == 1 && idx == 5;
  if (a.dir == BD_W && b.dir == BD_W) {
    if (a.i >= 2 && b.i >= 2) return a.i == b.i && a.j + b.j == 1 && idx == 1;
    if (a.j >= 2 && b.j >= 2) return a.j == b.j && a.i + b.i == 1 && idx == 5;
    return false;
  }
  return false;
}

// p_refinement.rs:49-64
static void permutations(const Elem& e, BasisDir dir, std::vector<std::array<uint8_t, 2>>& out) {
  out.clear();
  int ni = e.ni, nj = e.nj;
  if (dir == BD_U) {
    for (int i = 0; i < ni; i++)
      for (int j = 0; j <= nj; j++) out.push_back({(uint8_t)i, (uint8_t)j});
  } else if (dir == BD_V) {
    for (int i = 0; i <= ni; i++)
      for (int j = 0; j < nj; j++) out.push_back({(uint8_t)i, (uint8_t)j});
  } else {
    for (int i = 0; i <= ni; i++)
      for (int j = 0; j <= nj; j++) out.push_back({(uint8_t)i, (uint8_t)j});
  }
}

struct Domain {
  Mesh mesh;
  size_t ndofs = 0;
  std::vector<std::vector<BasisSpec>> basis_specs;
  // dof -> addresses (elem_id, elem_idx)
  std::vector<std::vector<std::pair<size_t, size_t>>> dofs;

  // domain.rs:69-159
  void from_mesh(const Mesh& m) {
    mesh = m;
    mesh.set_edge_activation();
    size_t next_dof = 0, next_bs = 0;
    basis_specs.assign(mesh.elems.size(), {});
    std::map<size_t, std::vector<BasisSpec>> elem_bs, edge_bs;
    std::vector<std::array<uint8_t, 2>> perms;
    for (auto& el : mesh.elems) {   // domain.rs:201-235
      for (BasisDir dir : {BD_U, BD_V, BD_W}) {
        permutations(el, dir, perms);
        for (auto& ij : perms) {
          BasisSpec bs = make_spec(next_bs++, ij[0], ij[1], dir, el);
          if (bs.loc == LOC_ELEM) elem_bs[el.id].push_back(bs);
          else if (bs.loc == LOC_EDGE) edge_bs[bs.loc_id].push_back(bs);
        }
      }
    }
    auto push = [&](BasisSpec bs, size_t dof) {   // domain.rs:356-368
      size_t e = bs.elem_id;
      size_t idx = basis_specs[e].size();
      if (bs.dof_id >= 0 || bs.elem_idx >= 0) throw std::runtime_error("spec already assigned");
      bs.dof_id = (long)dof;
      bs.elem_idx = (long)idx;
      basis_specs[e].push_back(bs);
      return std::make_pair(e, idx);
    };
    for (auto& kv : elem_bs) {
      if (!mesh.elems[kv.first].has_children) {
        basis_specs[kv.first].clear();
        for (auto& bs : kv.second) {
          if (bs.dir == BD_U || bs.dir == BD_V) {
            size_t d = next_dof++;
            dofs.push_back({push(bs, d)});
          }
        }
      }
    }
    for (auto& kv : edge_bs) {
      const Edge& ed = mesh.edges[kv.first];
      if (!ed.active) continue;
      std::vector<BasisSpec> rel;
      for (auto& bs : kv.second)
        if ((bs.dir == BD_U || bs.dir == BD_V) &&
            (bs.elem_id == ed.active_elems[0] || bs.elem_id == ed.active_elems[1]))
          rel.push_back(bs);
      std::vector<std::array<size_t, 2>> pairs;
      for (size_t a = 0; a < rel.size(); a++)
        for (size_t b = a + 1; b < rel.size(); b++)
          if (matches_with_edge(rel[a], rel[b])) { pairs.push_back({a, b}); break; }
      for (auto& p : pairs) {
        size_t d = next_dof++;
        auto a0 = push(rel[p[0]], d);
        auto a1 = push(rel[p[1]], d);
        dofs.push_back({a0, a1});
      }
    }
    ndofs = next_dof;
  }
};

// ---------------------------------------------------------------------------
// glq.rs:179-249  Gauss-Legendre points by the Golub-Welsch eigenproblem.
// The symmetric tridiagonal eigenproblem is solved with implicit QL + Wilkinson
// shifts (the textbook tql2 recurrence), keeping the full eigenvector matrix.
// ---------------------------------------------------------------------------
static void tridiag_eigen(int n, std::vector<double>& d, std::vector<double>& e, std::vector<double>& z) {
  // d: diagonal (n), e: subdiagonal in e[1..n-1], z: n x n row-major identity on entry
  for (int i = 1; i < n; i++) e[i - 1] = e[i];
  if (n > 0) e[n - 1] = 0.0;
  double f = 0.0, tst1 = 0.0;
  for (int l = 0; l < n; l++) {
    tst1 = std::max(tst1, std::fabs(d[l]) + std::fabs(e[l]));
    int m = l;
    while (m < n) {
      if (std::fabs(e[m]) <= 2.220446049250313e-16 * tst1) break;
      m++;
    }
    if (m == n) m = n - 1;
    if (m > l) {
      int iter = 0;
      do {
        if (++iter > 200) throw std::runtime_error("tql2 no convergence");
        double g = d[l];
        double p = (d[l + 1] - g) / (2.0 * e[l]);
        double r = std::hypot(p, 1.0);
        if (p < 0) r = -r;
        d[l] = e[l] / (p + r);
        d[l + 1] = e[l] * (p + r);
        double dl1 = d[l + 1];
        double h = g - d[l];
        for (int i = l + 2; i < n; i++) d[i] -= h;
        f += h;
        p = d[m];
        double c = 1.0, c2 = c, c3 = c, el1 = e[l + 1], s = 0.0, s2 = 0.0;
        for (int i = m - 1; i >= l; i--) {
          c3 = c2;
          c2 = c;
          s2 = s;
          g = c * e[i];
          h = c * p;
          r = std::hypot(p, e[i]);
          e[i + 1] = s * r;
          s = e[i] / r;
          c = p / r;
          p = c * d[i] - s * g;
          d[i + 1] = h + s * (c * g + s * d[i]);
          for (int k = 0; k < n; k++) {
            h = z[k * n + i + 1];
            z[k * n + i + 1] = s * z[k * n + i] + c * h;
            z[k * n + i] = c * z[k * n + i] - s * h;
          }
        }
        p = -s * s2 * c3 * el1 * e[l] / dl1;
        e[l] = s * p;
        d[l] = c * p;
      } while (std::fabs(e[l]) > 2.220446049250313e-16 * tst1);
    }
    d[l] = d[l] + f;
    e[l] = 0.0;
  }
}

static void gauss_quadrature_points(int n, std::vector<double>& pts, std::vector<double>& wts) {
  std::vector<double> d(n, 0.0), e(n, 0.0), z((size_t)n * n, 0.0);
  for (int i = 1; i < n; i++) e[i] = 0.5 / std::sqrt(1.0 - std::pow(2.0 * i, -2.0));   // glq.rs:180-182
  for (int i = 0; i < n; i++) z[(size_t)i * n + i] = 1.0;
  tridiag_eigen(n, d, e, z);
  std::vector<std::pair<double, double>> xw(n);
  for (int k = 0; k < n; k++) xw[k] = {d[k], z[k] * z[k] * 2.0};   // row 0 of eigenvector matrix
  std::sort(xw.begin(), xw.end(), [](auto& a, auto& b) { return a.first < b.first; });
  pts.resize(n);
  wts.resize(n);
  for (int k = 0; k < n; k++) {
    pts[k] = xw[k].first;
    wts[k] = xw[k].second;
  }
}

static int default_ngq(int max_order) {   // basis.rs:172-177
  float conv = (float)(max_order * 4);
  int p2 = (int)std::ceil(std::log2(conv));
  return (int)std::lround(std::pow(2.0f, (float)p2));
}

// ---------------------------------------------------------------------------
// Shape-function spaces (hierarchical_basis_fns.rs)
// ---------------------------------------------------------------------------
struct ShapeSpace {   // norm = N, tang = T, with first (and, when sampled for integrate_by_parts, second) derivatives
  std::vector<std::vector<double>> n, nd, t, td, nd2, td2;
};

// HierPoly without 2nd derivatives: hierarchical_basis_fns.rs:102-162
static ShapeSpace hier_poly(int nmax, const std::vector<double>& x) {
  ShapeSpace s;
  size_t np = x.size();
  for (int k = 0; k <= nmax; k++) {
    double kf = (double)k;
    std::vector<double> pw(np), pwd(np), po(np), pod(np);
    if (k == 0) {
      for (size_t p = 0; p < np; p++) { po[p] = 1.0 - x[p]; pod[p] = -1.0; pw[p] = 1.0; pwd[p] = 0.0; }
    } else if (k == 1) {
      for (size_t p = 0; p < np; p++) { po[p] = 1.0 + x[p]; pod[p] = 1.0; pw[p] = x[p]; pwd[p] = 1.0; }
    } else {
      for (size_t p = 0; p < np; p++) {
        pw[p] = s.n[k - 1][p] * x[p];
        pwd[p] = kf * s.n[k - 1][p];
      }
      if (k % 2 == 0) {
        for (size_t p = 0; p < np; p++) { po[p] = pw[p] - 1.0; pod[p] = pwd[p]; }
      } else {
        for (size_t p = 0; p < np; p++) { po[p] = pw[p] - x[p]; pod[p] = pwd[p] - 1.0; }
      }
    }
    s.n.push_back(pw);
    s.nd.push_back(pwd);
    s.t.push_back(po);
    s.td.push_back(pod);
  }
  return s;
}

// Legendre-based space restating HierMaxOrtho (hierarchical_basis_fns.rs:201-647),
// the stand-in for KOLeg. Coefficient tables: hierarchical_basis_fns.rs:206-252.
static const double EUC_NORM_COEFFS[12] = {0.968246, 2.561738, 0.838525, 4.248161, 0.816397, 5.882766,
                                           0.808509, 1.0, 1.0, 1.0, 1.0, 1.0};
static const int Q_DENOM[12] = {1, 3, 6, 10, 15, 21, 28, 36, 40, 55, 66, 72};
static double q_num(int index, int k) {
  // Q_NUMERATORS[index][k]: alternating-zero pattern with the last entry = Q_DENOMINATORS-style top
  // hierarchical_basis_fns.rs:210-223
  static const int rows[12][14] = {
      {-1, 0, 1},
      {0, -3, 0, 3},
      {-1, 0, -5, 0, 6},
      {0, -3, 0, -7, 0, 10},
      {-1, 0, -5, 0, -9, 0, 15},
      {0, -3, 0, -7, 0, -11, 0, 21},
      {-1, 0, -5, 0, -9, 0, -13, 0, 28},
      {0, -3, 0, -7, 0, -11, 0, -15, 0, 36},
      {-1, 0, -5, 0, -9, 0, -13, 0, -17, 0, 40},
      {0, -3, 0, -7, 0, -11, 0, -15, 0, -19, 0, 55},
      {-1, 0, -5, 0, -9, 0, -13, 0, -17, 0, -21, 0, 66},
      {0, -3, 0, -7, 0, -11, 0, -15, 0, -19, 0, -23, 0, 72}};
  return (double)rows[index][k];
}
static ShapeSpace koleg(int nmax, const std::vector<double>& x) {
  if (nmax > 12) throw std::runtime_error("KOLeg supports orders <= 12");
  size_t np = x.size();
  std::vector<std::vector<double>> L(nmax + 1, std::vector<double>(np)), Ld(nmax + 1, std::vector<double>(np));
  for (int i = 0; i <= nmax; i++) {   // hierarchical_basis_fns.rs:420-455
    double f = (double)i;
    for (size_t p = 0; p < np; p++) {
      if (i == 0) { L[i][p] = 1.0; Ld[i][p] = 0.0; }
      else if (i == 1) { L[i][p] = x[p]; Ld[i][p] = 1.0; }
      else {
        L[i][p] = ((2.0 * f - 1.0) * x[p] * L[i - 1][p] - (f - 1.0) * L[i - 2][p]) / f;
        Ld[i][p] = f * L[i - 1][p] + x[p] * Ld[i - 1][p];
      }
    }
  }
  ShapeSpace s;
  s.n = L;
  s.nd = Ld;
  for (int i = 0; i <= nmax; i++) {   // hierarchical_basis_fns.rs:300-352
    std::vector<double> q(np, 0.0), qd(np, 0.0);
    if (i == 0) { for (size_t p = 0; p < np; p++) { q[p] = 1.0 - x[p]; qd[p] = -1.0; } }
    else if (i == 1) { for (size_t p = 0; p < np; p++) { q[p] = 1.0 + x[p]; qd[p] = 1.0; } }
    else {
      int index = i - 2;   // Q_WEIGHTS[i-2] has i+1 entries (get_q_weight_vector::<i+1>)
      int dim = i + 1;
      for (int k = 0; k < dim; k++) {
        double w = q_num(index, k) / (double)Q_DENOM[index];
        for (size_t p = 0; p < np; p++) {
          q[p] += w * L[k][p];
          qd[p] += w * Ld[k][p];
        }
      }
      for (size_t p = 0; p < np; p++) {
        q[p] *= EUC_NORM_COEFFS[index];
        qd[p] *= EUC_NORM_COEFFS[index];
      }
    }
    s.t.push_back(q);
    s.td.push_back(qd);
  }
  return s;
}

// Second derivatives of the shape spaces, as the samplers built with compute_2nd_derivs = true hold them.
// HierPoly::new_with_d2 (hierarchical_basis_fns.rs:24-100): norm_d2 = d2(x^n) (2, 6x, n(n-1)x^(n-2));
// tang_d2 returns the same table (hierarchical_basis_fns.rs:194-197).
static void add_d2_hier_poly(ShapeSpace& s, int nmax, const std::vector<double>& x) {
  size_t np = x.size();
  for (int k = 0; k <= nmax; k++) {
    std::vector<double> d2(np, 0.0);
    if (k == 2) {
      for (size_t p = 0; p < np; p++) d2[p] = 2.0;
    } else if (k == 3) {
      for (size_t p = 0; p < np; p++) d2[p] = 6.0 * x[p];
    } else if (k > 3) {
      const double kf = (double)k;
      for (size_t p = 0; p < np; p++) d2[p] = kf * (kf - 1.0) * s.n[k - 2][p];
    }
    s.nd2.push_back(d2);
  }
  s.td2 = s.nd2;
}
// LegendrePoly::with_specs_with_2nd_derivs (hierarchical_basis_fns.rs:466-590): P_2'' = 3, P_n'' =
// (2x P_n' - n(n+1) P_n) / (1 - x^2) with the denominator replaced by 1 at x = +-1; the Q functions'
// second derivatives are the weighted Legendre sums (QFunction::with_specs_with_2nd_derivs 356-395,
// weighted_double_prime_sum 620-644)
static void add_d2_koleg(ShapeSpace& s, int nmax, const std::vector<double>& x) {
  size_t np = x.size();
  std::vector<double> den(np);
  for (size_t p = 0; p < np; p++) den[p] = 1.0 - std::pow(x[p], 2);
  if (std::fabs(std::fabs(x[0]) - 1.0) < 1e-15) den[0] = 1.0;
  if (std::fabs(std::fabs(x[np - 1]) - 1.0) < 1e-15) den[np - 1] = 1.0;
  std::vector<std::vector<double>> L2(nmax + 1, std::vector<double>(np, 0.0));
  for (int i = 2; i <= nmax; i++) {
    const double f = (double)i;
    for (size_t p = 0; p < np; p++)
      L2[i][p] = i == 2 ? 3.0 : (2.0 * x[p] * s.nd[i][p] - (f * (f + 1.0)) * s.n[i][p]) / den[p];
  }
  s.nd2 = L2;
  for (int i = 0; i <= nmax; i++) {
    std::vector<double> q(np, 0.0);
    if (i >= 2) {
      int index = i - 2;
      for (int k = 0; k < i + 1; k++) {
        double w = q_num(index, k) / (double)Q_DENOM[index];
        for (size_t p = 0; p < np; p++) q[p] += w * L2[k][p];
      }
      for (size_t p = 0; p < np; p++) q[p] *= EUC_NORM_COEFFS[index];
    }
    s.td2.push_back(q);
  }
}

// ---------------------------------------------------------------------------
// HierCurlBasisFn (basis.rs:209-423) — for affine Elems the Jacobian is constant
// but it is still evaluated per point, as the reference does.
// ---------------------------------------------------------------------------
struct M2 { double u0, u1, v0, v1; };
struct BasisFn {
  std::vector<M2> jac, jac_inv;   // nq_u x nq_v, row-major [m][n]
  std::vector<double> det;
  double ps[2];
  ShapeSpace us, vs;
  int nv;
  const M2& ji(int m, int n) const { return jac_inv[(size_t)m * nv + n]; }
  const M2& jj(int m, int n) const { return jac[(size_t)m * nv + n]; }
  double dt(int m, int n) const { return det[(size_t)m * nv + n]; }
};

static BasisFn defined_over(const Mesh& mesh, const Elem& el, const Elem* desc, const std::vector<double>& up,
                            const std::vector<double>& vp, int imax, int jmax, int basis, bool d2 = false) {
  BasisFn b;
  std::vector<double> us = up, vs = vp;
  double su = 1.0, sv = 1.0;
  if (desc && desc->id != el.id) {
    Range2 r = mesh.relative_parametric_range(*desc, el.id);
    // glq.rs:238-249
    su = (r[0][1] - r[0][0]) / 2.0;
    double ou = (r[0][1] + r[0][0]) / 2.0;
    sv = (r[1][1] - r[1][0]) / 2.0;
    double ov = (r[1][1] + r[1][0]) / 2.0;
    for (auto& x : us) x = x * su + ou;
    for (auto& x : vs) x = x * sv + ov;
  }
  Range2 pr = mesh.parametric_range(el);
  const Element& elt = mesh.elements[el.element];
  auto map_range = [](double val, double in_min, double in_max, double out_min, double out_max) {
    return (val - in_min) * (out_max - out_min) / (in_max - in_min) + out_min;   // element.rs:62-64
  };
  double xmin = map_range(pr[0][0], -1.0, 1.0, elt.points[0].x, elt.points[3].x);
  double xmax = map_range(pr[0][1], -1.0, 1.0, elt.points[0].x, elt.points[3].x);
  double ymin = map_range(pr[1][0], -1.0, 1.0, elt.points[0].y, elt.points[3].y);
  double ymax = map_range(pr[1][1], -1.0, 1.0, elt.points[0].y, elt.points[3].y);
  double dxdu = (xmax - xmin) / 2.0, dydv = (ymax - ymin) / 2.0;   // element.rs:33-50
  b.nv = (int)vs.size();
  for (size_t m = 0; m < us.size(); m++) {
    for (size_t n = 0; n < vs.size(); n++) {
      M2 t = {dxdu, 0.0, 0.0, dydv};
      double d = t.u0 * t.v1 - t.u1 * t.v0;   // space.rs:137-140
      M2 ti = {t.v1 / d, (-1.0 * t.u1) / d, (-1.0 * t.v0) / d, t.u0 / d};   // space.rs:142-147
      b.jac.push_back(t);
      b.jac_inv.push_back(ti);
      b.det.push_back(d);
    }
  }
  b.ps[0] = su;
  b.ps[1] = sv;
  b.us = basis == 0 ? hier_poly(imax, us) : koleg(imax, us);
  b.vs = basis == 0 ? hier_poly(jmax, vs) : koleg(jmax, vs);
  if (d2) {
    if (basis == 0) {
      add_d2_hier_poly(b.us, imax, us);
      add_d2_hier_poly(b.vs, jmax, vs);
    } else {
      add_d2_koleg(b.us, imax, us);
      add_d2_koleg(b.vs, jmax, vs);
    }
  }
  return b;
}

struct V2 { double x, y; };
// basis.rs:225-252
static inline V2 f_u(const BasisFn& b, int i, int j, int m, int n) {
  const M2& ji = b.ji(m, n);
  return {(ji.u0 * b.us.n[i][m]) * b.vs.t[j][n], (ji.u1 * b.us.n[i][m]) * b.vs.t[j][n]};
}
static inline V2 f_v(const BasisFn& b, int i, int j, int m, int n) {
  const M2& ji = b.ji(m, n);
  return {(ji.v0 * b.us.t[i][m]) * b.vs.n[j][n], (ji.v1 * b.us.t[i][m]) * b.vs.n[j][n]};
}
static inline V2 f_u_d1(const BasisFn& b, int i, int j, int m, int n, const double* ps) {
  const M2& ji = b.ji(m, n);
  V2 a = {ji.u0 * (b.us.n[i][m] * b.vs.td[j][n]), ji.u1 * (b.us.nd[i][m] * b.vs.t[j][n])};
  return {a.x * ps[0], a.y * ps[1]};
}
static inline V2 f_v_d1(const BasisFn& b, int i, int j, int m, int n, const double* ps) {
  const M2& ji = b.ji(m, n);
  V2 a = {ji.v0 * (b.us.t[i][m] * b.vs.nd[j][n]), ji.v1 * (b.us.td[i][m] * b.vs.n[j][n])};
  return {a.x * ps[0], a.y * ps[1]};
}
static inline double curl(V2 a) { return a.x * -1.0 + a.y * 1.0; }   // CURL_OP integrals.rs:240

// integrals.rs:249-271
static inline double max_uv(const BasisFn& p, const BasisFn& q, int m, int n) {
  double rp = p.jj(m, n).u0 / p.jj(m, n).v1, rq = q.jj(m, n).u0 / q.jj(m, n).v1;
  return (double)(p.dt(m, n) >= q.dt(m, n)) * rp + (double)(p.dt(m, n) < q.dt(m, n)) * rq;
}
static inline double max_vu(const BasisFn& p, const BasisFn& q, int m, int n) {
  double rp = p.jj(m, n).v1 / p.jj(m, n).u0, rq = q.jj(m, n).v1 / q.jj(m, n).u0;
  return (double)(p.dt(m, n) >= q.dt(m, n)) * rp + (double)(p.dt(m, n) < q.dt(m, n)) * rq;
}

// glq.rs:19-32 real_gauss_quad, inlined with the same association order
template <class F>
static inline double gauss_quad(const std::vector<double>& uw, const std::vector<double>& vw, F f) {
  double sol = 0.0;
  for (size_t m = 0; m < uw.size(); m++) {
    double inner = 0.0;
    for (size_t n = 0; n < vw.size(); n++) inner += f((int)m, (int)n) * vw[n];
    sol += inner * uw[m];
  }
  return sol;
}

// CurlCurl::integrate integrals.rs:26-92
static double curl_curl(const std::vector<double>& uw, const std::vector<double>& vw, BasisDir pd, BasisDir qd,
                        int pi, int pj, int qi, int qj, const BasisFn& p, const BasisFn& q, double mu_re) {
  double v = 0.0;
  if (pd == BD_U && qd == BD_U)
    v = gauss_quad(uw, vw, [&](int m, int n) {
      return curl(f_u_d1(p, pi, pj, m, n, q.ps)) * curl(f_u_d1(q, qi, qj, m, n, p.ps)) * max_uv(p, q, m, n);
    });
  else if (pd == BD_U && qd == BD_V)
    v = gauss_quad(uw, vw, [&](int m, int n) {
      return curl(f_u_d1(p, pi, pj, m, n, q.ps)) * curl(f_v_d1(q, qi, qj, m, n, p.ps));
    });
  else if (pd == BD_V && qd == BD_U)
    v = gauss_quad(uw, vw, [&](int m, int n) {
      return curl(f_v_d1(p, pi, pj, m, n, q.ps)) * curl(f_u_d1(q, qi, qj, m, n, p.ps));
    });
  else if (pd == BD_V && qd == BD_V)
    v = gauss_quad(uw, vw, [&](int m, int n) {
      return curl(f_v_d1(p, pi, pj, m, n, q.ps)) * curl(f_v_d1(q, qi, qj, m, n, p.ps)) * max_vu(p, q, m, n);
    });
  return (1.0 / mu_re) * v;
}

// L2Inner::integrate integrals.rs:292-354
static double l2_inner(const std::vector<double>& uw, const std::vector<double>& vw, BasisDir pd, BasisDir qd,
                       int pi, int pj, int qi, int qj, const BasisFn& p, const BasisFn& q, double eps_re) {
  auto dot = [](V2 a, V2 b) { return a.x * b.x + a.y * b.y; };
  auto pm = [&](int m, int n) { return std::max(p.dt(m, n), q.dt(m, n)); };
  double v = 0.0;
  if (pd == BD_U && qd == BD_U)
    v = gauss_quad(uw, vw, [&](int m, int n) { return dot(f_u(p, pi, pj, m, n), f_u(q, qi, qj, m, n)) * pm(m, n); });
  else if (pd == BD_U && qd == BD_V)
    v = gauss_quad(uw, vw, [&](int m, int n) { return dot(f_u(p, pi, pj, m, n), f_v(q, qi, qj, m, n)) * pm(m, n); });
  else if (pd == BD_V && qd == BD_U)
    v = gauss_quad(uw, vw, [&](int m, int n) { return dot(f_v(p, pi, pj, m, n), f_u(q, qi, qj, m, n)) * pm(m, n); });
  else if (pd == BD_V && qd == BD_V)
    v = gauss_quad(uw, vw, [&](int m, int n) { return dot(f_v(p, pi, pj, m, n), f_v(q, qi, qj, m, n)) * pm(m, n); });
  return eps_re * (p.ps[0] * p.ps[1]) * (q.ps[0] * q.ps[1]) * v;
}

// ---------------------------------------------------------------------------
// integrate_by_parts (integrals.rs:94-237 CurlCurl, 356-418 L2Inner) on samplers with second
// derivatives: GLQ points with the endpoints -1 and +1 appended (weight 1.0, glq.rs:215-222), the
// face term over the interior points (real_gauss_quad_inner glq.rs:53-77) and four edge terms
// (real_gauss_quad_edge glq.rs:101-156). basis.rs:254-292 for the second derivatives.
// ---------------------------------------------------------------------------
static void glq_with_endpoints(int n, std::vector<double>& pts, std::vector<double>& wts) {
  gauss_quadrature_points(n, pts, wts);
  pts.insert(pts.begin(), -1.0);
  pts.push_back(1.0);
  wts.insert(wts.begin(), 1.0);
  wts.push_back(1.0);
}
static inline V2 f_u_d2(const BasisFn& b, int i, int j, int m, int n, const double* ps) {
  const M2& ji = b.ji(m, n);
  V2 a = {ji.u0 * (b.us.n[i][m] * b.vs.td2[j][n]), ji.u1 * (b.us.nd2[i][m] * b.vs.t[j][n])};
  return {a.x * ps[0] * ps[0], a.y * ps[1] * ps[1]};
}
static inline V2 f_v_d2(const BasisFn& b, int i, int j, int m, int n, const double* ps) {
  const M2& ji = b.ji(m, n);
  V2 a = {ji.v0 * (b.us.t[i][m] * b.vs.nd2[j][n]), ji.v1 * (b.us.td2[i][m] * b.vs.n[j][n])};
  return {a.x * ps[0] * ps[0], a.y * ps[1] * ps[1]};
}
static inline V2 f_u_dd(const BasisFn& b, int i, int j, int m, int n, const double* ps) {
  const M2& ji = b.ji(m, n);
  return {ji.u0 * b.us.nd[i][m] * b.vs.td[j][n] * ps[0] * ps[1], ji.u1 * b.us.nd[i][m] * b.vs.td[j][n] * ps[0] * ps[1]};
}
static inline V2 f_v_dd(const BasisFn& b, int i, int j, int m, int n, const double* ps) {
  const M2& ji = b.ji(m, n);
  return {ji.v0 * b.us.td[i][m] * b.vs.nd[j][n] * ps[0] * ps[1], ji.v1 * b.us.td[i][m] * b.vs.nd[j][n] * ps[0] * ps[1]};
}
template <class F>
static inline double gauss_quad_inner(const std::vector<double>& uw, const std::vector<double>& vw, F f) {
  double sol = 0.0;
  for (size_t m = 1; m + 1 < uw.size(); m++) {
    double inner = 0.0;
    for (size_t n = 1; n + 1 < vw.size(); n++) inner += f((int)m, (int)n) * vw[n];
    sol += inner * uw[m];
  }
  return sol;
}
template <class F>
static inline double gauss_quad_edge(const std::vector<double>& uw, const std::vector<double>& vw, int edge, F f) {
  double sol = 0.0;
  const int nu = (int)uw.size(), nv = (int)vw.size();
  if (edge == 0)
    for (int m = 1; m < nu - 1; m++) sol += f(m, 0) * uw[m];
  else if (edge == 1)
    for (int m = nu - 2; m >= 1; m--) sol += f(m, nv - 1) * uw[m];
  else if (edge == 2)
    for (int n = nv - 2; n >= 1; n--) sol += f(0, n) * vw[n];
  else
    for (int n = 1; n < nv - 1; n++) sol += f(nu - 1, n) * vw[n];
  return sol;
}
static const V2 EDGE_UNIT[4] = {{-1.0, 0.0}, {1.0, 0.0}, {0.0, -1.0}, {0.0, 1.0}};   // integrals.rs:242-247

// out: face, edge 0..3 (IntegralResult::ByParts)
static void curl_curl_by_parts(const std::vector<double>& uw, const std::vector<double>& vw, BasisDir pd,
                               BasisDir qd, int pi, int pj, int qi, int qj, const BasisFn& p, const BasisFn& q,
                               double mu_re, double* out) {
  auto dot = [](V2 a, V2 b) { return a.x * b.x + a.y * b.y; };
  const double gp = p.ps[0] * p.ps[1], gq = q.ps[0] * q.ps[1];
  double face = 0.0;
  if (pd == BD_U && qd == BD_U)
    face = gauss_quad_inner(uw, vw, [&](int m, int n) {
             V2 d2 = f_u_d2(p, pi, pj, m, n, q.ps), dd = f_u_dd(p, pi, pj, m, n, q.ps);
             V2 pv = {dd.y + d2.x, d2.y + dd.x};
             return dot(pv, f_u(q, qi, qj, m, n)) / std::pow(gq, 2) * max_uv(p, q, m, n);
           }) * -1.0;
  else if (pd == BD_U && qd == BD_V)
    face = gauss_quad_inner(uw, vw, [&](int m, int n) {
      V2 d2 = f_u_d2(p, pi, pj, m, n, q.ps), dd = f_u_dd(p, pi, pj, m, n, q.ps);
      V2 pv = {dd.y + d2.x, d2.y + dd.x};
      return dot(pv, f_v(q, qi, qj, m, n)) / std::pow(gq, 2);
    });
  else if (pd == BD_V && qd == BD_U)
    face = gauss_quad_inner(uw, vw, [&](int m, int n) {
      V2 d2 = f_v_d2(p, pi, pj, m, n, q.ps), dd = f_v_dd(p, pi, pj, m, n, q.ps);
      V2 pv = {dd.y + d2.x, d2.y + dd.x};
      return dot(pv, f_u(q, qi, qj, m, n)) / std::pow(gq, 2);
    });
  else if (pd == BD_V && qd == BD_V)
    face = gauss_quad_inner(uw, vw, [&](int m, int n) {
             V2 d2 = f_v_d2(p, pi, pj, m, n, q.ps), dd = f_v_dd(p, pi, pj, m, n, q.ps);
             V2 pv = {dd.y + d2.x, d2.y + dd.x};
             return dot(pv, f_v(q, qi, qj, m, n)) / std::pow(gq, 2) * max_vu(p, q, m, n);
           }) * -1.0;
  out[0] = (1.0 / mu_re) * gp * gq * face;
  for (int e = 0; e < 4; e++) {
    const double pe = e < 2 ? p.ps[0] : p.ps[1], qe = e < 2 ? q.ps[0] : q.ps[1];
    double v = 0.0;
    if (pd == BD_U && qd == BD_U && e < 2)
      v = gauss_quad_edge(uw, vw, e, [&](int m, int n) {
        return curl(f_u_d1(p, pi, pj, m, n, q.ps)) * dot(f_u(q, qi, qj, m, n), EDGE_UNIT[e]) / gq * max_uv(p, q, m, n);
      });
    else if (pd == BD_V && qd == BD_U && e < 2)
      v = gauss_quad_edge(uw, vw, e, [&](int m, int n) {
        return curl(f_v_d1(p, pi, pj, m, n, q.ps)) * dot(f_u(q, qi, qj, m, n), EDGE_UNIT[e]) / gq;
      });
    else if (pd == BD_U && qd == BD_V && e >= 2)
      v = gauss_quad_edge(uw, vw, e, [&](int m, int n) {
            return curl(f_u_d1(p, pi, pj, m, n, q.ps)) * dot(f_v(q, qi, qj, m, n), EDGE_UNIT[e]) / gq;
          }) * -1.0;
    else if (pd == BD_V && qd == BD_V && e >= 2)
      v = gauss_quad_edge(uw, vw, e, [&](int m, int n) {
            return curl(f_v_d1(p, pi, pj, m, n, q.ps)) * dot(f_v(q, qi, qj, m, n), EDGE_UNIT[e]) / gq *
                   max_vu(p, q, m, n);
          }) * -1.0;
    out[1 + e] = -1.0 * (1.0 / mu_re) * pe * qe * v;
  }
}

// L2Inner::integrate_by_parts: the full integral over the interior points
static double l2_inner_by_parts(const std::vector<double>& uw, const std::vector<double>& vw, BasisDir pd,
                                BasisDir qd, int pi, int pj, int qi, int qj, const BasisFn& p, const BasisFn& q,
                                double eps_re) {
  auto dot = [](V2 a, V2 b) { return a.x * b.x + a.y * b.y; };
  auto pm = [&](int m, int n) { return std::max(p.dt(m, n), q.dt(m, n)); };
  double v = 0.0;
  if (pd == BD_U && qd == BD_U)
    v = gauss_quad_inner(uw, vw, [&](int m, int n) { return dot(f_u(p, pi, pj, m, n), f_u(q, qi, qj, m, n)) * pm(m, n); });
  else if (pd == BD_U && qd == BD_V)
    v = gauss_quad_inner(uw, vw, [&](int m, int n) { return dot(f_u(p, pi, pj, m, n), f_v(q, qi, qj, m, n)) * pm(m, n); });
  else if (pd == BD_V && qd == BD_U)
    v = gauss_quad_inner(uw, vw, [&](int m, int n) { return dot(f_v(p, pi, pj, m, n), f_u(q, qi, qj, m, n)) * pm(m, n); });
  else if (pd == BD_V && qd == BD_V)
    v = gauss_quad_inner(uw, vw, [&](int m, int n) { return dot(f_v(p, pi, pj, m, n), f_v(q, qi, qj, m, n)) * pm(m, n); });
  return eps_re * (p.ps[0] * p.ps[1]) * (q.ps[0] * q.ps[1]) * v;
}

// ---------------------------------------------------------------------------
// galerkin.rs:33-187 + sparse_matrix.rs:68-120 + linalg.rs:59-81
// ---------------------------------------------------------------------------
typedef std::map<std::pair<uint32_t, uint32_t>, double> SparseMap;

static inline void insert_sym(SparseMap& m, size_t r, size_t c, double v) {
  std::pair<uint32_t, uint32_t> key = r <= c ? std::make_pair((uint32_t)r, (uint32_t)c)
                                             : std::make_pair((uint32_t)c, (uint32_t)r);
  auto it = m.find(key);
  if (it != m.end()) it->second += v;
  else m.emplace(key, v);
}

struct GEPResult {
  size_t n = 0;
  std::vector<uint32_t> rows, cols;
  std::vector<double> a, b;
};

static void galerkin_elem(const Domain& dom, size_t eid, const std::vector<double>& up, const std::vector<double>& uw,
                          const std::vector<double>& vp, const std::vector<double>& vw, int imax, int jmax,
                          int basis, SparseMap& la, SparseMap& lb) {
  const Mesh& mesh = dom.mesh;
  const Elem& el = mesh.elems[eid];
  const Element& elt = mesh.elements[el.element];
  BasisFn bl = defined_over(mesh, el, nullptr, up, vp, imax, jmax, basis);
  const auto& L = dom.basis_specs[eid];
  std::vector<size_t> desc = mesh.descendant_elems(eid);
  SparseMap ga, gb;
  for (size_t i = 0; i < L.size(); i++) {
    const BasisSpec& p = L[i];
    for (size_t k = i; k < L.size(); k++) {
      const BasisSpec& q = L[k];
      double a = curl_curl(uw, vw, p.dir, q.dir, p.i, p.j, q.i, q.j, bl, bl, elt.mu_re);
      double b = l2_inner(uw, vw, p.dir, q.dir, p.i, p.j, q.i, q.j, bl, bl, elt.eps_re);
      insert_sym(la, (size_t)p.dof_id, (size_t)q.dof_id, a);
      insert_sym(lb, (size_t)p.dof_id, (size_t)q.dof_id, b);
    }
  }
  // the reference samples (E over D) and (D local) inside the p loop; the values are the same for every p
  std::vector<BasisFn> bp, bq;
  for (size_t d : desc) {
    bp.push_back(defined_over(mesh, el, &mesh.elems[d], up, vp, imax, jmax, basis));
    bq.push_back(defined_over(mesh, mesh.elems[d], nullptr, up, vp, imax, jmax, basis));
  }
  for (const BasisSpec& p : L) {
    for (size_t di = 0; di < desc.size(); di++) {
      for (const BasisSpec& q : dom.basis_specs[desc[di]]) {
        double a = curl_curl(uw, vw, p.dir, q.dir, p.i, p.j, q.i, q.j, bp[di], bq[di], elt.mu_re);
        double b = l2_inner(uw, vw, p.dir, q.dir, p.i, p.j, q.i, q.j, bp[di], bq[di], elt.eps_re);
        insert_sym(la, (size_t)p.dof_id, (size_t)q.dof_id, a);
        insert_sym(lb, (size_t)p.dof_id, (size_t)q.dof_id, b);
      }
    }
  }
}

// nthreads > 1: elems are processed by a thread pool (like the rayon fan-out) and the
// per-elem maps are merged on the calling thread in elem order.
static GEPResult galerkin(const Domain& dom, int basis, int nu, int nv, int nthreads) {
  if (dom.ndofs == 0) throw std::runtime_error("EmptyDOFSet");
  auto mo = dom.mesh.max_expansion_orders();
  int imax = mo[0], jmax = mo[1];
  if (nu <= 0) nu = default_ngq(imax);
  if (nv <= 0) nv = default_ngq(jmax);
  std::vector<double> up, uw, vp, vw;
  gauss_quadrature_points(nu, up, uw);
  gauss_quadrature_points(nv, vp, vw);
  size_t ne = dom.mesh.elems.size();
  std::vector<SparseMap> las(ne), lbs(ne);
  if (nthreads <= 1) {
    for (size_t e = 0; e < ne; e++) galerkin_elem(dom, e, up, uw, vp, vw, imax, jmax, basis, las[e], lbs[e]);
  } else {
    std::vector<std::thread> th;
    std::atomic<size_t> next{0};
    for (int t = 0; t < nthreads; t++)
      th.emplace_back([&]() {
        for (;;) {
          size_t e = next.fetch_add(1);
          if (e >= ne) break;
          galerkin_elem(dom, e, up, uw, vp, vw, imax, jmax, basis, las[e], lbs[e]);
        }
      });
    for (auto& t : th) t.join();
  }
  SparseMap A, B;
  for (size_t e = 0; e < ne; e++) {   // sparse_matrix.rs:106-120 consume_matrix
    for (auto& kv : las[e]) {
      auto it = A.find(kv.first);
      if (it != A.end()) it->second += kv.second;
      else A.emplace(kv.first, kv.second);
    }
    for (auto& kv : lbs[e]) {
      auto it = B.find(kv.first);
      if (it != B.end()) it->second += kv.second;
      else B.emplace(kv.first, kv.second);
    }
    SparseMap().swap(las[e]);
    SparseMap().swap(lbs[e]);
  }
  GEPResult r;
  r.n = dom.ndofs;
  for (auto& kv : A) {
    r.rows.push_back(kv.first.first);
    r.cols.push_back(kv.first.second);
    r.a.push_back(kv.second);
    r.b.push_back(B.at(kv.first));
  }
  return r;
}

// The Galerkin visit set of galerkin_elem with integrate_by_parts in place of integrate: per upper key
// (collisions summed in elem order) the CurlCurl face term, its four edge terms and the L2Inner value.
struct ByPartsResult {
  std::vector<uint32_t> rows, cols;
  std::vector<double> vals;   // 6 per key: face, edge 0..3, B
};
static ByPartsResult galerkin_by_parts(const Domain& dom, int basis, int nu, int nv) {
  if (dom.ndofs == 0) throw std::runtime_error("EmptyDOFSet");
  auto mo = dom.mesh.max_expansion_orders();
  int imax = mo[0], jmax = mo[1];
  if (nu <= 0) nu = default_ngq(imax);
  if (nv <= 0) nv = default_ngq(jmax);
  std::vector<double> up, uw, vp, vw;
  glq_with_endpoints(nu, up, uw);
  glq_with_endpoints(nv, vp, vw);
  const Mesh& mesh = dom.mesh;
  std::map<std::pair<uint32_t, uint32_t>, std::array<double, 6>> acc;
  auto add = [&](size_t r, size_t c, const double* v) {
    std::pair<uint32_t, uint32_t> key = r <= c ? std::make_pair((uint32_t)r, (uint32_t)c)
                                               : std::make_pair((uint32_t)c, (uint32_t)r);
    auto it = acc.find(key);
    if (it == acc.end()) {
      std::array<double, 6> a;
      for (int k = 0; k < 6; k++) a[k] = v[k];
      acc.emplace(key, a);
    } else {
      for (int k = 0; k < 6; k++) it->second[k] += v[k];
    }
  };
  for (size_t eid = 0; eid < mesh.elems.size(); eid++) {
    const Elem& el = mesh.elems[eid];
    const Element& elt = mesh.elements[el.element];
    const auto& L = dom.basis_specs[eid];
    if (L.empty()) continue;
    BasisFn bl = defined_over(mesh, el, nullptr, up, vp, imax, jmax, basis, true);
    double v[6];
    for (size_t i = 0; i < L.size(); i++)
      for (size_t k = i; k < L.size(); k++) {
        const BasisSpec& ps = L[i];
        const BasisSpec& qs = L[k];
        curl_curl_by_parts(uw, vw, ps.dir, qs.dir, ps.i, ps.j, qs.i, qs.j, bl, bl, elt.mu_re, v);
        v[5] = l2_inner_by_parts(uw, vw, ps.dir, qs.dir, ps.i, ps.j, qs.i, qs.j, bl, bl, elt.eps_re);
        add((size_t)ps.dof_id, (size_t)qs.dof_id, v);
      }
    std::vector<size_t> desc = mesh.descendant_elems(eid);
    for (size_t d : desc) {
      BasisFn bp = defined_over(mesh, el, &mesh.elems[d], up, vp, imax, jmax, basis, true);
      BasisFn bq = defined_over(mesh, mesh.elems[d], nullptr, up, vp, imax, jmax, basis, true);
      for (const BasisSpec& ps : L)
        for (const BasisSpec& qs : dom.basis_specs[d]) {
          curl_curl_by_parts(uw, vw, ps.dir, qs.dir, ps.i, ps.j, qs.i, qs.j, bp, bq, elt.mu_re, v);
          v[5] = l2_inner_by_parts(uw, vw, ps.dir, qs.dir, ps.i, ps.j, qs.i, qs.j, bp, bq, elt.eps_re);
          add((size_t)ps.dof_id, (size_t)qs.dof_id, v);
        }
    }
  }
  ByPartsResult r;
  for (auto& kv : acc) {
    r.rows.push_back(kv.first.first);
    r.cols.push_back(kv.first.second);
    for (int k = 0; k < 6; k++) r.vals.push_back(kv.second[k]);
  }
  return r;
}

// fields.rs:386-389
static std::vector<double> uniform_range(double min, double max, size_t n) {
  double step = (max - min) / ((double)(n - 1));
  std::vector<double> r(n);
  for (size_t i = 0; i < n; i++) r[i] = ((double)i) * step + min;
  return r;
}

// UniformFieldSpace::xy_fields (fields.rs:63-122). Leaves in ascending id; per leaf a d0 x d1 grid
// [m][n] (m along u). The reference allocates its per-leaf arrays [d1][d0] and indexes them [m][n],
// which only runs for d0 == d1; this restatement uses [m][n] for any d0, d1.
static void xy_fields(const Domain& dom, int basis, size_t d0, size_t d1, const std::vector<double>& sol,
                      std::vector<double>& xo, std::vector<double>& yo) {
  if (sol.size() != dom.ndofs) throw std::runtime_error("MismatchedSolutionSize");
  const Mesh& mesh = dom.mesh;
  std::vector<double> pu = uniform_range(-1.0, 1.0, d0), pv = uniform_range(-1.0, 1.0, d1);
  auto mo = mesh.max_expansion_orders();
  xo.clear();
  yo.clear();
  for (const Elem& leaf : mesh.elems) {
    if (leaf.has_children) continue;
    std::vector<double> xv(d0 * d1, 0.0), yv(d0 * d1, 0.0);
    // ancestor_elems(leaf, true) (mesh.rs:520-541): the leaf, then each parent up to the root
    std::vector<size_t> chain{leaf.id};
    for (auto it = leaf.ancestors.rbegin(); it != leaf.ancestors.rend(); ++it) chain.push_back(it->first);
    for (size_t a : chain) {
      BasisFn bf = defined_over(mesh, mesh.elems[a], &leaf, pu, pv, mo[0], mo[1], basis);
      for (const BasisSpec& bs : dom.basis_specs[a]) {
        for (size_t m = 0; m < d0; m++) {
          for (size_t n = 0; n < d1; n++) {
            V2 f = {0.0, 0.0};
            if (bs.dir == BD_U) f = f_u(bf, bs.i, bs.j, (int)m, (int)n);
            else if (bs.dir == BD_V) f = f_v(bf, bs.i, bs.j, (int)m, (int)n);
            double c = sol[(size_t)bs.dof_id];
            xv[m * d1 + n] += f.x * c;
            yv[m * d1 + n] += f.y * c;
          }
        }
      }
    }
    xo.insert(xo.end(), xv.begin(), xv.end());
    yo.insert(yo.end(), yv.begin(), yv.end());
  }
}

}  // namespace oracle

// ---------------------------------------------------------------------------
// C ABI for the test harness (ctypes). Handles are opaque pointers.
// ---------------------------------------------------------------------------
using namespace oracle;

struct OracleState {
  Mesh mesh;
  std::unique_ptr<Domain> dom;
  GEPResult gep;
  ByPartsResult bp;
  std::vector<double> glq_p, glq_w;
};

static thread_local std::string g_err;

#define ORACLE_TRY(...)                   \
  try {                                   \
    __VA_ARGS__;                          \
    return 0;                             \
  } catch (const std::exception& ex) {    \
    g_err = ex.what();                    \
    return -1;                            \
  }

extern "C" {

const char* oracle_last_error() { return g_err.c_str(); }

void* oracle_mesh_new(int64_t n_nodes, const double* xy, int64_t n_el, const int64_t* node_ids,
                      const double* mats) {
  try {
    auto* s = new OracleState();
    s->mesh.from_arrays((size_t)n_nodes, xy, (size_t)n_el, node_ids, mats);
    return s;
  } catch (const std::exception& ex) {
    g_err = ex.what();
    return nullptr;
  }
}
void oracle_free(void* h) { delete (OracleState*)h; }

void* oracle_mesh_unit() {
  auto* s = new OracleState();
  s->mesh.unit();
  return s;
}

int oracle_set_orders(void* h, const int64_t* ids, int64_t n, int i, int j) {
  auto* s = (OracleState*)h;
  ORACLE_TRY({
    std::vector<size_t> v;
    if (ids == nullptr)
      for (auto& e : s->mesh.elems) v.push_back(e.id);
    else
      for (int64_t k = 0; k < n; k++) v.push_back((size_t)ids[k]);
    s->mesh.set_expansion_orders(v, i, j);
  })
}
int oracle_p_refine(void* h, const int64_t* ids, int64_t n, int di, int dj) {
  auto* s = (OracleState*)h;
  ORACLE_TRY({
    std::vector<size_t> v;
    bool global = ids == nullptr;
    if (global)
      for (auto& e : s->mesh.elems) v.push_back(e.id);
    else
      for (int64_t k = 0; k < n; k++) v.push_back((size_t)ids[k]);
    s->mesh.p_refine(v, di, dj, global);
  })
}
int oracle_h_refine(void* h, const int64_t* ids, int64_t n, int kind, int ext) {
  auto* s = (OracleState*)h;
  ORACLE_TRY({
    HRef r{kind, ext};
    if (ids == nullptr) s->mesh.global_h_refinement(r);
    else {
      std::vector<size_t> v;
      for (int64_t k = 0; k < n; k++) v.push_back((size_t)ids[k]);
      s->mesh.h_refine_elems(v, r);
    }
  })
}
int oracle_execute_h(void* h, const int64_t* ids, const int32_t* kinds, int64_t n) {
  auto* s = (OracleState*)h;
  ORACLE_TRY({
    std::vector<std::pair<size_t, HRef>> refs;
    for (int64_t k = 0; k < n; k++) refs.push_back({(size_t)ids[k], HRef{kinds[k], -1}});
    s->mesh.execute_h_refinements(refs);
  })
}
int64_t oracle_num_elems(void* h) { return (int64_t)((OracleState*)h)->mesh.elems.size(); }
int64_t oracle_num_edges(void* h) { return (int64_t)((OracleState*)h)->mesh.edges.size(); }
int64_t oracle_num_nodes(void* h) { return (int64_t)((OracleState*)h)->mesh.nodes.size(); }

// per elem: [is_leaf, ni, nj, parent, nodes0..3, edges0..3, h_u, h_v]
int oracle_elem_info(void* h, int64_t* out) {
  auto* s = (OracleState*)h;
  ORACLE_TRY({
    for (size_t e = 0; e < s->mesh.elems.size(); e++) {
      const Elem& el = s->mesh.elems[e];
      int64_t* o = out + 14 * e;
      o[0] = el.has_children ? 0 : 1;
      o[1] = el.ni;
      o[2] = el.nj;
      o[3] = el.ancestors.empty() ? -1 : (int64_t)el.ancestors.back().first;
      for (int k = 0; k < 4; k++) o[4 + k] = (int64_t)el.nodes[k];
      for (int k = 0; k < 4; k++) o[8 + k] = (int64_t)el.edges[k];
      o[12] = el.h_levels.u;
      o[13] = el.h_levels.v;
    }
  })
}

int oracle_domain(void* h, int64_t* ndofs) {
  auto* s = (OracleState*)h;
  ORACLE_TRY({
    s->dom.reset(new Domain());
    s->dom->from_mesh(s->mesh);
    *ndofs = (int64_t)s->dom->ndofs;
  })
}
int64_t oracle_num_specs(void* h) {
  auto* s = (OracleState*)h;
  int64_t c = 0;
  for (auto& v : s->dom->basis_specs) c += (int64_t)v.size();
  return c;
}
// per spec (elem order, then elem_idx): [elem_id, elem_idx, i, j, dir, dof_id]
int oracle_specs(void* h, int64_t* out) {
  auto* s = (OracleState*)h;
  ORACLE_TRY({
    size_t k = 0;
    for (size_t e = 0; e < s->dom->basis_specs.size(); e++)
      for (auto& bs : s->dom->basis_specs[e]) {
        int64_t* o = out + 6 * k++;
        o[0] = (int64_t)e;
        o[1] = bs.elem_idx;
        o[2] = bs.i;
        o[3] = bs.j;
        o[4] = (int64_t)bs.dir;
        o[5] = bs.dof_id;
      }
  })
}

int oracle_galerkin(void* h, int basis, int nu, int nv, int nthreads, int64_t* nnz_upper) {
  auto* s = (OracleState*)h;
  ORACLE_TRY({
    if (!s->dom) throw std::runtime_error("domain not built");
    if ((nu > 0 && nu < 4) || (nv > 0 && nv < 4)) throw std::runtime_error("InvalidGLQSettings");
    s->gep = galerkin(*s->dom, basis, nu, nv, nthreads);
    *nnz_upper = (int64_t)s->gep.rows.size();
  })
}
int oracle_galerkin_by_parts(void* h, int basis, int nu, int nv, int64_t* nnz_upper) {
  auto* s = (OracleState*)h;
  ORACLE_TRY({
    if (!s->dom) throw std::runtime_error("domain not built");
    if ((nu > 0 && nu < 4) || (nv > 0 && nv < 4)) throw std::runtime_error("InvalidGLQSettings");
    s->bp = galerkin_by_parts(*s->dom, basis, nu, nv);
    *nnz_upper = (int64_t)s->bp.rows.size();
  })
}
int oracle_by_parts_export(void* h, int32_t* rows, int32_t* cols, double* vals6) {
  auto* s = (OracleState*)h;
  ORACLE_TRY({
    for (size_t k = 0; k < s->bp.rows.size(); k++) {
      rows[k] = (int32_t)s->bp.rows[k];
      cols[k] = (int32_t)s->bp.cols[k];
    }
    std::copy(s->bp.vals.begin(), s->bp.vals.end(), vals6);
  })
}
// the doc examples of real_gauss_quad_inner / real_gauss_quad_edge (glq.rs:36-52, 79-100): u^2 v^2 over
// n GLQ points per axis plus the endpoints; out = [inner, edge 0, edge 1, edge 2, edge 3]
int oracle_quad_doc(int n, double* out5) {
  ORACLE_TRY({
    std::vector<double> up, uw, vp, vw;
    glq_with_endpoints(n, up, uw);
    glq_with_endpoints(n, vp, vw);
    auto f = [&](int m, int k) { return std::pow(up[m], 2) * std::pow(vp[k], 2); };
    out5[0] = gauss_quad_inner(uw, vw, f);
    for (int e = 0; e < 4; e++) out5[1 + e] = gauss_quad_edge(uw, vw, e, f);
  })
}
// Per Elem (x0, y0, x1, y1) from its lower-left and upper-right nodes (Elem::nodes order is
// [lower-left, lower-right, upper-left, upper-right], elem.rs:12-36); used only to order the
// oracle's own sparse factorizations (nested dissection), never in any value it computes.
int oracle_elem_bounds(void* h, double* out) {
  auto* s = (OracleState*)h;
  ORACLE_TRY({
    for (size_t e = 0; e < s->mesh.elems.size(); e++) {
      const Elem& el = s->mesh.elems[e];
      const Point& a = s->mesh.nodes[el.nodes[0]].coords;
      const Point& b = s->mesh.nodes[el.nodes[3]].coords;
      out[4 * e + 0] = a.x;
      out[4 * e + 1] = a.y;
      out[4 * e + 2] = b.x;
      out[4 * e + 3] = b.y;
    }
  })
}
int oracle_num_leaves(void* h) {
  auto* s = (OracleState*)h;
  int n = 0;
  for (const Elem& e : s->mesh.elems) n += e.has_children ? 0 : 1;
  return n;
}
int oracle_xy_fields(void* h, int basis, int d0, int d1, const double* sol, int64_t nsol, double* xo, double* yo) {
  auto* s = (OracleState*)h;
  ORACLE_TRY({
    if (!s->dom) throw std::runtime_error("domain not built");
    if (d0 < 2 || d1 < 2) throw std::runtime_error("densities below 2");
    std::vector<double> v(sol, sol + nsol), x, y;
    xy_fields(*s->dom, basis, (size_t)d0, (size_t)d1, v, x, y);
    std::copy(x.begin(), x.end(), xo);
    std::copy(y.begin(), y.end(), yo);
  })
}
int oracle_gep_export(void* h, int32_t* rows, int32_t* cols, double* a, double* b) {
  auto* s = (OracleState*)h;
  ORACLE_TRY({
    for (size_t k = 0; k < s->gep.rows.size(); k++) {
      rows[k] = (int32_t)s->gep.rows[k];
      cols[k] = (int32_t)s->gep.cols[k];
      a[k] = s->gep.a[k];
      b[k] = s->gep.b[k];
    }
  })
}

int oracle_glq(int n, double* pts, double* wts) {
  ORACLE_TRY({
    std::vector<double> p, w;
    gauss_quadrature_points(n, p, w);
    for (int k = 0; k < n; k++) { pts[k] = p[k]; wts[k] = w[k]; }
  })
}

// shape tables: basis 0 = HierPoly, 1 = KOLeg; out: 4 tables (N, N', T, T') of (nmax+1) x np
int oracle_shapes(int basis, int nmax, int np, const double* x, double* out) {
  ORACLE_TRY({
    std::vector<double> xs(x, x + np);
    ShapeSpace s = basis == 0 ? hier_poly(nmax, xs) : koleg(nmax, xs);
    const std::vector<std::vector<double>>* tabs[4] = {&s.n, &s.nd, &s.t, &s.td};
    for (int t = 0; t < 4; t++)
      for (int k = 0; k <= nmax; k++)
        for (int p = 0; p < np; p++) out[((size_t)t * (nmax + 1) + k) * np + p] = (*tabs[t])[k][p];
  })
}

int oracle_default_ngq(int max_order) { return default_ngq(max_order); }

}  // extern "C"
