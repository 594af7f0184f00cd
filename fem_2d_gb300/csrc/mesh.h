// Refinement-by-superposition mesh: the structure Domain::from_mesh and the Galerkin driver read.
//
// Follows src/fem_domain/domain/mesh.rs and its submodules. Ids of Elems, Edges and Nodes are
// allocated in exactly the reference's order (they decide DoF numbering); the containers are flat
// vectors, and an Edge keeps, per side, only the list of (h-level rank, elem) pairs it needs to
// find the active pair (edge.rs:203-222).
#pragma once
#include <array>
#include <cstdint>
#include <string>
#include <vector>

namespace fem2d {

// Coordinates compared the way Point/FloatRep do (space.rs:349-382): the fractional part is rounded
// to 1e-12 and the comparison is on (sign, bits of the rounded magnitude).
struct QKey {
  bool pos;
  uint64_t bits;
  static QKey of(double v);
  int cmp(const QKey& o) const;
  bool operator==(const QKey& o) const { return pos == o.pos && bits == o.bits; }
};

struct Pt {
  double x = 0, y = 0;
  QKey kx{true, 0}, ky{true, 0};
  Pt() = default;
  Pt(double x_, double y_) : x(x_), y(y_), kx(QKey::of(x_)), ky(QKey::of(y_)) {}
  bool same(const Pt& o) const { return kx == o.kx && ky == o.ky; }
};

enum Axis : uint8_t { AX_U = 0, AX_V = 1 };
// position of a child inside its parent (HRefLoc, h_refinement.rs:197-252)
enum Loc : uint8_t { L_SW = 0, L_SE, L_NW, L_NE, L_W, L_E, L_S, L_N };

struct RootElement {   // element.rs:7-12: the base quad of an Elem tree
  double x0, y0, x3, y3;   // points[0] and points[3]
  double eps_re, eps_im, mu_re, mu_im;
};

struct MEdge {
  int64_t n0, n1;
  bool boundary;
  Axis dir;
  double length;
  int64_t child[2] = {-1, -1};
  int64_t parent = -1;
  int64_t mid_node = -1;
  // per side: (rank key, elem id); rank = (hi << 8) | lo of edge_ranking (h_refinement.rs:31-36)
  std::vector<std::pair<uint16_t, int64_t>> side[2];
  bool active = false;
  int64_t act[2] = {-1, -1};
};

struct MElem {
  int64_t nodes[4];
  int64_t edges[4];
  int64_t root;                 // index into Mesh::roots
  uint8_t hu = 0, hv = 0;       // HLevels
  uint8_t ni = 1, nj = 1;       // PolyOrders (default 1,1)
  int8_t nchild = 0;
  int64_t child[4] = {-1, -1, -1, -1};
  std::vector<int64_t> anc;     // ancestor ids, root first
  std::vector<uint8_t> locs;    // loc of the next-level Elem inside anc[k]
  bool leaf() const { return nchild == 0; }
};

struct MNode {
  Pt p;
  bool boundary;
};

class Mesh {
 public:
  std::vector<RootElement> roots;
  std::vector<MElem> elems;
  std::vector<MEdge> edges;
  std::vector<MNode> nodes;

  static Mesh from_json(const std::string& text);
  static Mesh unit();

  void set_expansion(const std::vector<int64_t>& ids, int i, int j);
  void p_refine(const std::vector<int64_t>& ids, int di, int dj, bool clamp_to_window);
  // kinds: 0 T, 1 U, 2 V; ext: -1 or child index
  void execute_h_refinements(const std::vector<int64_t>& ids, const std::vector<int>& kinds,
                             const std::vector<int>& exts);
  void global_h_refinement(int kind, int ext);
  void h_refine_elems(const std::vector<int64_t>& ids, int kind, int ext);
  void set_edge_activation();

  bool refineable(int64_t e) const;
  std::array<int, 2> max_orders() const;
  // parametric range of Elem e inside its root, [[u0,u1],[v0,v1]] (elem.rs:191-197)
  std::array<double, 4> param_range(int64_t e) const;
  // range of e inside ancestor a (elem.rs:170-188)
  std::array<double, 4> relative_range(int64_t e, int64_t a) const;
  // descendants of e in depth-first preorder, e excluded (mesh.rs:470-493)
  void descendants(int64_t e, std::vector<int64_t>& out) const;

 private:
  void attach(int64_t edge, int64_t elem);
  int64_t split_edge(int64_t pe, int64_t& next_node, int64_t& next_edge, int64_t ch[2]);
  int64_t join_nodes(int64_t a, int64_t b, int64_t& next_edge);
  bool activate_tree(int64_t e);
};

// Jacobian of an Elem's map from its own parametric square to real space (element.rs:33-50) and the
// inverse-Jacobian diagonal the basis functions carry (space.rs:137-147): a = dx/du, b = dy/dv,
// det = a*b, ji_u0 = b/det, ji_v1 = a/det (evaluated in exactly that order).
struct ElemJac {
  double a, b, det, ji_u0, ji_v1;
};
ElemJac elem_jacobian(const Mesh& m, int64_t e);

}  // namespace fem2d
