// Host-side mesh planner for the GB300 BEM library.
//
// Turns a triangle mesh into the device-ready layout used by the assembly
// kernels:
//  * element geometry (normals, areas, surface curls) as in the reference's
//    BoundaryMesh / surface_curls (src/blab/solvers/julia_local/src/
//    BeatEngineCore.jl:236-256, 685-702);
//  * the regular triangle rule (BeatEngineCore.jl:517-549) and the remapped
//    Duffy rules for vertex-sharing pairs (BeatEngineCore.jl:551-915), with the
//    same point order and orientation keys so the discretisation is identical;
//  * test-face tiles: faces ordered by recursive coordinate bisection of their
//    centroids and cut into compact tiles.  Each tile owns a block of
//    "extended rows" (one per distinct vertex of the tile); a vertex shared by
//    several tiles has one primary extended row (which defines its matrix row)
//    and halo rows in the other tiles.  The assembly kernel accumulates test
//    faces into extended rows without atomics, and the column gather folds
//    halo rows back into matrix rows in a fixed order;
//  * lane groups: each tile's faces are packed into groups of 32 faces that
//    share no vertex, so the 32 lanes of a warp can accumulate one group into
//    shared memory without conflicts.
#include "bem_internal.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstddef>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <thread>

namespace bem {
namespace {

using V3 = std::array<double, 3>;
inline V3 sub(const V3& a, const V3& b) { return {a[0] - b[0], a[1] - b[1], a[2] - b[2]}; }
inline double dot(const V3& a, const V3& b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
inline V3 cross(const V3& a, const V3& b) {
  return {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
}

// Regular rule (BeatEngineCore.jl:517-549): literal constants of the order-4
// six-point rule, including the asymmetric final digits of two points.
void regular_rule(int order, std::vector<double>& pts, std::vector<double>& w) {
  if (order <= 1) {
    pts = {1.0 / 3.0, 1.0 / 3.0};
    w = {0.5};
  } else if (order == 4) {
    pts = {0.4459484909159651, 0.4459484909159651, 0.0915762135097710, 0.0915762135097700,
           0.1081030181680700, 0.4459484909159651, 0.4459484909159651, 0.1081030181680700,
           0.8168475729804590, 0.0915762135097700, 0.0915762135097710, 0.8168475729804580};
    const double ws[6] = {0.2233815896780110, 0.1099517436553220, 0.2233815896780110,
                          0.2233815896780110, 0.1099517436553220, 0.1099517436553220};
    w.clear();
    for (double x : ws) w.push_back(0.5 * x);
  } else {
    pts = {1.0 / 6.0, 1.0 / 6.0, 2.0 / 3.0, 1.0 / 6.0, 1.0 / 6.0, 2.0 / 3.0};
    w = {1.0 / 6.0, 1.0 / 6.0, 1.0 / 6.0};
  }
}

// Gauss-Legendre on [0,1] (BeatEngineCore.jl:551-569).
bool gauss01(int order, std::vector<double>& x, std::vector<double>& w) {
  if (order == 1) {
    x = {0.5};
    w = {1.0};
  } else if (order == 2) {
    double a = 0.5 / std::sqrt(3.0);
    x = {0.5 - a, 0.5 + a};
    w = {0.5, 0.5};
  } else if (order == 3) {
    double a = std::sqrt(3.0 / 5.0) / 2.0;
    x = {0.5 - a, 0.5, 0.5 + a};
    w = {5.0 / 18.0, 4.0 / 9.0, 5.0 / 18.0};
  } else if (order == 4) {
    double x1 = std::sqrt(3.0 / 7.0 - 2.0 / 7.0 * std::sqrt(6.0 / 5.0)) / 2.0;
    double x2 = std::sqrt(3.0 / 7.0 + 2.0 / 7.0 * std::sqrt(6.0 / 5.0)) / 2.0;
    double w1 = (18.0 + std::sqrt(30.0)) / 72.0;
    double w2 = (18.0 - std::sqrt(30.0)) / 72.0;
    x = {0.5 - x2, 0.5 - x1, 0.5 + x1, 0.5 + x2};
    w = {w2, w1, w1, w2};
  } else {
    return false;
  }
  return true;
}

// One Duffy point as (test xi, test eta, trial xi, trial eta, w).
using DPoint = std::array<double, 5>;

// Duffy rules on [0,1]^4 mapped to triangle pairs (BeatEngineCore.jl:571-631):
// coincident (6 sub-maps), edge-adjacent (5), vertex-adjacent (2).
std::vector<DPoint> duffy_base(int order, int kind) {
  std::vector<double> x, w;
  gauss01(order, x, w);
  const int n = (int)x.size();
  std::vector<DPoint> out;
  auto push = [&](double tx, double ty, double rx, double ry, double weight) {
    out.push_back({tx - ty, ty, rx - ry, ry, weight});
  };
  for (int ti = 0; ti < n * n; ++ti) {
    for (int ri = 0; ri < n * n; ++ri) {
      const double xsi = x[ti % n], e1 = x[ti / n], e2 = x[ri % n], e3 = x[ri / n];
      const double base = (w[ti / n] * w[ti % n]) * (w[ri / n] * w[ri % n]);
      const double e12 = e1 * e2, e123 = e12 * e3;
      if (kind == 1) {
        double wt = base * xsi * xsi * xsi * e1 * e1 * e2;
        push(xsi, xsi * (1.0 - e1 + e12), xsi * (1.0 - e123), xsi * (1.0 - e1), wt);
        push(xsi * (1.0 - e123), xsi * (1.0 - e1), xsi, xsi * (1.0 - e1 + e12), wt);
        push(xsi, xsi * (e1 - e12 + e123), xsi * (1.0 - e12), xsi * (e1 - e12), wt);
        push(xsi * (1.0 - e12), xsi * (e1 - e12), xsi, xsi * (e1 - e12 + e123), wt);
        push(xsi * (1.0 - e123), xsi * (e1 - e123), xsi, xsi * (e1 - e12), wt);
        push(xsi, xsi * (e1 - e12), xsi * (1.0 - e123), xsi * (e1 - e123), wt);
      } else if (kind == 2) {
        double wt = base * xsi * xsi * xsi * e1 * e1;
        push(xsi, xsi * e1 * e3, xsi * (1.0 - e12), xsi * e1 * (1.0 - e2), wt);
        push(xsi, xsi * e1, xsi * (1.0 - e123), xsi * e1 * e2 * (1.0 - e3), wt * e2);
        push(xsi * (1.0 - e12), xsi * e1 * (1.0 - e2), xsi, xsi * e123, wt * e2);
        push(xsi * (1.0 - e123), xsi * e12 * (1.0 - e3), xsi, xsi * e1, wt * e2);
        push(xsi * (1.0 - e123), xsi * e1 * (1.0 - e2 * e3), xsi, xsi * e12, wt * e2);
      } else {
        double wt = base * xsi * xsi * xsi * e2;
        push(xsi, xsi * e1, xsi * e2, xsi * e2 * e3, wt);
        push(xsi * e2, xsi * e2 * e3, xsi, xsi * e1, wt);
      }
    }
  }
  return out;
}

// Shared-vertex / shared-edge reparametrisations (BeatEngineCore.jl:633-655),
// vertex ids 1-based.
inline void remap_vertex(double& u, double& v, int id) {
  if (id == 2) {
    u = 1.0 - u - v;
  } else if (id == 3) {
    v = 1.0 - u - v;
  }
}
inline void remap_edge(double& u, double& v, int a, int b) {
  static const double ref[3][2] = {{0.0, 0.0}, {1.0, 0.0}, {0.0, 1.0}};
  const int c = 6 - a - b;
  const double* p0 = ref[a - 1];
  const double* p1 = ref[b - 1];
  const double* p2 = ref[c - 1];
  double nu = p0[0] + u * (p1[0] - p0[0]) + v * (p2[0] - p0[0]);
  double nv = p0[1] + u * (p1[1] - p0[1]) + v * (p2[1] - p0[1]);
  u = nu;
  v = nv;
}

struct Adjacency {
  int kind, ta, tb, ra, rb;
};
// BeatEngineCore.jl:453-479
Adjacency classify(const int* fa, const int* fb) {
  int sa[9], sb[9], n = 0;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      if (fa[i] == fb[j]) {
        sa[n] = i + 1;
        sb[n] = j + 1;
        ++n;
      }
  if (n >= 3) return {1, 0, 0, 0, 0};
  if (n == 2) {
    if (sb[1] < sb[0]) {
      std::swap(sa[0], sa[1]);
      std::swap(sb[0], sb[1]);
    }
    return {2, sa[0], sa[1], sb[0], sb[1]};
  }
  if (n == 1) return {3, sa[0], 0, sb[0], 0};
  return {0, 0, 0, 0, 0};
}

// Worker threads of the planner's parallel loops: the hardware threads, at most
// 8 (16 measured slower on a 16-core Grace host); one for meshes too small to gain
// from it.  BEM_PLAN_THREADS (1-64) overrides the count; the plan does not depend on it.
int plan_threads(int nf) {
  if (const char* e = std::getenv("BEM_PLAN_THREADS")) {
    const int t = std::atoi(e);
    if (t >= 1 && t <= 64) return t;
  }
  const unsigned hc = std::thread::hardware_concurrency();
  if (nf < 2000) return 1;
  return (int)std::max(1u, std::min(hc ? hc : 1u, 8u));
}

// f(begin, end, slice) over T contiguous slices of [0, n), on T threads (the
// calling thread takes the first slice).
template <class F>
void parallel_slices(long long n, int T, F&& f) {
  if (T <= 1) {
    f(0, n, 0);
    return;
  }
  std::vector<std::thread> th;
  th.reserve(T - 1);
  for (int i = 1; i < T; ++i) th.emplace_back([&f, n, T, i]() { f(n * i / T, n * (i + 1) / T, i); });
  f(0, n / T, 0);
  for (auto& x : th) x.join();
}

// Recursive coordinate bisection of face centroids into leaves of <= cap faces.
void rcb(std::vector<int>& ids, int lo, int hi, const std::vector<double>& cent, int cap,
         std::vector<std::pair<int, int>>& leaves) {
  if (hi - lo <= cap) {
    leaves.push_back({lo, hi});
    return;
  }
  double mn[3] = {1e300, 1e300, 1e300}, mx[3] = {-1e300, -1e300, -1e300};
  for (int i = lo; i < hi; ++i)
    for (int d = 0; d < 3; ++d) {
      mn[d] = std::min(mn[d], cent[3 * ids[i] + d]);
      mx[d] = std::max(mx[d], cent[3 * ids[i] + d]);
    }
  int axis = 0;
  for (int d = 1; d < 3; ++d)
    if (mx[d] - mn[d] > mx[axis] - mn[axis]) axis = d;
  // split so that the left part holds a whole number of tiles when possible
  int n = hi - lo;
  int tiles = (n + cap - 1) / cap;
  int left_tiles = tiles / 2;
  int mid = lo + std::max(1, std::min(n - 1, (int)((long long)n * left_tiles / tiles)));
  std::nth_element(ids.begin() + lo, ids.begin() + mid, ids.begin() + hi, [&](int a, int b) {
    double ca = cent[3 * a + axis], cb = cent[3 * b + axis];
    return ca < cb || (ca == cb && a < b);
  });
  rcb(ids, lo, mid, cent, cap, leaves);
  rcb(ids, mid, hi, cent, cap, leaves);
}

}  // namespace

// Symmetry set-up (BeatEngineCore.jl:323-439): the mesh is the fundamental
// domain (x >= 0, and y >= 0 for xy).  Vertices within the plane tolerance
// (max(1e-9, 1e-6 x bounding-box diagonal)) of a symmetry plane are snapped onto
// it, a vertex on the negative side of an active plane is an error, each
// vertex's planes are recorded (fix_mask) and its orbit weight is 2 per plane.
static std::string apply_symmetry(MeshPlan& P) {
  const int nv = P.nv;
  P.transforms = P.symmetry == 0 ? std::vector<int>{0} : P.symmetry == 1 ? std::vector<int>{0, 1}
                                                                          : std::vector<int>{0, 1, 2, 3};
  P.fix_mask.assign(nv, 0);
  std::vector<double> w(nv, 1.0);
  if (P.symmetry != 0) {
    double lo[3] = {P.verts[0], P.verts[1], P.verts[2]}, hi[3] = {lo[0], lo[1], lo[2]};
    for (int v = 1; v < nv; ++v)
      for (int d = 0; d < 3; ++d) {
        lo[d] = std::min(lo[d], P.verts[3 * v + d]);
        hi[d] = std::max(hi[d], P.verts[3 * v + d]);
      }
    const double diag = std::sqrt((hi[0] - lo[0]) * (hi[0] - lo[0]) + (hi[1] - lo[1]) * (hi[1] - lo[1]) +
                                  (hi[2] - lo[2]) * (hi[2] - lo[2]));
    const double tol = std::max(1e-9, diag * 1e-6);
    const int axes = P.symmetry == 1 ? 1 : 2;
    for (int v = 0; v < nv; ++v)
      for (int a = 0; a < axes; ++a) {
        double& c = P.verts[3 * v + a];
        if (c < -tol) {
          const char* name = a == 0 ? "X" : "Y";
          return std::string("Mesh is not in the positive ") + name + " fundamental domain for " +
                 (P.symmetry == 1 ? "X" : "XY") + " symmetry. Vertex " + std::to_string(v + 1) + " has " +
                 (a == 0 ? "x" : "y") + "=" + std::to_string(c) + " m.";
        }
        if (std::fabs(c) <= tol) {
          c = 0.0;
          P.fix_mask[v] |= (unsigned char)(1 << a);
          w[v] *= 2.0;
        }
      }
  }
  P.row_weight = w;  // vertex order here; permuted to matrix rows once vertex_row is known
  return std::string();
}

// Adjacency of a test face with the image of a trial face under tr: the shared
// vertices are common indices fixed by tr (on the mesh, the image of a trial
// vertex coincides with a test vertex exactly when it is that vertex and lies on
// the planes tr reflects across).  Same result layout as classify().
Adjacency classify_image(const int* fa, const int* fb, const std::vector<unsigned char>& fix, int tr) {
  int sa[9], sb[9], n = 0;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      if (fa[i] == fb[j] && (fix[fb[j]] & tr) == tr) {
        sa[n] = i + 1;
        sb[n] = j + 1;
        ++n;
      }
  if (n >= 3) return {1, 0, 0, 0, 0};
  if (n == 2) {
    if (sb[1] < sb[0]) {
      std::swap(sa[0], sa[1]);
      std::swap(sb[0], sb[1]);
    }
    return {2, sa[0], sa[1], sb[0], sb[1]};
  }
  if (n == 1) return {3, sa[0], 0, sb[0], 0};
  return {0, 0, 0, 0, 0};
}

// Pack faces (given by their three tile-local vertex rows) into groups of at
// most kLanes faces in which no two faces share a vertex.  Target: the minimum
// ceil(n / kLanes) groups.  Faces are dealt round-robin (consecutive faces of a
// spatially ordered tile are often neighbours, so this spreads them), each to
// the first group from its own start that has room and no shared vertex; a
// face that fits nowhere is placed through a chain of displacements (below),
// and otherwise opens an extra group.
// Returns groups of indices into `fl`.
static std::vector<std::vector<int>> pack_lane_groups(const std::vector<std::array<int, 3>>& fl, int n_rows) {
  const int n = (int)fl.size();
  const int G = std::max(1, (n + kLanes - 1) / kLanes);
  std::vector<std::vector<int>> groups(G);
  std::vector<std::vector<int>> owner(G, std::vector<int>(n_rows, -1));  // row -> face in group
  // distinct faces of group g sharing a vertex with f: 0, 1 (that face in *who) or 2 (two or more)
  auto clashes = [&](int g, int f, int* who) {
    int first = -1;
    for (int a = 0; a < 3; ++a) {
      const int o = owner[g][fl[f][a]];
      if (o < 0) continue;
      if (first < 0)
        first = o;
      else if (o != first)
        return 2;
    }
    *who = first;
    return first < 0 ? 0 : 1;
  };
  auto put = [&](int g, int f) {
    groups[g].push_back(f);
    for (int a = 0; a < 3; ++a) owner[g][fl[f][a]] = f;
  };
  auto take = [&](int g, int f) {
    groups[g].erase(std::find(groups[g].begin(), groups[g].end(), f));
    for (int a = 0; a < 3; ++a) owner[g][fl[f][a]] = -1;
  };
  auto fits = [&](int g, int f) {
    int who = -1;
    return (int)groups[g].size() < kLanes && clashes(g, f, &who) == 0;
  };
  std::vector<int> left;
  for (int f = 0; f < n; ++f) {
    int placed = -1;
    for (int i = 0; i < G && placed < 0; ++i) {
      const int g = (f + i) % G;
      if (fits(g, f)) placed = g;
    }
    if (placed >= 0)
      put(placed, f);
    else
      left.push_back(f);
  }
  // Augmenting chains: f enters group g1 displacing its single clashing face
  // y1, y1 enters g2 displacing y2, ..., the last face enters a group with room
  // and no clash.  Breadth-first over faces, groups distinct along a chain.
  std::vector<int> group_of(n, -1);
  for (int g = 0; g < G; ++g)
    for (int f : groups[g]) group_of[f] = g;
  std::vector<int> still;
  std::vector<int> parent(n), via(n), stamp(n, -1);
  for (int f : left) {
    std::vector<int> queue{f};
    stamp[f] = f;
    parent[f] = -1;
    via[f] = -1;
    int end_face = -1, end_group = -1;
    for (size_t qi = 0; qi < queue.size() && end_face < 0 && queue.size() < 4096; ++qi) {
      const int x = queue[qi];
      // groups already on x's chain may not be reused
      auto on_chain = [&](int g) {
        for (int y = x; y >= 0; y = parent[y])
          if (via[y] == g || group_of[y] == g) return true;
        return false;
      };
      for (int g = 0; g < G && end_face < 0; ++g) {
        if (on_chain(g)) continue;
        int y = -1;
        const int c = clashes(g, x, &y);
        if (c == 0 && (int)groups[g].size() < kLanes) {
          end_face = x;
          end_group = g;
        } else if (c == 1 && stamp[y] != f) {
          stamp[y] = f;
          parent[y] = x;
          via[y] = g;  // y leaves g, x takes its place
          queue.push_back(y);
        }
      }
    }
    if (end_face < 0) {
      still.push_back(f);
      continue;
    }
    // apply from the end: end_face -> end_group, then each displaced face's
    // predecessor takes its slot
    int x = end_face, g = end_group;
    while (x >= 0) {
      const int from = x == f ? -1 : via[x];  // group x is displaced from
      if (from >= 0) take(from, x);
      put(g, x);
      group_of[x] = g;
      g = from;
      x = parent[x];
    }
  }
  // extra groups, first fit
  for (int f : still) {
    int placed = -1;
    for (int g = G; g < (int)groups.size() && placed < 0; ++g)
      if (fits(g, f)) placed = g;
    if (placed < 0) {
      groups.emplace_back();
      owner.emplace_back(n_rows, -1);
      placed = (int)groups.size() - 1;
    }
    put(placed, f);
  }
  std::vector<std::vector<int>> out;
  for (auto& g : groups)
    if (!g.empty()) out.push_back(std::move(g));
  return out;
}

std::string build_mesh_plan(const double* verts_in, int nv, const int* faces, int nf, int regular_order,
                            int singular_order, int tile_faces, MeshPlan& P, int symmetry) {
  if (nv <= 0 || nf <= 0) return "mesh must have at least one vertex and one face";
  if (regular_order < 1 || regular_order > 4) return "regular quadrature order must be 1..4";
  if (singular_order < 1 || singular_order > 4) return "Duffy 1D Gauss order must be between 1 and 4";
  if (symmetry < 0 || symmetry > 2) return "symmetry must be 0 (off), 1 (x) or 2 (xy)";
  if (tile_faces < 32) tile_faces = 32;
  P = MeshPlan();
  P.nv = nv;
  P.nf = nf;
  P.regular_order = regular_order;
  P.singular_order = singular_order;
  P.symmetry = symmetry;
  P.verts.assign(verts_in, verts_in + 3 * (size_t)nv);
  P.faces.assign(faces, faces + 3 * (size_t)nf);
  for (int i = 0; i < 3 * nf; ++i)
    if (faces[i] < 0 || faces[i] >= nv) return "face references a vertex index out of range";
  for (int i = 0; i < 3 * nv; ++i)
    if (!std::isfinite(verts_in[i])) return "vertex coordinates must be finite";
  {
    std::string e = apply_symmetry(P);
    if (!e.empty()) return e;
  }
  const double* verts = P.verts.data();  // snapped to the symmetry planes

  regular_rule(regular_order, P.rule_pts, P.rule_w);
  const int Q = (int)P.rule_w.size();
  P.Q = Q;
  for (int q = 0; q < Q; ++q) {
    double u = P.rule_pts[2 * q], v = P.rule_pts[2 * q + 1];
    double phi[3] = {1.0 - u - v, u, v};
    for (int a = 0; a < 3; ++a) {
      P.m10[a] += P.rule_w[q] * phi[a];
      for (int b = 0; b < 3; ++b) P.m11[3 * a + b] += P.rule_w[q] * phi[a] * phi[b];
    }
  }

  // ---- geometry (BeatEngineCore.jl:236-256, 685-702)
  P.area.resize(nf);
  P.normal.resize(3 * (size_t)nf);
  P.curls.resize(9 * (size_t)nf);
  std::vector<double> cent(3 * (size_t)nf);
  P.faces32.resize(nf);
  P.faces64.resize(nf);
  const int Tg = plan_threads(nf);
  std::vector<char> degenerate(Tg, 0);
  parallel_slices(nf, Tg, [&](long long fb, long long fe, int ti) {
    for (int f = (int)fb; f < (int)fe; ++f) {
      V3 v[3];
      for (int a = 0; a < 3; ++a)
        for (int d = 0; d < 3; ++d) v[a][d] = verts[3 * faces[3 * f + a] + d];
      V3 e1 = sub(v[1], v[0]), e2 = sub(v[2], v[0]);
      V3 cp = cross(e1, e2);
      double nn = std::sqrt(dot(cp, cp));
      if (!(nn > 0.0)) {
        degenerate[ti] = 1;
        return;
      }
      V3 n = {cp[0] / nn, cp[1] / nn, cp[2] / nn};
      P.area[f] = nn / 2.0;
      double g11 = dot(e1, e1), g12 = dot(e1, e2), g22 = dot(e2, e2);
      double det = g11 * g22 - g12 * g12;
      double i11 = g22 / det, i12 = -g12 / det, i22 = g11 / det;
      const double rg[3][2] = {{-1.0, -1.0}, {1.0, 0.0}, {0.0, 1.0}};
      V3 curl[3];
      for (int a = 0; a < 3; ++a) {
        double c1 = i11 * rg[a][0] + i12 * rg[a][1], c2 = i12 * rg[a][0] + i22 * rg[a][1];
        V3 g = {e1[0] * c1 + e2[0] * c2, e1[1] * c1 + e2[1] * c2, e1[2] * c1 + e2[2] * c2};
        curl[a] = cross(n, g);
      }
      V3 c = {(v[0][0] + v[1][0] + v[2][0]) / 3.0, (v[0][1] + v[1][1] + v[2][1]) / 3.0,
              (v[0][2] + v[1][2] + v[2][2]) / 3.0};
      for (int d = 0; d < 3; ++d) {
        cent[3 * f + d] = c[d];
        P.normal[3 * f + d] = n[d];
      }
      for (int a = 0; a < 3; ++a)
        for (int d = 0; d < 3; ++d) P.curls[9 * f + 3 * a + d] = curl[a][d];

      FaceF32& F = P.faces32[f];
      FaceF64& G = P.faces64[f];
      std::fill((float*)&F, (float*)&F + 40, 0.0f);
      std::fill((double*)&G, (double*)&G + sizeof(FaceF64) / 8, 0.0);
      for (int d = 0; d < 3; ++d) {
        F.anchor_hi[d] = (float)c[d];
        F.anchor_lo[d] = (float)(c[d] - (double)F.anchor_hi[d]);
        F.normal[d] = (float)n[d];
        G.anchor[d] = c[d];
        G.normal[d] = n[d];
      }
      F.area2 = (float)nn;
      G.area2 = nn;
      for (int a = 0; a < 3; ++a)
        for (int d = 0; d < 3; ++d) {
          F.curls[3 * a + d] = (float)curl[a][d];
          G.curls[3 * a + d] = curl[a][d];
        }
      for (int q = 0; q < Q; ++q) {
        double u = P.rule_pts[2 * q], w2 = P.rule_pts[2 * q + 1];
        for (int d = 0; d < 3; ++d) {
          // quadrature point as in local_to_global (BeatEngineCore.jl:678-681)
          double x = (1.0 - u - w2) * v[0][d] + u * v[1][d] + w2 * v[2][d];
          F.off[3 * q + d] = (float)(x - c[d]);
          G.off[3 * q + d] = x - c[d];
        }
      }
      for (int a = 0; a < 3; ++a) {
        F.verts[a] = faces[3 * f + a];
        G.verts[a] = faces[3 * f + a];
      }
    }
  });
  for (char d : degenerate)
    if (d) return "mesh contains a degenerate (zero-area) triangle";

  // ---- test-face tiles by recursive coordinate bisection
  std::vector<int> order(nf);
  std::iota(order.begin(), order.end(), 0);
  std::vector<std::pair<int, int>> leaves;
  rcb(order, 0, nf, cent, tile_faces, leaves);
  P.tile_faces = tile_faces;
  P.n_tiles = (int)leaves.size();
  std::vector<int> face_tile(nf);
  std::vector<std::vector<int>> tile_face_list(P.n_tiles);
  for (int t = 0; t < P.n_tiles; ++t) {
    std::vector<int> fl(order.begin() + leaves[t].first, order.begin() + leaves[t].second);
    std::sort(fl.begin(), fl.end());
    for (int f : fl) face_tile[f] = t;
    tile_face_list[t] = fl;
  }
  // primary tile of a vertex = first tile (in tile order) containing it
  std::vector<int> primary(nv, -1);
  for (int t = 0; t < P.n_tiles; ++t)
    for (int f : tile_face_list[t])
      for (int a = 0; a < 3; ++a)
        if (primary[faces[3 * f + a]] < 0) primary[faces[3 * f + a]] = t;
  for (int v = 0; v < nv; ++v)
    if (primary[v] < 0) primary[v] = -2;  // unreferenced vertex: gets its own row below
  // tile-local rows: primary vertices first (first-appearance order), then halo vertices
  P.face_ext.assign(3 * (size_t)nf, -1);
  P.tile_row_base.assign(P.n_tiles + 1, 0);
  P.vertex_row.assign(nv, -1);
  P.row_vertex.clear();
  std::vector<std::vector<int>> tile_rows(P.n_tiles);
  std::vector<int> face_loc(3 * (size_t)nf, -1);  // tile-local row of each face vertex
  {
    std::vector<int> loc(nv, -1);  // tile-local row of a vertex while its tile is built
    std::vector<int> prim, halo;
    for (int t = 0; t < P.n_tiles; ++t) {
      prim.clear();
      halo.clear();
      for (int f : tile_face_list[t])
        for (int a = 0; a < 3; ++a) {
          const int v = faces[3 * f + a];
          if (loc[v] == -1) {
            loc[v] = -2;  // seen; the row index is assigned below
            (primary[v] == t ? prim : halo).push_back(v);
          }
        }
      for (int v : prim) {
        P.vertex_row[v] = (int)P.row_vertex.size();
        P.row_vertex.push_back(v);
      }
      std::vector<int>& rows = tile_rows[t];
      rows = prim;
      rows.insert(rows.end(), halo.begin(), halo.end());
      for (size_t i = 0; i < rows.size(); ++i) loc[rows[i]] = (int)i;
      for (int f : tile_face_list[t])
        for (int a = 0; a < 3; ++a) face_loc[3 * f + a] = loc[faces[3 * f + a]];
      for (int v : rows) loc[v] = -1;
      P.tile_row_base[t + 1] = P.tile_row_base[t] + (int)rows.size();
      P.max_tile_rows = std::max(P.max_tile_rows, (int)rows.size());
    }
  }
  for (int v = 0; v < nv; ++v)
    if (P.vertex_row[v] < 0) {  // vertex used by no face: identity-free zero row
      P.vertex_row[v] = (int)P.row_vertex.size();
      P.row_vertex.push_back(v);
    }
  {  // orbit weights to matrix-row order
    std::vector<double> rw(nv, 1.0);
    for (int v = 0; v < nv; ++v) rw[P.vertex_row[v]] = P.row_weight[v];
    P.row_weight.swap(rw);
  }
  P.n_ext = P.tile_row_base[P.n_tiles];
  P.ext_row.resize(P.n_ext);
  P.ext_is_halo.resize(P.n_ext);
  for (int t = 0; t < P.n_tiles; ++t)
    for (size_t i = 0; i < tile_rows[t].size(); ++i) {
      int v = tile_rows[t][i];
      P.ext_row[P.tile_row_base[t] + i] = P.vertex_row[v];
      P.ext_is_halo[P.tile_row_base[t] + i] = primary[v] == t ? 0 : 1;
    }
  for (int f = 0; f < nf; ++f) {
    int t = face_tile[f];
    for (int a = 0; a < 3; ++a) P.face_ext[3 * f + a] = P.tile_row_base[t] + face_loc[3 * f + a];
  }
  // halo gather lists, grouped by target row (ascending ext id within a row)
  {
    std::vector<std::pair<int, int>> h;  // (row, ext)
    for (int e = 0; e < P.n_ext; ++e)
      if (P.ext_is_halo[e]) h.push_back({P.ext_row[e], e});
    std::sort(h.begin(), h.end());
    P.halo_ext.clear();
    P.halo_row.clear();
    P.halo_row_ptr.assign(1, 0);
    P.halo_slot_of_ext.assign(P.n_ext, -1);
    for (size_t i = 0; i < h.size(); ++i) {
      if (i == 0 || h[i].first != h[i - 1].first) {
        if (i) P.halo_row_ptr.push_back((int)i);
        P.halo_row.push_back(h[i].first);
      }
      P.halo_slot_of_ext[h[i].second] = (int)i;
      P.halo_ext.push_back(h[i].second);
    }
    P.halo_row_ptr.push_back((int)h.size());
    if (h.empty()) P.halo_row_ptr.assign(1, 0);
  }
  // lane groups: each tile's faces packed into ceil(n / 32) vertex-disjoint
  // groups of 32 where possible (pack_lane_groups), so few lanes idle.
  // The tiles are packed independently, on the planner's threads, and appended in
  // tile order.
  P.tile_group_ptr.assign(1, 0);
  P.lane_slots.clear();
  std::vector<std::vector<std::vector<int>>> tile_groups(P.n_tiles);
  parallel_slices(P.n_tiles, std::min(plan_threads(nf), std::max(1, P.n_tiles)), [&](long long tb, long long te, int) {
    for (long long t = tb; t < te; ++t) {
      std::vector<std::array<int, 3>> fl;
      fl.reserve(tile_face_list[t].size());
      for (int f : tile_face_list[t]) fl.push_back({face_loc[3 * f], face_loc[3 * f + 1], face_loc[3 * f + 2]});
      tile_groups[t] = pack_lane_groups(fl, (int)tile_rows[t].size());
      for (auto& g : tile_groups[t])
        for (int& i : g) i = tile_face_list[t][i];
    }
  });
  for (int t = 0; t < P.n_tiles; ++t) {
    const std::vector<std::vector<int>>& groups = tile_groups[t];
    for (auto& g : groups) {
      for (int l = 0; l < kLanes; ++l) {
        LaneSlot s;
        if (l < (int)g.size()) {
          int f = g[l];
          s.face = f;
          for (int a = 0; a < 3; ++a) s.loc[a] = face_loc[3 * f + a];
        } else {
          s.face = -1;
          s.loc[0] = s.loc[1] = s.loc[2] = 0;
        }
        P.lane_slots.push_back(s);
      }
    }
    P.tile_group_ptr.push_back(P.tile_group_ptr.back() + (int)groups.size());
  }
  // the same groups, field-major: word w of lane l's face record at [grp][w][l]
  static_assert(offsetof(FaceF32, anchor_lo) == 4 * kFwAnchorLo && offsetof(FaceF32, normal) == 4 * kFwNormal &&
                    offsetof(FaceF32, area2) == 4 * kFwArea2 && offsetof(FaceF32, curls) == 4 * kFwCurls &&
                    offsetof(FaceF32, off) == 4 * kFwOff && offsetof(FaceF32, verts) == 4 * kFwVerts &&
                    sizeof(FaceF32) == 4 * kFaceWords,
                "FaceF32 word offsets");
  {
    const size_t ng = P.lane_slots.size() / kLanes;
    P.group_faces32.resize(ng * kFaceWords * kLanes);
    parallel_slices((long long)ng, plan_threads(nf), [&](long long gb, long long ge, int) {
    for (long long g = gb; g < ge; ++g)
      for (int l = 0; l < kLanes; ++l) {
        const int f = P.lane_slots[g * kLanes + l].face;
        float w[kFaceWords];
        if (f >= 0) {
          std::memcpy(w, &P.faces32[f], sizeof(w));
        } else {
          std::memset(w, 0, sizeof(w));
          const int none = -1;
          for (int a = 0; a < 3; ++a) std::memcpy(&w[kFwVerts + a], &none, sizeof(int));
        }
        for (int i = 0; i < kFaceWords; ++i) P.group_faces32[(g * kFaceWords + i) * kLanes + l] = w[i];
      }
    });
  }
  // column gather CSR: vertex j <- (g, b)
  P.col_ptr.assign(nv + 1, 0);
  for (int i = 0; i < 3 * nf; ++i) P.col_ptr[faces[i] + 1]++;
  for (int v = 0; v < nv; ++v) P.col_ptr[v + 1] += P.col_ptr[v];
  P.col_fb.assign(3 * (size_t)nf, 0);
  {
    std::vector<int> fill(P.col_ptr.begin(), P.col_ptr.end() - 1);
    for (int f = 0; f < nf; ++f)
      for (int b = 0; b < 3; ++b) P.col_fb[fill[faces[3 * f + b]]++] = 3 * f + b;
  }

  // ---- singular pairs and remapped Duffy rules (BeatEngineCore.jl:784-915)
  std::vector<std::vector<int>> v2f(nv);
  for (int f = 0; f < nf; ++f)
    for (int a = 0; a < 3; ++a) v2f[faces[3 * f + a]].push_back(f);
  std::vector<DPoint> base[4];
  for (int k = 1; k <= 3; ++k) base[k] = duffy_base(singular_order, k);
  // Candidate pairs, enumerated over (transform, test face) in order.  The index
  // range is cut into contiguous slices enumerated by worker threads; each slice
  // keeps its pairs in order with their adjacency keys (kind, ta, tb, ra, rb;
  // every field < 4), and the rules are then numbered in order of first
  // appearance over the slices in order, so the result does not depend on the
  // number of threads.
  const int ntr = (int)P.transforms.size();
  const long long n_idx = (long long)ntr * nf;
  const int T = plan_threads(nf);
  struct Slice {
    std::vector<SingularPair> pairs;
    std::vector<short> keys;
    int image_pairs = 0;
  };
  std::vector<Slice> slices(T);
  parallel_slices(n_idx, T, [&](long long b, long long e, int ti) {
    Slice& sl = slices[ti];
    sl.pairs.reserve((size_t)(16 * (e - b)));
    sl.keys.reserve((size_t)(16 * (e - b)));
    std::vector<long long> seen(nf, -1);  // candidate stamp: the index that last listed the face
    std::vector<int> cand;
    for (long long idx = b; idx < e; ++idx) {
      const int tr = P.transforms[(int)(idx / nf)];
      const int t = (int)(idx % nf);
      cand.clear();
      for (int a = 0; a < 3; ++a) {
        const int v = faces[3 * t + a];
        if (tr != 0 && (P.fix_mask[v] & tr) != tr) continue;  // images touch the test face only on the planes
        for (int r : v2f[v])
          if (seen[r] != idx) {
            seen[r] = idx;
            cand.push_back(r);
          }
      }
      for (int r : cand) {
        Adjacency adj = tr == 0 ? classify(&faces[3 * t], &faces[3 * r])
                                : classify_image(&faces[3 * t], &faces[3 * r], P.fix_mask, tr);
        if (adj.kind == 0) continue;
        const int key = adj.kind == 1 ? 256
                        : adj.kind == 2 ? 512 + 64 * adj.ta + 16 * adj.tb + 4 * adj.ra + adj.rb
                                        : 768 + 64 * adj.ta + 4 * adj.ra;
        SingularPair sp;
        sp.test = t;
        sp.trial = r;
        sp.rule = -1;
        sp.kind = adj.kind;
        sp.tr = tr;
        sp.pad = 0;
        sp.jac = (2.0 * P.area[t]) * (2.0 * P.area[r]);
        sp.nprod = P.normal[3 * t] * tr_sx(tr) * P.normal[3 * r] +
                   P.normal[3 * t + 1] * tr_sy(tr) * P.normal[3 * r + 1] + P.normal[3 * t + 2] * P.normal[3 * r + 2];
        if (tr != 0) ++sl.image_pairs;
        sl.pairs.push_back(sp);
        sl.keys.push_back((short)key);
      }
    }
  });
  // rules in order of first appearance; rule_of_key is -1 until a key is seen
  std::vector<int> rule_of_key(4 * 256, -1);
  int n_rules = 0;
  P.rule_ptr.assign(1, 0);
  P.duffy.clear();
  size_t n_pairs = 0;
  for (Slice& sl : slices) {
    P.image_pairs += sl.image_pairs;
    n_pairs += sl.pairs.size();
    for (size_t i = 0; i < sl.pairs.size(); ++i) {
      const int key = sl.keys[i];
      int rule = rule_of_key[key];
      if (rule < 0) {
        rule = rule_of_key[key] = n_rules++;
        const int kind = key >> 8, ta = (key >> 6) & 3, tb = (key >> 4) & 3, ra = (key >> 2) & 3, rb = key & 3;
        for (const DPoint& q : base[kind]) {
          double tu = q[0], tv = q[1], ru = q[2], rv = q[3];
          if (kind == 2) {
            remap_edge(tu, tv, ta, tb);
            remap_edge(ru, rv, ra, rb);
          } else if (kind == 3) {
            remap_vertex(tu, tv, ta);
            remap_vertex(ru, rv, ra);
          }
          P.duffy.insert(P.duffy.end(), {tu, tv, ru, rv, q[4]});
        }
        P.rule_ptr.push_back((int)(P.duffy.size() / 5));
      }
      sl.pairs[i].rule = rule;
    }
  }
  // pairs grouped by trial face, generation order kept within a face (a stable
  // counting sort; each slice scatters its own pairs after the slices before it)
  {
    std::vector<std::vector<int>> cnt(T, std::vector<int>(nf, 0));
    parallel_slices(T, T, [&](long long b, long long e, int) {
      for (long long ti = b; ti < e; ++ti)
        for (const auto& sp : slices[ti].pairs) cnt[ti][sp.trial]++;
    });
    P.pairs_by_trial_ptr.assign(nf + 1, 0);
    for (int f = 0; f < nf; ++f) {
      int run = P.pairs_by_trial_ptr[f];
      for (int ti = 0; ti < T; ++ti) {
        const int c = cnt[ti][f];
        cnt[ti][f] = run;  // this slice's first position for trial face f
        run += c;
      }
      P.pairs_by_trial_ptr[f + 1] = run;
    }
    P.pairs.resize(n_pairs);
    parallel_slices(T, T, [&](long long b, long long e, int) {
      for (long long ti = b; ti < e; ++ti)
        for (const auto& sp : slices[ti].pairs) P.pairs[cnt[ti][sp.trial]++] = sp;
    });
  }
  P.pairs_by_test_ptr.assign(nf + 1, 0);
  for (const auto& sp : P.pairs) P.pairs_by_test_ptr[sp.test + 1]++;
  for (int f = 0; f < nf; ++f) P.pairs_by_test_ptr[f + 1] += P.pairs_by_test_ptr[f];
  P.pairs_by_test.assign(P.pairs.size(), 0);
  {
    std::vector<int> fill(P.pairs_by_test_ptr.begin(), P.pairs_by_test_ptr.end() - 1);
    for (size_t i = 0; i < P.pairs.size(); ++i) P.pairs_by_test[fill[P.pairs[i].test]++] = (int)i;
  }
  // singular scatter plan: every (trial column 3 g + b, extended row e) entry the
  // pairs of trial face g add into, with its contributions in pair order (pair k,
  // then test vertex a), so a thread per entry adds them in the order one thread
  // per trial face would have.  The entries of trial face g are its own columns, so
  // each face's entries and contributions are planned on their own: in slices of
  // trial faces on the planner's threads, numbered in order of first appearance
  // within the face and concatenated in face order (the same plan as one walk over
  // all faces).
  {
    struct ScatSlice {
      std::vector<int> col, row, cnt, src;
      double r2 = 0.0;     // largest squared vertex distance of a pair
      long long npts = 0;  // Duffy points of the pairs
    };
    const int Ts = plan_threads(nf);
    std::vector<ScatSlice> ss(Ts);
    parallel_slices(nf, Ts, [&](long long gb, long long ge, int ti) {
      ScatSlice& S = ss[ti];
      const size_t npairs_slice = (size_t)(P.pairs_by_trial_ptr[ge] - P.pairs_by_trial_ptr[gb]);
      S.src.reserve(9 * npairs_slice);
      S.col.reserve(4 * npairs_slice);
      S.row.reserve(4 * npairs_slice);
      S.cnt.reserve(4 * npairs_slice);
      std::vector<int> entry_of(3 * (size_t)std::max(P.n_ext, 1), -1);
      std::vector<int> touched, off;
      for (long long g = gb; g < ge; ++g) {
        const int k0 = P.pairs_by_trial_ptr[g], k1 = P.pairs_by_trial_ptr[g + 1];
        const int e0 = (int)S.col.size();
        touched.clear();
        for (int k = k0; k < k1; ++k) {
          const int f = P.pairs[k].test;
          {
            const SingularPair& sp = P.pairs[k];
            const double sx = tr_sx(sp.tr), sy = tr_sy(sp.tr);
            for (int a = 0; a < 3; ++a) {
              const double* t = &P.verts[3 * (size_t)P.faces[3 * (size_t)f + a]];
              for (int b = 0; b < 3; ++b) {
                const double* q = &P.verts[3 * (size_t)P.faces[3 * (size_t)g + b]];
                const double dx = sx * q[0] - t[0], dy = sy * q[1] - t[1], dz = q[2] - t[2];
                S.r2 = std::max(S.r2, dx * dx + dy * dy + dz * dz);
              }
            }
            S.npts += P.rule_ptr[sp.rule + 1] - P.rule_ptr[sp.rule];
          }
          for (int a = 0; a < 3; ++a) {
            const int e = P.face_ext[3 * (size_t)f + a];
            for (int b = 0; b < 3; ++b) {
              int& slot = entry_of[3 * (size_t)e + b];
              if (slot < 0) {
                slot = (int)S.col.size();
                S.col.push_back(3 * (int)g + b);
                S.row.push_back(e);
                S.cnt.push_back(0);
                touched.push_back(3 * e + b);
              }
              S.cnt[slot]++;
            }
          }
        }
        // this face's contributions grouped by entry, each entry's in walk order
        const int ne_g = (int)S.col.size() - e0;
        off.assign(ne_g, 0);
        size_t run = S.src.size();
        for (int i = 0; i < ne_g; ++i) {
          off[i] = (int)run;
          run += S.cnt[e0 + i];
        }
        S.src.resize(run);
        for (int k = k0; k < k1; ++k) {
          const int f = P.pairs[k].test;
          for (int a = 0; a < 3; ++a) {
            const int e = P.face_ext[3 * (size_t)f + a];
            for (int b = 0; b < 3; ++b) S.src[off[entry_of[3 * (size_t)e + b] - e0]++] = 12 * k + 3 * a + b;
          }
        }
        for (int t : touched) entry_of[t] = -1;
      }
    });
    size_t ne = 0, nc = 0;
    double r2 = 0.0;
    P.singular_points = 0;
    for (const ScatSlice& S : ss) {
      ne += S.col.size();
      nc += S.src.size();
      r2 = std::max(r2, S.r2);
      P.singular_points += S.npts;
    }
    P.pair_radius = std::sqrt(r2);
    P.scat_col.resize(ne);
    P.scat_row.resize(ne);
    P.scat_ptr.resize(ne + 1);
    P.scat_src.resize(nc);
    std::vector<size_t> eo(Ts + 1, 0), co(Ts + 1, 0);
    for (int t = 0; t < Ts; ++t) {
      eo[t + 1] = eo[t] + ss[t].col.size();
      co[t + 1] = co[t] + ss[t].src.size();
    }
    P.scat_ptr[0] = 0;
    // each slice into its own range (the copies, and the first touch of the fresh
    // pages, spread over the threads)
    parallel_slices(Ts, Ts, [&](long long b, long long e, int) {
      for (long long t = b; t < e; ++t) {
        const ScatSlice& S = ss[t];
        std::copy(S.col.begin(), S.col.end(), P.scat_col.begin() + eo[t]);
        std::copy(S.row.begin(), S.row.end(), P.scat_row.begin() + eo[t]);
        std::copy(S.src.begin(), S.src.end(), P.scat_src.begin() + co[t]);
        int run = (int)co[t];
        for (size_t i = 0; i < S.cnt.size(); ++i) {
          run += S.cnt[i];
          P.scat_ptr[eo[t] + i + 1] = run;
        }
      }
    });
  }
  return std::string();
}

}  // namespace bem
