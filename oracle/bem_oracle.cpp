// CPU oracle for the exterior Burton-Miller Galerkin P1/DP0 Helmholtz BEM path.
//
// TEST INFRASTRUCTURE ONLY.  This file restates, in C++17 + OpenMP, the
// algorithm of the reference's BEAT CPU backend so that the CUDA path can be
// checked against it.  It is never linked into, loaded by, or called from the
// product library; only tests, __graft_entry__.smoke() and bench.py's
// cpu_baseline / reference arm use it.
//
// Parity status: the reference engine is Julia and cannot run on these
// machines, and the reference ships no numeric golden vectors for this path,
// so numeric parity with the reference itself is unpinned.  What is pinned is
// listed in the tests (literal rule constants, fixture-mesh counts, the
// reference's own consistency relations, analytic solutions).
//
// Every function cites the reference lines it follows (paths relative to
// src/blab/solvers/julia_local/):
//   triangle_rule            src/BeatEngineCore.jl:517-549
//   gauss_rule_1d            src/BeatEngineCore.jl:551-569
//   duffy_rule               src/BeatEngineCore.jl:571-631
//   remap_shared_vertex/edge src/BeatEngineCore.jl:633-655
//   adjacency_info           src/BeatEngineCore.jl:453-479
//   singular cache           src/BeatEngineCore.jl:784-915
//   surface_gradients/curls  src/BeatEngineCore.jl:685-702
//   l2 identity (mass)       src/BeatEngineCore.jl:731-749, 952-979
//   regular pair integral    src/BeatEngineCpuAssembly.jl:278-373
//   singular pair integral   src/BeatEngineCpuAssembly.jl:151-218, 447-486
//   colored threading        src/BeatEngineCpuAssembly.jl:102-130, 636-803
//   field evaluation         src/BeatEngineCpuField.jl:1-45, BeatEngineCore.jl:1240-1280
//   symmetry                 src/BeatEngineCore.jl:323-439, 481-505, 917-943,
//                            src/BeatEngineCpuAssembly.jl:411-445, 488-634
//
// The template parameter T is the working precision: float restates the
// reference's production FP32 path ("BEAT CPU restated"); double is the FP64
// oracle of the same discretisation.

#include <algorithm>
#include <array>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <map>
#include <set>
#include <tuple>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

template <typename T> using V3 = std::array<T, 3>;
template <typename T> using V2 = std::array<T, 2>;
template <typename T> using C = std::complex<T>;

template <typename T> inline V3<T> sub(const V3<T>& a, const V3<T>& b) { return {a[0] - b[0], a[1] - b[1], a[2] - b[2]}; }
template <typename T> inline T dot(const V3<T>& a, const V3<T>& b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
template <typename T> inline V3<T> cross(const V3<T>& a, const V3<T>& b) {
  return {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
}
template <typename T> inline T norm(const V3<T>& a) { return std::sqrt(dot(a, a)); }

// ---------------------------------------------------------------- rules ----

template <typename T> struct TriRule {
  std::vector<V2<T>> pts;
  std::vector<T> w;
};

// BeatEngineCore.jl:517-549 (literal constants kept exactly, including the
// asymmetric last digits of the order-4 points).
template <typename T> TriRule<T> triangle_rule(int order) {
  TriRule<T> r;
  if (order <= 1) {
    r.pts = {{T(1) / T(3), T(1) / T(3)}};
    r.w = {T(0.5)};
  } else if (order == 4) {
    r.pts = {{T(0.4459484909159651), T(0.4459484909159651)}, {T(0.0915762135097710), T(0.0915762135097700)},
             {T(0.1081030181680700), T(0.4459484909159651)}, {T(0.4459484909159651), T(0.1081030181680700)},
             {T(0.8168475729804590), T(0.0915762135097700)}, {T(0.0915762135097710), T(0.8168475729804580)}};
    const T ws[6] = {T(0.2233815896780110), T(0.1099517436553220), T(0.2233815896780110),
                     T(0.2233815896780110), T(0.1099517436553220), T(0.1099517436553220)};
    for (int i = 0; i < 6; ++i) r.w.push_back(T(0.5) * ws[i]);
  } else {
    r.pts = {{T(1) / T(6), T(1) / T(6)}, {T(2) / T(3), T(1) / T(6)}, {T(1) / T(6), T(2) / T(3)}};
    r.w = {T(1) / T(6), T(1) / T(6), T(1) / T(6)};
  }
  return r;
}

// BeatEngineCore.jl:551-569
template <typename T> void gauss_rule_1d(int order, std::vector<T>& x, std::vector<T>& w) {
  if (order == 1) {
    x = {T(0.5)};
    w = {T(1.0)};
  } else if (order == 2) {
    T a = T(0.5) / std::sqrt(T(3.0));
    x = {T(0.5) - a, T(0.5) + a};
    w = {T(0.5), T(0.5)};
  } else if (order == 3) {
    T a = std::sqrt(T(3.0) / T(5.0)) / T(2.0);
    x = {T(0.5) - a, T(0.5), T(0.5) + a};
    w = {T(5.0) / T(18.0), T(4.0) / T(9.0), T(5.0) / T(18.0)};
  } else if (order == 4) {
    T x1 = std::sqrt(T(3.0) / T(7.0) - T(2.0) / T(7.0) * std::sqrt(T(6.0) / T(5.0))) / T(2.0);
    T x2 = std::sqrt(T(3.0) / T(7.0) + T(2.0) / T(7.0) * std::sqrt(T(6.0) / T(5.0))) / T(2.0);
    T w1 = (T(18.0) + std::sqrt(T(30.0))) / T(72.0);
    T w2 = (T(18.0) - std::sqrt(T(30.0))) / T(72.0);
    x = {T(0.5) - x2, T(0.5) - x1, T(0.5) + x1, T(0.5) + x2};
    w = {w2, w1, w1, w2};
  } else {
    x.clear();
    w.clear();
  }
}

template <typename T> struct DuffyRule {
  std::vector<V2<T>> test, trial;
  std::vector<T> w;
};

// BeatEngineCore.jl:627-631
template <typename T> inline void append_duffy(DuffyRule<T>& r, T tx, T ty, T rx, T ry, T weight) {
  r.test.push_back({tx - ty, ty});
  r.trial.push_back({rx - ry, ry});
  r.w.push_back(weight);
}

// kind: 1 coincident, 2 edge adjacent, 3 vertex adjacent.  BeatEngineCore.jl:571-625
template <typename T> DuffyRule<T> duffy_rule(int order, int kind) {
  std::vector<T> xr, wr;
  gauss_rule_1d<T>(order, xr, wr);
  std::vector<V2<T>> tp;
  std::vector<T> tw;
  for (size_t i = 0; i < xr.size(); ++i)
    for (size_t j = 0; j < xr.size(); ++j) {
      tp.push_back({xr[j], xr[i]});
      tw.push_back(wr[i] * wr[j]);
    }
  DuffyRule<T> r;
  const T one = T(1.0);
  for (size_t ti = 0; ti < tp.size(); ++ti)
    for (size_t ri = 0; ri < tp.size(); ++ri) {
      T xsi = tp[ti][0], eta1 = tp[ti][1], eta2 = tp[ri][0], eta3 = tp[ri][1];
      T eta12 = eta1 * eta2, eta123 = eta12 * eta3;
      T base = tw[ti] * tw[ri];
      if (kind == 1) {
        T w = base * xsi * xsi * xsi * eta1 * eta1 * eta2;
        append_duffy(r, xsi, xsi * (one - eta1 + eta12), xsi * (one - eta123), xsi * (one - eta1), w);
        append_duffy(r, xsi * (one - eta123), xsi * (one - eta1), xsi, xsi * (one - eta1 + eta12), w);
        append_duffy(r, xsi, xsi * (eta1 - eta12 + eta123), xsi * (one - eta12), xsi * (eta1 - eta12), w);
        append_duffy(r, xsi * (one - eta12), xsi * (eta1 - eta12), xsi, xsi * (eta1 - eta12 + eta123), w);
        append_duffy(r, xsi * (one - eta123), xsi * (eta1 - eta123), xsi, xsi * (eta1 - eta12), w);
        append_duffy(r, xsi, xsi * (eta1 - eta12), xsi * (one - eta123), xsi * (eta1 - eta123), w);
      } else if (kind == 2) {
        T w = base * xsi * xsi * xsi * eta1 * eta1;
        append_duffy(r, xsi, xsi * eta1 * eta3, xsi * (one - eta12), xsi * eta1 * (one - eta2), w);
        append_duffy(r, xsi, xsi * eta1, xsi * (one - eta123), xsi * eta1 * eta2 * (one - eta3), w * eta2);
        append_duffy(r, xsi * (one - eta12), xsi * eta1 * (one - eta2), xsi, xsi * eta123, w * eta2);
        append_duffy(r, xsi * (one - eta123), xsi * eta12 * (one - eta3), xsi, xsi * eta1, w * eta2);
        append_duffy(r, xsi * (one - eta123), xsi * eta1 * (one - eta2 * eta3), xsi, xsi * eta12, w * eta2);
      } else {
        T w = base * xsi * xsi * xsi * eta2;
        append_duffy(r, xsi, xsi * eta1, xsi * eta2, xsi * eta2 * eta3, w);
        append_duffy(r, xsi * eta2, xsi * eta2 * eta3, xsi, xsi * eta1, w);
      }
    }
  return r;
}

// BeatEngineCore.jl:633-655 (vertex ids are 1-based as in the reference)
template <typename T> inline V2<T> remap_vertex(const V2<T>& p, int id) {
  if (id == 2) return {T(1.0) - p[0] - p[1], p[1]};
  if (id == 3) return {p[0], T(1.0) - p[0] - p[1]};
  return p;
}
template <typename T> inline V2<T> remap_edge(const V2<T>& p, int a, int b) {
  const V2<T> ref[3] = {{T(0), T(0)}, {T(1), T(0)}, {T(0), T(1)}};
  int rem = 6 - a - b;
  V2<T> v0 = ref[a - 1], v1 = ref[b - 1], v2 = ref[rem - 1];
  return {v0[0] + p[0] * (v1[0] - v0[0]) + p[1] * (v2[0] - v0[0]), v0[1] + p[0] * (v1[1] - v0[1]) + p[1] * (v2[1] - v0[1])};
}

struct AdjInfo {
  int kind;  // 0 regular, 1 coincident, 2 edge, 3 vertex
  int ta, tb, ra, rb;  // 1-based local vertex ids (0 when unused)
};

// BeatEngineCore.jl:453-479
inline AdjInfo adjacency_info(const int* fa, const int* fb) {
  int sa[9], sb[9], n = 0;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      if (fa[i] == fb[j]) {
        sa[n] = i + 1;
        sb[n] = j + 1;
        ++n;
      }
  if (n == 3) return {1, 0, 0, 0, 0};
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

// ------------------------------------------------------------------ mesh ----

template <typename T> struct Elem {
  int face[3];
  V3<T> v[3];
  V3<T> normal;
  V3<T> curls[3];
  T area;
};

// surface_gradients / surface_curls, BeatEngineCore.jl:685-702
template <typename T> void surface_curls(Elem<T>& e) {
  V3<T> e1 = sub(e.v[1], e.v[0]), e2 = sub(e.v[2], e.v[0]);
  T g11 = dot(e1, e1), g12 = dot(e1, e2), g22 = dot(e2, e2);
  T det = g11 * g22 - g12 * g12;
  T i11 = g22 / det, i12 = -g12 / det, i22 = g11 / det;
  // lift = [e1 e2] * inv(gram); grads = lift * ref_grad
  const T rg[3][2] = {{T(-1), T(-1)}, {T(1), T(0)}, {T(0), T(1)}};
  for (int a = 0; a < 3; ++a) {
    T c1 = i11 * rg[a][0] + i12 * rg[a][1];
    T c2 = i12 * rg[a][0] + i22 * rg[a][1];
    V3<T> g = {e1[0] * c1 + e2[0] * c2, e1[1] * c1 + e2[1] * c2, e1[2] * c1 + e2[2] * c2};
    e.curls[a] = cross(e.normal, g);
  }
}

// BoundaryMesh constructor, BeatEngineCore.jl:236-256
template <typename T> std::vector<Elem<T>> build_elements(const double* verts, const int* faces, int nf) {
  std::vector<Elem<T>> el(nf);
  for (int f = 0; f < nf; ++f) {
    Elem<T>& e = el[f];
    for (int a = 0; a < 3; ++a) {
      e.face[a] = faces[3 * f + a];
      for (int d = 0; d < 3; ++d) e.v[a][d] = T(verts[3 * e.face[a] + d]);
    }
    V3<T> cp = cross(sub(e.v[1], e.v[0]), sub(e.v[2], e.v[0]));
    T nn = norm(cp);
    e.area = nn / T(2.0);
    e.normal = {cp[0] / nn, cp[1] / nn, cp[2] / nn};
    surface_curls(e);
  }
  return el;
}

// ------------------------------------------------------------- symmetry ----
// BeatEngineCore.jl:323-439: transforms (x: S = diag(-1, 1, 1); y: diag(1, -1, 1);
// xy: diag(-1, -1, 1)), reflected points / normals S p, curls det(S) S c, the
// plane tolerance max(1e-9, 1e-6 x bounding-box diagonal), snapping of
// near-plane vertices onto the planes, and the P1 orbit weights (2 per plane).
struct SymTransform {
  int sx, sy, det;
};
inline std::vector<SymTransform> image_transforms(int mode) {
  if (mode == 1) return {{-1, 1, -1}};
  if (mode == 2) return {{-1, 1, -1}, {1, -1, -1}, {-1, -1, 1}};
  return {};
}
inline double symmetry_tolerance(const double* verts, int nv) {
  if (nv <= 0) return 1e-9;
  double lo[3] = {verts[0], verts[1], verts[2]}, hi[3] = {verts[0], verts[1], verts[2]};
  for (int v = 1; v < nv; ++v)
    for (int d = 0; d < 3; ++d) {
      lo[d] = std::min(lo[d], verts[3 * v + d]);
      hi[d] = std::max(hi[d], verts[3 * v + d]);
    }
  const double diag = std::sqrt((hi[0] - lo[0]) * (hi[0] - lo[0]) + (hi[1] - lo[1]) * (hi[1] - lo[1]) +
                                (hi[2] - lo[2]) * (hi[2] - lo[2]));
  return std::max(1e-9, diag * 1e-6);
}
// snapped vertex copy and P1 orbit weights (p1_symmetry_orbit_weights)
inline std::vector<double> snap_symmetry(const double* verts, int nv, int mode, std::vector<double>& weights) {
  std::vector<double> out(verts, verts + 3 * (size_t)nv);
  weights.assign(nv, 1.0);
  if (mode == 0) return out;
  const double tol = symmetry_tolerance(verts, nv);
  const int axes = mode == 1 ? 1 : 2;
  for (int v = 0; v < nv; ++v)
    for (int a = 0; a < axes; ++a)
      if (std::fabs(out[3 * v + a]) <= tol) {
        out[3 * v + a] = 0.0;
        weights[v] *= 2.0;
      }
  return out;
}
template <typename T> inline V3<T> reflect_point(const SymTransform& t, const V3<T>& p) {
  return {T(t.sx) * p[0], T(t.sy) * p[1], p[2]};
}
template <typename T> Elem<T> reflect_element(const Elem<T>& e, const SymTransform& t) {
  Elem<T> r = e;
  for (int a = 0; a < 3; ++a) {
    r.v[a] = reflect_point(t, e.v[a]);
    r.curls[a] = {T(t.det * t.sx) * e.curls[a][0], T(t.det * t.sy) * e.curls[a][1], T(t.det) * e.curls[a][2]};
  }
  r.normal = reflect_point(t, e.normal);
  return r;
}
// geometric_adjacency_info, BeatEngineCore.jl:481-505 (1-based local vertex ids)
template <typename T> AdjInfo geometric_adjacency(const V3<T>* a, const V3<T>* b, T tol) {
  int sa[9], sb[9], n = 0;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      if (norm(sub(a[i], b[j])) <= tol) {
        sa[n] = i + 1;
        sb[n] = j + 1;
        ++n;
      }
  if (n >= 3) return {1, sa[0], sa[1], sb[0], sb[1]};
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

template <typename T> inline V3<T> local_to_global(const V3<T>* v, const V2<T>& p) {
  T a = T(1) - p[0] - p[1];
  return {a * v[0][0] + p[0] * v[1][0] + p[1] * v[2][0], a * v[0][1] + p[0] * v[1][1] + p[1] * v[2][1],
          a * v[0][2] + p[0] * v[1][2] + p[1] * v[2][2]};
}
template <typename T> inline V3<T> p1_values(const V2<T>& p) { return {T(1) - p[0] - p[1], p[0], p[1]}; }

inline bool elements_adjacent(const int* a, const int* b) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      if (a[i] == b[j]) return true;
  return false;
}

// Greedy element coloring, BeatEngineCpuAssembly.jl:102-130
std::vector<std::vector<int>> color_groups(const int* faces, int nf, int nv) {
  std::vector<std::set<int>> vcol(nv);
  std::vector<std::vector<int>> groups;
  for (int f = 0; f < nf; ++f) {
    std::set<int> used;
    for (int a = 0; a < 3; ++a) used.insert(vcol[faces[3 * f + a]].begin(), vcol[faces[3 * f + a]].end());
    int c = 1;
    while (used.count(c)) ++c;
    while ((int)groups.size() < c) groups.emplace_back();
    groups[c - 1].push_back(f);
    for (int a = 0; a < 3; ++a) vcol[faces[3 * f + a]].insert(c);
  }
  return groups;
}

// Singular pair list with rules remapped per orientation, BeatEngineCore.jl:784-915
template <typename T> struct SingularCache {
  struct Pair {
    int test, trial, rule;
    T jac, nprod;
  };
  std::vector<std::vector<Pair>> by_test;
  std::vector<DuffyRule<T>> rules;
  int count = 0;
};

template <typename T>
SingularCache<T> build_singular_cache(const std::vector<Elem<T>>& el, const int* faces, int nf, int nv, int order) {
  SingularCache<T> sc;
  sc.by_test.resize(nf);
  std::vector<std::vector<int>> v2e(nv);
  for (int f = 0; f < nf; ++f)
    for (int a = 0; a < 3; ++a) v2e[faces[3 * f + a]].push_back(f);
  DuffyRule<T> base[4] = {DuffyRule<T>(), duffy_rule<T>(order, 1), duffy_rule<T>(order, 2), duffy_rule<T>(order, 3)};
  std::map<std::tuple<int, int, int, int, int>, int> rule_index;
  for (int t = 0; t < nf; ++t) {
    std::vector<int> cand;
    std::set<int> seen;
    for (int a = 0; a < 3; ++a)
      for (int r : v2e[faces[3 * t + a]])
        if (!seen.count(r)) {
          seen.insert(r);
          cand.push_back(r);
        }
    for (int r : cand) {
      AdjInfo info = adjacency_info(faces + 3 * t, faces + 3 * r);
      if (info.kind == 0) continue;
      std::tuple<int, int, int, int, int> key =
          info.kind == 1 ? std::make_tuple(1, 0, 0, 0, 0)
          : info.kind == 2 ? std::make_tuple(2, info.ta, info.tb, info.ra, info.rb)
                           : std::make_tuple(3, info.ta, 0, info.ra, 0);
      auto it = rule_index.find(key);
      int ri;
      if (it == rule_index.end()) {
        const DuffyRule<T>& b = base[info.kind];
        DuffyRule<T> rr;
        rr.w = b.w;
        for (size_t q = 0; q < b.w.size(); ++q) {
          if (info.kind == 1) {
            rr.test.push_back(b.test[q]);
            rr.trial.push_back(b.trial[q]);
          } else if (info.kind == 2) {
            rr.test.push_back(remap_edge(b.test[q], info.ta, info.tb));
            rr.trial.push_back(remap_edge(b.trial[q], info.ra, info.rb));
          } else {
            rr.test.push_back(remap_vertex(b.test[q], info.ta));
            rr.trial.push_back(remap_vertex(b.trial[q], info.ra));
          }
        }
        sc.rules.push_back(rr);
        ri = (int)sc.rules.size() - 1;
        rule_index[key] = ri;
      } else {
        ri = it->second;
      }
      T jac = (T(2.0) * el[t].area) * (T(2.0) * el[r].area);
      T np = dot(el[t].normal, el[r].normal);
      sc.by_test[t].push_back({t, r, ri, jac, np});
      sc.count++;
    }
  }
  return sc;
}

// Operators are returned row-major: S, Kp are (nv x nf), D, H are (nv x nv).
template <typename T> struct Ops {
  C<T>* S;
  C<T>* D;
  C<T>* Kp;
  C<T>* H;
  int nv, nf;
  C<T>& s(int r, int c) { return S[(size_t)r * nf + c]; }
  C<T>& kp(int r, int c) { return Kp[(size_t)r * nf + c]; }
  C<T>& d(int r, int c) { return D[(size_t)r * nv + c]; }
  C<T>& h(int r, int c) { return H[(size_t)r * nv + c]; }
};

// _beat_cpu_green, BeatEngineCpuAssembly.jl:1-6
template <typename T> inline C<T> green(T radius, T inv_radius, T k) {
  T phase = k * radius;
  T scale = (T(1) / (T(4.0) * T(M_PI))) * inv_radius;
  return C<T>(std::cos(phase) * scale, std::sin(phase) * scale);
}

}  // namespace

// ----------------------------------------------------------- C interface ----
namespace {

template <typename T> struct Assembler {
  // Accumulates pair integrals into row-major S, Kp (nv x nf), D, H (nv x nv).
  C<T>*S, *D, *Kp, *H;
  int nv, nf;
  T k, k2;
  const TriRule<T>* rule;
  std::vector<V3<T>> basis;

  // _beat_cpu_accumulate_regular_pair_signed!, BeatEngineCpuAssembly.jl:278-373
  // (sign -1 subtracts, for the image singular delta)
  void regular_pair(const Elem<T>& te, const Elem<T>& re, const std::vector<V3<T>>& tq_pts,
                    const std::vector<V3<T>>& rq_pts, T sign) {
    const int Q = (int)rule->w.size();
    C<T> sb[3] = {}, ab[3] = {}, db[3][3] = {}, hb[3][3] = {};
    T cp[3][3];
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) cp[a][b] = dot(te.curls[a], re.curls[b]);
    const T nprod = dot(te.normal, re.normal);
    const T jac = T(4.0) * te.area * re.area;
    for (int tq = 0; tq < Q; ++tq) {
      const V3<T>& x = tq_pts[tq];
      const T tw = rule->w[tq];
      for (int rq = 0; rq < Q; ++rq) {
        V3<T> rv = sub(rq_pts[rq], x);
        T radius = norm(rv);
        if (radius == T(0)) continue;
        T inv_r = T(1) / radius;
        C<T> g = green(radius, inv_r, k);
        C<T> gs = g * C<T>(-inv_r, k);
        T trial_dot = dot(rv, re.normal) * inv_r;
        T test_dot = -dot(rv, te.normal) * inv_r;
        C<T> dv = gs * trial_dot, av = gs * test_dot;
        T weight = tw * rule->w[rq] * jac;
        C<T> wg = g * weight, wd = dv * weight, wa = av * weight;
        for (int a = 0; a < 3; ++a) {
          T tv = basis[tq][a];
          sb[a] += tv * wg;
          ab[a] += tv * wa;
          for (int b = 0; b < 3; ++b) {
            T bp = tv * basis[rq][b];
            db[a][b] += bp * wd;
            hb[a][b] += (cp[a][b] - k2 * bp * nprod) * wg;
          }
        }
      }
    }
    for (int a = 0; a < 3; ++a) {
      const size_t row = te.face[a];
      S[row * nf + re_dp0] += sign * sb[a];
      Kp[row * nf + re_dp0] += sign * ab[a];
      for (int b = 0; b < 3; ++b) {
        const size_t col = re.face[b];
        D[row * nv + col] += sign * db[a][b];
        H[row * nv + col] += sign * hb[a][b];
      }
    }
  }
  int re_dp0 = 0;  // DP0 dof (face index) of the trial element of the current pair

  // _beat_cpu_accumulate_pair!, BeatEngineCpuAssembly.jl:151-218
  void singular_pair(const Elem<T>& te, const Elem<T>& re, const DuffyRule<T>& du, T jac, T nprod) {
    T cp[3][3];
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) cp[a][b] = dot(te.curls[a], re.curls[b]);
    for (size_t q = 0; q < du.w.size(); ++q) {
      V3<T> tb = p1_values(du.test[q]), rb = p1_values(du.trial[q]);
      V3<T> x = local_to_global(te.v, du.test[q]);
      V3<T> y = local_to_global(re.v, du.trial[q]);
      V3<T> rv = sub(y, x);
      T radius = norm(rv);
      if (radius == T(0)) continue;
      T inv_r = T(1) / radius;
      C<T> g = green(radius, inv_r, k);
      C<T> gs = g * C<T>(-inv_r, k);
      T trial_dot = dot(rv, re.normal) * inv_r;
      T test_dot = -dot(rv, te.normal) * inv_r;
      C<T> dv = gs * trial_dot, av = gs * test_dot;
      T weight = du.w[q] * jac;
      for (int a = 0; a < 3; ++a) {
        const size_t row = te.face[a];
        T tv = tb[a];
        S[row * nf + re_dp0] += tv * g * weight;
        Kp[row * nf + re_dp0] += tv * av * weight;
        for (int b = 0; b < 3; ++b) {
          const size_t col = re.face[b];
          T bp = tv * rb[b];
          D[row * nv + col] += bp * dv * weight;
          H[row * nv + col] += (cp[a][b] - k2 * bp * nprod) * g * weight;
        }
      }
    }
  }
};

// A Duffy rule remapped to an adjacency orientation (BeatEngineCore.jl:633-655, 856-873)
template <typename T> DuffyRule<T> remapped_rule(const DuffyRule<T>& b, const AdjInfo& info) {
  DuffyRule<T> rr;
  rr.w = b.w;
  for (size_t q = 0; q < b.w.size(); ++q) {
    if (info.kind == 1) {
      rr.test.push_back(b.test[q]);
      rr.trial.push_back(b.trial[q]);
    } else if (info.kind == 2) {
      rr.test.push_back(remap_edge(b.test[q], info.ta, info.tb));
      rr.trial.push_back(remap_edge(b.trial[q], info.ra, info.rb));
    } else {
      rr.test.push_back(remap_vertex(b.test[q], info.ta));
      rr.trial.push_back(remap_vertex(b.trial[q], info.ra));
    }
  }
  return rr;
}

// assemble_regular_galerkin_operators_cpu, BeatEngineCpuAssembly.jl:636-870:
// regular pairs, their symmetry images (all pairs, :675-735), singular pairs,
// the image singular delta (Duffy minus regular for image pairs that touch,
// :805-857), then the P1 orbit row weights (:627-634, :861).
template <typename T>
int assemble_impl(const double* verts_in, int nv, const int* faces, int nf, double kd, int reg_order, int sing_order,
                  int symmetry, C<T>* S, C<T>* D, C<T>* Kp, C<T>* H, int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
  std::vector<double> weights;
  const std::vector<double> verts = snap_symmetry(verts_in, nv, symmetry, weights);
  std::vector<Elem<T>> el = build_elements<T>(verts.data(), faces, nf);
  TriRule<T> rule = triangle_rule<T>(reg_order);
  const int Q = (int)rule.w.size();
  std::vector<std::vector<V3<T>>> qpts(nf, std::vector<V3<T>>(Q));
  for (int f = 0; f < nf; ++f)
    for (int q = 0; q < Q; ++q) qpts[f][q] = local_to_global(el[f].v, rule.pts[q]);
  std::memset((void*)S, 0, sizeof(C<T>) * (size_t)nv * nf);
  std::memset((void*)Kp, 0, sizeof(C<T>) * (size_t)nv * nf);
  std::memset((void*)D, 0, sizeof(C<T>) * (size_t)nv * nv);
  std::memset((void*)H, 0, sizeof(C<T>) * (size_t)nv * nv);
  std::vector<std::vector<int>> groups = color_groups(faces, nf, nv);
  Assembler<T> base;
  base.S = S;
  base.D = D;
  base.Kp = Kp;
  base.H = H;
  base.nv = nv;
  base.nf = nf;
  base.k = T(kd);
  base.k2 = base.k * base.k;
  base.rule = &rule;
  for (int q = 0; q < Q; ++q) base.basis.push_back(p1_values(rule.pts[q]));
  const std::vector<SymTransform> images = image_transforms(symmetry);

  // Regular pairs, BeatEngineCpuAssembly.jl:375-409, 682-713; images :411-445, 715-735
  for (int ti = -1; ti < (int)images.size(); ++ti) {
    std::vector<Elem<T>> trial_el = el;
    std::vector<std::vector<V3<T>>> trial_q = qpts;
    if (ti >= 0)
      for (int f = 0; f < nf; ++f) {
        trial_el[f] = reflect_element(el[f], images[ti]);
        for (int q = 0; q < Q; ++q) trial_q[f][q] = reflect_point(images[ti], qpts[f][q]);
      }
    for (const auto& group : groups) {
#pragma omp parallel for schedule(dynamic, 1)
      for (long gi = 0; gi < (long)group.size(); ++gi) {
        Assembler<T> as = base;
        const int t = group[gi];
        for (int r = 0; r < nf; ++r) {
          if (ti < 0 && elements_adjacent(el[t].face, el[r].face)) continue;
          as.re_dp0 = r;
          as.regular_pair(el[t], trial_el[r], qpts[t], trial_q[r], T(1));
        }
      }
    }
  }

  if (sing_order > 0) {
    // Singular pairs, BeatEngineCpuAssembly.jl:151-218, 447-486, 764-797
    SingularCache<T> sc = build_singular_cache<T>(el, faces, nf, nv, sing_order);
    for (const auto& group : groups) {
#pragma omp parallel for schedule(dynamic, 1)
      for (long gi = 0; gi < (long)group.size(); ++gi) {
        Assembler<T> as = base;
        const int t = group[gi];
        for (const auto& pr : sc.by_test[t]) {
          as.re_dp0 = pr.trial;
          as.singular_pair(el[pr.test], el[pr.trial], sc.rules[pr.rule], pr.jac, pr.nprod);
        }
      }
    }
    // Image singular delta: image_singular_candidates / _beat_cpu_image_singular_cache
    // (BeatEngineCore.jl:917-943, BeatEngineCpuAssembly.jl:488-527, 565-625)
    DuffyRule<T> dbase[4] = {DuffyRule<T>(), duffy_rule<T>(sing_order, 1), duffy_rule<T>(sing_order, 2),
                             duffy_rule<T>(sing_order, 3)};
    const T tol = T(1e-8);
    for (const SymTransform& tr : images) {
      std::vector<Elem<T>> img(nf);
      std::vector<std::vector<V3<T>>> img_q(nf, std::vector<V3<T>>(Q));
      for (int f = 0; f < nf; ++f) {
        img[f] = reflect_element(el[f], tr);
        for (int q = 0; q < Q; ++q) img_q[f][q] = reflect_point(tr, qpts[f][q]);
      }
      std::vector<std::vector<std::pair<int, AdjInfo>>> by_test(nf);
      for (int t = 0; t < nf; ++t)
        for (int r = 0; r < nf; ++r) {
          AdjInfo info = geometric_adjacency(el[t].v, img[r].v, tol);
          if (info.kind != 0) by_test[t].push_back({r, info});
        }
      for (const auto& group : groups) {
#pragma omp parallel for schedule(dynamic, 1)
        for (long gi = 0; gi < (long)group.size(); ++gi) {
          Assembler<T> as = base;
          const int t = group[gi];
          for (const auto& pr : by_test[t]) {
            const int r = pr.first;
            const DuffyRule<T> du = remapped_rule(dbase[pr.second.kind], pr.second);
            const T jac = (T(2.0) * el[t].area) * (T(2.0) * el[r].area);
            as.re_dp0 = r;
            as.singular_pair(el[t], img[r], du, jac, dot(el[t].normal, img[r].normal));
            as.regular_pair(el[t], img[r], qpts[t], img_q[r], T(-1));
          }
        }
      }
    }
  }
  if (symmetry != 0)
    for (int v = 0; v < nv; ++v) {
      const T w = T(weights[v]);
      for (int c = 0; c < nf; ++c) {
        S[(size_t)v * nf + c] *= w;
        Kp[(size_t)v * nf + c] *= w;
      }
      for (int c = 0; c < nv; ++c) {
        D[(size_t)v * nv + c] *= w;
        H[(size_t)v * nv + c] *= w;
      }
    }
  return 0;
}

// l2_identity_element_matrix + assemble_l2_identity_matrix, BeatEngineCore.jl:731-749, 952-979
// (rows weighted by the P1 orbit weights under symmetry, BeatEngineCore.jl:974-977)
template <typename T>
int mass_impl(const double* verts_in, int nv, const int* faces, int nf, int reg_order, int symmetry, T* M11, T* M10) {
  std::vector<double> weights;
  const std::vector<double> verts = snap_symmetry(verts_in, nv, symmetry, weights);
  std::vector<Elem<T>> el = build_elements<T>(verts.data(), faces, nf);
  TriRule<T> rule = triangle_rule<T>(reg_order);
  std::memset(M11, 0, sizeof(T) * (size_t)nv * nv);
  std::memset(M10, 0, sizeof(T) * (size_t)nv * nf);
  for (int f = 0; f < nf; ++f) {
    T blk11[3][3] = {}, blk10[3] = {};
    T js = T(2.0) * el[f].area;
    for (size_t q = 0; q < rule.w.size(); ++q) {
      V3<T> phi = p1_values(rule.pts[q]);
      for (int i = 0; i < 3; ++i) {
        for (int j = 0; j < 3; ++j) blk11[i][j] += phi[i] * phi[j] * rule.w[q] * js;
        blk10[i] += phi[i] * T(1.0) * rule.w[q] * js;
      }
    }
    for (int i = 0; i < 3; ++i) {
      size_t row = el[f].face[i];
      for (int j = 0; j < 3; ++j) M11[row * nv + el[f].face[j]] += blk11[i][j];
      M10[row * nf + f] += blk10[i];
    }
  }
  if (symmetry != 0)
    for (int v = 0; v < nv; ++v) {
      for (int c = 0; c < nv; ++c) M11[(size_t)v * nv + c] *= T(weights[v]);
      for (int c = 0; c < nf; ++c) M10[(size_t)v * nf + c] *= T(weights[v]);
    }
  return 0;
}

// evaluate_galerkin_field_cpu, BeatEngineCpuField.jl:1-45 (sources built as in
// build_field_evaluation_cache, BeatEngineCore.jl:1240-1280, including the
// symmetry images of every face)
template <typename T>
int field_impl(const double* verts_in, int nv, const int* faces, int nf, int reg_order, int symmetry, double kd,
               const C<T>* pressure, const C<T>* qn, const double* pts, int npts, C<T>* out, int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
  const T k = T(kd);
  std::vector<double> weights;
  const std::vector<double> verts = snap_symmetry(verts_in, nv, symmetry, weights);
  std::vector<Elem<T>> el = build_elements<T>(verts.data(), faces, nf);
  TriRule<T> rule = triangle_rule<T>(reg_order);
  const int Q = (int)rule.w.size();
  std::vector<SymTransform> trs = {{1, 1, 1}};
  for (const SymTransform& t : image_transforms(symmetry)) trs.push_back(t);
  const size_t ns = (size_t)nf * Q * trs.size();
  std::vector<V3<T>> sp(ns), sn(ns), bv(ns);
  std::vector<T> sw(ns);
  std::vector<int> se(ns);
  size_t s = 0;
  for (int f = 0; f < nf; ++f) {
    T js = T(2.0) * el[f].area;
    for (const SymTransform& tr : trs)
      for (int q = 0; q < Q; ++q, ++s) {
        sp[s] = reflect_point(tr, local_to_global(el[f].v, rule.pts[q]));
        sn[s] = reflect_point(tr, el[f].normal);
        sw[s] = rule.w[q] * js;
        se[s] = f;
        bv[s] = p1_values(rule.pts[q]);
      }
  }
#pragma omp parallel for schedule(static)
  for (long p = 0; p < npts; ++p) {
    V3<T> x = {T(pts[3 * p]), T(pts[3 * p + 1]), T(pts[3 * p + 2])};
    C<T> pot(0);
    for (size_t i = 0; i < ns; ++i) {
      V3<T> rv = sub(sp[i], x);
      T radius = norm(rv);
      if (radius == T(0)) continue;
      T phase = k * radius;
      T gsc = T(1) / (T(4.0) * T(M_PI) * radius);
      C<T> g(std::cos(phase) * gsc, std::sin(phase) * gsc);
      T nproj = dot(rv, sn[i]) / radius;
      C<T> dl = g * (C<T>(0, k) - T(1) / radius) * nproj;
      const int* fc = el[se[i]].face;
      C<T> ps = (bv[i][0] * pressure[fc[0]] + bv[i][1] * pressure[fc[1]] + bv[i][2] * pressure[fc[2]]) * sw[i];
      C<T> qs = qn[se[i]] * sw[i];
      pot += dl * ps - g * qs;
    }
    out[p] = pot;
  }
  return 0;
}

}  // namespace

extern "C" {

// Operators, row-major complex interleaved: S, Kp (nv x nf); D, H (nv x nv).
int oracle_assemble_f64(const double* verts, int nv, const int* faces, int nf, double k, int reg_order, int sing_order,
                        int symmetry, double* S, double* D, double* Kp, double* H, int nthreads) {
  return assemble_impl<double>(verts, nv, faces, nf, k, reg_order, sing_order, symmetry, reinterpret_cast<C<double>*>(S),
                               reinterpret_cast<C<double>*>(D), reinterpret_cast<C<double>*>(Kp),
                               reinterpret_cast<C<double>*>(H), nthreads);
}
int oracle_assemble_f32(const double* verts, int nv, const int* faces, int nf, double k, int reg_order, int sing_order,
                        int symmetry, float* S, float* D, float* Kp, float* H, int nthreads) {
  return assemble_impl<float>(verts, nv, faces, nf, k, reg_order, sing_order, symmetry, reinterpret_cast<C<float>*>(S),
                              reinterpret_cast<C<float>*>(D), reinterpret_cast<C<float>*>(Kp),
                              reinterpret_cast<C<float>*>(H), nthreads);
}
int oracle_mass_f64(const double* verts, int nv, const int* faces, int nf, int reg_order, int symmetry, double* M11,
                    double* M10) {
  return mass_impl<double>(verts, nv, faces, nf, reg_order, symmetry, M11, M10);
}
int oracle_mass_f32(const double* verts, int nv, const int* faces, int nf, int reg_order, int symmetry, float* M11,
                    float* M10) {
  return mass_impl<float>(verts, nv, faces, nf, reg_order, symmetry, M11, M10);
}
int oracle_field_f64(const double* verts, int nv, const int* faces, int nf, int reg_order, int symmetry, double k,
                     const double* pressure, const double* qn, const double* pts, int npts, double* out, int nthreads) {
  return field_impl<double>(verts, nv, faces, nf, reg_order, symmetry, k, reinterpret_cast<const C<double>*>(pressure),
                            reinterpret_cast<const C<double>*>(qn), pts, npts, reinterpret_cast<C<double>*>(out), nthreads);
}
int oracle_field_f32(const double* verts, int nv, const int* faces, int nf, int reg_order, int symmetry, double k,
                     const float* pressure, const float* qn, const double* pts, int npts, float* out, int nthreads) {
  return field_impl<float>(verts, nv, faces, nf, reg_order, symmetry, k, reinterpret_cast<const C<float>*>(pressure),
                           reinterpret_cast<const C<float>*>(qn), pts, npts, reinterpret_cast<C<float>*>(out), nthreads);
}

// Rule export for tests: writes up to cap points; returns the point count.
int oracle_triangle_rule(int order, double* pts, double* w, int cap) {
  TriRule<double> r = triangle_rule<double>(order);
  int n = (int)r.w.size();
  for (int i = 0; i < n && i < cap; ++i) {
    pts[2 * i] = r.pts[i][0];
    pts[2 * i + 1] = r.pts[i][1];
    w[i] = r.w[i];
  }
  return n;
}
int oracle_duffy_rule(int order, int kind, double* test, double* trial, double* w, int cap) {
  DuffyRule<double> r = duffy_rule<double>(order, kind);
  int n = (int)r.w.size();
  for (int i = 0; i < n && i < cap; ++i) {
    test[2 * i] = r.test[i][0];
    test[2 * i + 1] = r.test[i][1];
    trial[2 * i] = r.trial[i][0];
    trial[2 * i + 1] = r.trial[i][1];
    w[i] = r.w[i];
  }
  return n;
}
// Number of vertex-sharing (singular) pairs, for tests.
int oracle_singular_pair_count(const double* verts, int nv, const int* faces, int nf, int order) {
  std::vector<Elem<double>> el = build_elements<double>(verts, faces, nf);
  return build_singular_cache<double>(el, faces, nf, nv, order).count;
}
int oracle_color_count(const int* faces, int nf, int nv) { return (int)color_groups(faces, nf, nv).size(); }

}  // extern "C"
