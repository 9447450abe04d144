// Internal (non-ABI) structures shared by the host mesh planner and the
// kernel launchers of the GB300 BEM library.
#pragma once

#include <cstdint>
#include <memory>
#include <string>
#include <utility>
#include <vector>

namespace bem {

// std::allocator whose value-initialisation of a trivial element does nothing, so
// a vector resized before being filled in parallel is not first zero-filled (and
// its pages are first touched by the threads that fill them).
template <typename T> struct UninitAlloc : std::allocator<T> {
  template <typename U> struct rebind {
    using other = UninitAlloc<U>;
  };
  UninitAlloc() = default;
  template <typename U> UninitAlloc(const UninitAlloc<U>&) noexcept {}
  template <typename U> void construct(U*) noexcept {}
  template <typename U, typename... A> void construct(U* p, A&&... a) { ::new ((void*)p) U(std::forward<A>(a)...); }
};
template <typename T> using FillVec = std::vector<T, UninitAlloc<T>>;

// Regular (6-point) rule and Duffy rules use the reference's orders; the
// planner supports regular orders 1 (1 point), 2/3 (3 points) and 4 (6 points)
// and singular (Duffy) orders 1..4.
constexpr int kMaxQ = 6;
constexpr int kLanes = 32;

// Compensated-FP32 face record, 40 words (160 B, 16-byte aligned).
//   anchor_hi/anchor_lo : face centroid as an unevaluated float sum (double-float)
//   off                 : quadrature points minus the centroid (float, |off| ~ h)
//   normal, area2 (=2A), curls[3], verts[3] (global vertex ids for adjacency)
struct alignas(16) FaceF32 {
  float anchor_hi[3];
  float anchor_lo[3];
  float normal[3];
  float area2;
  float curls[9];
  float off[kMaxQ * 3];
  int verts[3];
};
static_assert(sizeof(FaceF32) == 160, "FaceF32 layout");
// FaceF32 as 40 four-byte words (the field-major copy of the lane groups)
constexpr int kFaceWords = 40;
constexpr int kFwAnchorHi = 0, kFwAnchorLo = 3, kFwNormal = 6, kFwArea2 = 9, kFwCurls = 10, kFwOff = 19, kFwVerts = 37;

// FP64 face record (288 B).
struct alignas(16) FaceF64 {
  double anchor[3];
  double normal[3];
  double area2;
  double curls[9];
  double off[kMaxQ * 3];
  int verts[3];
  int pad;
};
static_assert(sizeof(FaceF64) % 16 == 0, "FaceF64 layout");

// One lane slot of a tile group: test face id and the tile-local rows of its
// three vertices (-1 face id = empty slot).
struct alignas(16) LaneSlot {
  int face;
  int loc[3];
};

// Singular (vertex-sharing) pair.
struct SingularPair {
  int test, trial, rule, kind;  // kind 1 coincident, 2 edge, 3 vertex
  int tr;                       // symmetry transform of the trial face (0 identity, 1 x, 2 y, 3 xy)
  int pad;
  double jac;                   // (2 A_test)(2 A_trial)
  double nprod;                 // n_test . (S n_trial)
};

// Symmetry transform tr (bit 0: x -> -x, bit 1: y -> -y): S = diag(sx, sy, 1),
// reflected points and normals are S p, reflected surface curls det(S) S c
// (BeatEngineCore.jl:323-355).  A vertex is fixed by tr when it lies on every
// plane tr reflects across: (fix_mask & tr) == tr.
inline int tr_sx(int tr) { return (tr & 1) ? -1 : 1; }
inline int tr_sy(int tr) { return (tr & 2) ? -1 : 1; }

struct MeshPlan {
  int nv = 0, nf = 0, Q = 0, regular_order = 4, singular_order = 4;
  // symmetry: 0 off, 1 x (half model, x >= 0), 2 xy (quarter model, x, y >= 0)
  int symmetry = 0;
  std::vector<int> transforms;          // {0} | {0, 1} | {0, 1, 2, 3}
  std::vector<unsigned char> fix_mask;  // per vertex: bit 0 on x = 0, bit 1 on y = 0
  std::vector<double> row_weight;       // per matrix row: symmetry orbit weight of its vertex (1, 2, 4)
  int image_pairs = 0;                  // singular pairs of a test face with a reflected trial face
  // regular rule on the reference triangle
  std::vector<double> rule_pts;  // Q x 2
  std::vector<double> rule_w;    // Q
  // per-face records
  std::vector<FaceF32> faces32;
  std::vector<FaceF64> faces64;
  std::vector<int> faces;  // nf x 3 (input vertex ids)
  std::vector<double> verts;  // nv x 3
  std::vector<double> area;   // nf
  std::vector<double> normal;  // nf x 3
  std::vector<double> curls;   // nf x 9
  // test-face tiles (the extended-row layout)
  int tile_faces = 0;                 // max faces per tile
  int n_tiles = 0;
  int max_tile_rows = 0;              // max distinct vertices in one tile
  std::vector<int> tile_group_ptr;    // n_tiles + 1, in units of groups
  std::vector<LaneSlot> lane_slots;   // n_groups x 32
  std::vector<float> group_faces32;   // n_groups x kFaceWords x 32: the test face of each lane slot, field-major
  std::vector<int> tile_row_base;     // n_tiles + 1: extended-row offset of each tile
  int n_ext = 0;                      // total extended rows
  std::vector<int> ext_row;           // n_ext: matrix row (permuted order) of each extended row
  std::vector<int> ext_is_halo;       // n_ext: 1 when the extended row is not the vertex's primary slot
  // row permutation: matrix row r holds the equation of vertex row_vertex[r]
  std::vector<int> row_vertex;        // nv
  std::vector<int> vertex_row;        // nv
  // halo gather: extended rows that are not primary, grouped by target matrix row
  std::vector<int> halo_ext;          // n_halo: extended row ids, sorted by target row
  std::vector<int> halo_row;          // n_halo_rows: target matrix rows (distinct)
  std::vector<int> halo_row_ptr;      // n_halo_rows + 1 into halo_ext
  std::vector<int> halo_slot_of_ext;  // n_ext: index into halo_ext or -1
  // column gather: for vertex j, the (trial face, local vertex) pairs g*3+b
  std::vector<int> col_ptr;           // nv + 1
  std::vector<int> col_fb;            // 3 nf
  // per-(face, local vertex) extended row of that face's tile
  std::vector<int> face_ext;          // nf x 3
  // singular pairs sorted by trial face, with CSR by trial face and by test face
  std::vector<SingularPair> pairs;
  std::vector<int> pairs_by_trial_ptr;  // nf + 1 (pairs are sorted by trial)
  std::vector<int> pairs_by_test;       // pair ids grouped by test face
  std::vector<int> pairs_by_test_ptr;   // nf + 1
  // singular scatter: the distinct extended-row entries (column 3 g + b of trial
  // face g, extended row e) that the pairs' 3 x 3 blocks add into, each with its
  // contributions (block element 12 k + 3 a + b of pair k) in pair order
  FillVec<int> scat_col, scat_row;  // per entry
  FillVec<int> scat_ptr;            // entries + 1
  FillVec<int> scat_src;            // 9 per pair
  double pair_radius = 0.0;         // largest vertex distance of a pair (its trial face reflected for image pairs)
  long long singular_points = 0;    // Duffy points over all pairs
  // Duffy rules: concatenated points; rule r occupies [rule_ptr[r], rule_ptr[r+1])
  std::vector<int> rule_ptr;
  std::vector<double> duffy;  // 5 doubles per point: test xi, test eta, trial xi, trial eta, w
  // mass element constants: m11[a][b] = sum_q w_q phi_a phi_b ; m10[a] = sum_q w_q phi_a
  double m11[9] = {0};
  double m10[3] = {0};
};

// Build the plan; returns an empty string on success, else an error message.
std::string build_mesh_plan(const double* verts, int nv, const int* faces, int nf, int regular_order,
                            int singular_order, int tile_faces, MeshPlan& plan, int symmetry = 0);

}  // namespace bem
