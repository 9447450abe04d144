// Test driver: runs the mesh planner of the library on a mesh read from a
// binary file (int32 nv, nf; float64 vertices[nv][3]; int32 faces[nf][3]) and
// prints the tile and lane-group layout as text for the Python checks.
// Arguments: mesh file, faces per tile, optional symmetry (0 none, 1 x, 2 xy).
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "bem_internal.h"

int main(int argc, char** argv) {
  if (argc < 3) return 2;
  FILE* f = std::fopen(argv[1], "rb");
  if (!f) return 2;
  int nv = 0, nf = 0;
  bool ok = std::fread(&nv, 4, 1, f) == 1 && std::fread(&nf, 4, 1, f) == 1;
  std::vector<double> v(3 * (size_t)nv);
  std::vector<int> fc(3 * (size_t)nf);
  ok = ok && std::fread(v.data(), 8, v.size(), f) == v.size() && std::fread(fc.data(), 4, fc.size(), f) == fc.size();
  std::fclose(f);
  if (!ok) return 2;
  bem::MeshPlan p;
  const int symmetry = argc > 3 ? std::atoi(argv[3]) : 0;  // 0 none, 1 x, 2 xy
  const std::string err = bem::build_mesh_plan(v.data(), nv, fc.data(), nf, 4, 4, std::atoi(argv[2]), p, symmetry);
  if (!err.empty()) {
    std::printf("error %s\n", err.c_str());
    return 1;
  }
  std::printf("tiles %d\n", p.n_tiles);
  for (int t = 0; t < p.n_tiles; ++t) {
    std::printf("tile %d rows %d groups %d\n", t, p.tile_row_base[t + 1] - p.tile_row_base[t],
                p.tile_group_ptr[t + 1] - p.tile_group_ptr[t]);
    for (int g = p.tile_group_ptr[t]; g < p.tile_group_ptr[t + 1]; ++g)
      for (int l = 0; l < bem::kLanes; ++l) {
        const bem::LaneSlot& s = p.lane_slots[(size_t)g * bem::kLanes + l];
        if (s.face >= 0) std::printf("slot %d %d %d %d %d\n", g, s.face, s.loc[0], s.loc[1], s.loc[2]);
      }
  }
  // singular pairs (trial, test), the faces' extended rows and the scatter plan
  std::printf("npairs %zu next %d\n", p.pairs.size(), p.n_ext);
  std::printf("radius %.17g points %lld\n", p.pair_radius, p.singular_points);
  for (size_t k = 0; k < p.pairs.size(); ++k)
    std::printf("pair %d %d %d %d\n", p.pairs[k].trial, p.pairs[k].test, p.pairs[k].tr,
                p.rule_ptr[p.pairs[k].rule + 1] - p.rule_ptr[p.pairs[k].rule]);
  for (int f = 0; f < nf; ++f) std::printf("fext %d %d %d\n", p.face_ext[3 * f], p.face_ext[3 * f + 1], p.face_ext[3 * f + 2]);
  for (size_t i = 0; i < p.scat_col.size(); ++i) {
    std::printf("scat %d %d", p.scat_col[i], p.scat_row[i]);
    for (int s = p.scat_ptr[i]; s < p.scat_ptr[i + 1]; ++s) std::printf(" %d", p.scat_src[s]);
    std::printf("\n");
  }
  return 0;
}
