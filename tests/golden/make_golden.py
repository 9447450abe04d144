"""Generate the golden fixtures under tests/golden from the reference's own files.

Reads (text only, nothing executed) from a Boundary Lab checkout:
  src/blab/solvers/julia_local/src/BeatEngineCore.jl  -> literal constants of
      triangle_rule order 4 (lines 517-549)
  src/blab/solvers/julia_local/test_meshes/*.msh      -> per-file triangle and
      node counts, the first 16 triangles of sample.msh (the element subset
      the reference's CPU pipeline test uses, runtests.jl:79-146), and the
      whole of sample_half.msh (the x-symmetry CPU-vs-CUDA case,
      runtests.jl:148-206), sample_quarter.msh and sample_detailed.msh (the
      default mesh of scripts/benchmark_cuda.jl:46) as compact .npz fixtures
Usage: python tests/golden/make_golden.py [/path/to/boundary-lab]
       (default: $BOUNDARY_LAB_REFERENCE, else a "reference" directory beside
       this repository)
"""

from __future__ import annotations

import json
import os
import re
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


def triangle_rule_constants(core_jl: Path) -> dict:
    text = core_jl.read_text()
    start = text.index("function triangle_rule(")
    body = text[start: text.index("\nend", start)]
    block = body[body.index("elseif order == 4"): body.index("return TriangleRule(\n        [\n            SVector{2,T}(T(1) / T(6)")]
    nums = [float(x) for x in re.findall(r"T\((\d+\.\d+)\)", block)]
    # 6 points x 2 coordinates, then the 0.5 factor, then 6 weights
    pts = nums[:12]
    assert abs(nums[12] - 0.5) < 1e-15
    weights = nums[13:19]
    return {"points": [pts[i:i + 2] for i in range(0, 12, 2)], "weight_factor": 0.5, "weights": weights,
            "source": "src/blab/solvers/julia_local/src/BeatEngineCore.jl:520-538"}


def gmsh_counts(path: Path) -> dict:
    lines = path.read_text().splitlines()
    ns, ne = lines.index("$Nodes"), lines.index("$Elements")
    nodes = sum(1 for ln in lines[ns + 2: lines.index("$EndNodes")] if len(ln.split()) >= 4)
    tris = sum(1 for ln in lines[ne + 2: lines.index("$EndElements")]
               if len(ln.split()) >= 8 and ln.split()[1] == "2")
    return {"nodes": nodes, "triangles": tris}


def subset16(path: Path) -> dict:
    lines = path.read_text().splitlines()
    ns, ne = lines.index("$Nodes"), lines.index("$Elements")
    coords = {}
    for ln in lines[ns + 2: lines.index("$EndNodes")]:
        p = ln.split()
        if len(p) >= 4:
            coords[int(p[0])] = [float(p[1]), float(p[2]), float(p[3])]
    tris = []
    for ln in lines[ne + 2: lines.index("$EndElements")]:
        p = ln.split()
        if len(p) >= 8 and p[1] == "2":
            tris.append((int(p[3]), [int(p[-3]), int(p[-2]), int(p[-1])]))
        if len(tris) == 16:
            break
    used = sorted({n for _, t in tris for n in t})
    index = {n: i for i, n in enumerate(used)}
    return {"vertices_mm": [coords[n] for n in used], "faces": [[index[n] for n in t] for _, t in tris],
            "tags": [tag for tag, _ in tris], "source": "first 16 triangles of test_meshes/sample.msh"}


def fixture_mesh(path: Path) -> dict:
    """Every node and triangle of a Gmsh 2.2 file, as the reference's loader reads them
    (load_gmsh22_with_tags, BeatEngineCore.jl:193-234): nodes in file order, triangles
    (element type 2) with their node ids mapped to 0-based node positions, physical tag
    = the element's first tag.  Coordinates are kept as parsed (millimetres); the tests
    apply the reference's Float32 parse and scale."""
    lines = path.read_text().splitlines()
    ns, ne = lines.index("$Nodes"), lines.index("$Elements")
    index, nodes = {}, []
    for ln in lines[ns + 2: lines.index("$EndNodes")]:
        p = ln.split()
        if len(p) >= 4:
            nodes.append([float(p[1]), float(p[2]), float(p[3])])
            index[int(p[0])] = len(nodes) - 1
    faces, tags = [], []
    for ln in lines[ne + 2: lines.index("$EndElements")]:
        p = ln.split()
        if len(p) < 8 or p[1] != "2":
            continue
        ids = [index.get(int(x), -1) for x in p[-3:]]
        if min(ids) < 0:
            continue
        faces.append(ids)
        tags.append(int(p[3]))
    return {"nodes_mm": np.asarray(nodes, np.float64), "faces": np.asarray(faces, np.int32),
            "tags": np.asarray(tags, np.int32)}


def main(root: str) -> None:
    root = Path(root)
    jl = root / "src/blab/solvers/julia_local"
    (HERE / "triangle_rule_order4.json").write_text(json.dumps(triangle_rule_constants(jl / "src/BeatEngineCore.jl"), indent=1))
    counts = {p.name: gmsh_counts(p) for p in sorted((jl / "test_meshes").glob("*.msh"))}
    (HERE / "reference_mesh_counts.json").write_text(json.dumps(counts, indent=1))
    (HERE / "sample_subset16.json").write_text(json.dumps(subset16(jl / "test_meshes/sample.msh")))
    for name in ("sample_half", "sample_quarter", "sample_detailed"):
        np.savez_compressed(HERE / f"{name}.npz", **fixture_mesh(jl / "test_meshes" / f"{name}.msh"))
    print("wrote", sorted(p.name for p in HERE.iterdir() if p.suffix in (".json", ".npz")))


def default_root() -> str:
    env = os.environ.get("BOUNDARY_LAB_REFERENCE")
    return env if env else str(HERE.parents[2] / "reference")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else default_root())
