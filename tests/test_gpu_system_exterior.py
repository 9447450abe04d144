"""Physical-system exterior path on the GPU: the same compiled-system request on the
CUDA engine and on the FP64 CPU oracle.  Two excitation ports (the piston and the
rest of the box, each an ideal velocity source) so the multi-port solve, the
per-component impedance and the per-output point slicing are all exercised.

Tolerances (relative 2-norm): float32 requests (mixed form) 1e-5 on the field,
the boundary pressure and the impedance; float64 requests 1e-9."""

import sys
from pathlib import Path

import numpy as np
import pytest

from conftest import pkg_module

pytestmark = pytest.mark.gpu
TESTS = Path(__file__).resolve().parent
se = pkg_module("system_exterior")
meshes = pkg_module("meshes")


def oracle_factory(**kw):
    sys.path.insert(0, str(TESTS))
    import oracle_engine

    return oracle_engine.make_engine(**kw)


@pytest.fixture(scope="module")
def box_file(tmp_path_factory):
    box = meshes.box_with_piston((0.3, 0.2, 0.25), 600, 0.05, "+z")
    path = tmp_path_factory.mktemp("sysgpu") / "box.msh"
    meshes.write_gmsh22(path, box.vertices * 1000.0, box.faces, box.tags)
    return path


def request(path, precision):
    boundaries = [{"id": f"boundary:{name}", "name": name, "region_id": "region:ext", "kind": "moving",
                   "group": {"mesh_id": "mesh:box", "dimension": 2, "tag": tag, "name": None}, "parameters": {}}
                  for name, tag in (("wall", 1), ("piston", 2))]
    components = [{"id": f"component:{name}", "name": name, "kind": "ideal_velocity_source",
                   "boundary_ids": [f"boundary:{name}"],
                   "parameters": {"boundary_motion_weights": {f"boundary:{name}": w}}}
                  for name, w in (("piston", 1.0), ("wall", 0.25))]
    ports = [{"id": f"port:{name}", "name": name, "component_id": f"component:{name}", "kind": "normal_velocity"}
             for name in ("piston", "wall")]
    system = {"id": "system:box", "name": "box", "contract_version": 1, "meshes": [
        {"id": "mesh:box", "name": "box", "file": str(path), "purpose": "bem_surface", "scale_to_m": 0.001,
         "translation_m": [0.0, 0.0, 0.05]}],
        "regions": [{"id": "region:ext", "name": "air", "kind": "unbounded_air", "mesh_ids": ["mesh:box"],
                     "sound_speed_m_per_s": 343.0, "density_kg_per_m3": 1.205, "loss_model": {}}],
        "boundaries": boundaries, "interfaces": [], "components": components, "excitation_ports": ports,
        "assumptions": []}
    return {"schema_version": 1, "compiled_system": system, "frequencies_hz": [600.0, 2400.0],
            "excitation_port_ids": ["port:piston", "port:wall"],
            "outputs": [{"id": "far", "quantity": "exterior_pressure",
                         "options": {"points_m": [[0, 0, 2.0], [2.0, 0, 0], [0, 1.5, 1.3]]}},
                        {"id": "near", "quantity": "exterior_pressure", "options": {"points_m": [[0.05, 0.0, 0.4]]}},
                        {"id": "bem", "quantity": "bem_boundary_pressure"},
                        {"id": "z", "quantity": "radiation_impedance"}],
            "solver_options": {"precision": precision, "bem_backend": "cuda"}}


def values(result):
    out = {}
    for q in result["quantities"]:
        v = q["values"]
        out[q["id"]] = (np.asarray(v["real"]) + 1j * np.asarray(v["imag"])).reshape(v["shape"])
    return out


@pytest.mark.parametrize("precision,tol", [("float32", 1e-5), ("float64", 1e-9)])
def test_system_request_matches_oracle(native, box_file, precision, tol):
    req = request(box_file, precision)
    job = se.ExteriorSystemJob(req)
    try:
        got = list(job.results())
    finally:
        job.close()
    ref_job = se.ExteriorSystemJob(req, engine_factory=oracle_factory)
    try:
        ref = list(ref_job.results())
    finally:
        ref_job.close()
    assert len(got) == 2
    for g, r in zip(got, ref):
        assert g["freq_hz"] == r["freq_hz"]
        gv, rv = values(g), values(r)
        assert gv["far"].shape == (2, 3) and gv["near"].shape == (2, 1) and gv["z"].shape == (2,)
        for key in ("far", "near", "bem", "z"):
            err = np.linalg.norm(gv[key] - rv[key]) / np.linalg.norm(rv[key])
            assert err < tol, (precision, g["freq_hz"], key, err)
        assert g["diagnostics"]["engine_form"] == ("mixed" if precision == "float32" else "fp64")
        assert g["quantities"][0]["values"]["dtype"] == ("complex64" if precision == "float32" else "complex128")
