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


def test_system_path_matches_legacy_path_on_the_gpu(native, box_file):
    """The reference's own cross-check (tests/test_physical_compiler.py:786-868) on the CUDA
    engine: the system path's field on the axis and its piston impedance equal the legacy
    exterior job's on the same mesh and drive (float32 wire of the legacy result)."""
    job_mod = pkg_module("job")
    req = request(box_file, "float64")
    sysreq = dict(req)
    sysreq["excitation_port_ids"] = ["port:piston"]
    sysreq["compiled_system"] = dict(req["compiled_system"])
    sysreq["compiled_system"]["components"] = [c for c in req["compiled_system"]["components"]
                                               if c["id"] == "component:piston"]
    sysreq["compiled_system"]["excitation_ports"] = [p for p in req["compiled_system"]["excitation_ports"]
                                                     if p["id"] == "port:piston"]
    sysreq["outputs"] = [{"id": "far", "quantity": "exterior_pressure", "options": {"points_m": [[0.0, 0.0, 2.05]]}},
                         {"id": "z", "quantity": "radiation_impedance"}]
    job = se.ExteriorSystemJob(sysreq)
    try:
        got = list(job.results())
    finally:
        job.close()
    # legacy: the mesh without the system's 5 cm translation, so its on-axis point at 2 m is the
    # system's (0, 0, 2.05)
    cfg = {"mesh_file": str(box_file), "scale_factor": 0.001, "rho": 1.205, "sound_speed": 343.0,
           "step_size": 90.0, "distance": 2.0,
           "radiators": [{"name": "piston", "tag": 2, "channel": "main"}], "channels": [{"name": "main"}],
           "flat_target_normalization_enabled": False}
    legacy = list(job_mod.ExteriorJob({"config": cfg, "frequencies_hz": req["frequencies_hz"]}).results())
    for g, leg in zip(got, legacy):
        v = values(g)
        hp = leg["result"]["horizontal_pressure"]
        h0 = complex(hp["real"][0][2], hp["imag"][0][2])  # 0 degrees
        assert abs(v["far"][0, 0] - h0) / abs(h0) < 1e-5
        zl = complex(*leg["result"]["impedance"][0])
        assert abs(v["z"][0] - zl) / abs(zl) < 1e-5
