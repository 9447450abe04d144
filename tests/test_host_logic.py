"""Host-side request logic (request.py, the solver.jl restatement) and meshes (CPU only)."""

import re
from pathlib import Path

import numpy as np
import pytest

from conftest import pkg_module

rq = pkg_module("request")
meshes = pkg_module("meshes")
ROOT = Path(__file__).resolve().parents[1]


def test_polar_points_default():
    angles, h, v, on_axis = rq.polar_observation_points({})
    assert angles.dtype == np.float32 and len(angles) == 73
    assert angles[0] == -180 and angles[-1] == 180 and angles[on_axis] == 0
    assert np.allclose(h[on_axis], [0, 0, 2.0]) and np.allclose(v[on_axis], [0, 0, 2.0])
    assert np.allclose(np.linalg.norm(h, axis=1), 2.0)


def test_polar_points_partial_range_appends_max():
    angles, *_ = rq.polar_observation_points({"min_angle": -10, "max_angle": 12, "step_size": 5})
    assert list(angles) == [-10, -5, 0, 5, 10, 12]


@pytest.mark.parametrize("cfg,msg", [({"step_size": 0}, "positive"), ({"min_angle": 5, "max_angle": 10}, "include 0"),
                                     ({"min_angle": -200}, "within"), ({"distance": -1}, "distance")])
def test_polar_validation(cfg, msg):
    with pytest.raises(rq.RequestError, match=msg):
        rq.polar_observation_points(cfg)


def test_spherical_observation_metadata():
    assert rq.spherical_observation({}) is None
    pts, meta = rq.spherical_observation({"spherical_sampling_enabled": True, "spherical_sampling_points": 50,
                                          "distance": 2.0, "axial_offset": 0.1})
    assert pts.shape == (50, 3)
    assert np.allclose(np.linalg.norm(pts - [0, 0, 0.1], axis=1), 2.0)
    assert meta["theta_polar_rad"].dtype == np.float32
    assert np.all((meta["phi_azimuth_rad"] >= 0) & (meta["phi_azimuth_rad"] < 2 * np.pi + 1e-6))


@pytest.mark.parametrize("order", [1, 2, 4, 6])
@pytest.mark.parametrize("ctype", ["lowpass", "highpass"])
def test_butterworth_is_minus_3db_at_cutoff(order, ctype):
    r = rq.crossover_response({"type": ctype, "filter": "butterworth", "order": order, "frequency_hz": 1000.0}, 1000.0)
    assert abs(abs(r) - 2 ** -0.5) < 1e-12
    far = rq.crossover_response({"type": ctype, "order": order, "frequency_hz": 1000.0}, 1e6 if ctype == "highpass" else 1.0)
    assert abs(abs(far) - 1) < 1e-3


@pytest.mark.parametrize("order", [2, 4, 6])
def test_linkwitz_riley_is_minus_6db_and_sums_flat(order):
    lp = rq.crossover_response({"type": "lowpass", "filter": "linkwitz_riley", "order": order, "frequency_hz": 800.0}, 800.0)
    hp = rq.crossover_response({"type": "highpass", "filter": "linkwitz_riley", "order": order, "frequency_hz": 800.0}, 800.0)
    assert abs(abs(lp) - 0.5) < 1e-12 and abs(abs(hp) - 0.5) < 1e-12
    for f in (100.0, 800.0, 5000.0):
        lp = rq.crossover_response({"type": "lowpass", "filter": "linkwitz_riley", "order": order, "frequency_hz": 800.0}, f)
        hp = rq.crossover_response({"type": "highpass", "filter": "linkwitz_riley", "order": order, "frequency_hz": 800.0}, f)
        s = lp + hp if order % 4 == 0 else lp - hp
        assert abs(abs(s) - 1.0) < 1e-9


def test_crossover_validation():
    with pytest.raises(rq.RequestError, match="order"):
        rq.validate_crossover_config("w", {"type": "lowpass", "frequency_hz": 100, "order": 3})
    with pytest.raises(rq.RequestError, match="Linkwitz"):
        rq.validate_crossover_config("w", {"type": "lowpass", "frequency_hz": 100, "order": 1, "filter": "linkwitz_riley"})
    with pytest.raises(rq.RequestError, match="frequency_hz"):
        rq.validate_crossover_config("w", {"type": "highpass"})


def test_channel_drive_level_polarity_delay():
    d = rq.channel_drive({"level_db": 6.0, "polarity": -1, "delay_ms": 0.25, "hpf": None, "lpf": None}, 1000.0)
    assert abs(abs(d) - 10 ** (6 / 20)) < 1e-12
    assert abs(np.angle(-d) - (-2 * np.pi * 1000 * 0.25e-3)) < 1e-9


def test_interpolate_reference_wraps():
    angles = np.arange(-180, 181, 90, dtype=np.float32)  # -180..180
    vals = np.array([1, 2, 3, 4, 1], complex)
    assert rq.interpolate_complex_reference(vals, angles, 0.0) == 3
    assert abs(rq.interpolate_complex_reference(vals, angles, 45.0) - 3.5) < 1e-12
    assert abs(rq.interpolate_complex_reference(vals, angles, 225.0) - 1.5) < 1e-12


def test_flat_target_normalises_on_axis():
    angles, *_ = rq.polar_observation_points({"step_size": 30})
    rng = np.random.default_rng(0)
    h = [rng.normal(size=len(angles)) + 1j * rng.normal(size=len(angles))]
    syn = rq.synthesize_channel_basis(["main"], h, h, None, {}, 1000.0, angles, 0.0, True)
    on = int(np.argmin(np.abs(angles)))
    assert abs(syn.horizontal_norm[on]) < 1e-5
    assert abs(syn.horizontal_spl[on] - 20 * np.log10(1 / 20e-6)) < 1e-3


def test_impedance_for_uniform_pressure():
    v, f = meshes.icosphere(0.1, 1)
    mesh = meshes.BoundaryMesh(v, f, np.full(len(f), 2))
    rad = [{"name": "r", "tag": 2, "mesh_id": 1}]
    z = rq.impedance_for_radiators(mesh.faces, mesh.areas, mesh.tags, mesh.element_mesh_ids,
                                   np.full(mesh.n_vertices, 2.0 + 1.0j), rad, [1.0 + 0j])
    force = (2 + 1j) * mesh.areas.sum() * 10
    assert np.allclose(z[0], [force.real / 2, -force.imag / 2], rtol=1e-6)
    z0 = rq.impedance_for_radiators(mesh.faces, mesh.areas, mesh.tags, mesh.element_mesh_ids,
                                    np.ones(mesh.n_vertices), rad, [0j])
    assert np.all(np.isnan(z0[0]))


def test_radiators_channels_and_drive_patterns():
    cfg = {"mesh_file": "x.msh", "radiators": [{"name": "a", "tag": 2, "channel": "lf"},
                                               {"name": "b", "tag": 3, "channel": "hf", "velocity_offset_db": 6}],
           "channels": [{"name": "lf"}, {"name": "hf", "level_db": -3}]}
    mi = rq.mesh_inputs_from_config(cfg)
    rads = rq.radiator_inputs_from_config(cfg, mi)
    chans = rq.channel_inputs_from_config(cfg)
    rq.validate_radiator_channels(rads, chans)
    tags = np.array([1, 2, 2, 3, 3])
    ids = np.ones(5, np.int32)
    pat = rq.face_drive_pattern(rads, rq.channel_unit_drives(rads, "hf"), 5, tags, ids)
    assert np.allclose(pat, [0, 0, 0, 10 ** 0.3, 10 ** 0.3])
    with pytest.raises(rq.RequestError, match="unknown channel"):
        rq.validate_radiator_channels(rads, {"lf": {}})
    with pytest.raises(rq.RequestError, match="No elements"):
        rq.validate_radiator_elements([{"name": "z", "tag": 9, "mesh_id": 1, "mesh": "mesh"}], tags, ids)


def test_wavelength_quadrature_is_rejected_like_the_reference_gpu_backends():
    with pytest.raises(rq.RequestError, match="BEAT CPU"):
        rq.regular_quadrature_mode({"regular_quadrature_mode": "wavelength"})
    assert rq.regular_quadrature_mode({}) == "fixed"


# ------------------------------------------------------------------- meshes --


def _closed_and_consistent(mesh):
    edges = {}
    for a, b, c in mesh.faces:
        for e in ((a, b), (b, c), (c, a)):
            edges[e] = edges.get(e, 0) + 1
    return all(v == 1 for v in edges.values()) and all((b, a) in edges for a, b in edges)


@pytest.mark.parametrize("name", ["sphere1280", "box5k"])
def test_generated_meshes_are_closed_outward(name):
    mesh = meshes.config_mesh(name)
    assert _closed_and_consistent(mesh)
    assert mesh.signed_volume() > 0
    assert np.any(mesh.tags == meshes.RADIATOR_TAG)


def test_box_sizes_and_seeded_pistons():
    assert abs(meshes.box_with_piston(target_faces=10000).n_faces - 10000) < 100
    a = meshes.seeded_piston_mesh(2000, 5)
    b = meshes.seeded_piston_mesh(2000, 5)
    assert np.array_equal(a.faces, b.faces) and np.array_equal(a.tags, b.tags)
    assert _closed_and_consistent(a)


def test_gmsh_roundtrip_and_loader_rules(tmp_path):
    mesh = meshes.sphere_with_cap(0.1, 1)
    p = tmp_path / "m.msh"
    meshes.write_gmsh22(p, mesh.vertices * 1000, mesh.faces, mesh.tags)
    text = p.read_text().replace("$EndElements", "99 1 2 5 5 1 2\n100 2 1 7 1 2 3\n$EndElements")
    text = text.replace(f"$Elements\n{mesh.n_faces}", f"$Elements\n{mesh.n_faces + 2}")
    p.write_text(text)
    back = meshes.read_gmsh22(p, 0.001)
    # the line element (type 1) and the 7-token triangle are skipped, as BeatEngineCore.jl:219-231
    assert back.n_faces == mesh.n_faces
    assert np.allclose(back.vertices, mesh.vertices)
    assert np.array_equal(back.tags, mesh.tags)


def test_combine_meshes_without_welding():
    a = meshes.sphere_with_cap(0.1, 1)
    c = meshes.combine_meshes([a, a], [(0, 0, 0), (1.0, 0, 0)])
    assert c.n_vertices == 2 * a.n_vertices and c.n_faces == 2 * a.n_faces
    assert np.array_equal(c.faces[a.n_faces:], a.faces + a.n_vertices)
    assert set(c.element_mesh_ids) == {1, 2}
    assert np.allclose(c.vertices[a.n_vertices:], a.vertices + [1.0, 0, 0])


def test_horn_in_box_is_closed():
    mesh = meshes.horn_in_box(target_faces=4000)
    assert _closed_and_consistent(mesh)
    assert np.any(mesh.tags == meshes.RADIATOR_TAG)


# ---------------------------------------------------------------------- ABI --


def test_library_exports_every_header_symbol():
    build = pkg_module("build")
    lib_path = build.build()
    native = pkg_module("native")
    lib = native.load()
    header = (ROOT / "include" / "gb300_bem.h").read_text()
    declared = set(re.findall(r"^\s*(?:int|void|const char\*|long long|void\*)\s+\**(bem_\w+)\s*\(", header, re.M))
    assert declared and declared == set(native.EXPORTED_SYMBOLS)
    for name in declared:
        assert hasattr(lib, name), name
    assert lib.bem_abi_version() == 3
    assert lib_path.exists()


def test_no_gpu_context_fails_cleanly():
    import ctypes

    native = pkg_module("native")
    from conftest import cuda_available

    if cuda_available():
        pytest.skip("a GPU is present")
    lib = native.load()
    h = ctypes.c_void_p()
    assert lib.bem_create_context(0, ctypes.byref(h)) == 2  # BEM_ERR_CUDA, no crash
    assert lib.bem_estimate_device_bytes(5000, 10000, 130000, 1, 2146, 16, 1) > 16 * 5000 * 5000 * 8
