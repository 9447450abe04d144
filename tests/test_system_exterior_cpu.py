"""Physical-system exterior path (system_exterior.py, worker.py) on CPU.

The numerical engine is the FP64 CPU oracle behind the product's engine hook, so
these tests check the request handling, tag mapping, excitations, quadrature
selection, quantity wire and worker protocol of coupled_solver.jl:267-569.  The
consistency check is the reference's own
(tests/test_physical_compiler.py:786-868): the system path's field at a point and
its radiation impedance equal the legacy exterior path's on the same mesh.
"""

import json
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

from conftest import pkg_module

TESTS = Path(__file__).resolve().parent
ROOT = TESTS.parent
WORKER = ROOT / "boundary-lab_gb300" / "worker.py"
se = pkg_module("system_exterior")
meshes = pkg_module("meshes")
job_mod = pkg_module("job")


def oracle_factory(**kw):
    sys.path.insert(0, str(TESTS))
    import oracle_engine

    return oracle_engine.make_engine(**kw)


@pytest.fixture(scope="module")
def sphere_file(tmp_path_factory):
    mesh = meshes.sphere_with_cap(0.1, 1, 40.0)  # 80 faces, tag 2 = cap, 1 = rest
    path = tmp_path_factory.mktemp("sys") / "sphere.msh"
    meshes.write_gmsh22(path, mesh.vertices * 1000.0, mesh.faces, mesh.tags)
    return path


def system_request(mesh_files, *, precision="float64", backend="cuda", outputs=None, freqs=(400.0, 1300.0),
                   weights=None, symmetry="off", extra_options=None):
    """A compiled exterior system in the wire form of system_contract.py:177-196: one unbounded
    region over the given surfaces; boundary:cap (tag 2 of the first mesh) moving, the rest rigid."""
    mesh_entries, boundaries = [], []
    for i, (path, translation) in enumerate(mesh_files):
        mid = f"mesh:{i}"
        mesh_entries.append({"id": mid, "name": f"m{i}", "file": str(path), "purpose": "bem_surface",
                             "scale_to_m": 0.001, "translation_m": list(translation)})
        for tag, kind in ((1, "rigid"), (2, "moving" if i == 0 else "rigid")):
            bid = "boundary:cap" if (i == 0 and tag == 2) else f"boundary:{i}:{tag}"
            boundaries.append({"id": bid, "name": bid, "region_id": "region:ext", "kind": kind,
                               "group": {"mesh_id": mid, "dimension": 2, "tag": tag, "name": None}, "parameters": {}})
    params = {"motion_profile": "uniform"}
    if weights is not None:
        params["boundary_motion_weights"] = weights
    system = {
        "id": "system:test", "name": "test", "contract_version": 1, "source_model_version": 1, "metadata": {},
        "meshes": mesh_entries,
        "regions": [{"id": "region:ext", "name": "Exterior", "kind": "unbounded_air", "mesh_ids":
                     [m["id"] for m in mesh_entries], "volume_groups": [], "sound_speed_m_per_s": 343.0,
                     "density_kg_per_m3": 1.205, "loss_model": {}}],
        "boundaries": boundaries, "interfaces": [], "assumptions": [],
        "components": [{"id": "component:cap", "name": "Cap", "kind": "ideal_velocity_source",
                        "boundary_ids": ["boundary:cap"], "parameters": params}],
        "excitation_ports": [{"id": "excitation:cap", "name": "cap", "component_id": "component:cap",
                              "kind": "normal_velocity"}],
    }
    if outputs is None:
        outputs = [{"id": "output:field", "quantity": "exterior_pressure", "target_ids": [],
                    "options": {"points_m": [[0.0, 0.0, 2.0], [2.0, 0.0, 0.0], [0.0, 1.0, -1.5]]}},
                   {"id": "output:bem", "quantity": "bem_boundary_pressure", "target_ids": [], "options": {}},
                   {"id": "output:neumann", "quantity": "bem_boundary_neumann", "target_ids": ["x"], "options": {}},
                   {"id": "output:impedance", "quantity": "radiation_impedance", "target_ids": [], "options": {}}]
    return {"schema_version": 1, "compiled_system": system, "frequencies_hz": list(freqs),
            "excitation_port_ids": ["excitation:cap"], "outputs": outputs,
            "solver_options": {"precision": precision, "bem_backend": backend, "symmetry": symmetry,
                               "quadrature_order": 4, "singular_order": 4, **(extra_options or {})}}


def wire_values(q):
    v = q["values"]
    arr = np.asarray(v["real"], np.float64) + 1j * np.asarray(v["imag"], np.float64)
    return arr.reshape(v["shape"])


def check_result_contract(result, n_ports):
    """The checks of system_contract.py:125-156 on one result dict."""
    assert result["schema_version"] == 1 and result["freq_hz"] > 0
    ids = [q["id"] for q in result["quantities"]]
    assert len(ids) == len(set(ids))
    for q in result["quantities"]:
        vals = wire_values(q)
        assert q["id"] and q["quantity"] and q["unit"]
        assert len(q["axes"]) == vals.ndim
        if "excitation" in q["axes"]:
            assert vals.shape[q["axes"].index("excitation")] == n_ports
    json.dumps(result, allow_nan=False)


def run(request, **kw):
    job = se.ExteriorSystemJob(request, engine_factory=oracle_factory, **kw)
    try:
        return list(job.results()), job
    finally:
        job.close()


def test_system_path_matches_the_legacy_path(sphere_file):
    """Field and impedance equal the legacy exterior job's on the same mesh and drive (the
    reference's own cross-check), and the boundary traces are the oracle's."""
    req = system_request([(sphere_file, (0, 0, 0))])
    results, job = run(req)
    assert [r["freq_hz"] for r in results] == [400.0, 1300.0]
    for r in results:
        check_result_contract(r, 1)
        d = r["diagnostics"]
        assert d["formulation"] == "exterior_burton_miller_neumann" and d["bounded_region_count"] == 0
        assert d["regular_quadrature_mode"] == "fixed" and d["regular_quadrature_order"] == 4
    q = {x["id"]: x for x in results[0]["quantities"]}
    assert q["output:field"]["values"]["dtype"] == "complex128"
    assert q["output:field"]["axes"] == ["excitation", "observation"] and q["output:field"]["unit"] == "Pa"
    assert q["output:field"]["metadata"] == {"points_m": [[0.0, 0.0, 2.0], [2.0, 0.0, 0.0], [0.0, 1.0, -1.5]]}
    assert q["output:neumann"]["target_id"] == "x" and q["output:bem"]["target_id"] is None
    assert wire_values(q["output:bem"]).shape == (1, job.mesh.n_vertices)
    neumann = wire_values(q["output:neumann"])[0]
    omega = 2 * np.pi * 400.0
    assert np.allclose(neumann[job.mesh.tags == 2], 1j * 1.205 * omega) and np.all(neumann[job.mesh.tags == 1] == 0)
    # legacy path: radiator = tag 2, unit channel, observation at 2 m on the axes
    cfg = {"mesh_file": str(sphere_file), "scale_factor": 0.001, "rho": 1.205, "sound_speed": 343.0,
           "step_size": 90.0, "distance": 2.0, "radiators": [{"name": "cap", "tag": 2, "channel": "main"}],
           "channels": [{"name": "main"}], "flat_target_normalization_enabled": False}
    legacy = list(job_mod.ExteriorJob({"config": cfg, "frequencies_hz": [400.0, 1300.0]},
                                      engine_factory=oracle_factory).results())
    for r, leg in zip(results, legacy):
        q = {x["id"]: x for x in r["quantities"]}
        h = np.asarray(leg["result"]["horizontal_pressure"]["real"][0]) + \
            1j * np.asarray(leg["result"]["horizontal_pressure"]["imag"][0])
        # horizontal angles -180, -90, 0, 90, 180: 0 deg is (0, 0, 2) on the axis
        field = wire_values(q["output:field"])[0]
        assert abs(field[0] - h[2]) / abs(h[2]) < 1e-6
        z = wire_values(q["output:impedance"])[0]
        zl = complex(*leg["result"]["impedance"][0])
        assert abs(z - zl) / abs(zl) < 1e-6
    # boundary traces against the oracle directly
    from oracle import oracle

    omega = 2 * np.pi * 1300.0
    drive = (job.mesh.tags == 2).astype(complex)
    sol = oracle.solve_frequency(job.mesh, omega / 343.0, (drive * 1j * 1.205 * omega)[:, None],
                                 np.array([[0.0, 0.0, 2.0]]))
    q = {x["id"]: x for x in results[1]["quantities"]}
    p = wire_values(q["output:bem"])[0]
    assert np.linalg.norm(p - sol.pressure[:, 0]) / np.linalg.norm(sol.pressure[:, 0]) < 1e-12


def test_float32_request_answers_complex64(sphere_file):
    results, _ = run(system_request([(sphere_file, (0, 0, 0))], precision="float32", freqs=(700.0,)))
    for q in results[0]["quantities"]:
        assert q["values"]["dtype"] == "complex64"
    assert results[0]["diagnostics"]["precision"] == "float32"


def test_meshes_are_combined_with_fresh_solver_tags(sphere_file):
    """Two copies of the surface (the second shifted by 1 m): solver tags 1..4 in order of first
    appearance; the moving boundary is tag 2 of the first mesh only."""
    req = system_request([(sphere_file, (0, 0, 0)), (sphere_file, (1000.0, 0, 0))], freqs=(500.0,))
    region = se.aggregate_bem_region(req["compiled_system"]["meshes"], req["compiled_system"]["regions"][0],
                                     req["compiled_system"]["boundaries"])
    single = meshes.read_gmsh22(sphere_file, 0.001)
    n = single.n_faces
    first = {t: i + 1 for i, t in enumerate(dict.fromkeys(single.tags.tolist()))}
    assert region.mesh.n_faces == 2 * n
    assert region.mesh.tags[:n].tolist() == [first[t] for t in single.tags.tolist()]
    assert region.mesh.tags[n:].tolist() == [first[t] + 2 for t in single.tags.tolist()]
    assert np.allclose(region.mesh.vertices[single.n_vertices:], single.vertices + [1000.0, 0, 0])
    assert region.boundary_tag_by_id["boundary:cap"] == first[2]
    assert region.boundary_tag_by_id["boundary:1:2"] == first[2] + 2
    assert region.face_offset_by_mesh_id == {"mesh:0": 0, "mesh:1": n}
    results, job = run(req)
    neumann = wire_values({x["id"]: x for x in results[0]["quantities"]}["output:neumann"])[0]
    assert np.count_nonzero(neumann) == np.count_nonzero(single.tags == 2)


def test_motion_weights_scale_the_drive(sphere_file):
    a, _ = run(system_request([(sphere_file, (0, 0, 0))], freqs=(900.0,)))
    b, _ = run(system_request([(sphere_file, (0, 0, 0))], freqs=(900.0,), weights={"boundary:cap": 2.5}))
    qa = {x["id"]: wire_values(x) for x in a[0]["quantities"]}
    qb = {x["id"]: wire_values(x) for x in b[0]["quantities"]}
    for key in ("output:field", "output:bem", "output:neumann", "output:impedance"):
        np.testing.assert_allclose(qb[key], 2.5 * qa[key], rtol=1e-10, atol=1e-30)


def test_wavelength_quadrature_on_the_cpu_backend(sphere_file):
    """bem_backend cpu defaults to wavelength mode: order 1 / 2 / base by k h (p90 of the face
    areas), one engine per order; cuda rejects wavelength mode."""
    mesh = se.aggregate_bem_region(*[system_request([(sphere_file, (0, 0, 0))])["compiled_system"][k]
                                     for k in ("meshes",)], {"id": "region:ext", "mesh_ids": ["mesh:0"]},
                                   []).mesh
    h = np.sqrt(np.quantile(mesh.areas, 0.9))
    f_of_kh = lambda kh: kh / h * 343.0 / (2 * np.pi)  # noqa: E731
    opts = {"wavelength_kh_q1_max": 0.5, "wavelength_kh_q2_max": 1.5}
    freqs = [f_of_kh(0.3), f_of_kh(1.0), f_of_kh(1.2), f_of_kh(2.0)]
    orders = [se.exterior_quadrature_selection(opts, mesh, f, 343.0, 4, "cpu").order for f in freqs]
    assert orders == [1, 2, 2, 4]
    assert se.exterior_quadrature_selection({}, mesh, freqs[0], 343.0, 4, "cpu").order == 2  # q1 = 0, q2 = 2
    stats = {"median": np.median(mesh.areas), "p75": np.quantile(mesh.areas, 0.75),
             "p90": np.quantile(mesh.areas, 0.9), "max": np.max(mesh.areas)}
    for stat, area in stats.items():
        for f in np.geomspace(50.0, 20000.0, 40):
            kh = 2 * np.pi * f / 343.0 * np.sqrt(area)
            want = 1 if kh <= 0.5 else 2 if kh <= 1.5 else 4
            got = se.exterior_quadrature_selection({"wavelength_mesh_stat": stat, **opts}, mesh, f, 343.0, 4, "cpu")
            assert got.order == want, (stat, f)
    prepared = []

    def recording_factory(**kw):
        eng = oracle_factory(**kw)
        prep = eng.prepare

        def prepare(*a, **k):
            prepared.append(a[4])
            return prep(*a, **k)

        eng.prepare = prepare
        return eng

    req = system_request([(sphere_file, (0, 0, 0))], backend="cpu", freqs=freqs, extra_options=opts)
    job = se.ExteriorSystemJob(req, engine_factory=recording_factory)
    results = list(job.results())
    job.close()
    assert [r["diagnostics"]["regular_quadrature_order"] for r in results] == [1, 2, 2, 4]
    assert all(r["diagnostics"]["regular_quadrature_mode"] == "wavelength" for r in results)
    assert sorted(prepared) == [1, 2, 4]
    with pytest.raises(se.SystemRequestError, match="only on the CPU backend"):
        list(se.ExteriorSystemJob(system_request([(sphere_file, (0, 0, 0))], extra_options={
            "regular_quadrature_mode": "wavelength"}), engine_factory=oracle_factory).results())
    for bad, msg in (({"regular_quadrature_mode": "adaptive"}, "Unsupported regular quadrature mode"),
                     ({"wavelength_mesh_stat": "p50"}, "Unsupported wavelength mesh stat"),
                     ({"wavelength_kh_q1_max": -1.0}, "must be non-negative"),
                     ({"wavelength_kh_q1_max": 2.0}, "must exceed")):
        with pytest.raises(se.SystemRequestError, match=msg):
            se.exterior_quadrature_selection(bad, mesh, 500.0, 343.0, 4, "cpu")


def test_half_model_with_symmetry_matches_the_full_model(tmp_path):
    box = meshes.box_with_piston((0.3, 0.2, 0.25), 300, 0.05, "+z")
    half = meshes.fundamental_domain(box, "x")
    full, _ = meshes.mirror_to_full(half, "x")
    paths = {}
    for name, m in (("half", half), ("full", full)):
        paths[name] = tmp_path / f"{name}.msh"
        meshes.write_gmsh22(paths[name], m.vertices * 1000.0, m.faces, m.tags)
    pts = [[0.0, 0.0, 2.0], [0.7, 0.3, 1.5]]
    out = [{"id": "f", "quantity": "exterior_pressure", "options": {"points_m": pts}},
           {"id": "z", "quantity": "radiation_impedance"}]
    got = {}
    for name, sym in (("half", "x"), ("full", "off")):
        res, _ = run(system_request([(paths[name], (0, 0, 0))], outputs=out, freqs=(800.0,), symmetry=sym))
        got[name] = {q["id"]: wire_values(q) for q in res[0]["quantities"]}
        assert res[0]["diagnostics"]["symmetry"] == sym
    assert np.linalg.norm(got["half"]["f"] - got["full"]["f"]) / np.linalg.norm(got["full"]["f"]) < 5e-5
    np.testing.assert_allclose(got["half"]["z"], got["full"]["z"], rtol=5e-5)


def test_rejections(sphere_file):
    base = lambda **kw: system_request([(sphere_file, (0, 0, 0))], **kw)  # noqa: E731

    def expect(request, msg):
        with pytest.raises(se.SystemRequestError, match=msg):
            job = se.ExteriorSystemJob(request, engine_factory=oracle_factory)
            try:
                list(job.results())
            finally:
                job.close()

    r = base()
    r["schema_version"] = 2
    expect(r, "Unsupported system solve request schema")
    r = base()
    r["compiled_system"]["regions"][0]["kind"] = "bounded_air"
    expect(r, "Interior FEM")
    r = base()
    r["compiled_system"]["regions"].append({**r["compiled_system"]["regions"][0], "id": "region:2"})
    expect(r, "exactly one unbounded region")
    r = base()
    r["compiled_system"]["regions"].append({**r["compiled_system"]["regions"][0], "id": "r2", "kind": "bounded_air"})
    expect(r, "Coupled FEM-BEM")
    expect(base(precision="float16"), "Exterior precision must be float32 or float64.")
    expect(base(backend="metal"), "Exterior BEM backend must be cpu, cuda, or rocm.")
    expect(base(symmetry="z"), "Unsupported symmetry mode: z. Expected off, x, or xy.")
    r = base()
    r["compiled_system"]["regions"][0]["sound_speed_m_per_s"] = 0.0
    expect(r, "sound speed and density must be positive")
    r = base()
    r["compiled_system"]["regions"][0]["mesh_ids"] = []
    expect(r, "at least one BEM mesh")
    r = base()
    r["compiled_system"]["regions"][0]["mesh_ids"] = ["mesh:nope"]
    expect(r, "Unknown mesh id: mesh:nope")
    r = base()
    r["compiled_system"]["meshes"][0]["purpose"] = "fem_volume"
    expect(r, "must be BEM surfaces")
    r = base()
    r["compiled_system"]["boundaries"][0]["group"]["mesh_id"] = "mesh:other"
    expect(r, "outside its unbounded region")
    r = base()
    r["compiled_system"]["boundaries"][0]["group"]["tag"] = 9
    expect(r, "tag 9 is not present in BEM mesh 'mesh:0'")
    r = base()
    r["compiled_system"]["excitation_ports"][0]["kind"] = "pressure"
    expect(r, "must be a normal-velocity port")
    r = base()
    r["compiled_system"]["components"][0]["kind"] = "electrodynamic_driver"
    expect(r, "must reference an ideal velocity source")
    r = base()
    r["compiled_system"]["components"][0]["boundary_ids"] = ["boundary:0:1"]  # rigid only
    expect(r, "has no moving boundaries")
    expect(base(weights={"boundary:cap": -1.0}), "finite and positive")
    r = base()
    r["excitation_port_ids"] = ["excitation:nope"]
    expect(r, "Unknown excitation port id: excitation:nope")
    expect(base(outputs=[{"id": "a", "quantity": "fem_pressure"}]), "Unsupported exterior output quantity: fem_pressure")
    expect(base(outputs=[{"id": "a", "quantity": "exterior_pressure", "options": {}}]),
           "exterior_pressure output requires options.points_m.")


def test_cancel_between_frequencies(sphere_file, tmp_path):
    cancel = tmp_path / "cancel"
    req = system_request([(sphere_file, (0, 0, 0))], freqs=(300.0, 600.0, 900.0))
    req["cancel_path"] = str(cancel)
    job = se.ExteriorSystemJob(req, engine_factory=oracle_factory)
    it = job.results()
    next(it)
    cancel.write_text("")
    with pytest.raises(se.SystemJobCancelled) as info:
        list(it)
    job.close()
    assert info.value.solved_count == 1
    with pytest.raises(se.SystemJobCancelled) as info:  # cancelled before the first frequency
        list(se.ExteriorSystemJob(req, engine_factory=oracle_factory).results())
    assert info.value.solved_count == 0


def _worker_env():
    env = dict(os.environ)
    env["GB300_BEM_ENGINE"] = "oracle_engine:make_engine"
    env["PYTHONPATH"] = os.pathsep.join([str(TESTS), str(ROOT)])
    return env


def test_worker_event_mode_and_one_shot(sphere_file, tmp_path):
    req = system_request([(sphere_file, (0, 0, 0))], freqs=(450.0, 950.0))
    path = tmp_path / "request.json"
    path.write_text(json.dumps(req))
    bad = tmp_path / "bad.json"
    bad.write_text(json.dumps({**req, "schema_version": 3}))
    lines = "\n".join(json.dumps({"request": str(p), "operation": "solve"}) for p in (path, bad)) + "\n"
    proc = subprocess.run([sys.executable, str(WORKER), "--worker"], input=lines, capture_output=True, text=True,
                          env=_worker_env(), timeout=600)
    events = [json.loads(x) for x in proc.stdout.splitlines() if x.strip()]
    assert [e["type"] for e in events] == ["ready", "result", "result", "completed", "failed"], proc.stderr[-2000:]
    assert events[3]["solved_count"] == 2
    assert "Unsupported system solve request schema" in events[4]["error"]
    for e in events[1:3]:
        check_result_contract(e["result"], 1)
    # one-shot: request on stdin, one result object per line, exit 0
    proc = subprocess.run([sys.executable, str(WORKER)], input=json.dumps(req), capture_output=True, text=True,
                          env=_worker_env(), timeout=600)
    assert proc.returncode == 0, proc.stderr[-2000:]
    plain = [json.loads(x) for x in proc.stdout.splitlines() if x.strip()]
    assert [r["freq_hz"] for r in plain] == [450.0, 950.0]
    assert plain[0]["quantities"] == events[1]["result"]["quantities"]
    proc = subprocess.run([sys.executable, str(WORKER)], input=json.dumps({**req, "schema_version": 3}),
                          capture_output=True, text=True, env=_worker_env(), timeout=600)
    assert proc.returncode == 1 and "Unsupported system solve request schema" in proc.stderr


def test_in_process_backend_session(sphere_file):
    """Gb300SystemBackend: metadata from the request, one SystemFrequencyResult per frequency
    with the wire's arrays, float32 precision as the production backend sets it; stop() ends
    the stream between frequencies; a bad request surfaces as RuntimeError."""
    req = system_request([(sphere_file, (0, 0, 0))], freqs=(350.0, 700.0, 1400.0))
    backend = se.Gb300SystemBackend(engine_factory=oracle_factory)
    session = backend.create_system_session(req)
    assert session.metadata.system_id == "system:test"
    assert session.metadata.excitation_port_ids == ("excitation:cap",)
    assert session.metadata.available_quantity_ids == ("output:field", "output:bem", "output:neumann",
                                                       "output:impedance")
    results = list(session.solve_stream())
    assert [r.freq_hz for r in results] == [350.0, 700.0, 1400.0]
    q = {x.id: x for x in results[0].quantities}
    assert q["output:field"].values.dtype == np.complex64 and q["output:field"].values.shape == (1, 3)
    assert q["output:impedance"].axes == ("radiator",) and q["output:impedance"].values.shape == (1,)
    assert results[0].diagnostics["precision"] == "float32"
    session = backend.create_system_session(req)
    got = []
    for r in session.solve_stream():
        got.append(r)
        session.stop()
    assert len(got) == 1
    bad = system_request([(sphere_file, (0, 0, 0))])
    bad["schema_version"] = 5
    with pytest.raises(RuntimeError, match="Unsupported system solve request schema"):
        backend.create_system_session(bad)

