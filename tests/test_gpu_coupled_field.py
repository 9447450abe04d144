"""Retained-trace field evaluation on the GPU (the reference's bem_field operation):
against the FP64 oracle field with the 3-point rule, with symmetry, through the
worker protocol, and the domain cache."""

import json
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

from conftest import pkg_module

pytestmark = pytest.mark.gpu

meshes = pkg_module("meshes")
cf = pkg_module("coupled_field")
ROOT = Path(__file__).resolve().parent.parent


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


def _traces(mesh, seed, dtype):
    rng = np.random.default_rng(seed)
    p = (rng.normal(size=mesh.n_vertices) + 1j * rng.normal(size=mesh.n_vertices)).astype(dtype)
    q = (rng.normal(size=mesh.n_faces) + 1j * rng.normal(size=mesh.n_faces)).astype(dtype)
    return p, q


def _points(n=40, r=0.6):
    rng = np.random.default_rng(5)
    d = rng.normal(size=(n, 3))
    return r * d / np.linalg.norm(d, axis=1, keepdims=True)


def _oracle_field(mesh, p, q, freq, pts, symmetry="off"):
    from oracle import oracle

    v32 = np.asarray(mesh.vertices, np.float32).astype(np.float64)
    m32 = meshes.BoundaryMesh(v32, mesh.faces, mesh.tags) if hasattr(meshes, "BoundaryMesh") else mesh
    k = 2 * np.pi * freq / 343.0
    return oracle.field(m32, np.asarray(p, np.complex128), np.asarray(q, np.complex128), k,
                        np.asarray(pts, np.float32).astype(np.float64), regular_order=2, symmetry=symmetry)


@pytest.mark.parametrize("dtype,tol", [(np.complex128, 1e-9), (np.complex64, 1e-5)])
def test_field_matches_oracle(dtype, tol):
    box = meshes.box_with_piston((0.3, 0.2, 0.25), 600, 0.05, "+z")
    p, q = _traces(box, 1, dtype)
    pts = _points()
    ev = cf.FieldEvaluator()
    try:
        req = cf.BemFieldEvaluationRequest("box", pts, box.vertices, box.faces, p, q, 2500.0, 343.0)
        u = cf.evaluate_bem_field(req, evaluator=ev)
        assert u.dtype == dtype and u.shape == (len(pts),)
        assert rel(u, _oracle_field(box, p, q, 2500.0, pts)) < tol
    finally:
        ev.release()


def test_symmetric_field_matches_oracle():
    box = meshes.box_with_piston((0.3, 0.2, 0.25), 600, 0.05, "+z")
    half = meshes.fundamental_domain(box, "x")
    p, q = _traces(half, 2, np.complex128)
    pts = _points()
    ev = cf.FieldEvaluator()
    try:
        req = cf.BemFieldEvaluationRequest("half", pts, half.vertices, half.faces, p, q, 1800.0, 343.0, symmetry="x")
        u = cf.evaluate_bem_field(req, evaluator=ev)
        assert rel(u, _oracle_field(half, p, q, 1800.0, pts, symmetry="x")) < 1e-9
    finally:
        ev.release()


def test_domain_cache():
    box = meshes.box_with_piston((0.3, 0.2, 0.25), 600, 0.05, "+z")
    p, q = _traces(box, 3, np.complex64)
    pts = _points(8)
    ev = cf.FieldEvaluator(max_domains=2)
    try:
        for key in ("a", "a", "b", "a", "c"):
            cf.evaluate_bem_field(cf.BemFieldEvaluationRequest(key, pts, box.vertices, box.faces, p, q, 900.0, 343.0),
                                  evaluator=ev)
        assert list(ev._meshes) == ["a|float32|off|q2", "c|float32|off|q2"]  # b was least recently used
    finally:
        ev.release()


def test_worker_bem_field(tmp_path):
    box = meshes.box_with_piston((0.3, 0.2, 0.25), 600, 0.05, "+z")
    p, q = _traces(box, 4, np.complex64)
    pts = _points(16)
    req = cf.BemFieldEvaluationRequest("wk", pts, box.vertices, box.faces, p, q, 3000.0, 343.0)
    path = tmp_path / "request.json"
    cf.write_evaluation_request(path, req)
    line = json.dumps({"request": str(path), "operation": "bem_field"}) + "\n"
    run = subprocess.run([sys.executable, str(ROOT / "boundary-lab_gb300" / "worker.py"), "--worker"], input=line,
                         capture_output=True, text=True, timeout=300, env=dict(os.environ))
    events = [json.loads(x) for x in run.stdout.splitlines() if x.strip()]
    kinds = [e["type"] for e in events]
    assert kinds == ["ready", "field_result", "completed"], run.stdout + run.stderr
    values = cf.read_binary_array(tmp_path, events[1]["values_binary"])
    ev = cf.FieldEvaluator()
    try:
        direct = cf.evaluate_bem_field(req, evaluator=ev)
    finally:
        ev.release()
    assert values.dtype == np.complex64 and np.array_equal(values, direct)
