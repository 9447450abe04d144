"""Retained-trace field requests on the CPU: the reference's validation messages
(src/blab/solvers/coupled_field.py:107-153) and the binary-array wire files of the
coupled worker's bem_field operation (coupled_field.py:155-233,
julia_local/coupled_solver.jl:2283-2339)."""

import json

import numpy as np
import pytest

from conftest import pkg_module

cf = pkg_module("coupled_field")


def _request(**over):
    rng = np.random.default_rng(0)
    base = dict(
        domain_key="enclosure-1",
        points_m=rng.normal(size=(5, 3)),
        boundary_points_m=rng.normal(size=(4, 3)),
        boundary_triangles=np.array([[0, 1, 2], [0, 2, 3]]),
        boundary_pressure=(rng.normal(size=4) + 1j * rng.normal(size=4)).astype(np.complex64),
        boundary_normal_derivative=(rng.normal(size=2) + 1j * rng.normal(size=2)).astype(np.complex64),
        frequency_hz=1000.0,
        sound_speed_m_per_s=343.0,
    )
    base.update(over)
    return cf.BemFieldEvaluationRequest(**base)


@pytest.mark.parametrize(
    "over,message",
    [
        (dict(points_m=np.zeros((5, 2))), "Exterior evaluation points must have shape (point, 3)."),
        (dict(boundary_points_m=np.zeros(4)), "BEM boundary points must have shape (bem_node, 3)."),
        (dict(boundary_triangles=np.zeros((2, 4), int)), "BEM boundary triangles must have shape (bem_face, 3)."),
        (dict(boundary_pressure=np.zeros(3, np.complex64)), "BEM boundary pressure must contain one value per boundary node."),
        (dict(boundary_normal_derivative=np.zeros(3, np.complex64)),
         "BEM boundary normal derivative must contain one value per boundary face."),
        (dict(boundary_pressure=np.zeros(4)), "BEM boundary traces must be complex arrays."),
        (dict(frequency_hz=0.0), "Exterior field frequency must be finite and greater than zero."),
        (dict(frequency_hz=float("nan")), "Exterior field frequency must be finite and greater than zero."),
        (dict(sound_speed_m_per_s=-1.0), "Exterior-region sound speed must be finite and greater than zero."),
        (dict(symmetry="z"), "Exterior field symmetry must be off, x, or xy."),
        (dict(domain_key="  "), "Exterior field requests require a non-empty domain cache key."),
    ],
)
def test_validation_messages(over, message):
    with pytest.raises(ValueError) as exc:
        cf.validated_evaluation_request(_request(**over))
    assert str(exc.value) == message


def test_precision_from_trace_dtype():
    s, a = cf.validated_evaluation_request(_request())
    assert s["precision"] == "float32" and a["boundary_pressure"].dtype == np.complex64
    r = _request(boundary_pressure=np.zeros(4, np.complex128), boundary_normal_derivative=np.zeros(2, np.complex128))
    s, a = cf.validated_evaluation_request(r)
    assert s["precision"] == "float64" and a["boundary_normal_derivative"].dtype == np.complex128
    assert s["quadrature_order"] == 2 and a["points_m"].dtype == np.float32 and a["boundary_triangles"].dtype == np.int64


def test_wire_round_trip(tmp_path):
    req = _request(symmetry="XY")
    path = tmp_path / "request.json"
    cf.write_evaluation_request(path, req)
    payload = json.loads(path.read_text())
    assert payload["binary_array_schema_version"] == 1 and payload["binary_result_file"] == "field-result.bin"
    assert set(payload["binary_arrays"]) == {"points_m", "boundary_points_m", "boundary_triangles",
                                             "boundary_pressure", "boundary_normal_derivative"}
    scalars, arrays = cf.request_from_wire(payload, path)
    assert scalars["symmetry"] == "xy" and scalars["precision"] == "float32" and scalars["domain_key"] == "enclosure-1"
    np.testing.assert_array_equal(arrays["points_m"], np.asarray(req.points_m, np.float32))
    np.testing.assert_array_equal(arrays["boundary_triangles"], req.boundary_triangles)
    np.testing.assert_array_equal(arrays["boundary_pressure"], req.boundary_pressure)
    values = (np.arange(5) + 1j).astype(np.complex64)
    desc = cf.write_binary_result(payload, path, values)
    assert desc["dtype"] == "complex64" and desc["shape"] == [5] and desc["nbytes"] == 40
    np.testing.assert_array_equal(cf.read_binary_array(tmp_path, desc), values)


def test_wire_rejections(tmp_path):
    path = tmp_path / "request.json"
    cf.write_evaluation_request(path, _request())
    payload = json.loads(path.read_text())
    with pytest.raises(RuntimeError, match="schema"):
        cf.request_from_wire({**payload, "binary_array_schema_version": 2}, path)
    bad = json.loads(json.dumps(payload))
    bad["binary_arrays"]["points_m"]["file"] = "../x.bin"
    with pytest.raises(RuntimeError, match="path"):
        cf.request_from_wire(bad, path)
    bad = json.loads(json.dumps(payload))
    bad["binary_arrays"]["points_m"]["nbytes"] += 4
    with pytest.raises(RuntimeError, match="metadata"):
        cf.request_from_wire(bad, path)
    bad = json.loads(json.dumps(payload))
    del bad["binary_arrays"]["boundary_pressure"]
    with pytest.raises(RuntimeError, match="boundary_pressure"):
        cf.request_from_wire(bad, path)
    with pytest.raises(RuntimeError, match="quadrature order"):
        cf.request_from_wire({**payload, "quadrature_order": 4}, path)
    with pytest.raises(RuntimeError, match="result path"):
        cf.write_binary_result({"binary_result_file": "a/b.bin"}, path, np.zeros(1, np.complex64))


def test_backend_id_checked():
    with pytest.raises(ValueError, match="gb300_cuda"):
        cf.evaluate_bem_field(_request(), backend_id="beat_cpu")
