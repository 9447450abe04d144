"""Exterior-field evaluation from retained BEM boundary traces on the GB300 backend.

The reference evaluates the field of a physical-system solve's retained boundary
traces (P1 pressure per boundary node, DP0 normal derivative per boundary face)
through the Julia coupled worker's ``bem_field`` operation
(``src/blab/solvers/coupled_field.py:39-82``; the worker side is
``evaluate_bem_field_request`` / ``retained_bem_field_evaluation_cache``,
``src/blab/solvers/julia_local/coupled_solver.jl:2371-2497``).  This module keeps
that interface - the same request type, validation and messages, the same
binary-array files for the worker protocol, a cache of uploaded boundary meshes
keyed by the request's domain key (at most two, as the reference's
``MAX_BEM_FIELD_EVALUATION_CACHES``) - and evaluates on the GPU through
``bem_evaluate_field`` of the C ABI.

The reference sends coordinates as float32 and uses the 3-point rule
(``quadrature_order = 2``); both are kept.  complex128 traces select the plain
FP64 form, anything else the mixed form (compensated FP32 field, complex64
result), as the reference's float64 / float32 precision switch.
"""

from __future__ import annotations

import importlib
import threading
from collections import OrderedDict
from dataclasses import dataclass
from pathlib import Path
from typing import BinaryIO

import numpy as np

_FIELD_ARRAYS_FILENAME = "field-arrays.bin"
_FIELD_RESULT_FILENAME = "field-result.bin"
_BINARY_ARRAY_SCHEMA_VERSION = 1
_QUADRATURE_ORDER = 2  # the reference's retained-field rule (coupled_field.py payload)
_MAX_CACHED_DOMAINS = 2  # MAX_BEM_FIELD_EVALUATION_CACHES, coupled_solver.jl:15


def _native():
    return importlib.import_module(__name__.rsplit(".", 1)[0] + ".native")


@dataclass(frozen=True)
class BemFieldEvaluationRequest:
    domain_key: str
    points_m: np.ndarray
    boundary_points_m: np.ndarray
    boundary_triangles: np.ndarray
    boundary_pressure: np.ndarray
    boundary_normal_derivative: np.ndarray
    frequency_hz: float
    sound_speed_m_per_s: float
    symmetry: str = "off"


def validated_evaluation_request(request: BemFieldEvaluationRequest) -> tuple[dict[str, object], dict[str, np.ndarray]]:
    """The request as (scalars, arrays) in the reference's wire types, with its checks
    and messages (coupled_field.py:107-153)."""
    points = np.asarray(request.points_m, dtype=np.float32)
    boundary_points = np.asarray(request.boundary_points_m, dtype=np.float32)
    triangles = np.asarray(request.boundary_triangles, dtype=np.int64)
    pressure = np.asarray(request.boundary_pressure)
    normal = np.asarray(request.boundary_normal_derivative)
    if points.ndim != 2 or points.shape[1] != 3:
        raise ValueError("Exterior evaluation points must have shape (point, 3).")
    if boundary_points.ndim != 2 or boundary_points.shape[1] != 3:
        raise ValueError("BEM boundary points must have shape (bem_node, 3).")
    if triangles.ndim != 2 or triangles.shape[1] != 3:
        raise ValueError("BEM boundary triangles must have shape (bem_face, 3).")
    if pressure.shape != (boundary_points.shape[0],):
        raise ValueError("BEM boundary pressure must contain one value per boundary node.")
    if normal.shape != (triangles.shape[0],):
        raise ValueError("BEM boundary normal derivative must contain one value per boundary face.")
    if pressure.dtype.kind != "c" or normal.dtype.kind != "c":
        raise ValueError("BEM boundary traces must be complex arrays.")
    if not np.isfinite(request.frequency_hz) or request.frequency_hz <= 0.0:
        raise ValueError("Exterior field frequency must be finite and greater than zero.")
    if not np.isfinite(request.sound_speed_m_per_s) or request.sound_speed_m_per_s <= 0.0:
        raise ValueError("Exterior-region sound speed must be finite and greater than zero.")
    symmetry = str(request.symmetry).strip().lower()
    if symmetry not in {"off", "x", "xy"}:
        raise ValueError("Exterior field symmetry must be off, x, or xy.")
    dtype = np.result_type(pressure.dtype, normal.dtype)
    if dtype not in {np.dtype(np.complex64), np.dtype(np.complex128)}:
        dtype = np.dtype(np.complex64)
    domain_key = str(request.domain_key).strip()
    if not domain_key:
        raise ValueError("Exterior field requests require a non-empty domain cache key.")
    scalars = {
        "domain_key": domain_key,
        "frequency_hz": float(request.frequency_hz),
        "sound_speed_m_per_s": float(request.sound_speed_m_per_s),
        "symmetry": symmetry,
        "precision": "float64" if dtype == np.dtype(np.complex128) else "float32",
        "quadrature_order": _QUADRATURE_ORDER,
    }
    arrays = {
        "points_m": np.ascontiguousarray(points, dtype=np.dtype("<f4")),
        "boundary_points_m": np.ascontiguousarray(boundary_points, dtype=np.dtype("<f4")),
        "boundary_triangles": np.ascontiguousarray(triangles, dtype=np.dtype("<i8")),
        "boundary_pressure": np.ascontiguousarray(pressure, dtype=dtype.newbyteorder("<")),
        "boundary_normal_derivative": np.ascontiguousarray(normal, dtype=dtype.newbyteorder("<")),
    }
    return scalars, arrays


class FieldEvaluator:
    """Uploaded boundary meshes by domain key (least recently used first out)."""

    def __init__(self, device: int = 0, max_domains: int = _MAX_CACHED_DOMAINS):
        self.device = device
        self.max_domains = max_domains
        self._lock = threading.Lock()
        self._ctx = None
        self._meshes: OrderedDict[str, object] = OrderedDict()

    def _mesh(self, key: str, vertices: np.ndarray, triangles: np.ndarray, symmetry: str):
        native = _native()
        if self._ctx is None:
            native.load()
            self._ctx = native.Context(self.device)
        mesh = self._meshes.get(key)
        if mesh is not None:
            self._meshes.move_to_end(key)
            return mesh
        mesh = self._ctx.upload_mesh(vertices, triangles, regular_order=_QUADRATURE_ORDER, singular_order=1,
                                     symmetry=symmetry)
        self._meshes[key] = mesh
        while len(self._meshes) > self.max_domains:
            _, old = self._meshes.popitem(last=False)
            old.release()
        return mesh

    def evaluate(self, scalars: dict[str, object], arrays: dict[str, np.ndarray]) -> np.ndarray:
        """u(points) for validated scalars / arrays (validated_evaluation_request)."""
        native = _native()
        fp64 = scalars["precision"] == "float64"
        precision = native.BEM_PRECISION_FP64 if fp64 else native.BEM_PRECISION_MIXED
        key = f"{scalars['domain_key']}|{scalars['precision']}|{scalars['symmetry']}|q{scalars['quadrature_order']}"
        vertices = np.asarray(arrays["boundary_points_m"], np.float32).astype(np.float64)
        triangles = np.asarray(arrays["boundary_triangles"], np.int64).astype(np.int32)
        pressure = np.asarray(arrays["boundary_pressure"])
        normal = np.asarray(arrays["boundary_normal_derivative"])
        points = np.asarray(arrays["points_m"], np.float32).astype(np.float64)
        with self._lock:
            mesh = self._mesh(key, vertices, triangles, str(scalars["symmetry"]))
            if pressure.shape != (mesh.n_vertices,):
                raise RuntimeError("Retained BEM pressure does not align with boundary vertices.")
            if normal.shape != (mesh.n_faces,):
                raise RuntimeError("Retained BEM normal derivative does not align with boundary faces.")
            real = np.float64 if fp64 else np.float32
            k = real(2 * np.pi) * real(scalars["frequency_hz"]) / real(scalars["sound_speed_m_per_s"])
            values = mesh.evaluate_field(float(k), pressure, normal, points, precision)
        return values.astype(np.complex128 if fp64 else np.complex64)

    def release(self) -> None:
        with self._lock:
            for mesh in self._meshes.values():
                mesh.release()
            self._meshes.clear()
            self._ctx = None


_default_evaluator: FieldEvaluator | None = None
_default_lock = threading.Lock()


def _evaluator() -> FieldEvaluator:
    global _default_evaluator
    with _default_lock:
        if _default_evaluator is None:
            _default_evaluator = FieldEvaluator()
        return _default_evaluator


def evaluate_bem_field(request: BemFieldEvaluationRequest, *, backend_id: str = "gb300_cuda",
                       evaluator: FieldEvaluator | None = None) -> np.ndarray:
    """Evaluate one synthesized BEM response on arbitrary exterior points
    (coupled_field.py:39-82): complex [n_points], complex64 for float32 traces."""
    if str(backend_id).strip().lower() not in {"gb300_cuda", "gb300"}:
        raise ValueError("Retained BEM fields of this module run on the gb300_cuda backend.")
    scalars, arrays = validated_evaluation_request(request)
    values = (evaluator or _evaluator()).evaluate(scalars, arrays)
    if values.dtype.kind != "c" or values.shape != (np.asarray(request.points_m).shape[0],):
        raise RuntimeError("The field evaluation returned an invalid exterior pressure array.")
    return values


# ---------------------------------------------------------------- wire files --
# The coupled worker's binary arrays (coupled_field.py:155-233, coupled_solver.jl:2283-2339):
# a request JSON carries descriptors {file, offset, nbytes, dtype, shape, order, byte_order}
# of little-endian row-major arrays in one file beside it.


def write_binary_arrays(path: Path, arrays: dict[str, np.ndarray]) -> dict[str, dict[str, object]]:
    descriptors: dict[str, dict[str, object]] = {}
    with Path(path).open("wb") as handle:
        for name, values in arrays.items():
            array = np.ascontiguousarray(values)
            offset = handle.tell()
            _write_array_bytes(handle, array)
            descriptors[name] = {
                "file": Path(path).name,
                "offset": offset,
                "nbytes": int(array.nbytes),
                "dtype": array.dtype.name,
                "shape": list(array.shape),
                "order": "C",
                "byte_order": "little",
            }
    return descriptors


def _write_array_bytes(handle: BinaryIO, array: np.ndarray) -> None:
    view = memoryview(array)
    if not view.contiguous:
        raise ValueError("Binary field arrays must be contiguous.")
    handle.write(view.cast("B"))


_WIRE_DTYPES = {"float32", "float64", "int64", "complex64", "complex128"}


def read_binary_array(directory: Path, raw: object) -> np.ndarray:
    """One array of a request or result descriptor (checks of coupled_solver.jl:2283-2317)."""
    if not isinstance(raw, dict):
        raise RuntimeError("Invalid binary array descriptor.")
    filename = str(raw.get("file", ""))
    if not filename or Path(filename).name != filename:
        raise RuntimeError("Invalid binary array path.")
    if str(raw.get("order", "")) != "C" or str(raw.get("byte_order", "")) != "little":
        raise RuntimeError("Binary arrays must be little-endian and row-major.")
    try:
        name = str(raw["dtype"])
        if name not in _WIRE_DTYPES:
            raise ValueError(name)
        dtype = np.dtype(name).newbyteorder("<")
        shape = tuple(int(value) for value in raw["shape"])
        offset = int(raw.get("offset", 0))
        nbytes = int(raw["nbytes"])
    except (KeyError, TypeError, ValueError) as exc:
        raise RuntimeError("Invalid binary array descriptor.") from exc
    count = int(np.prod(shape, dtype=np.int64))
    if any(d < 0 for d in shape) or offset < 0 or nbytes != count * dtype.itemsize:
        raise RuntimeError("Inconsistent binary array metadata.")
    path = Path(directory) / filename
    if not path.is_file() or path.stat().st_size < offset + nbytes:
        raise RuntimeError("Incomplete binary array file.")
    return np.fromfile(path, dtype=dtype, count=count, offset=offset).reshape(shape)


def request_from_wire(request: dict, request_path: Path) -> tuple[dict[str, object], dict[str, np.ndarray]]:
    """(scalars, arrays) of a worker ``bem_field`` request JSON and its binary arrays."""
    if int(request.get("binary_array_schema_version", 0)) != _BINARY_ARRAY_SCHEMA_VERSION:
        raise RuntimeError("Unsupported BEM field binary-array schema.")
    descriptors = request.get("binary_arrays")
    if not isinstance(descriptors, dict):
        raise RuntimeError("BEM field request is missing binary-array metadata.")
    directory = Path(request_path).parent
    arrays = {}
    for name in ("points_m", "boundary_points_m", "boundary_triangles", "boundary_pressure",
                 "boundary_normal_derivative"):
        if name not in descriptors:
            raise RuntimeError(f"BEM field request is missing binary array {name!r}.")
        arrays[name] = read_binary_array(directory, descriptors[name])
    scalars = {
        "domain_key": str(request.get("domain_key", "")).strip(),
        "frequency_hz": float(request["frequency_hz"]),
        "sound_speed_m_per_s": float(request["sound_speed_m_per_s"]),
        "symmetry": str(request.get("symmetry", "off")).strip().lower(),
        "precision": str(request.get("precision", "float32")).lower(),
        "quadrature_order": int(request.get("quadrature_order", _QUADRATURE_ORDER)),
    }
    if not scalars["domain_key"]:
        raise RuntimeError("Exterior field request is missing its domain cache key.")
    if scalars["precision"] not in {"float32", "float64"}:
        raise RuntimeError("Exterior field precision must be float32 or float64.")
    if scalars["symmetry"] not in {"off", "x", "xy"}:
        raise RuntimeError("Exterior field symmetry must be off, x, or xy.")
    if scalars["quadrature_order"] != _QUADRATURE_ORDER:
        raise RuntimeError("Exterior field requests use quadrature order 2.")
    if not (scalars["frequency_hz"] > 0.0):
        raise RuntimeError("Exterior field frequency must be positive.")
    if not (scalars["sound_speed_m_per_s"] > 0.0):
        raise RuntimeError("Exterior field sound speed must be positive.")
    return scalars, arrays


def write_binary_result(request: dict, request_path: Path, values: np.ndarray) -> dict[str, object]:
    """The ``values_binary`` descriptor of a ``field_result`` event (coupled_solver.jl:2319-2339)."""
    filename = str(request.get("binary_result_file", ""))
    if not filename or Path(filename).name != filename:
        raise RuntimeError("BEM field request has an invalid binary result path.")
    array = np.ascontiguousarray(values)
    if array.dtype not in (np.dtype(np.complex64), np.dtype(np.complex128)):
        raise RuntimeError(f"Unsupported BEM field result precision: {array.dtype}")
    path = Path(request_path).parent / filename
    with path.open("wb") as handle:
        _write_array_bytes(handle, array.astype(array.dtype.newbyteorder("<"), copy=False))
    return {"file": filename, "offset": 0, "nbytes": int(array.nbytes), "dtype": array.dtype.name,
            "shape": list(array.shape), "order": "C", "byte_order": "little"}


def write_evaluation_request(request_path: Path, request: BemFieldEvaluationRequest) -> None:
    """The worker request files for a BemFieldEvaluationRequest (coupled_field.py:92-104)."""
    import json

    scalars, arrays = validated_evaluation_request(request)
    payload = dict(scalars)
    payload["bem_backend"] = "gb300"
    array_path = Path(request_path).with_name(_FIELD_ARRAYS_FILENAME)
    payload["binary_array_schema_version"] = _BINARY_ARRAY_SCHEMA_VERSION
    payload["binary_arrays"] = write_binary_arrays(array_path, arrays)
    payload["binary_result_file"] = _FIELD_RESULT_FILENAME
    Path(request_path).write_text(json.dumps(payload, separators=(",", ":")), encoding="utf-8")


__all__ = ["BemFieldEvaluationRequest", "FieldEvaluator", "evaluate_bem_field", "validated_evaluation_request",
           "request_from_wire", "write_binary_result", "write_evaluation_request", "read_binary_array",
           "write_binary_arrays"]
