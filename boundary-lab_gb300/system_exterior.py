"""Physical-system exterior solve on the GB300 engine.

The reference's coupled worker takes a compiled physical system
(src/blab/system_contract.py: ``compiled_system`` with meshes, regions,
boundaries, components and excitation ports).  When the system has exactly one
unbounded air region and no bounded one, it runs its BEM-only branch
(src/blab/solvers/julia_local/coupled_solver.jl:1465-1493 dispatch,
``solve_exterior_request`` :267-569).  That branch:

* combines the region's BEM surface meshes and gives every source physical tag
  its own solver tag (``aggregate_bem_region`` :47-87,
  ``combine_boundary_meshes`` BeatEngineCore.jl:266-313);
* drives each excitation port's moving boundaries with normal velocity equal to
  their motion weight (``exterior_excitations`` :196-232, ``exterior_neumann``
  :234-243);
* per frequency, solves the Burton-Miller system once per port and answers the
  requested ``quantities``: ``exterior_pressure`` at given points,
  ``bem_boundary_pressure`` (P1 nodes), ``bem_boundary_neumann`` (faces),
  ``radiation_impedance`` per component.

``ExteriorSystemJob`` does the same with these differences:

* every port is solved against one LU factorisation per frequency;
* frequencies run in batches on the GPU;
* ``float32`` requests run the mixed form (FP32 assembly, FP64-refined LU), which is
  at least as accurate as the reference's FP32 solve, and answer in complex64.

Requests with bounded regions (interior FEM and coupled FEM-BEM) are rejected:
they are not the exterior BEM path.
"""

from __future__ import annotations

import os
import threading
import time
from dataclasses import dataclass, field
from typing import Any, Callable, Iterator

import numpy as np

from . import meshes as meshmod
from .engine import engine_from_env

SYSTEM_SOLVE_REQUEST_VERSION = 1
SYSTEM_RESULT_VERSION = 1
QUANTITIES = ("exterior_pressure", "bem_boundary_pressure", "bem_boundary_neumann", "radiation_impedance")


class SystemRequestError(ValueError):
    """A request the exterior path cannot run; the message is the reference's where it has one."""


class SystemJobCancelled(Exception):
    def __init__(self, solved_count: int):
        super().__init__(f"cancelled after {solved_count} frequencies")
        self.solved_count = solved_count


def object_by_id(items, object_id: str, label: str) -> dict:
    """coupled_solver.jl:17-22."""
    for item in items:
        if str(item["id"]) == object_id:
            return item
    raise SystemRequestError(f"Unknown {label} id: {object_id}")


def normalized_symmetry_mode(mode) -> str:
    """BeatEngineCore.jl:317-321."""
    text = str(mode).strip().lower()
    if text not in ("off", "x", "xy"):
        raise SystemRequestError(f"Unsupported symmetry mode: {mode}. Expected off, x, or xy.")
    return text


@dataclass
class BemRegion:
    mesh: meshmod.BoundaryMesh          # combined surface, tags = solver tags
    boundary_tag_by_id: dict[str, int]
    vertex_offset_by_mesh_id: dict[str, int]
    face_offset_by_mesh_id: dict[str, int]


def aggregate_bem_region(meshes, region: dict, boundaries) -> BemRegion:
    """The unbounded region's surfaces in one mesh; solver tags numbered from 1 in order of
    first appearance, mesh after mesh (coupled_solver.jl:40-87, BeatEngineCore.jl:266-313)."""
    mesh_ids = [str(m) for m in region.get("mesh_ids", [])]
    if not mesh_ids:
        raise SystemRequestError("Unbounded region must contain at least one BEM mesh.")
    resources = [object_by_id(meshes, mid, "mesh") for mid in mesh_ids]
    if not all(str(r["purpose"]) == "bem_surface" for r in resources):
        raise SystemRequestError("Unbounded region meshes must be BEM surfaces.")
    verts, faces, tags = [], [], []
    tag_maps: dict[str, dict[int, int]] = {}
    v_off, f_off = {}, {}
    next_tag, nv, nf = 1, 0, 0
    for mid, res in zip(mesh_ids, resources):
        part = meshmod.read_gmsh22(str(res["file"]), float(res["scale_to_m"]))
        translation = np.asarray(res.get("translation_m", (0.0, 0.0, 0.0)), dtype=np.float64)
        v_off[mid], f_off[mid] = nv, nf
        local: dict[int, int] = {}
        for t in part.tags.tolist():
            if t not in local:
                local[t] = next_tag
                next_tag += 1
        tag_maps[mid] = local
        verts.append(part.vertices + translation)
        faces.append(part.faces + nv)
        tags.append(np.asarray([local[t] for t in part.tags.tolist()], dtype=np.int32))
        nv += len(part.vertices)
        nf += len(part.faces)
    combined = meshmod.BoundaryMesh(np.vstack(verts), np.vstack(faces), np.concatenate(tags))
    boundary_tag_by_id: dict[str, int] = {}
    for boundary in boundaries:
        if str(boundary["region_id"]) != str(region["id"]):
            continue
        bid = str(boundary["id"])
        group = boundary["group"]
        mid = str(group["mesh_id"])
        if mid not in tag_maps:
            raise SystemRequestError(f"Exterior boundary {bid!r} references mesh {mid!r} outside its unbounded "
                                     "region.")
        source_tag = int(group["tag"])
        solver_tag = tag_maps[mid].get(source_tag, 0)
        if solver_tag <= 0:
            raise SystemRequestError(f"Exterior boundary {bid!r} tag {source_tag} is not present in BEM mesh "
                                     f"{mid!r}.")
        boundary_tag_by_id[bid] = solver_tag
    return BemRegion(combined, boundary_tag_by_id, v_off, f_off)


@dataclass
class Excitation:
    port_id: str
    component_id: str
    tags: list[int]
    amplitudes: list[float]


def exterior_excitations(port_ids, ports, components, boundaries, boundary_tag_by_id: dict[str, int],
                         region: dict) -> list[Excitation]:
    """One normal-velocity excitation per port: the moving boundaries of its ideal velocity
    source, each at its motion weight (coupled_solver.jl:196-232)."""
    out = []
    for port_id in port_ids:
        port = object_by_id(ports, port_id, "excitation port")
        if str(port["kind"]) != "normal_velocity":
            raise SystemRequestError(f"Exterior excitation port {port_id} must be a normal-velocity port.")
        component = object_by_id(components, str(port["component_id"]), "component")
        if str(component["kind"]) != "ideal_velocity_source":
            raise SystemRequestError(f"Exterior excitation port {port_id} must reference an ideal velocity source.")
        weights = (component.get("parameters") or {}).get("boundary_motion_weights", {}) or {}
        tags, amps = [], []
        for bid in [str(b) for b in component.get("boundary_ids", [])]:
            boundary = object_by_id(boundaries, bid, "boundary")
            if str(boundary["region_id"]) != str(region["id"]):
                raise SystemRequestError(f"Exterior component {str(component['id'])!r} references a boundary "
                                         "outside its region.")
            if str(boundary["kind"]) != "moving":
                continue
            tag = boundary_tag_by_id.get(bid, 0)
            if tag <= 0:
                raise SystemRequestError(f"Exterior moving boundary {bid} did not resolve to a BEM tag.")
            amp = float(weights.get(bid, 1.0))
            if not (np.isfinite(amp) and amp > 0.0):
                raise SystemRequestError("Exterior boundary motion weights must be finite and positive.")
            tags.append(tag)
            amps.append(amp)
        if not tags:
            raise SystemRequestError(f"Exterior component {str(component['id'])!r} has no moving boundaries.")
        out.append(Excitation(port_id, str(component["id"]), tags, amps))
    return out


def excitation_drive(mesh: meshmod.BoundaryMesh, excitation: Excitation) -> np.ndarray:
    """Normal velocity per face (the Neumann datum is i rho omega times this, coupled_solver.jl:234-243);
    a face matched by several boundaries takes the last one's weight."""
    drive = np.zeros(mesh.n_faces, dtype=np.complex128)
    for tag, amp in zip(excitation.tags, excitation.amplitudes):
        drive[mesh.tags == tag] = amp
    return drive


@dataclass
class QuadratureSelection:
    order: int
    mode: str


def exterior_quadrature_selection(options: dict, mesh: meshmod.BoundaryMesh, frequency_hz: float,
                                  sound_speed: float, base_order: int, backend: str) -> QuadratureSelection:
    """Regular rule order for one frequency (coupled_solver.jl:161-194): the base order, or with
    ``wavelength`` mode (CPU backend only) order 1 / 2 / base by k h, h = sqrt of a statistic of
    the face areas."""
    default_mode = "wavelength" if backend == "cpu" else "fixed"
    mode = str(options.get("regular_quadrature_mode", default_mode)).lower()
    if mode not in ("fixed", "wavelength"):
        raise SystemRequestError(f"Unsupported regular quadrature mode: {mode}. Expected fixed or wavelength.")
    if backend != "cpu" and mode != "fixed":
        raise SystemRequestError("Wavelength-driven regular quadrature is currently available only on the CPU "
                                 "backend.")
    if mode == "fixed":
        return QuadratureSelection(base_order, mode)
    stat = str(options.get("wavelength_mesh_stat", "p90")).lower()
    areas = np.asarray(mesh.areas, dtype=np.float64)
    if stat == "median":
        area = float(np.median(areas))
    elif stat in ("p75", "p90"):
        area = float(np.quantile(areas, 0.75 if stat == "p75" else 0.90))
    elif stat == "max":
        area = float(np.max(areas))
    else:
        raise SystemRequestError(f"Unsupported wavelength mesh stat: {stat}.")
    kh = float(2.0 * np.pi * frequency_hz / sound_speed) * np.sqrt(area)
    q1 = float(options.get("wavelength_kh_q1_max", 0.0))
    q2 = float(options.get("wavelength_kh_q2_max", 2.0))
    if q1 < 0.0:
        raise SystemRequestError("wavelength_kh_q1_max must be non-negative.")
    if not q2 > q1:
        raise SystemRequestError("wavelength_kh_q2_max must exceed wavelength_kh_q1_max.")
    return QuadratureSelection(1 if kh <= q1 else 2 if kh <= q2 else base_order, mode)


def component_impedance(mesh: meshmod.BoundaryMesh, pressure: np.ndarray, excitation: Excitation,
                        symmetry: str) -> complex:
    """Radiation impedance of one component (coupled_solver.jl:254-265): F = sum over its faces
    of mean vertex pressure x area, times the symmetry factor and 10; Z = (Re F, -Im F) / 2."""
    sel = np.isin(mesh.tags, np.asarray(excitation.tags, dtype=np.int32))
    f = mesh.faces[sel]
    p_avg = (pressure[f[:, 0]] + pressure[f[:, 1]] + pressure[f[:, 2]]) / 3.0
    force = np.sum(p_avg * mesh.areas[sel]) * {"off": 1, "x": 2, "xy": 4}[symmetry] * 10.0
    return complex(force.real / 2.0, -force.imag / 2.0)


def complex_array_wire(values, complex_dtype) -> dict:
    """{"dtype", "shape", "real", "imag"}, values row-major (coupled_solver.jl:125-142)."""
    arr = np.asarray(values).astype(complex_dtype)
    return {"dtype": np.dtype(complex_dtype).name, "shape": list(arr.shape),
            "real": arr.real.ravel().tolist(), "imag": arr.imag.ravel().tolist()}


def quantity_wire(output: dict, values, unit: str, axes: list[str], complex_dtype, metadata=None) -> dict:
    """coupled_solver.jl:144-154."""
    targets = output.get("target_ids") or []
    return {"id": str(output["id"]), "quantity": str(output["quantity"]), "unit": unit,
            "target_id": None if not targets else str(targets[0]), "axes": axes,
            "values": complex_array_wire(values, complex_dtype), "metadata": metadata or {}}


class ExteriorSystemJob:
    """One exterior physical-system request: validation at construction, solve per frequency in
    ``results()`` (yields the reference's result dicts)."""

    def __init__(self, request: dict, *, engine_factory: Callable | None = None, device: int = 0,
                 batch: int = 0, chunk: int = 16):
        if int(request.get("schema_version", 0)) != SYSTEM_SOLVE_REQUEST_VERSION:
            raise SystemRequestError("Unsupported system solve request schema.")
        self.request = request
        self.cancel_path = request.get("cancel_path")
        system = request["compiled_system"]
        regions = system.get("regions", [])
        bounded = [r for r in regions if str(r["kind"]) == "bounded_air"]
        unbounded = [r for r in regions if str(r["kind"]) == "unbounded_air"]
        if not unbounded:
            raise SystemRequestError("Interior FEM systems (bounded regions only) are not part of the exterior BEM "
                                     "path this backend serves.")
        if len(unbounded) != 1:
            raise SystemRequestError("Coupled backend currently requires exactly one unbounded region.")
        if bounded:
            raise SystemRequestError("Coupled FEM-BEM systems (bounded and unbounded regions) are not part of the "
                                     "exterior BEM path this backend serves.")
        self.system = system
        self.region = unbounded[0]
        options = request.get("solver_options") or {}
        self.options = options
        precision = str(options.get("precision", "float32")).lower()
        if precision not in ("float32", "float64"):
            raise SystemRequestError("Exterior precision must be float32 or float64.")
        self.precision_name = precision
        self.complex_dtype = np.complex64 if precision == "float32" else np.complex128
        self.engine_precision = "mixed" if precision == "float32" else "fp64"
        backend = str(options.get("bem_backend", "cpu")).lower()
        if backend not in ("cpu", "cuda", "rocm"):
            raise SystemRequestError("Exterior BEM backend must be cpu, cuda, or rocm.")
        self.bem_backend = backend
        self.symmetry = normalized_symmetry_mode(options.get("symmetry", "off"))
        dtype = np.float32 if precision == "float32" else np.float64
        self.sound_speed = float(dtype(self.region["sound_speed_m_per_s"]))
        self.density = float(dtype(self.region["density_kg_per_m3"]))
        if not (self.sound_speed > 0.0 and self.density > 0.0):
            raise SystemRequestError("Exterior sound speed and density must be positive.")
        self.port_ids = [str(p) for p in request.get("excitation_port_ids", [])]
        self.frequencies = np.asarray(request.get("frequencies_hz", []), dtype=dtype).reshape(-1)
        self.outputs = list(request.get("outputs", []) or [])
        for output in self.outputs:
            q = str(output["quantity"])
            if q not in QUANTITIES:
                raise SystemRequestError(f"Unsupported exterior output quantity: {q}")
            if q == "exterior_pressure" and not (output.get("options") or {}).get("points_m"):
                raise SystemRequestError("exterior_pressure output requires options.points_m.")
        self.base_order = int(options.get("quadrature_order", 4))
        self.singular_order = int(options.get("singular_order", 4))
        self.engine_factory = engine_factory or engine_from_env
        self.device = device
        self.batch = batch
        self.chunk = chunk
        self.engines: dict[int, object] = {}
        self.mesh: meshmod.BoundaryMesh | None = None

    # --------------------------------------------------------------- setup --
    def setup(self) -> None:
        t0 = time.perf_counter()
        region = aggregate_bem_region(self.system.get("meshes", []), self.region, self.system.get("boundaries", []))
        mesh = meshmod.snap_symmetry_planes(region.mesh, self.symmetry)
        try:
            meshmod.validate_symmetry_fundamental_domain(mesh, self.symmetry)
        except ValueError as exc:
            raise SystemRequestError(str(exc)) from exc
        self.mesh = mesh
        self.excitations = exterior_excitations(self.port_ids, self.system.get("excitation_ports", []),
                                                self.system.get("components", []),
                                                self.system.get("boundaries", []), region.boundary_tag_by_id,
                                                self.region)
        self.drives = np.stack([excitation_drive(mesh, e) for e in self.excitations])
        # one observation set: the points of every exterior_pressure output, in output order
        self.point_slices: dict[str, slice] = {}
        pts = []
        n = 0
        for output in self.outputs:
            if str(output["quantity"]) == "exterior_pressure":
                p = np.asarray(output["options"]["points_m"], dtype=np.float64).reshape(-1, 3)
                self.point_slices[str(output["id"])] = slice(n, n + len(p))
                pts.append(p)
                n += len(p)
        # the engine needs one point at least; a far point stands in when no field is asked for
        self.points = np.vstack(pts) if pts else np.array([[0.0, 0.0, 1.0e3]])
        self.mesh_setup_s = time.perf_counter() - t0

    def _engine(self, order: int):
        if order not in self.engines:
            kwargs = {"device": self.device, "precision": self.engine_precision}
            if self.batch:
                kwargs["batch"] = self.batch
            engine = self.engine_factory(**kwargs)
            engine.prepare(self.mesh.vertices, self.mesh.faces, self.drives, self.points, order,
                           self.singular_order, symmetry=self.symmetry)
            self.engines[order] = engine
        return self.engines[order]

    def close(self) -> None:
        for engine in self.engines.values():
            engine.close()
        self.engines = {}

    def _cancel_requested(self, stop: Callable[[], bool] | None) -> bool:
        if stop is not None and stop():
            return True
        return bool(self.cancel_path) and os.path.isfile(str(self.cancel_path))

    # ------------------------------------------------------------- results --
    def results(self, stop: Callable[[], bool] | None = None) -> Iterator[dict]:
        """The result dict of each frequency in request order (coupled_solver.jl:361-549).
        Raises SystemJobCancelled when a cancel request is seen between frequencies."""
        if self._cancel_requested(stop):
            raise SystemJobCancelled(0)
        if self.mesh is None:
            self.setup()
        total = len(self.frequencies)
        selections = [exterior_quadrature_selection(self.options, self.mesh, float(f), self.sound_speed,
                                                    self.base_order, self.bem_backend) for f in self.frequencies]
        solved = 0
        while solved < total:
            if self._cancel_requested(stop):
                raise SystemJobCancelled(solved)
            order = selections[solved].order
            end = solved + 1
            while end < total and end - solved < self.chunk and selections[end].order == order:
                end += 1
            batch = self.frequencies[solved:end]
            res = self._engine(order).solve(batch.astype(np.float64), self.sound_speed, self.density)
            st = res.stats
            scale = 1.0 / len(batch)
            for i, freq in enumerate(batch):
                if i > 0 and self._cancel_requested(stop):
                    raise SystemJobCancelled(solved)
                t_post = time.perf_counter()
                quantities = self._quantities(float(freq), res.pressure[i], res.field[i])
                timings = {
                    "assembly_s": float(st.get("assembly_s", 0.0) * scale),
                    "solve_s": float(st.get("solve_s", 0.0) * scale),
                    "field_s": float(st.get("field_s", 0.0) * scale + time.perf_counter() - t_post),
                    "mesh_setup_s": float(self.mesh_setup_s) if solved == 0 else 0.0,
                    "cache_setup_s": 0.0,
                }
                sel = selections[solved]
                yield {
                    "schema_version": SYSTEM_RESULT_VERSION,
                    "freq_hz": float(freq),
                    "excitation_port_ids": list(self.port_ids),
                    "quantities": quantities,
                    "diagnostics": {
                        "precision": self.precision_name,
                        "bem_backend": self.bem_backend,
                        "symmetry": self.symmetry,
                        "formulation": "exterior_burton_miller_neumann",
                        "linear_solver": "gb300_dense_lu",
                        "bounded_region_count": 0,
                        "interface_count": 0,
                        "regular_quadrature_mode": sel.mode,
                        "regular_quadrature_order": sel.order,
                        "blas_threads": 1,
                        "engine": "gb300_cuda",
                        "engine_form": self.engine_precision,
                        "refine_steps": int(st.get("max_refine_steps", 0)),
                        "rel_residual": float(st.get("max_rel_residual", 0.0)),
                        "timings": timings,
                    },
                }
                solved += 1

    def _quantities(self, freq: float, pressure: np.ndarray, field: np.ndarray) -> list[dict]:
        """pressure [n_ports, n_vertices], field [n_ports, n_points] for one frequency."""
        omega = 2.0 * np.pi * freq
        out = []
        for output in self.outputs:
            q = str(output["quantity"])
            if q == "exterior_pressure":
                values = field[:, self.point_slices[str(output["id"])]]
                out.append(quantity_wire(output, values, "Pa", ["excitation", "observation"], self.complex_dtype,
                                         metadata={"points_m": output["options"]["points_m"]}))
            elif q == "bem_boundary_pressure":
                out.append(quantity_wire(output, pressure, "Pa", ["excitation", "bem_node"], self.complex_dtype))
            elif q == "bem_boundary_neumann":
                neumann = self.drives * (1j * self.density * omega)
                out.append(quantity_wire(output, neumann, "Pa/m", ["excitation", "bem_face"], self.complex_dtype))
            else:  # radiation_impedance, one value per component of the system
                by_component = {e.component_id: (e, pressure[i]) for i, e in enumerate(self.excitations)}
                values = []
                for component in self.system.get("components", []):
                    cid = str(component["id"])
                    if cid not in by_component:
                        raise SystemRequestError(f"radiation_impedance needs an excitation of component {cid!r}.")
                    e, p = by_component[cid]
                    values.append(component_impedance(self.mesh, p, e, self.symmetry))
                out.append(quantity_wire(output, np.asarray(values, dtype=np.complex128), "Pa*s/m^3", ["radiator"],
                                         self.complex_dtype))
        return out


def is_system_request(request: dict) -> bool:
    return isinstance(request, dict) and "compiled_system" in request


# ------------------------------------------------------ in-process backend --
# The reference's system-solver protocol (system_contract.py:41-108): a backend whose
# create_system_session(request) returns a session with ``metadata`` and
# ``solve_stream()`` yielding SystemFrequencyResult.  The reference's own classes are
# used when its package imports; these stand in otherwise.

@dataclass(frozen=True)
class QuantityResult:
    id: str
    quantity: str
    unit: str
    values: np.ndarray
    target_id: str | None = None
    axes: tuple = ()
    metadata: dict = field(default_factory=dict)


@dataclass(frozen=True)
class SystemFrequencyResult:
    freq_hz: float
    quantities: tuple
    excitation_port_ids: tuple = ()
    diagnostics: dict = field(default_factory=dict)


@dataclass(frozen=True)
class SystemSolveMetadata:
    system_id: str
    assumptions: tuple
    excitation_port_ids: tuple = ()
    available_quantity_ids: tuple = ()


def _reference_contract():
    try:
        import blab.system_contract as contract  # type: ignore  # noqa: PLC0415

        return contract
    except Exception:  # noqa: BLE001 - standalone use
        return None


def array_from_wire(raw: dict) -> np.ndarray:
    """The inverse of complex_array_wire (system_contract.py:372-386)."""
    dtype = np.dtype(str(raw["dtype"]))
    shape = tuple(int(v) for v in raw.get("shape", ()))
    if dtype.kind == "c":
        real_dtype = np.empty((), dtype=dtype).real.dtype
        values = (np.asarray(raw.get("real", ()), real_dtype) + 1j * np.asarray(raw.get("imag", ()), real_dtype))
        values = values.astype(dtype, copy=False)
    else:
        values = np.asarray(raw.get("real", ()), dtype=dtype)
    return values.reshape(shape)


def system_frequency_result_from_wire(raw: dict):
    ref = _reference_contract()
    if ref is not None:
        return ref.system_frequency_result_from_dict(raw)
    return SystemFrequencyResult(
        freq_hz=float(raw["freq_hz"]),
        quantities=tuple(QuantityResult(id=str(q["id"]), quantity=str(q["quantity"]), unit=str(q["unit"]),
                                        values=array_from_wire(q["values"]),
                                        target_id=None if q.get("target_id") is None else str(q["target_id"]),
                                        axes=tuple(str(a) for a in q.get("axes", ())),
                                        metadata=dict(q.get("metadata", {})))
                         for q in raw.get("quantities", ())),
        excitation_port_ids=tuple(str(v) for v in raw.get("excitation_port_ids", ())),
        diagnostics=dict(raw.get("diagnostics", {})),
    )


def system_request_to_wire(request) -> dict:
    """A SystemSolveRequest (the reference's dataclass) or its wire dict, as a wire dict."""
    if isinstance(request, dict):
        return dict(request)
    ref = _reference_contract()
    if ref is None:
        raise TypeError("a SystemSolveRequest object needs Boundary Lab's system_contract; pass the wire dict")
    return ref.system_solve_request_to_dict(request)


class Gb300SystemSession:
    def __init__(self, request, wire: dict, *, engine_factory: Callable | None, device: int, batch: int):
        self._stop = threading.Event()
        self._status = getattr(request, "status_callback", None)
        system = wire["compiled_system"]
        assumptions = (request.compiled_system.assumptions if not isinstance(request, dict)
                       else tuple(system.get("assumptions", ())))
        self._metadata = SystemSolveMetadata(system_id=str(system["id"]), assumptions=assumptions,
                                             excitation_port_ids=tuple(wire.get("excitation_port_ids", ())),
                                             available_quantity_ids=tuple(str(o["id"]) for o in wire.get("outputs",
                                                                                                      ())))
        try:
            self._job = ExteriorSystemJob(wire, engine_factory=engine_factory, device=device, batch=batch)
        except Exception as exc:
            raise RuntimeError(str(exc)) from exc

    @property
    def metadata(self) -> SystemSolveMetadata:
        return self._metadata

    def solve_stream(self, *, stop_requested: Callable[[], bool] | None = None) -> Iterator:
        def stop() -> bool:
            return self._stop.is_set() or (stop_requested is not None and stop_requested())

        try:
            for result in self._job.results(stop=stop):
                if stop():
                    return
                yield system_frequency_result_from_wire(result)
        except SystemJobCancelled:
            return
        except Exception as exc:
            raise RuntimeError(str(exc)) from exc
        finally:
            self._job.close()

    def stop(self) -> None:
        self._stop.set()


class Gb300SystemBackend:
    """Exterior physical-system solves on the GB300 (the exterior branch of the reference's
    PhysicalSystemProductionBackend, coupled_backend.py:811-843): the request's precision and
    BEM backend are set as that backend sets them, then the solve runs in-process."""

    backend_id = "gb300_cuda"
    label = "GB300 exterior BEM (physical system)"

    def __init__(self, *, precision: str = "float32", device: int = 0, batch: int = 0,
                 engine_factory: Callable | None = None, **_ignored: Any):
        self.precision = precision
        self.device = device
        self.batch = batch
        self.engine_factory = engine_factory

    def create_system_session(self, request) -> Gb300SystemSession:
        wire = system_request_to_wire(request)
        options = dict(wire.get("solver_options") or {})
        options["precision"] = self.precision
        options["bem_backend"] = "cuda"
        wire["solver_options"] = options
        return Gb300SystemSession(request, wire, engine_factory=self.engine_factory, device=self.device,
                                  batch=self.batch)

