"""One exterior solve job: the reference's solve_request_impl
(src/blab/solvers/julia_local/solver.jl:680-1020) on the GB300 engine.

``ExteriorJob`` turns a request dict (the JSON the reference's adapter writes,
beat_engine_backend.py:144-155) into the reference's event payloads:
``initialized`` metadata, ``status`` messages, one ``result`` payload per
frequency with exactly the fields of solver.jl:957-996, and the terminal
events.  The in-process backend session and the NDJSON worker both use it.

Differences from the reference, by design:
  * frequencies are solved in batches on the GPU (results are still emitted in
    request order, one event per frequency); cancellation is checked between
    batches and between emitted results;
  * every channel's excitation is solved against one LU factorisation per
    frequency (the reference refactors per channel, solver.jl:889-909).
Symmetry modes x / xy follow the reference: the combined mesh is snapped to
the symmetry planes and validated as a fundamental domain (solver.jl:718-719),
the operators, right-hand sides and field include the reflected images, and
impedance is scaled by the symmetry reduction factor (solver.jl:607-631).
"""

from __future__ import annotations

import os
import time
from typing import Callable, Iterator

import numpy as np

from . import meshes as meshmod
from . import request as rq
from .engine import engine_from_env

BACKEND_ID = "gb300_cuda"


class JobCancelled(Exception):
    def __init__(self, solved_count: int):
        super().__init__(f"cancelled after {solved_count} frequencies")
        self.solved_count = solved_count


class ExteriorJob:
    def __init__(self, request: dict, *, engine_factory: Callable | None = None,
                 status: Callable[[str], None] | None = None, precision: str = "mixed", device: int = 0,
                 batch: int = 0, admission=None):
        schema = int(rq.get_value(request, "schema_version", 1))
        if schema not in (1, 2):
            raise rq.RequestError(f"Unsupported solve request schema_version {schema}.")
        if "config" not in request:
            raise rq.RequestError("Solve request must include config.")
        self.config = request["config"]
        self.symmetry = rq.symmetry_mode_from_config(self.config)
        self.frequencies = np.asarray(request.get("frequencies_hz", []), dtype=np.float32).reshape(-1)
        if self.frequencies.size == 0:
            raise rq.RequestError("frequencies_hz must contain at least one frequency.")
        if not np.all(np.isfinite(self.frequencies)) or np.any(self.frequencies <= 0):
            raise rq.RequestError("frequencies_hz must contain only finite, positive values.")
        self.cancel_path = request.get("cancel_path")
        self.quadrature_mode = rq.regular_quadrature_mode(self.config)
        self.status = status or (lambda message: None)
        self.mesh_inputs = rq.mesh_inputs_from_config(self.config)
        self.radiators = rq.radiator_inputs_from_config(self.config, self.mesh_inputs)
        self.channels = rq.channel_inputs_from_config(self.config)
        rq.validate_radiator_channels(self.radiators, self.channels)
        self.angles, self.horizontal, self.vertical, self.on_axis = rq.polar_observation_points(self.config)
        self.sphere = rq.spherical_observation(self.config)
        self.channel_names = sorted({r.get("channel", "main") for r in self.radiators})
        self.rho = float(rq.get_value(self.config, "rho", 1.21))
        self.sound_speed = float(rq.get_value(self.config, "sound_speed", 343.0))
        self.flat_target = bool(rq.get_value(self.config, "flat_target_normalization_enabled", True))
        self.ref_angle = float(rq.get_value(self.config, "flat_target_reference_angle_deg", 0.0))
        self.regular_order = int(rq.get_value(self.config, "quadrature_order", 4))
        self.singular_order = int(rq.get_value(self.config, "singular_order", 4))
        self.precision = precision
        self.engine_factory = engine_factory or engine_from_env
        self.device = device
        self.batch = batch
        self.engine = None
        self.mesh = None
        # optional device-memory admission shared by concurrent jobs: acquire(bytes) -> token,
        # release(token); the job holds its footprint from setup to close
        self.admission = admission
        self._admitted = None

    # ------------------------------------------------------------ metadata --
    def initialized_payload(self) -> dict:
        return {
            "polar_angle_deg": [float(a) for a in self.angles],
            "radiator_names": [r["name"] for r in self.radiators],
            "sphere_metadata": None if self.sphere is None else {
                key: np.asarray(val, np.float32).tolist() for key, val in self.sphere[1].items()
            },
        }

    # --------------------------------------------------------------- setup --
    def setup(self) -> None:
        self.status(f"GB300 BEM loading {len(self.mesh_inputs)} mesh{'' if len(self.mesh_inputs) == 1 else 'es'}")
        parts = [meshmod.read_gmsh22(m.path, m.scale) for m in self.mesh_inputs]
        self.mesh = meshmod.combine_meshes(parts, [m.translation for m in self.mesh_inputs])
        self.mesh = meshmod.snap_symmetry_planes(self.mesh, self.symmetry)
        try:
            meshmod.validate_symmetry_fundamental_domain(self.mesh, self.symmetry)
        except ValueError as exc:
            raise rq.RequestError(str(exc)) from exc
        rq.validate_radiator_elements(self.radiators, self.mesh.tags, self.mesh.element_mesh_ids)
        drives = np.stack([
            rq.face_drive_pattern(self.radiators, rq.channel_unit_drives(self.radiators, name), self.mesh.n_faces,
                                  self.mesh.tags, self.mesh.element_mesh_ids)
            for name in self.channel_names
        ])
        parts_pts = [self.horizontal, self.vertical] + ([self.sphere[0]] if self.sphere is not None else [])
        self.points = np.vstack(parts_pts)
        self.status("Initializing GB300 BEM (mesh plan, singular moments)")
        kwargs = {"device": self.device, "precision": self.precision}
        if self.batch:
            kwargs["batch"] = self.batch
        self.engine = self.engine_factory(**kwargs)
        self.engine.prepare(self.mesh.vertices, self.mesh.faces, drives, self.points, self.regular_order,
                            self.singular_order, symmetry=self.symmetry)
        if self.admission is not None:
            footprint = getattr(self.engine, "device_bytes", None)
            need = int(footprint(len(self.frequencies))) if callable(footprint) else 0
            if need > self.admission.free_bytes():
                self.status("Waiting for GPU memory")
            self._admitted = self.admission.acquire(need)

    def close(self) -> None:
        if self.engine is not None:
            self.engine.close()
            self.engine = None
        if self._admitted is not None:
            self.admission.release(self._admitted)
            self._admitted = None

    def _cancel_requested(self, stop: Callable[[], bool] | None) -> bool:
        if stop is not None and stop():
            return True
        return bool(self.cancel_path) and os.path.isfile(str(self.cancel_path))

    # -------------------------------------------------------------- results --
    def results(self, stop: Callable[[], bool] | None = None, chunk: int | None = None) -> Iterator[dict]:
        """Yield the `result` event payload of each frequency in request order.
        Raises JobCancelled when a cancel request is seen between frequencies.
        ``chunk`` is the number of frequencies per engine call; by default the engine's
        preferred chunk (one full batch of the sweep), else 16."""
        if self.engine is None:
            self.setup()
        nh, nv = len(self.horizontal), len(self.vertical)
        total = len(self.frequencies)
        tune = getattr(self.engine, "tune_sweep", None)
        if callable(tune):  # the tuner sees the whole sweep, not its first chunk
            tune(self.frequencies.astype(np.float64), self.sound_speed, self.rho)
        if chunk is None:
            preferred = getattr(self.engine, "preferred_chunk", None)
            chunk = int(preferred(total)) if callable(preferred) else 16
        chunk = max(1, int(chunk))
        solved = 0
        while solved < total:
            if self._cancel_requested(stop):
                raise JobCancelled(solved)
            batch = self.frequencies[solved: solved + chunk]
            t0 = time.perf_counter()
            res = self.engine.solve(batch.astype(np.float64), self.sound_speed, self.rho)
            wall = time.perf_counter() - t0
            st = res.stats
            n = len(batch)
            device_total = st.get("assembly_s", 0.0) + st.get("solve_s", 0.0) + st.get("field_s", 0.0)
            scale = 1.0 / n
            for i, freq in enumerate(batch):
                if i > 0 and self._cancel_requested(stop):
                    raise JobCancelled(solved)
                t_post = time.perf_counter()
                payload = self._post_process(float(freq), res.pressure[i], res.field[i], nh, nv)
                post = time.perf_counter() - t_post
                payload["timings"] = {
                    "assembly_s": float(np.float32(st.get("assembly_s", wall) * scale)),
                    "solve_s": float(np.float32(st.get("solve_s", 0.0) * scale)),
                    "field_s": float(np.float32(st.get("field_s", 0.0) * scale + post)),
                }
                payload["diagnostics"] = {
                    "convergence_info": 0,
                    "message": ("GB300 dense LU, FP64 iterative refinement" if self.precision == "mixed"
                                else "GB300 dense LU (FP64)"),
                    "backend": BACKEND_ID,
                    "symmetry": self.symmetry,
                    "regular_assembly_mode": "gb300_fused_tiles",
                    "precision": self.precision,
                    "refine_steps": int(st.get("max_refine_steps", 0)),
                    "rel_residual": float(st.get("max_rel_residual", 0.0)),
                    "batch_wall_s": float(wall),
                    "batch_device_s": float(device_total),
                    "regular_quadrature_mode": self.quadrature_mode,
                    "regular_quadrature_order": self.regular_order,
                    "regular_quadrature_base_order": self.regular_order,
                }
                solved += 1
                yield {"solved_count": solved, "total_count": total, "result": payload}

    def _post_process(self, freq: float, pressure: np.ndarray, field: np.ndarray, nh: int, nv: int) -> dict:
        """Channel synthesis, SPL and impedance for one frequency (solver.jl:922-996)."""
        names = self.channel_names
        h_rows = [field[c, :nh] for c in range(len(names))]
        v_rows = [field[c, nh:nh + nv] for c in range(len(names))]
        s_rows = [field[c, nh + nv:] for c in range(len(names))] if self.sphere is not None else None
        syn = rq.synthesize_channel_basis(names, h_rows, v_rows, s_rows, self.channels, freq, self.angles,
                                          self.ref_angle, self.flat_target)
        drives = rq.radiator_drives_from_channel_basis(self.radiators, self.channels, freq, syn.corrections)
        mixed = sum(pressure[c] * syn.weights[c] for c in range(len(names)))
        impedance = rq.impedance_for_radiators(self.mesh.faces, self.mesh.areas, self.mesh.tags,
                                               self.mesh.element_mesh_ids, mixed, self.radiators, drives,
                                               self.symmetry)
        return {
            "freq_hz": float(np.float32(freq)),
            "horizontal_spl_norm_db": syn.horizontal_norm.tolist(),
            "vertical_spl_norm_db": syn.vertical_norm.tolist(),
            "impedance": impedance,
            "horizontal_spl_db": syn.horizontal_spl.tolist(),
            "vertical_spl_db": syn.vertical_spl.tolist(),
            "sphere_spl_norm_db": None if syn.sphere_norm is None else syn.sphere_norm.tolist(),
            "channel_names": list(names),
            "horizontal_pressure": rq.complex_rows_to_wire(h_rows),
            "vertical_pressure": rq.complex_rows_to_wire(v_rows),
            "sphere_pressure": None if s_rows is None else rq.complex_rows_to_wire(s_rows),
        }
