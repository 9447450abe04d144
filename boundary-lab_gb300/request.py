"""Host side of an exterior solve request: the reference's solver.jl request
handling, restated for the GB300 backend.

Everything here runs on the host once per job or once per frequency on small
vectors; the heavy per-frequency numerics go through the C ABI.  Function
names follow solver.jl so the mapping is direct (all line numbers refer to
src/blab/solvers/julia_local/solver.jl):

  mesh_inputs_from_config         :152-179   radiator_inputs_from_config :185-233
  channel_inputs_from_config      :235-250   validate_crossover_config   :50-68
  butterworth_poles / _response   :271-291   crossover_response          :293-309
  channel_drive                   :311-318   polar_observation_points    :320-348
  spherical_observation           :350-388   drive_for_radiator          :390-406
  radiator_faces                  :408-410, 420-432, 450-458
  pressure_to_spl                 :488-490   complex_rows_to_wire        :492-497
  interpolate_complex_reference   :499-525   flat_target_corrections     :527-544
  synthesize_channel_basis        :546-588   channel_unit_drives         :590-597
  radiator_drives_from_channel_basis :599-605
  impedance_for_radiators         :607-631   regular_quadrature_mode     :93-101

The reference evaluates these in Float32 (FloatType = Float32, solver.jl:694)
and ships Float32 on the wire; here they are evaluated in float64 and rounded
to float32 where the reference's wire format is float32.
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Any, Iterable

import numpy as np


class RequestError(ValueError):
    """Invalid solve request (the reference raises these as Julia errors -> `failed` events)."""


def get_value(raw: dict, key: str, default=None):
    return raw[key] if isinstance(raw, dict) and key in raw and raw[key] is not None else default


# --------------------------------------------------------------- config ----


def validate_crossover_config(owner: str, crossover) -> None:
    if crossover is None:
        return
    ctype = str(get_value(crossover, "type", "none")).lower()
    if ctype not in ("none", "lowpass", "highpass"):
        raise RequestError(f"{owner} crossover type must be none, lowpass, or highpass.")
    if ctype == "none":
        return
    freq = get_value(crossover, "frequency_hz", None)
    if freq is None or not float(freq) > 0.0:
        raise RequestError(f"{owner} crossover frequency_hz must be > 0.")
    filt = str(get_value(crossover, "filter", "butterworth")).lower()
    if filt not in ("butterworth", "linkwitz_riley"):
        raise RequestError(f"{owner} crossover filter must be butterworth or linkwitz_riley.")
    order = int(get_value(crossover, "order", 1))
    if order not in (1, 2, 4, 6):
        raise RequestError(f"{owner} crossover order must be 1, 2, 4, or 6.")
    if filt == "linkwitz_riley" and order not in (2, 4, 6):
        raise RequestError(f"{owner} Linkwitz-Riley order must be 2, 4, or 6.")


def symmetry_mode_from_config(config: dict) -> str:
    mode = str(get_value(config, "symmetry", "off")).strip().lower()
    if mode not in ("off", "x", "xy"):
        raise RequestError(f"Unsupported symmetry mode: {mode}. Expected off, x, or xy.")
    return mode


def regular_quadrature_mode(config: dict) -> str:
    """GPU backends support the fixed rule only (solver.jl:93-101)."""
    mode = str(get_value(config, "regular_quadrature_mode", get_value(config, "quadrature_mode", "fixed"))).strip().lower()
    if mode not in ("fixed", "wavelength"):
        raise RequestError(f"Unsupported regular quadrature mode: {mode}. Expected fixed or wavelength.")
    if mode == "wavelength":
        raise RequestError("Wavelength-driven regular quadrature is currently implemented only for the BEAT CPU backend.")
    return mode


@dataclass
class MeshInput:
    path: str
    scale: float
    name: str
    translation: tuple[float, float, float]


def mesh_inputs_from_config(config: dict) -> list[MeshInput]:
    meshes = get_value(config, "meshes", []) or []
    if meshes:
        out, seen = [], set()
        for index, mesh in enumerate(meshes, start=1):
            name = str(get_value(mesh, "name", f"mesh_{index}"))
            if name in seen:
                raise RequestError(f"Duplicate mesh name: {name}")
            seen.add(name)
            translation = get_value(mesh, "translation_m", [0.0, 0.0, 0.0])
            if len(translation) != 3:
                raise RequestError(f"Mesh '{name}' translation_m must contain three values.")
            out.append(MeshInput(
                str(mesh["file"]),
                float(get_value(mesh, "scale_factor", get_value(config, "scale_factor", 0.001))),
                name,
                tuple(float(t) for t in translation),
            ))
        return out
    if "mesh_file" not in config or not config["mesh_file"]:
        raise RequestError("config must provide mesh_file or meshes")
    return [MeshInput(str(config["mesh_file"]), float(get_value(config, "scale_factor", 0.001)), "mesh", (0.0, 0.0, 0.0))]


def _crossover_dict(raw) -> dict:
    return dict(raw) if isinstance(raw, dict) else {"type": "none"}


def radiator_inputs_from_config(config: dict, mesh_inputs: list[MeshInput]) -> list[dict]:
    raw = get_value(config, "radiators", []) or []
    lookup = {m.name: i + 1 for i, m in enumerate(mesh_inputs)}
    if not raw:
        return [{
            "name": "Radiator", "tag": int(get_value(config, "tag_throat", 2)), "mesh": mesh_inputs[0].name,
            "mesh_id": 1, "channel": "main", "velocity_offset_db": 0.0, "level_db": 0.0, "polarity": 1,
            "delay_ms": 0.0, "hpf": {"type": "none"}, "lpf": {"type": "none"},
        }]
    out = []
    for radiator in raw:
        name = str(get_value(radiator, "name", "Radiator"))
        mesh_name = get_value(radiator, "mesh", None)
        if mesh_name is None:
            if len(mesh_inputs) != 1:
                raise RequestError(f"Radiator '{name}' must specify 'mesh' when multiple meshes are configured.")
            mesh_name = mesh_inputs[0].name
        mesh_name = str(mesh_name)
        if mesh_name not in lookup:
            raise RequestError(f"Radiator '{name}' references unknown mesh '{mesh_name}'.")
        validate_crossover_config(name, get_value(radiator, "hpf", None))
        validate_crossover_config(name, get_value(radiator, "lpf", None))
        out.append({
            "name": name, "tag": int(radiator["tag"]), "mesh": mesh_name, "mesh_id": lookup[mesh_name],
            "channel": str(get_value(radiator, "channel", "main")),
            "velocity_offset_db": float(get_value(radiator, "velocity_offset_db", 0.0)),
            "level_db": float(get_value(radiator, "level_db", 0.0)),
            "polarity": int(get_value(radiator, "polarity", 1)),
            "delay_ms": float(get_value(radiator, "delay_ms", 0.0)),
            "hpf": _crossover_dict(get_value(radiator, "hpf", {"type": "none"})),
            "lpf": _crossover_dict(get_value(radiator, "lpf", {"type": "none"})),
        })
    return out


def channel_inputs_from_config(config: dict) -> dict[str, dict]:
    channels = {}
    for channel in get_value(config, "channels", []) or []:
        name = str(channel["name"])
        validate_crossover_config(f"channel {name}", get_value(channel, "hpf", None))
        validate_crossover_config(f"channel {name}", get_value(channel, "lpf", None))
        channels[name] = {
            "level_db": float(get_value(channel, "level_db", 0.0)),
            "polarity": int(get_value(channel, "polarity", 1)),
            "delay_ms": float(get_value(channel, "delay_ms", 0.0)),
            "hpf": _crossover_dict(get_value(channel, "hpf", {"type": "none"})),
            "lpf": _crossover_dict(get_value(channel, "lpf", {"type": "none"})),
        }
    return channels


def validate_radiator_channels(radiators: list[dict], channels: dict) -> None:
    if not channels:
        return
    for radiator in radiators:
        if radiator.get("channel", "main") not in channels:
            raise RequestError(f"Radiator '{radiator['name']}' references unknown channel '{radiator['channel']}'.")


# ------------------------------------------------------------ crossovers ----


def butterworth_poles(order: int) -> np.ndarray:
    k = np.arange(1, order + 1)
    return np.exp(1j * (np.pi / 2 + (2 * k - 1) * np.pi / (2 * order)))


def butterworth_response(ctype: str, order: int, cutoff_hz: float, freq: float) -> complex:
    omega = 2 * np.pi * freq
    omega_c = 2 * np.pi * float(cutoff_hz)
    s = 1j * omega
    response = 1.0 + 0j
    for pole in butterworth_poles(order):
        if ctype == "lowpass":
            sp = omega_c * pole
            response *= (-sp) / (s - sp)
        else:
            sp = omega_c / pole
            response *= s / (s - sp)
    return complex(response)


def crossover_response(crossover, freq: float) -> complex:
    if crossover is None:
        return 1.0 + 0j
    ctype = str(get_value(crossover, "type", "none")).lower()
    if ctype == "none":
        return 1.0 + 0j
    filt = str(get_value(crossover, "filter", "butterworth")).lower()
    order = int(get_value(crossover, "order", 1))
    cutoff = get_value(crossover, "frequency_hz", None)
    if cutoff is None:
        raise RequestError(f"Crossover frequency_hz must be set for {ctype}.")
    if filt == "linkwitz_riley":
        section = butterworth_response(ctype, order // 2, cutoff, freq)
        return section * section
    return butterworth_response(ctype, order, cutoff, freq)


def channel_drive(channel: dict, freq: float) -> complex:
    omega = 2 * np.pi * freq
    level = 10.0 ** (float(channel["level_db"]) / 20.0)
    delay = np.exp(-1j * omega * float(channel["delay_ms"]) / 1000.0)
    xo = crossover_response(channel.get("hpf"), freq) * crossover_response(channel.get("lpf"), freq)
    return complex(float(channel["polarity"]) * level * delay * xo)


def drive_for_radiator(radiator: dict, channels: dict, freq: float) -> complex:
    channel = channels.get(radiator.get("channel", "main"))
    if channel is not None:
        return channel_drive(channel, freq) * 10.0 ** (float(radiator["velocity_offset_db"]) / 20.0)
    omega = 2 * np.pi * freq
    level = 10.0 ** ((float(radiator["level_db"]) + float(radiator["velocity_offset_db"])) / 20.0)
    delay = np.exp(-1j * omega * float(radiator["delay_ms"]) / 1000.0)
    xo = crossover_response(radiator.get("hpf"), freq) * crossover_response(radiator.get("lpf"), freq)
    return complex(float(radiator["polarity"]) * level * delay * xo)


# ---------------------------------------------------------- observations ----


def polar_observation_points(config: dict):
    """(angles float32, horizontal (n,3), vertical (n,3), on_axis_idx) of solver.jl:320-348."""
    step = float(get_value(config, "step_size", 5.0))
    amin = float(get_value(config, "min_angle", -180.0))
    amax = float(get_value(config, "max_angle", 180.0))
    if step <= 0:
        raise RequestError("step_size must be positive.")
    if amin < -180 or amax > 180:
        raise RequestError("polar angle range must stay within [-180, 180] degrees.")
    if amax < amin:
        raise RequestError("max_angle must be >= min_angle.")
    if not (amin <= 0 <= amax):
        raise RequestError("polar angle range must include 0 degrees.")
    # Julia range(a, stop=b, step=s): a + i*s for i = 0..floor((b-a)/s)
    count = int(math.floor((amax - amin) / step + 1e-10)) + 1
    angles = (amin + step * np.arange(count)).astype(np.float32)
    if angles.size == 0 or angles[-1] < np.float32(amax):
        angles = np.append(angles, np.float32(amax))
    angles = np.clip(angles, np.float32(amin), np.float32(amax)).astype(np.float32)
    distance = float(get_value(config, "distance", 2.0))
    if distance <= 0:
        raise RequestError("distance must be positive.")
    offset = float(get_value(config, "axial_offset", 0.0))
    rad = np.pi * angles.astype(np.float64) / 180.0
    horizontal = np.stack([distance * np.sin(rad), np.zeros_like(rad), distance * np.cos(rad) + offset], axis=1)
    vertical = np.stack([np.zeros_like(rad), distance * np.sin(rad), distance * np.cos(rad) + offset], axis=1)
    on_axis = int(np.argmin(np.abs(angles.astype(np.float64))))
    return angles, horizontal, vertical, on_axis


def fibonacci_sphere(n: int, radius: float, axial_offset: float = 0.0) -> np.ndarray:
    i = np.arange(n, dtype=np.float64)
    z = 1.0 - (2.0 * i + 1.0) / n
    xy = np.sqrt(np.maximum(1.0 - z * z, 0.0))
    phi = i * (np.pi * (3.0 - np.sqrt(5.0)))
    return np.stack([radius * xy * np.cos(phi), radius * xy * np.sin(phi), radius * z + axial_offset], axis=1)


def spherical_observation(config: dict):
    """Fibonacci sphere points + wire metadata of solver.jl:350-388, or None when disabled."""
    if not bool(get_value(config, "spherical_sampling_enabled", False)):
        return None
    n = int(get_value(config, "spherical_sampling_points", 6000))
    if n <= 0:
        raise RequestError("spherical_sampling_points must be positive.")
    distance = float(get_value(config, "distance", 2.0))
    if distance <= 0:
        raise RequestError("distance must be positive.")
    offset = float(get_value(config, "axial_offset", 0.0))
    points = fibonacci_sphere(n, distance, offset)
    i = np.arange(n, dtype=np.float64)
    z_unit = 1.0 - (2.0 * i + 1.0) / n
    theta = np.arccos(np.clip(z_unit, -1.0, 1.0)).astype(np.float32)
    phi = np.mod(np.arctan2(points[:, 1], points[:, 0]), 2 * np.pi).astype(np.float32)
    meta = {
        "r_distance_m": np.full(n, distance, dtype=np.float32),
        "theta_polar_rad": theta,
        "phi_azimuth_rad": phi,
    }
    return points, meta


# ------------------------------------------------------------- radiators ----


def radiator_faces(radiator: dict, tags: np.ndarray, element_mesh_ids: np.ndarray) -> np.ndarray:
    """Faces driven by a radiator: matching physical tag on the radiator's own mesh."""
    return np.nonzero((tags == int(radiator["tag"])) & (element_mesh_ids == int(radiator["mesh_id"])))[0]


def validate_radiator_elements(radiators, tags, element_mesh_ids) -> None:
    for radiator in radiators:
        if radiator_faces(radiator, tags, element_mesh_ids).size == 0:
            raise RequestError(
                f"No elements found for radiator '{radiator['name']}' tag={int(radiator['tag'])} on mesh '{radiator['mesh']}'."
            )


def channel_unit_drives(radiators: list[dict], channel_name: str) -> np.ndarray:
    return np.array([
        10.0 ** (float(r["velocity_offset_db"]) / 20.0) if r.get("channel", "main") == channel_name else 0.0
        for r in radiators
    ], dtype=np.complex128)


def face_drive_pattern(radiators, unit_drives, n_faces, tags, element_mesh_ids) -> np.ndarray:
    """Per-face complex drive; later radiators overwrite earlier ones on shared faces (solver.jl:451-458)."""
    q = np.zeros(n_faces, np.complex128)
    for radiator, drive in zip(radiators, unit_drives):
        q[radiator_faces(radiator, tags, element_mesh_ids)] = drive
    return q


# -------------------------------------------------------- post-processing ----


def pressure_to_spl(pressure: np.ndarray) -> np.ndarray:
    with np.errstate(divide="ignore"):
        return (20.0 * np.log10(np.abs(pressure) / 20e-6)).astype(np.float32)


def complex_rows_to_wire(rows) -> dict:
    return {
        "real": [np.asarray(row).real.astype(np.float32).tolist() for row in rows],
        "imag": [np.asarray(row).imag.astype(np.float32).tolist() for row in rows],
    }


def interpolate_complex_reference(values, angles_deg, reference_angle_deg: float) -> complex:
    values = np.asarray(values)
    if values.size == 0:
        return 0j
    if values.size == 1:
        return complex(values[0])
    ref = math.fmod(float(reference_angle_deg) + 180.0, 360.0)
    if ref < 0:
        ref += 360.0
    ref -= 180.0
    angles = np.asarray(angles_deg, dtype=np.float64)
    vals = values.astype(np.complex128)
    if np.isclose(angles[0], -180.0) and np.isclose(angles[-1], 180.0):
        angles = angles[:-1]
        vals = vals[:-1]
    ext_a = np.concatenate([angles - 360.0, angles, angles + 360.0])
    ext_v = np.concatenate([vals, vals, vals])
    for i in range(len(ext_a) - 1):
        left, right = ext_a[i], ext_a[i + 1]
        if left <= ref <= right:
            if np.isclose(left, right):
                return complex(ext_v[i])
            frac = (ref - left) / (right - left)
            return complex(ext_v[i] * (1.0 - frac) + ext_v[i + 1] * frac)
    return complex(ext_v[int(np.argmin(np.abs(ext_a - ref)))])


def flat_target_corrections(channel_names, horizontal_rows, angles_deg, reference_angle_deg, flat_target: bool):
    corrections = {}
    for idx, name in enumerate(channel_names):
        if not flat_target:
            corrections[name] = 1.0
            continue
        ref = interpolate_complex_reference(horizontal_rows[idx], angles_deg, reference_angle_deg)
        mag = abs(ref)
        corrections[name] = 1.0 if mag <= 1e-12 else 1.0 / mag
    return corrections


DEFAULT_CHANNEL = {"level_db": 0.0, "polarity": 1, "delay_ms": 0.0, "hpf": {"type": "none"}, "lpf": {"type": "none"}}


@dataclass
class Synthesis:
    horizontal_spl: np.ndarray
    vertical_spl: np.ndarray
    horizontal_norm: np.ndarray
    vertical_norm: np.ndarray
    sphere_norm: np.ndarray | None
    corrections: dict
    weights: np.ndarray


def synthesize_channel_basis(channel_names, horizontal_rows, vertical_rows, sphere_rows, channels, freq,
                             angles_deg, reference_angle_deg, flat_target: bool) -> Synthesis:
    corrections = flat_target_corrections(channel_names, horizontal_rows, angles_deg, reference_angle_deg, flat_target)
    weights = np.array([channel_drive(channels.get(name, DEFAULT_CHANNEL), freq) * corrections[name]
                        for name in channel_names], dtype=np.complex128)
    hp = sum(np.asarray(horizontal_rows[i]) * weights[i] for i in range(len(channel_names)))
    vp = sum(np.asarray(vertical_rows[i]) * weights[i] for i in range(len(channel_names)))
    hs, vs = pressure_to_spl(hp), pressure_to_spl(vp)
    on_axis = int(np.argmin(np.abs(np.asarray(angles_deg, dtype=np.float64))))
    reference = hs[on_axis]
    sphere_norm = None
    if sphere_rows is not None:
        sp = sum(np.asarray(sphere_rows[i]) * weights[i] for i in range(len(channel_names)))
        sphere_norm = (pressure_to_spl(sp) - reference).astype(np.float32)
    return Synthesis(hs, vs, (hs - reference).astype(np.float32), (vs - reference).astype(np.float32), sphere_norm,
                     corrections, weights)


def radiator_drives_from_channel_basis(radiators, channels, freq, corrections) -> np.ndarray:
    return np.array([drive_for_radiator(r, channels, freq) * corrections.get(r.get("channel", "main"), 1.0)
                     for r in radiators], dtype=np.complex128)


def symmetry_reduction_factor(mode: str) -> int:
    return {"off": 1, "x": 2, "xy": 4}[mode]


def impedance_for_radiators(faces, areas, tags, element_mesh_ids, pressure, radiators, drives,
                            symmetry_mode: str = "off") -> list[list[float]]:
    scale = symmetry_reduction_factor(symmetry_mode)
    out = []
    for radiator, drive in zip(radiators, drives):
        if abs(drive) <= 0.0:
            out.append([float("nan"), float("nan")])
            continue
        idx = radiator_faces(radiator, tags, element_mesh_ids)
        f = faces[idx]
        p_avg = (pressure[f[:, 0]] + pressure[f[:, 1]] + pressure[f[:, 2]]) / 3.0
        force = np.sum(p_avg * areas[idx] * scale) * 10.0
        z = force / drive
        out.append([float(np.float32(z.real / 2)), float(np.float32(-z.imag / 2))])
    return out
