"""The reference's solver-backend data contract (src/blab/solvers/base.py:13-110).

Whenever Boundary Lab's own package (``blab``) is importable at the moment a
class is looked up (``contract.FrequencyResult`` etc.), its class is used, so
sessions hand the application genuine ``FrequencyResult`` objects.  Otherwise
equivalent dataclasses with the same names and fields are used, so the backend
also runs standalone (for example on a GPU host without the application).
"""

from __future__ import annotations

from dataclasses import dataclass, field
from typing import Any, Callable

import numpy as np


@dataclass(frozen=True)
class _FrequencySolveTimings:
    assembly_s: float = 0.0
    solve_s: float = 0.0
    field_s: float = 0.0


@dataclass(frozen=True)
class _SolverDiagnostics:
    convergence_info: int | None = None
    message: str | None = None
    backend: str | None = None
    symmetry: str | None = None
    regular_assembly_mode: str | None = None


@dataclass(frozen=True)
class _FrequencyResult:
    freq_hz: float
    horizontal_spl_norm_db: np.ndarray
    vertical_spl_norm_db: np.ndarray
    impedance: np.ndarray
    horizontal_spl_db: np.ndarray | None = None
    vertical_spl_db: np.ndarray | None = None
    sphere_spl_norm_db: np.ndarray | None = None
    channel_names: np.ndarray | None = None
    horizontal_pressure: np.ndarray | None = None
    vertical_pressure: np.ndarray | None = None
    sphere_pressure: np.ndarray | None = None
    timings: _FrequencySolveTimings = field(default_factory=_FrequencySolveTimings)
    diagnostics: _SolverDiagnostics | None = None

    @property
    def has_channel_basis(self) -> bool:
        return self.channel_names is not None and self.horizontal_pressure is not None and self.vertical_pressure is not None


@dataclass(frozen=True)
class _SolveRequest:
    config: Any
    frequencies_hz: np.ndarray
    assets: tuple = ()
    status_callback: Callable[[str], None] | None = field(default=None, compare=False, repr=False)


@dataclass(frozen=True)
class _SolveMetadata:
    polar_angle_deg: np.ndarray
    radiator_names: np.ndarray
    sphere_metadata: dict[str, np.ndarray] | None = None


@dataclass(frozen=True)
class _SolverCapabilities:
    supports_spherical_sampling: bool = True
    supports_impedance: bool = True
    supports_burton_miller: bool = True
    supports_flat_target_normalization: bool = True
    supports_channel_resynthesis: bool = False
    supports_cancellation: bool = True
    supports_streaming: bool = True
    supports_remote_assets: bool = False
    supports_parallel_workers: bool = False
    supports_symmetry: bool = False
    is_remote: bool = False


_LOCAL = {
    "FrequencySolveTimings": _FrequencySolveTimings,
    "SolverDiagnostics": _SolverDiagnostics,
    "FrequencyResult": _FrequencyResult,
    "SolveRequest": _SolveRequest,
    "SolveMetadata": _SolveMetadata,
    "SolverCapabilities": _SolverCapabilities,
}


def have_blab() -> bool:
    try:
        import blab.solvers.base  # type: ignore  # noqa: F401

        return True
    except Exception:  # noqa: BLE001 - any import failure means standalone mode
        return False


def __getattr__(name: str):
    """Resolve a contract class at use time: the application's own class when its package is
    importable now, else the standalone equivalent."""
    if name in _LOCAL:
        try:
            import blab.solvers.base as base  # type: ignore

            return getattr(base, name)
        except Exception:  # noqa: BLE001
            return _LOCAL[name]
    raise AttributeError(name)


def frequency_result_from_event(raw: dict) -> "FrequencyResult":
    """FrequencyResult from the `result` payload of an NDJSON event (float32 wire, as protocol.py:263-278)."""

    def f32(x):
        return None if x is None else np.asarray(x, dtype=np.float32)

    def c64(x):
        if x is None:
            return None
        return (np.asarray(x["real"], np.float32) + 1j * np.asarray(x["imag"], np.float32)).astype(np.complex64)

    t = raw.get("timings") or {}
    d = raw.get("diagnostics")
    FrequencyResult = __getattr__("FrequencyResult")
    FrequencySolveTimings = __getattr__("FrequencySolveTimings")
    SolverDiagnostics = __getattr__("SolverDiagnostics")
    return FrequencyResult(
        freq_hz=float(raw["freq_hz"]),
        horizontal_spl_norm_db=f32(raw["horizontal_spl_norm_db"]),
        vertical_spl_norm_db=f32(raw["vertical_spl_norm_db"]),
        impedance=f32(raw["impedance"]),
        horizontal_spl_db=f32(raw.get("horizontal_spl_db")),
        vertical_spl_db=f32(raw.get("vertical_spl_db")),
        sphere_spl_norm_db=f32(raw.get("sphere_spl_norm_db")),
        channel_names=None if raw.get("channel_names") is None else np.asarray(raw["channel_names"]),
        horizontal_pressure=c64(raw.get("horizontal_pressure")),
        vertical_pressure=c64(raw.get("vertical_pressure")),
        sphere_pressure=c64(raw.get("sphere_pressure")),
        timings=FrequencySolveTimings(float(t.get("assembly_s", 0.0)), float(t.get("solve_s", 0.0)),
                                      float(t.get("field_s", 0.0))),
        diagnostics=None if d is None else SolverDiagnostics(
            convergence_info=d.get("convergence_info"), message=d.get("message"), backend=d.get("backend"),
            symmetry=d.get("symmetry"), regular_assembly_mode=d.get("regular_assembly_mode")),
    )
