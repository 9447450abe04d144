"""Test-only engine: the CPU oracle behind the engine interface of the product's
engine.py (prepare / solve / close), so session, worker and server logic can be
exercised on machines without a GPU.  Selected with
GB300_BEM_ENGINE=oracle_engine:make_engine (tests/ on sys.path)."""

from __future__ import annotations

import sys
from dataclasses import dataclass
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

from oracle import oracle  # noqa: E402


@dataclass
class _Result:
    pressure: np.ndarray
    field: np.ndarray
    stats: dict


class OracleEngine:
    name = "cpu_oracle"

    def __init__(self, device: int = 0, precision: str = "mixed", batch: int = 0, **_):
        self.mesh = None

    def prepare(self, vertices, faces, drives, points, regular_order=4, singular_order=4, symmetry="off"):
        self.symmetry = symmetry
        self.vertices = np.asarray(vertices, float)
        self.faces = np.asarray(faces, np.int32)
        self.drives = np.asarray(drives, np.complex128).reshape(-1, len(self.faces))
        self.points = np.asarray(points, float)
        self.orders = (regular_order, singular_order)

        class _M:
            pass

        self.mesh = _M()
        self.mesh.vertices, self.mesh.faces = self.vertices, self.faces

    def solve(self, freqs, sound_speed, rho):
        ps, us = [], []
        for f in np.asarray(freqs, float):
            omega = 2 * np.pi * f
            q = (self.drives * (1j * rho * omega)).T
            sol = oracle.solve_frequency(self.mesh, omega / sound_speed, q, self.points,
                                         regular_order=self.orders[0], singular_order=self.orders[1],
                                         symmetry=self.symmetry)
            ps.append(sol.pressure.T)
            us.append(sol.field.T)
        stats = {"assembly_s": 0.0, "solve_s": 0.0, "field_s": 0.0, "max_refine_steps": 0, "max_rel_residual": 0.0}
        return _Result(np.asarray(ps), np.asarray(us), stats)

    def close(self):
        self.mesh = None


def make_engine(**kwargs):
    return OracleEngine(**kwargs)
