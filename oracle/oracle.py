"""Python side of the CPU oracle (test infrastructure only).

Wraps ``liboracle.so`` (the C++ restatement of BEAT CPU assembly and field) and
adds the dense Burton-Miller system and its LU solve:

* ``burton_miller_matrices`` follows ``burton_miller_neumann_matrices``
  (src/blab/solvers/julia_local/src/BeatEngineCpuSolve.jl:45-53):
  ``lhs = 1/2 M11 - D + eta H``, ``rhs_op = -S - eta (K' + 1/2 M10)``, ``eta = i/k``.
* ``solve`` factors with LAPACK getrf (scipy's OpenBLAS) and solves with getrs,
  as ``lu!`` / ``\\`` do in BeatEngineCpuSolve.jl:56-76.  The reference pins
  OpenBLAS_jll 0.3.29; scipy bundles its own OpenBLAS build.
* ``neumann_data`` follows ``pressure_for_drives`` (solver.jl:434-459):
  ``q_f = i rho omega drive`` on radiator faces, zero elsewhere.
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass
from functools import lru_cache

import numpy as np
import scipy.linalg

from .build import build_oracle

_dp = ctypes.POINTER(ctypes.c_double)
_fp = ctypes.POINTER(ctypes.c_float)
_ip = ctypes.POINTER(ctypes.c_int)


@lru_cache(maxsize=1)
def lib() -> ctypes.CDLL:
    handle = ctypes.CDLL(str(build_oracle()))
    i, d = ctypes.c_int, ctypes.c_double
    handle.oracle_assemble_f64.argtypes = [_dp, i, _ip, i, d, i, i, i, _dp, _dp, _dp, _dp, i]
    handle.oracle_assemble_f32.argtypes = [_dp, i, _ip, i, d, i, i, i, _fp, _fp, _fp, _fp, i]
    handle.oracle_mass_f64.argtypes = [_dp, i, _ip, i, i, i, _dp, _dp]
    handle.oracle_mass_f32.argtypes = [_dp, i, _ip, i, i, i, _fp, _fp]
    handle.oracle_field_f64.argtypes = [_dp, i, _ip, i, i, i, d, _dp, _dp, _dp, i, _dp, i]
    handle.oracle_field_f32.argtypes = [_dp, i, _ip, i, i, i, d, _fp, _fp, _dp, i, _fp, i]
    handle.oracle_triangle_rule.argtypes = [i, _dp, _dp, i]
    handle.oracle_duffy_rule.argtypes = [i, i, _dp, _dp, _dp, i]
    handle.oracle_singular_pair_count.argtypes = [_dp, i, _ip, i, i]
    handle.oracle_color_count.argtypes = [_ip, i, i]
    for name in ("oracle_assemble_f64", "oracle_assemble_f32", "oracle_mass_f64", "oracle_mass_f32",
                 "oracle_field_f64", "oracle_field_f32", "oracle_triangle_rule", "oracle_duffy_rule",
                 "oracle_singular_pair_count", "oracle_color_count"):
        getattr(handle, name).restype = ctypes.c_int
    return handle


def _geom(mesh) -> tuple[np.ndarray, np.ndarray]:
    v = np.ascontiguousarray(mesh.vertices, dtype=np.float64)
    f = np.ascontiguousarray(mesh.faces, dtype=np.int32)
    return v, f


def _ptr(a: np.ndarray, t):
    return a.ctypes.data_as(t)


@dataclass
class Operators:
    single_layer: np.ndarray  # (N_p, N_f)
    double_layer: np.ndarray  # (N_p, N_p)
    adjoint_double_layer: np.ndarray  # (N_p, N_f)
    hypersingular: np.ndarray  # (N_p, N_p)


SYMMETRY = {"off": 0, "x": 1, "xy": 2}


def assemble(mesh, k: float, *, precision: str = "f64", regular_order: int = 4, singular_order: int = 4,
             threads: int = 0, symmetry: str = "off") -> Operators:
    """Galerkin S, D, K', H operators (BeatEngineCpuAssembly.jl:636-886); with symmetry
    "x" / "xy" the mesh is the fundamental domain and the images are included."""
    v, f = _geom(mesh)
    nv, nf = len(v), len(f)
    ctype = np.complex128 if precision == "f64" else np.complex64
    S = np.zeros((nv, nf), ctype)
    Kp = np.zeros((nv, nf), ctype)
    D = np.zeros((nv, nv), ctype)
    H = np.zeros((nv, nv), ctype)
    if precision == "f64":
        fn, pt = lib().oracle_assemble_f64, _dp
    else:
        fn, pt = lib().oracle_assemble_f32, _fp
    rc = fn(_ptr(v, _dp), nv, _ptr(f, _ip), nf, float(k), regular_order, singular_order, SYMMETRY[symmetry],
            _ptr(S, pt), _ptr(D, pt), _ptr(Kp, pt), _ptr(H, pt), threads)
    if rc != 0:
        raise RuntimeError(f"oracle assembly failed ({rc})")
    return Operators(S, D, Kp, H)


def mass(mesh, *, precision: str = "f64", regular_order: int = 4, symmetry: str = "off") -> tuple[np.ndarray, np.ndarray]:
    """Dense L2 identity matrices M11 (P1 x P1) and M10 (P1 x DP0) (BeatEngineCore.jl:952-979)."""
    v, f = _geom(mesh)
    nv, nf = len(v), len(f)
    rtype = np.float64 if precision == "f64" else np.float32
    M11 = np.zeros((nv, nv), rtype)
    M10 = np.zeros((nv, nf), rtype)
    if precision == "f64":
        lib().oracle_mass_f64(_ptr(v, _dp), nv, _ptr(f, _ip), nf, regular_order, SYMMETRY[symmetry], _ptr(M11, _dp),
                              _ptr(M10, _dp))
    else:
        lib().oracle_mass_f32(_ptr(v, _dp), nv, _ptr(f, _ip), nf, regular_order, SYMMETRY[symmetry], _ptr(M11, _fp),
                              _ptr(M10, _fp))
    return M11, M10


def burton_miller_matrices(ops: Operators, M11: np.ndarray, M10: np.ndarray, k: float) -> tuple[np.ndarray, np.ndarray]:
    """(lhs, rhs_operator) of BeatEngineCpuSolve.jl:45-53."""
    ctype = ops.double_layer.dtype
    eta = ctype.type(1j / k)
    half = ctype.type(0.5)
    lhs = half * M11.astype(ctype) - ops.double_layer + eta * ops.hypersingular
    rhs_op = -ops.single_layer - eta * (ops.adjoint_double_layer + half * M10.astype(ctype))
    return lhs, rhs_op


def solve(lhs: np.ndarray, rhs: np.ndarray) -> np.ndarray:
    """LU with partial pivoting (LAPACK getrf) then getrs, one or more right-hand sides."""
    lu, piv = scipy.linalg.lu_factor(lhs, check_finite=False)
    return scipy.linalg.lu_solve((lu, piv), rhs, check_finite=False)


def neumann_data(mesh, radiator_faces: np.ndarray, drive: complex, rho: float, omega: float, dtype=np.complex128) -> np.ndarray:
    """q_f = i rho omega drive on the radiator faces (solver.jl:450-459)."""
    q = np.zeros(len(mesh.faces), dtype)
    q[radiator_faces] = dtype(1j * rho * omega) * dtype(drive)
    return q


def field(mesh, pressure: np.ndarray, q: np.ndarray, k: float, points: np.ndarray, *, precision: str = "f64",
          regular_order: int = 4, threads: int = 0, symmetry: str = "off") -> np.ndarray:
    """Exterior potential u(x) = sum_s [dG/dn_y p(y_s) - G q_s] w_s (BeatEngineCpuField.jl:1-45)."""
    v, f = _geom(mesh)
    pts = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 3)
    if precision == "f64":
        p = np.ascontiguousarray(pressure, np.complex128)
        qq = np.ascontiguousarray(q, np.complex128)
        out = np.zeros(len(pts), np.complex128)
        rc = lib().oracle_field_f64(_ptr(v, _dp), len(v), _ptr(f, _ip), len(f), regular_order, SYMMETRY[symmetry], float(k),
                                    _ptr(p, _dp), _ptr(qq, _dp), _ptr(pts, _dp), len(pts), _ptr(out, _dp), threads)
    else:
        p = np.ascontiguousarray(pressure, np.complex64)
        qq = np.ascontiguousarray(q, np.complex64)
        out = np.zeros(len(pts), np.complex64)
        rc = lib().oracle_field_f32(_ptr(v, _dp), len(v), _ptr(f, _ip), len(f), regular_order, SYMMETRY[symmetry], float(k),
                                    _ptr(p, _fp), _ptr(qq, _fp), _ptr(pts, _dp), len(pts), _ptr(out, _fp), threads)
    if rc != 0:
        raise RuntimeError(f"oracle field failed ({rc})")
    return out


def triangle_rule(order: int) -> tuple[np.ndarray, np.ndarray]:
    pts = np.zeros((16, 2))
    w = np.zeros(16)
    n = lib().oracle_triangle_rule(order, _ptr(pts, _dp), _ptr(w, _dp), 16)
    return pts[:n], w[:n]


def duffy_rule(order: int, kind: int) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    cap = 6 * order**4
    t = np.zeros((cap, 2))
    r = np.zeros((cap, 2))
    w = np.zeros(cap)
    n = lib().oracle_duffy_rule(order, kind, _ptr(t, _dp), _ptr(r, _dp), _ptr(w, _dp), cap)
    return t[:n], r[:n], w[:n]


def singular_pair_count(mesh, order: int = 4) -> int:
    v, f = _geom(mesh)
    return int(lib().oracle_singular_pair_count(_ptr(v, _dp), len(v), _ptr(f, _ip), len(f), order))


def color_count(mesh) -> int:
    v, f = _geom(mesh)
    return int(lib().oracle_color_count(_ptr(f, _ip), len(f), len(v)))


@dataclass
class FrequencySolution:
    pressure: np.ndarray  # (N_p, n_rhs)
    field: np.ndarray  # (n_points, n_rhs)


def solve_frequency(mesh, k: float, q_columns: np.ndarray, points: np.ndarray, *, precision: str = "f64",
                    regular_order: int = 4, singular_order: int = 4, threads: int = 0,
                    symmetry: str = "off") -> FrequencySolution:
    """One exterior BM frequency solve: assemble, factor once, solve every right-hand side, field."""
    ops = assemble(mesh, k, precision=precision, regular_order=regular_order, singular_order=singular_order,
                   threads=threads, symmetry=symmetry)
    M11, M10 = mass(mesh, precision=precision, regular_order=regular_order, symmetry=symmetry)
    lhs, rhs_op = burton_miller_matrices(ops, M11, M10, k)
    q_columns = np.asarray(q_columns).reshape(len(mesh.faces), -1).astype(lhs.dtype)
    pressure = solve(lhs, rhs_op @ q_columns)
    fields = np.stack(
        [field(mesh, pressure[:, c], q_columns[:, c], k, points, precision=precision, regular_order=regular_order,
               threads=threads, symmetry=symmetry) for c in range(q_columns.shape[1])],
        axis=1,
    )
    return FrequencySolution(pressure, fields)
