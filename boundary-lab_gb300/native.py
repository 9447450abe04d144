"""ctypes binding of the C ABI in include/gb300_bem.h (libgb300_bem.so).

There is no fallback: if the shared library is missing or cannot be loaded,
every entry point raises ``NativeLibraryError``.  Build it with
``build.build()`` (or ``__graft_entry__.build()`` at the repository root).
"""

from __future__ import annotations

import ctypes
import threading
from pathlib import Path

import numpy as np

from . import build as _build

BEM_OK = 0
BEM_PRECISION_FP64 = 0
BEM_PRECISION_MIXED = 1
STATUS_NAMES = {
    0: "BEM_OK",
    1: "BEM_ERR_INVALID_ARGUMENT",
    2: "BEM_ERR_CUDA",
    3: "BEM_ERR_OUT_OF_MEMORY",
    4: "BEM_ERR_SINGULAR",
    5: "BEM_ERR_NOT_CONVERGED",
}
SYMMETRY_MODES = {"off": 0, "x": 1, "xy": 2}

EXPORTED_SYMBOLS = (
    "bem_abi_version",
    "bem_create_context",
    "bem_destroy_context",
    "bem_last_error",
    "bem_context_stream",
    "bem_upload_mesh",
    "bem_upload_mesh_symmetric",
    "bem_release_mesh",
    "bem_mesh_info",
    "bem_set_excitation",
    "bem_set_observation_points",
    "bem_default_options",
    "bem_solve_frequencies",
    "bem_solve_jobs",
    "bem_assemble_lhs",
    "bem_apply_rhs_operator",
    "bem_estimate_device_bytes",
    "bem_auto_batch",
    "bem_evaluate_field",
    "bem_evaluate_field_noalloc",
    "bem_lu_factor_dense",
    "bem_trim_context",
    "bem_context_scratch_bytes",
)


def evaluate_field_noalloc(d_vertices: int, n_vertices: int, d_faces: int, n_faces: int, k: float, d_pressure: int,
                           d_neumann: int, d_points: int, n_points: int, d_field_out: int, *,
                           precision: int = BEM_PRECISION_MIXED, regular_order: int = 4, stream: int = 0) -> None:
    """Field at n_points from caller-owned device buffers, without any device allocation
    (bem_evaluate_field_noalloc).  Pointers are integers (e.g. torch's data_ptr())."""
    lib = load()
    err = ctypes.create_string_buffer(256)
    rc = lib.bem_evaluate_field_noalloc(d_vertices, n_vertices, d_faces, n_faces, regular_order, float(k), d_pressure,
                                        d_neumann, d_points, n_points, int(precision), d_field_out,
                                        ctypes.c_void_p(stream) if stream else None, err, len(err))
    if rc != BEM_OK:
        raise BemError(rc, err.value.decode("utf-8", "replace"))


class NativeLibraryError(RuntimeError):
    """The GB300 BEM shared library is missing or failed to load."""


class BemError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class Job(ctypes.Structure):
    """bem_job: one mesh's frequencies and output buffers in a bem_solve_jobs call."""

    _fields_ = [
        ("mesh", ctypes.c_void_p),
        ("freqs_hz", ctypes.POINTER(ctypes.c_double)),
        ("n_freq", ctypes.c_int),
        ("pressure_out", ctypes.c_void_p),
        ("field_out", ctypes.c_void_p),
    ]


class SolveOptions(ctypes.Structure):
    _fields_ = [
        ("precision", ctypes.c_int),
        ("sound_speed", ctypes.c_double),
        ("rho", ctypes.c_double),
        ("refine_tol", ctypes.c_double),
        ("max_refine", ctypes.c_int),
        ("batch", ctypes.c_int),
        ("lu_block", ctypes.c_int),
        ("outputs_on_device", ctypes.c_int),
        ("profile", ctypes.c_int),
        ("lu_gemm", ctypes.c_int),
        ("lanes", ctypes.c_int),
    ]


class SolveStats(ctypes.Structure):
    _fields_ = [
        ("assembly_s", ctypes.c_double),
        ("solve_s", ctypes.c_double),
        ("field_s", ctypes.c_double),
        ("max_refine_steps", ctypes.c_int),
        ("max_rel_residual", ctypes.c_double),
        ("batches", ctypes.c_int),
        ("kernel_s", ctypes.c_double * 8),
        ("regular_pairs", ctypes.c_longlong),
        ("singular_pairs", ctypes.c_longlong),
        ("singular_points", ctypes.c_longlong),
        ("lu_gemm_used", ctypes.c_int),
        ("kernel_launches", ctypes.c_longlong),
        ("regular_flop", ctypes.c_double),
        ("singular_cheb_freqs", ctypes.c_longlong),
    ]

KERNEL_SLOTS = ("singular", "regular", "gather", "rhs", "lu", "solve", "field")


def stats_dict(stats: "SolveStats") -> dict:
    out = {name: getattr(stats, name) for name, _ in SolveStats._fields_ if name != "kernel_s"}
    out["kernel_s"] = {name: stats.kernel_s[i] for i, name in enumerate(KERNEL_SLOTS)}
    return out


_lock = threading.Lock()
_lib: ctypes.CDLL | None = None


def library_path() -> Path:
    return _build.LIBRARY


def load(build_if_missing: bool = False) -> ctypes.CDLL:
    """Load libgb300_bem.so (optionally building it first); raise if unavailable."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = library_path()
        if not path.exists():
            if build_if_missing:
                _build.build()
            else:
                raise NativeLibraryError(
                    f"{path} not found: build the CUDA library first (python -c 'import __graft_entry__ as g; g.build()')"
                )
        try:
            lib = ctypes.CDLL(str(path))
        except OSError as exc:
            raise NativeLibraryError(f"cannot load {path}: {exc}") from exc
        vp, ip, dp = ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double)
        lib.bem_abi_version.restype = ip
        lib.bem_create_context.argtypes = [ip, ctypes.POINTER(vp)]
        lib.bem_create_context.restype = ip
        lib.bem_destroy_context.argtypes = [vp]
        lib.bem_destroy_context.restype = None
        lib.bem_last_error.argtypes = [vp]
        lib.bem_last_error.restype = ctypes.c_char_p
        lib.bem_context_stream.argtypes = [vp]
        lib.bem_context_stream.restype = vp
        lib.bem_upload_mesh.argtypes = [vp, dp, ip, ctypes.POINTER(ctypes.c_int), ip, ip, ip, ctypes.POINTER(vp)]
        lib.bem_upload_mesh.restype = ip
        lib.bem_upload_mesh_symmetric.argtypes = [vp, dp, ip, ctypes.POINTER(ctypes.c_int), ip, ip, ip, ip,
                                                  ctypes.POINTER(vp)]
        lib.bem_upload_mesh_symmetric.restype = ip
        lib.bem_release_mesh.argtypes = [vp]
        lib.bem_release_mesh.restype = None
        lib.bem_mesh_info.argtypes = [vp, ctypes.POINTER(ip), ctypes.POINTER(ip), ctypes.POINTER(ip)]
        lib.bem_mesh_info.restype = ip
        lib.bem_set_excitation.argtypes = [vp, dp, ip]
        lib.bem_set_excitation.restype = ip
        lib.bem_set_observation_points.argtypes = [vp, dp, ip]
        lib.bem_set_observation_points.restype = ip
        lib.bem_default_options.argtypes = [ctypes.POINTER(SolveOptions)]
        lib.bem_default_options.restype = None
        lib.bem_solve_frequencies.argtypes = [vp, dp, ip, ctypes.POINTER(SolveOptions), vp, vp,
                                              ctypes.POINTER(SolveStats)]
        lib.bem_solve_frequencies.restype = ip
        lib.bem_solve_jobs.argtypes = [vp, ctypes.POINTER(Job), ip, ctypes.POINTER(SolveOptions),
                                       ctypes.POINTER(SolveStats)]
        lib.bem_solve_jobs.restype = ip
        lib.bem_assemble_lhs.argtypes = [vp, ctypes.c_double, ip, dp, dp]
        lib.bem_assemble_lhs.restype = ip
        lib.bem_apply_rhs_operator.argtypes = [vp, ctypes.c_double, ip, dp, dp, ip, dp]
        lib.bem_apply_rhs_operator.restype = ip
        lib.bem_lu_factor_dense.argtypes = [vp, ip, dp, ctypes.POINTER(ctypes.c_int), ip, ip]
        lib.bem_lu_factor_dense.restype = ip
        lib.bem_estimate_device_bytes.argtypes = [ip, ip, ip, ip, ip, ip, ip]
        lib.bem_estimate_device_bytes.restype = ctypes.c_longlong
        lib.bem_auto_batch.argtypes = [vp, ip, ip]
        lib.bem_auto_batch.restype = ip
        lib.bem_evaluate_field.argtypes = [vp, ctypes.c_double, ip, dp, dp, dp, ip, dp]
        lib.bem_evaluate_field.restype = ip
        lib.bem_trim_context.argtypes = [vp]
        lib.bem_trim_context.restype = ip
        lib.bem_context_scratch_bytes.argtypes = [vp]
        lib.bem_context_scratch_bytes.restype = ctypes.c_longlong
        # allocation-free field evaluation: every pointer is a caller-owned device buffer
        lib.bem_evaluate_field_noalloc.argtypes = [vp, ip, vp, ip, ip, ctypes.c_double, vp, vp, vp, ip, ip, vp, vp,
                                                   ctypes.c_char_p, ip]
        lib.bem_evaluate_field_noalloc.restype = ip
        if lib.bem_abi_version() != 3:
            raise NativeLibraryError(f"unexpected ABI version {lib.bem_abi_version()} in {path}")
        _lib = lib
        return lib


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _cplx_view(a: np.ndarray) -> np.ndarray:
    """complex128 array -> contiguous float64 view (interleaved re, im)."""
    a = np.ascontiguousarray(a, dtype=np.complex128)
    return a.view(np.float64)


class Context:
    """One CUDA device + stream, owning all device memory of its meshes."""

    def __init__(self, device: int = 0):
        self._lib = load()
        handle = ctypes.c_void_p()
        rc = self._lib.bem_create_context(int(device), ctypes.byref(handle))
        if rc != BEM_OK:
            raise BemError(rc, f"cannot create a CUDA context on device {device}")
        self._h = handle
        self.device = device

    def _check(self, rc: int) -> None:
        if rc != BEM_OK:
            msg = self._lib.bem_last_error(self._h)
            raise BemError(rc, msg.decode("utf-8", "replace") if msg else "")

    @property
    def stream_handle(self) -> int:
        """The context's cudaStream_t as an integer (for torch.cuda.ExternalStream)."""
        return int(self._lib.bem_context_stream(self._h) or 0)

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.bem_destroy_context(self._h)
            self._h = None

    def __del__(self):  # pragma: no cover - interpreter shutdown order
        try:
            self.close()
        except Exception:
            pass

    def upload_mesh(self, vertices: np.ndarray, faces: np.ndarray, regular_order: int = 4,
                    singular_order: int = 4, symmetry: str | int = "off") -> "Mesh":
        """Upload a mesh; symmetry "off", "x" (half model, x >= 0) or "xy" (quarter model)."""
        v = np.ascontiguousarray(vertices, dtype=np.float64).reshape(-1, 3)
        f = np.ascontiguousarray(faces, dtype=np.int32).reshape(-1, 3)
        sym = SYMMETRY_MODES[symmetry] if isinstance(symmetry, str) else int(symmetry)
        handle = ctypes.c_void_p()
        self._check(self._lib.bem_upload_mesh_symmetric(
            self._h, _dptr(v), len(v), f.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), len(f), int(regular_order),
            int(singular_order), sym, ctypes.byref(handle)))
        return Mesh(self, handle, len(v), len(f))

    def solve_jobs(self, jobs, *, precision: int = BEM_PRECISION_MIXED, sound_speed: float = 343.0, rho: float = 1.21,
                   refine_tol: float = 1e-10, max_refine: int = 8, batch: int = 0, lu_block: int = 0,
                   want_field: bool = True, profile: bool = False, lu_gemm: int = 0):
        """Solve several uploaded meshes together (bem_solve_jobs): ``jobs`` is a sequence of
        (Mesh, freqs_hz).  Returns ([(pressure, field) per job], stats dict), with the shapes
        of Mesh.solve."""
        items = (Job * len(jobs))()
        keep = []
        outs = []
        for i, (mesh, freqs) in enumerate(jobs):
            if mesh.ctx is not self:
                raise ValueError("every mesh of solve_jobs must belong to this context")
            f = np.ascontiguousarray(freqs, dtype=np.float64).reshape(-1)
            pressure = np.zeros((len(f), mesh.n_rhs, mesh.n_vertices), np.complex128)
            field = np.zeros((len(f), mesh.n_rhs, mesh.n_points), np.complex128) if want_field else None
            keep.append(f)
            outs.append((pressure, field))
            items[i].mesh = mesh._h
            items[i].freqs_hz = _dptr(f)
            items[i].n_freq = len(f)
            items[i].pressure_out = pressure.ctypes.data_as(ctypes.c_void_p)
            items[i].field_out = None if field is None else field.ctypes.data_as(ctypes.c_void_p)
        opt = SolveOptions()
        self._lib.bem_default_options(ctypes.byref(opt))
        opt.precision = int(precision)
        opt.sound_speed = float(sound_speed)
        opt.rho = float(rho)
        opt.refine_tol = float(refine_tol)
        opt.max_refine = int(max_refine)
        opt.batch = int(batch)
        opt.lu_block = int(lu_block)
        opt.profile = int(bool(profile))
        opt.lu_gemm = int(lu_gemm)
        stats = SolveStats()
        self._check(self._lib.bem_solve_jobs(self._h, items, len(jobs), ctypes.byref(opt), ctypes.byref(stats)))
        return outs, stats_dict(stats)

    def lu_factor_dense(self, a: np.ndarray, precision: int = BEM_PRECISION_FP64, lu_gemm: int = 0):
        """(LU, ipiv) of a dense complex matrix, LAPACK getrf conventions (0-based ipiv)."""
        a = np.asarray(a, dtype=np.complex128)
        n = a.shape[0]
        buf = np.asfortranarray(a).copy(order="F")
        ipiv = np.zeros(n, dtype=np.int32)
        self._check(self._lib.bem_lu_factor_dense(self._h, n, _dptr(buf.reshape(-1, order="F").view(np.float64)),
                                                  ipiv.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), int(precision),
                                                  int(lu_gemm)))
        return buf, ipiv

    def estimate_device_bytes(self, n_vertices: int, n_faces: int, n_pairs: int, n_rhs: int, n_points: int,
                              batch: int, precision: int) -> int:
        return int(self._lib.bem_estimate_device_bytes(n_vertices, n_faces, n_pairs, n_rhs, n_points, batch, precision))

    def trim(self) -> None:
        """Free this context's solve scratch and return unused pool memory (bem_trim_context)."""
        self._check(self._lib.bem_trim_context(self._h))

    @property
    def scratch_bytes(self) -> int:
        """Device bytes of solve scratch this context holds (bem_context_scratch_bytes)."""
        return int(self._lib.bem_context_scratch_bytes(self._h))


class Mesh:
    def __init__(self, ctx: Context, handle: ctypes.c_void_p, nv: int, nf: int):
        self.ctx = ctx
        self._h = handle
        self.n_vertices = nv
        self.n_faces = nf
        self.n_rhs = 0
        self.n_points = 0
        nvv, nff, npp = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        ctx._check(ctx._lib.bem_mesh_info(handle, ctypes.byref(nvv), ctypes.byref(nff), ctypes.byref(npp)))
        self.n_singular_pairs = npp.value

    def release(self) -> None:
        if self._h is not None and self.ctx._h is not None:
            self.ctx._lib.bem_release_mesh(self._h)
        self._h = None

    def auto_batch(self, n_freq: int, precision: int = BEM_PRECISION_MIXED) -> int:
        """The batch the solve uses with batch=0 for a sweep of n_freq frequencies;
        n_freq <= 0: the largest batch (the LU's cluster panels in one wave)."""
        b = int(self.ctx._lib.bem_auto_batch(self._h, precision, int(n_freq)))
        if b < 1:
            raise BemError(1, self.ctx._lib.bem_last_error(self.ctx._h).decode())
        return b

    def evaluate_field(self, k: float, pressure: np.ndarray, neumann: np.ndarray, points: np.ndarray,
                       precision: int = BEM_PRECISION_MIXED) -> np.ndarray:
        """Exterior field u(x) of retained boundary traces (pressure per vertex, normal
        derivative per face) at points [n][3]; returns complex128 [n]."""
        p = np.ascontiguousarray(pressure, dtype=np.complex128).reshape(self.n_vertices)
        q = np.ascontiguousarray(neumann, dtype=np.complex128).reshape(self.n_faces)
        pts = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 3)
        out = np.zeros(len(pts), np.complex128)
        self.ctx._check(self.ctx._lib.bem_evaluate_field(self._h, float(k), int(precision), _dptr(_cplx_view(p)),
                                                         _dptr(_cplx_view(q)), _dptr(pts), len(pts),
                                                         _dptr(_cplx_view(out))))
        return out

    def set_excitation(self, unit_drive: np.ndarray) -> None:
        d = np.asarray(unit_drive, dtype=np.complex128).reshape(-1, self.n_faces)
        self.ctx._check(self.ctx._lib.bem_set_excitation(self._h, _dptr(_cplx_view(d)), d.shape[0]))
        self.n_rhs = d.shape[0]

    def set_observation_points(self, points: np.ndarray) -> None:
        p = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 3)
        self.ctx._check(self.ctx._lib.bem_set_observation_points(self._h, _dptr(p), len(p)))
        self.n_points = len(p)

    def solve(self, freqs_hz, *, precision: int = BEM_PRECISION_MIXED, sound_speed: float = 343.0,
              rho: float = 1.21, refine_tol: float = 1e-10, max_refine: int = 8, batch: int = 0, lu_block: int = 0,
              want_pressure: bool = True, want_field: bool = True, profile: bool = False, lu_gemm: int = 0,
              lanes: int = 1):
        """Returns (pressure [n_freq, n_rhs, n_vertices], field [n_freq, n_rhs, n_points], stats dict).
        lanes = 2 runs a sweep of two or more batches on two streams (bem_solve_options.lanes)."""
        f = np.ascontiguousarray(freqs_hz, dtype=np.float64).reshape(-1)
        opt = SolveOptions()
        self.ctx._lib.bem_default_options(ctypes.byref(opt))
        opt.precision = int(precision)
        opt.sound_speed = float(sound_speed)
        opt.rho = float(rho)
        opt.refine_tol = float(refine_tol)
        opt.max_refine = int(max_refine)
        opt.batch = int(batch)
        opt.lu_block = int(lu_block)
        opt.profile = int(bool(profile))
        opt.lu_gemm = int(lu_gemm)
        opt.lanes = int(lanes)
        pressure = np.zeros((len(f), self.n_rhs, self.n_vertices), np.complex128) if want_pressure else None
        field = np.zeros((len(f), self.n_rhs, self.n_points), np.complex128) if want_field else None
        stats = SolveStats()
        rc = self.ctx._lib.bem_solve_frequencies(
            self._h, _dptr(f), len(f), ctypes.byref(opt),
            None if pressure is None else pressure.ctypes.data_as(ctypes.c_void_p),
            None if field is None else field.ctypes.data_as(ctypes.c_void_p),
            ctypes.byref(stats))
        self.ctx._check(rc)
        return pressure, field, stats_dict(stats)

    def solve_device(self, freqs_hz, pressure_ptr: int, field_ptr: int, **kw) -> dict:
        """Same as solve() but writes into device buffers (pointers on the context's device)."""
        f = np.ascontiguousarray(freqs_hz, dtype=np.float64).reshape(-1)
        opt = SolveOptions()
        self.ctx._lib.bem_default_options(ctypes.byref(opt))
        for key, value in kw.items():
            setattr(opt, key, value)
        opt.outputs_on_device = 1
        stats = SolveStats()
        self.ctx._check(self.ctx._lib.bem_solve_frequencies(
            self._h, _dptr(f), len(f), ctypes.byref(opt),
            ctypes.c_void_p(pressure_ptr) if pressure_ptr else None,
            ctypes.c_void_p(field_ptr) if field_ptr else None, ctypes.byref(stats)))
        return stats_dict(stats)

    def assemble_lhs(self, k: float, coeffs=(-1.0, None, 0.5), precision: int = BEM_PRECISION_FP64) -> np.ndarray:
        """Dense cD*D + cH*H + cM*M11 (default: the Burton-Miller LHS, cH = i/k)."""
        cD, cH, cM = coeffs
        if cH is None:
            cH = 1j / k
        c = np.array([complex(cD).real, complex(cD).imag, complex(cH).real, complex(cH).imag,
                      complex(cM).real, complex(cM).imag], dtype=np.float64)
        out = np.zeros((self.n_vertices, self.n_vertices), np.complex128)  # [col][row]
        self.ctx._check(self.ctx._lib.bem_assemble_lhs(self._h, float(k), int(precision), _dptr(c),
                                                       _dptr(out.view(np.float64))))
        return out.T.copy()

    def apply_rhs_operator(self, k: float, q: np.ndarray, coeffs=(-1.0, None, None),
                           precision: int = BEM_PRECISION_FP64) -> np.ndarray:
        """(cS*S + cK*K' + cM10*M10) q for q of shape (n_faces,) or (n_faces, n_rhs).
        Note: this replaces the mesh's excitation patterns."""
        cS, cK, cM10 = coeffs
        if cK is None:
            cK = -1j / k
        if cM10 is None:
            cM10 = -0.5j / k
        q = np.asarray(q, dtype=np.complex128)
        squeeze = q.ndim == 1
        qc = q.reshape(self.n_faces, -1).T.copy()  # [n_rhs][n_faces]
        c = np.array([complex(cS).real, complex(cS).imag, complex(cK).real, complex(cK).imag,
                      complex(cM10).real, complex(cM10).imag], dtype=np.float64)
        out = np.zeros((qc.shape[0], self.n_vertices), np.complex128)
        self.ctx._check(self.ctx._lib.bem_apply_rhs_operator(self._h, float(k), int(precision), _dptr(c),
                                                             _dptr(_cplx_view(qc)), qc.shape[0],
                                                             _dptr(out.view(np.float64))))
        self.n_rhs = qc.shape[0]
        return out[0] if squeeze else out.T.copy()
