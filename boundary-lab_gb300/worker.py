"""NDJSON worker speaking the reference BEAT worker protocol on the GB300 engine.

Same command line and events as src/blab/solvers/julia_local/solver.jl:
  python worker.py --request request.json   one job, then exit
  python worker.py --worker                 emit `ready`, then one job per stdin line
                                            {"request": "<path>", "operation": "solve"}
Events (one JSON object per stdout line): ready, initialized, status, result,
cancelled, completed, failed (solver.jl:12-24, 703-715, 807, 957-996, 1019-1036).
The coupled worker's `bem_field` operation (coupled_solver.jl:2516-2546) is served
too: the field of retained boundary traces, read from the request's binary arrays,
answered by a `field_result` event with a `values_binary` descriptor and `completed`
(the protocol of src/blab/solvers/coupled_field.py).
A `solve` request that carries a `compiled_system` (the physical-system contract,
src/blab/system_contract.py) runs the coupled worker's exterior BEM branch
(coupled_solver.jl:267-569, system_exterior.py): `result` events carry
`{"result": {schema_version, freq_hz, excitation_port_ids, quantities,
diagnostics}}`.  As the coupled solver, the worker started without arguments
reads one such request from stdin and prints one result object per line.
The cancel file named by the request's `cancel_path` is honoured between
frequencies.  Because the command line matches, the reference's own adapter
runs this worker unchanged:
  BeatEngineBackend(julia_executable=sys.executable, solver_script=<this file>, julia_project=None)
"""

from __future__ import annotations

import importlib
import json
import math
import os
import sys
from pathlib import Path


def _package():
    root = Path(__file__).resolve().parent.parent
    if str(root) not in sys.path:
        sys.path.insert(0, str(root))
    return importlib.import_module("boundary-lab_gb300")


def _clean(value):
    """JSON-safe copy: NaN/Inf become null (the reference's JSON writer cannot emit them either)."""
    if isinstance(value, float):
        return value if math.isfinite(value) else None
    if isinstance(value, dict):
        return {k: _clean(v) for k, v in value.items()}
    if isinstance(value, (list, tuple)):
        return [_clean(v) for v in value]
    return value


def emit(event_type: str, **payload) -> None:
    event = {"type": event_type, **payload}
    sys.stdout.write(json.dumps(_clean(event), separators=(",", ":")) + "\n")
    sys.stdout.flush()


def solve_request(request: dict) -> None:
    _package()
    job_mod = importlib.import_module("boundary-lab_gb300.job")
    precision = os.environ.get("GB300_BEM_PRECISION", "mixed")
    device = int(os.environ.get("GB300_BEM_DEVICE", "0"))
    job = job_mod.ExteriorJob(request, status=lambda m: emit("status", message=m), precision=precision,
                              device=device)
    emit("initialized", **job.initialized_payload())
    try:
        for event in job.results():
            emit("result", **event)
    except job_mod.JobCancelled as exc:
        emit("cancelled", solved_count=exc.solved_count)
        return
    finally:
        job.close()
    emit("completed", solved_count=len(job.frequencies))


def system_request(request: dict, *, event_mode: bool = True) -> None:
    """A physical-system solve (exterior BEM branch): `result` events, then `completed` or
    `cancelled` (coupled_solver.jl:2531-2534); plain result lines when not in event mode."""
    _package()
    se = importlib.import_module("boundary-lab_gb300.system_exterior")
    job = se.ExteriorSystemJob(request, device=int(os.environ.get("GB300_BEM_DEVICE", "0")))
    try:
        for result in job.results():
            if event_mode:
                emit("result", result=result)
            else:
                sys.stdout.write(json.dumps(_clean(result), separators=(",", ":")) + "\n")
                sys.stdout.flush()
    except se.SystemJobCancelled as exc:
        if event_mode:
            emit("cancelled", solved_count=exc.solved_count)
        return
    finally:
        job.close()
    if event_mode:
        emit("completed", solved_count=len(job.frequencies))


def dispatch_solve(request: dict) -> None:
    if "compiled_system" in request:
        system_request(request)
    else:
        solve_request(request)


_field_evaluator = None


def field_request(request: dict, request_path: str) -> None:
    """The `bem_field` operation: the exterior field of retained boundary traces."""
    global _field_evaluator
    _package()
    cf = importlib.import_module("boundary-lab_gb300.coupled_field")
    if _field_evaluator is None:
        _field_evaluator = cf.FieldEvaluator(device=int(os.environ.get("GB300_BEM_DEVICE", "0")))
    scalars, arrays = cf.request_from_wire(request, Path(request_path))
    values = _field_evaluator.evaluate(scalars, arrays)
    emit("field_result", values_binary=cf.write_binary_result(request, Path(request_path), values))
    emit("completed")


def worker_loop() -> None:
    global _field_evaluator
    emit("ready", protocol="boundary_lab_julia_worker", pid=os.getpid())
    for line in sys.stdin:
        text = line.strip()
        if not text:
            continue
        try:
            message = json.loads(text)
            request_path = str(message["request"])
            with open(request_path, encoding="utf-8") as fh:
                request = json.load(fh)
            operation = str(message.get("operation", "solve"))
            if operation == "bem_field":
                field_request(request, request_path)
            elif operation == "solve":
                if _field_evaluator is not None:  # a solve releases the retained field caches
                    _field_evaluator.release()
                    _field_evaluator = None
                dispatch_solve(request)
            else:
                raise ValueError(f"Unsupported worker operation: {operation}")
        except Exception as exc:  # noqa: BLE001 - every failure becomes a `failed` event
            emit("failed", error=f"{type(exc).__name__}: {exc}")


def main(argv: list[str]) -> int:
    request_path = None
    worker = False
    i = 0
    while i < len(argv):
        if argv[i] == "--request" and i + 1 < len(argv):
            request_path = argv[i + 1]
            i += 2
        elif argv[i] == "--worker":
            worker = True
            i += 1
        else:
            emit("failed", error=f"Unknown argument: {argv[i]}")
            return 1
    if not worker and request_path is None and not sys.stdin.isatty():
        # the coupled solver's one-shot form: a system request on stdin, plain result lines out,
        # errors on stderr with exit status 1 (coupled_solver.jl:2561-2575)
        try:
            request = json.loads(sys.stdin.read() or "null")
            if not isinstance(request, dict) or "compiled_system" not in request:
                emit("failed", error="Missing --request path.")
                return 1
            system_request(request, event_mode=False)
            return 0
        except Exception as exc:  # noqa: BLE001
            sys.stderr.write(f"{type(exc).__name__}: {exc}\n")
            return 1
    try:
        if worker:
            worker_loop()
            return 0
        if request_path is None:
            emit("failed", error="Missing --request path.")
            return 1
        with open(request_path, encoding="utf-8") as fh:
            dispatch_solve(json.load(fh))
        return 0
    except Exception as exc:  # noqa: BLE001
        emit("failed", error=f"{type(exc).__name__}: {exc}")
        return 1


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
