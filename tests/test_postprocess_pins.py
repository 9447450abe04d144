"""Pins of the host post-processing (request.py) against the reference.

request.py restates the Julia worker's post-processing function by function
(src/blab/solvers/julia_local/solver.jl:271-318, 488-631).  The Julia engine cannot
run here, but the reference's Python package holds independent implementations of
the same math, used by its job server and GUI for channel re-synthesis:

* ``blab.channel_synthesis`` (channel_synthesis.py:12-131): crossovers through
  scipy's analog Butterworth design (not the pole formula of solver.jl:271-292),
  channel drives, flat-target corrections with np.interp, and the SPL synthesis
  of a channel basis in complex64;

those pin crossover responses, channel drives and the reference-angle interpolation
to ~1e-12, and the synthesised SPL rows to float32 rounding.  SPL
(solver.jl:488-490) and the radiation impedance (solver.jl:607-631) are pinned with
hand-derived known answers, which need no reference checkout.
"""

import math

import numpy as np
import pytest

from conftest import pkg_module, reference_checkout

rq = pkg_module("request")


@pytest.fixture(scope="module")
def blab():
    ref = reference_checkout()
    if ref is None:
        pytest.skip("reference checkout not present")
    import sys

    sys.path.insert(0, str(ref / "src"))
    try:
        from blab import channel_synthesis, config  # noqa: F401
    except Exception as exc:  # noqa: BLE001
        pytest.skip(f"reference package not importable: {exc}")
    finally:
        sys.path.remove(str(ref / "src"))
    return channel_synthesis, config


CROSSOVERS = [("lowpass", "butterworth", o) for o in range(1, 9)] + \
             [("highpass", "butterworth", o) for o in range(1, 9)] + \
             [(t, "linkwitz_riley", o) for t in ("lowpass", "highpass") for o in (2, 4, 8)]


@pytest.mark.parametrize("ctype,filt,order", CROSSOVERS)
def test_crossover_matches_scipy_design(blab, ctype, filt, order):
    cs, cfg = blab
    for cutoff in (80.0, 1200.0, 3500.0):
        for freq in np.geomspace(20.0, 20000.0, 37):
            ours = rq.crossover_response({"type": ctype, "filter": filt, "order": order, "frequency_hz": cutoff},
                                         float(freq))
            ref = cs.crossover_response(cfg.CrossoverConfig(type=ctype, filter=filt, order=order,
                                                            frequency_hz=cutoff), float(freq))
            assert abs(ours - ref) <= 1e-11 * max(1.0, abs(ref)), (cutoff, freq)


def test_channel_drive_matches_reference(blab):
    cs, cfg = blab
    rng = np.random.default_rng(4)
    for _ in range(40):
        level, delay = float(rng.uniform(-12, 6)), float(rng.uniform(0, 3))
        pol = int(rng.choice([-1, 1]))
        hpf = {"type": "highpass", "filter": str(rng.choice(["butterworth", "linkwitz_riley"])), "order": 4,
               "frequency_hz": float(rng.uniform(50, 500))}
        lpf = {"type": "lowpass", "filter": "butterworth", "order": int(rng.integers(1, 5)),
               "frequency_hz": float(rng.uniform(1000, 8000))}
        freq = float(rng.uniform(20, 20000))
        ours = rq.channel_drive({"level_db": level, "polarity": pol, "delay_ms": delay, "hpf": hpf, "lpf": lpf}, freq)
        ref = cs.channel_drive(cfg.ChannelConfig(name="c", level_db=level, polarity=pol, delay_ms=delay,
                                                 hpf=cfg.CrossoverConfig(**hpf), lpf=cfg.CrossoverConfig(**lpf)), freq)
        assert abs(ours - ref) <= 1e-11 * abs(ref)


@pytest.mark.parametrize("grid", ["full_circle", "half_circle", "coarse"])
def test_reference_angle_interpolation_matches_reference(blab, grid):
    cs, _ = blab
    angles = {"full_circle": np.arange(-180.0, 180.1, 5.0), "half_circle": np.arange(0.0, 180.1, 5.0),
              "coarse": np.arange(-180.0, 180.1, 30.0)}[grid].astype(np.float32)
    rng = np.random.default_rng(len(angles))
    values = (rng.normal(size=len(angles)) + 1j * rng.normal(size=len(angles))).astype(np.complex64)
    for ref_angle in (0.0, 2.5, 7.25, -37.0, 179.0, 185.0, -190.0, 360.0, 725.5):
        ours = rq.interpolate_complex_reference(values, angles, ref_angle)
        ref = cs.complex_reference_pressure(values, angles, ref_angle)
        assert abs(ours - ref) <= 1e-6 * max(1.0, abs(ref)), ref_angle


def test_flat_target_corrections_match_reference(blab):
    cs, _ = blab
    angles = np.arange(-180.0, 180.1, 5.0).astype(np.float32)
    rng = np.random.default_rng(9)
    rows = (rng.normal(size=(3, len(angles))) + 1j * rng.normal(size=(3, len(angles)))).astype(np.complex64)
    rows[2] *= 1e-14  # below the 1e-12 floor: correction 1
    for ref_angle in (0.0, 12.5, -90.0):
        ours = rq.flat_target_corrections(["a", "b", "c"], rows, angles, ref_angle, True)
        ref = cs.flat_target_corrections(rows, angles, ref_angle, enabled=True)
        for i, name in enumerate("abc"):
            assert abs(ours[name] - float(ref[i])) <= 2e-7 * abs(float(ref[i]))
    off = rq.flat_target_corrections(["a", "b"], rows[:2], angles, 0.0, False)
    assert off == {"a": 1.0, "b": 1.0}
    assert np.all(cs.flat_target_corrections(rows[:2], angles, 0.0, enabled=False) == 1.0)


@pytest.mark.parametrize("flat", [True, False])
def test_channel_synthesis_matches_reference(blab, flat):
    """Two channels with crossovers, level, polarity and delay: the synthesised SPL rows
    (horizontal, vertical, normalised and sphere) equal the reference's complex64
    synthesis to float32 rounding (1e-4 dB)."""
    cs, cfg = blab
    angles = np.arange(-180.0, 180.1, 5.0).astype(np.float32)
    rng = np.random.default_rng(13)
    n = len(angles)
    base = np.exp(-0.5 * (angles / 70.0) ** 2)
    h = ((base + 0.1 * rng.normal(size=(2, n))) * np.exp(1j * rng.uniform(0, 2 * np.pi, size=(2, n)))).astype(np.complex64)
    v = ((base + 0.1 * rng.normal(size=(2, n))) * np.exp(1j * rng.uniform(0, 2 * np.pi, size=(2, n)))).astype(np.complex64)
    s = (rng.normal(size=(2, 300)) + 1j * rng.normal(size=(2, 300))).astype(np.complex64)
    chans = {
        "woofer": {"level_db": -1.5, "polarity": 1, "delay_ms": 0.0, "hpf": {"type": "none"},
                   "lpf": {"type": "lowpass", "filter": "linkwitz_riley", "order": 4, "frequency_hz": 1800.0}},
        "tweeter": {"level_db": -4.0, "polarity": -1, "delay_ms": 0.12, "lpf": {"type": "none"},
                    "hpf": {"type": "highpass", "filter": "linkwitz_riley", "order": 4, "frequency_hz": 1800.0}},
    }
    configs = tuple(cfg.ChannelConfig(name=k, level_db=c["level_db"], polarity=c["polarity"], delay_ms=c["delay_ms"],
                                      hpf=cfg.CrossoverConfig(**c["hpf"]), lpf=cfg.CrossoverConfig(**c["lpf"]))
                    for k, c in chans.items())
    names = ["tweeter", "woofer"]
    for freq in (900.0, 1800.0, 4100.0):
        ours = rq.synthesize_channel_basis(names, list(h), list(v), list(s), chans, freq, angles, 0.0, flat)
        ref = cs.synthesize_channel_basis_spl(freq_hz=freq, polar_angle_deg=angles, channel_names=np.array(names),
                                              horizontal_pressure=h, vertical_pressure=v, channel_configs=configs,
                                              flat_target_reference_angle_deg=0.0, flat_target_enabled=flat,
                                              sphere_pressure=s)
        for key, mine in (("horizontal_spl_db", ours.horizontal_spl), ("vertical_spl_db", ours.vertical_spl),
                          ("horizontal_spl_norm_db", ours.horizontal_norm),
                          ("vertical_spl_norm_db", ours.vertical_norm), ("sphere_spl_norm_db", ours.sphere_norm)):
            assert np.max(np.abs(np.asarray(mine, np.float64) - np.asarray(ref[key], np.float64))) < 1e-4, (freq, key)
        for i, name in enumerate(names):
            assert abs(ours.corrections[name] - float(ref["channel_corrections"][i])) <= 2e-7 * ours.corrections[name]


def test_pressure_to_spl_known_answers():
    """SPL = 20 log10(|p| / 20 uPa) as float32 (solver.jl:488-490): 20 uPa is 0 dB, every
    factor 10 adds 20 dB, 1 Pa is 20 log10(5e4) = 93.9794 dB, the phase does not matter."""
    p = np.array([20e-6, 2e-4, 2e-3 * 1j, 1.0, -1.0, (0.6 + 0.8j), 2e-6], np.complex128)
    spl = rq.pressure_to_spl(p)
    assert spl.dtype == np.float32
    want = np.array([0.0, 20.0, 40.0, 93.97940008672037, 93.97940008672037, 93.97940008672037, -20.0], np.float32)
    assert np.all(np.abs(spl - want) <= 2e-5)


def test_impedance_known_answers():
    """Radiation impedance (solver.jl:607-631): F = 10 x sum over the radiator's faces of
    mean(p at the face's vertices) x area x symmetry factor; Z = F / drive, reported as
    [Re Z / 2, -Im Z / 2] in float32, NaN for a zero drive.  Two faces of areas 0.5 and
    0.25 with uniform pressure (1 + 2i): F = 10 x 0.75 x (1 + 2i) = 7.5 + 15i."""
    faces = np.array([[0, 1, 2], [1, 3, 2], [4, 5, 6]])
    areas = np.array([0.5, 0.25, 9.0])
    tags = np.array([2, 2, 1])
    ids = np.ones(3, np.int32)
    pressure = np.full(7, 1 + 2j)
    pressure[6] = 100.0  # on a face of the other tag: not counted
    rad = [{"name": "r", "tag": 2, "mesh_id": 1}, {"name": "silent", "tag": 2, "mesh_id": 1}]
    z = rq.impedance_for_radiators(faces, areas, tags, ids, pressure, rad, np.array([1.0, 0.0]))
    assert z[0] == [3.75, -7.5]
    assert all(math.isnan(x) for x in z[1])
    # drive 2i: Z = (7.5 + 15i) / 2i = 7.5 - 3.75i -> [3.75, 1.875]
    z = rq.impedance_for_radiators(faces, areas, tags, ids, pressure, rad[:1], np.array([2j]))
    assert z[0] == [3.75, 1.875]
    # half model (symmetry x): the force counts the mirror image, factor 2
    z = rq.impedance_for_radiators(faces, areas, tags, ids, pressure, rad[:1], np.array([1.0]), "x")
    assert z[0] == [7.5, -15.0]
    # non-uniform pressure: the face mean of vertex values
    p2 = np.zeros(7, complex)
    p2[[0, 1, 2]] = [3.0, 0.0, 0.0]  # face 0 mean 1, face 1 mean 0
    z = rq.impedance_for_radiators(faces, areas, tags, ids, p2, rad[:1], np.array([1.0]))
    assert z[0] == [2.5, 0.0]
