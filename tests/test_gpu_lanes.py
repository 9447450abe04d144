"""Two-lane sweeps (bem_solve_options.lanes = 2): every other batch runs on a helper
context's stream from a second host thread.  Each batch is computed by the same kernels
on the same inputs whichever lane takes it, so the results are bitwise those of one
lane; the helper context's scratch is counted and trimmed with its owner's."""

import numpy as np
import pytest

from conftest import pkg_module

pytestmark = pytest.mark.gpu
meshes = pkg_module("meshes")
PTS = np.array([[0.0, 0.0, 2.0], [1.5, 0.3, 1.2], [-0.8, 1.1, -1.4], [2.0, 0.0, 0.0]])


@pytest.mark.parametrize("precision", [0, 1])
def test_two_lanes_match_one_lane(native, precision):
    mesh = meshes.box_with_piston((0.3, 0.2, 0.25), 600, 0.05, "+z")
    freqs = np.geomspace(300.0, 5000.0, 7)  # batches of 2: 4 batches, 2 per lane
    ctx = native.Context(0)
    try:
        m = ctx.upload_mesh(mesh.vertices, mesh.faces)
        m.set_excitation((mesh.tags == meshes.RADIATOR_TAG).astype(np.complex128)[None, :])
        m.set_observation_points(PTS)
        p1, u1, s1 = m.solve(freqs, precision=precision, sound_speed=343.0, rho=1.205, batch=2)
        p2, u2, s2 = m.solve(freqs, precision=precision, sound_speed=343.0, rho=1.205, batch=2, lanes=2)
        assert s1["batches"] == s2["batches"] == 4
        assert np.array_equal(p1, p2) and np.array_equal(u1, u2)
        assert ctx.scratch_bytes > 0
        ctx.trim()
        assert ctx.scratch_bytes == 0
        # a sweep of one batch runs on one lane whatever the option says
        p3, u3, s3 = m.solve(freqs[:2], precision=precision, sound_speed=343.0, rho=1.205, batch=2, lanes=2)
        assert s3["batches"] == 1 and np.array_equal(p3, p1[:2])
        m.release()
    finally:
        ctx.close()
