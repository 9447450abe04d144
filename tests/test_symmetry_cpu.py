"""Symmetric models on the CPU oracle (no GPU).

A half model with x symmetry (quarter model with xy symmetry) is the full model
restricted to its fundamental domain: the reference's symmetric assembly
(image pairs, the image singular delta, orbit row weights; BeatEngineCpuAssembly.jl:
411-445, 488-634) and field images (BeatEngineCore.jl:1240-1280) must give the
full model's surface pressure on the fundamental-domain vertices and its field
everywhere.  The full model is built by mirroring the fundamental domain, so both
discretise the same surface.  They differ only in quadrature orientation: a
mirrored face of the full mesh has its vertex order reversed (outward normal),
while the reference's reflected trial element keeps the order, so vertex-sharing
pairs across the plane use differently oriented Duffy rules.  That difference
is the Duffy rule's own error: it falls from 6e-4 at order 2 to 4e-5 at order 4
in the folded operators and to ~5e-6 in the solutions, which is the tolerance
used here (an error in the symmetric formulation itself is O(1)).
Also: the reference's snapping and validation rules.
"""

import numpy as np
import pytest

from conftest import pkg_module

meshes = pkg_module("meshes")


@pytest.fixture(scope="module")
def oracle_mod():
    from oracle.build import build_oracle
    from oracle import oracle

    build_oracle()
    return oracle


def _pts():
    return np.array([[0.4, 0.3, 1.5], [1.2, -0.8, 0.2], [-0.6, 0.5, -1.1], [0.0, 0.0, 2.0], [0.3, 0.0, 0.9]])


@pytest.mark.parametrize("mode", ["x", "xy"])
def test_symmetric_model_equals_full_model(oracle_mod, mode):
    box = meshes.box_with_piston((0.3, 0.2, 0.25), 600, 0.05, "+z")  # 8 x 6 cells: grid lines on x = 0, y = 0
    part = meshes.fundamental_domain(box, mode)
    full, index = meshes.mirror_to_full(part, mode)
    k = 2 * np.pi * 900.0 / 343.0
    q_part = np.where(part.tags == meshes.RADIATOR_TAG, 1j * 1.205 * 2 * np.pi * 900.0, 0).astype(np.complex128)
    q_full = np.where(full.tags == meshes.RADIATOR_TAG, 1j * 1.205 * 2 * np.pi * 900.0, 0).astype(np.complex128)
    pts = _pts()
    ref = oracle_mod.solve_frequency(full, k, q_full, pts)
    sym = oracle_mod.solve_frequency(part, k, q_part, pts, symmetry=mode)
    p_full = ref.pressure[index, 0]
    assert np.linalg.norm(sym.pressure[:, 0] - p_full) / np.linalg.norm(p_full) < 2e-5
    assert np.linalg.norm(sym.field[:, 0] - ref.field[:, 0]) / np.linalg.norm(ref.field[:, 0]) < 2e-5


def test_folded_operators_converge_with_duffy_order(oracle_mod):
    part = meshes.fundamental_domain(meshes.box_with_piston((0.3, 0.2, 0.25), 600, 0.05, "+z"), "x")
    full, index = meshes.mirror_to_full(part, "x")
    pos = {tuple(np.round(p, 12)): i for i, p in enumerate(part.vertices)}
    fold = np.array([pos[tuple(np.round(p * np.array([np.sign(p[0]) or 1.0, 1.0, 1.0]), 12))] for p in full.vertices])
    k = 2 * np.pi * 900.0 / 343.0
    gaps = []
    for order in (2, 4):
        d_full = oracle_mod.assemble(full, k, singular_order=order).double_layer
        d_sym = oracle_mod.assemble(part, k, singular_order=order, symmetry="x").double_layer
        folded = np.zeros_like(d_sym)
        for c in range(full.n_vertices):
            folded[:, fold[c]] += d_full[index, c]
        gaps.append(np.linalg.norm(folded - d_sym) / np.linalg.norm(d_sym))
    assert gaps[1] < 1e-4 and gaps[1] < gaps[0] / 10, gaps


def test_symmetric_operators_have_orbit_row_weights(oracle_mod):
    part = meshes.fundamental_domain(meshes.box_with_piston((0.3, 0.2, 0.25), 600, 0.05, "+z"), "x")
    M11, M10 = oracle_mod.mass(part, symmetry="x")
    M11_off, M10_off = oracle_mod.mass(part)
    w = meshes.p1_symmetry_orbit_weights(part, "x")
    assert set(np.unique(w)) == {1.0, 2.0}
    np.testing.assert_allclose(M11, w[:, None] * M11_off, rtol=1e-14)
    np.testing.assert_allclose(M10, w[:, None] * M10_off, rtol=1e-14)


def test_snapping_and_fundamental_domain_validation():
    v = np.array([[1e-12, 0.0, 0.0], [1.0, 0.0, 0.0], [0.5, 1.0, 0.0], [-3e-12, 1.0, 1.0]])
    f = np.array([[0, 1, 2], [0, 2, 3]], np.int32)
    mesh = meshes.BoundaryMesh(v, f, np.ones(2, np.int32))
    snapped = meshes.snap_symmetry_planes(mesh, "x")
    assert snapped.vertices[0, 0] == 0.0 and snapped.vertices[3, 0] == 0.0
    meshes.validate_symmetry_fundamental_domain(snapped, "x")
    bad = meshes.BoundaryMesh(v - np.array([0.1, 0, 0]), f, np.ones(2, np.int32))
    with pytest.raises(ValueError, match="positive X fundamental domain"):
        meshes.validate_symmetry_fundamental_domain(bad, "x")
    assert meshes.snap_symmetry_planes(mesh, "off") is mesh
