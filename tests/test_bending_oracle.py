"""The rest-dihedral bending option's CPU restatement (oracle/bending_oracle.py), pinned by finite
differences of its own energy, and reducing to the reference's bending energy at zero rest angle."""
import os
import sys

import numpy as np

from conftest import REPO

sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, os.path.join(REPO, "capsid-souffle_gb300"))
import bending_oracle as BO  # noqa: E402


def _curved_patch():
    from souffle_gb300 import geometry
    t = geometry.with_rest_dihedral(geometry.patch_n3(6.0))
    return t, BO.quads(t.edges, t.edge_type, [tuple(f) for f in t.faces])


def test_gradient_matches_finite_differences():
    t, qs = _curved_patch()
    assert len(qs) > 0
    beta0 = BO.rest_angles(t.bend_rest, qs)
    assert np.all(np.abs(beta0) > 1e-3)                  # the curved rest shape is not flat
    rng = np.random.default_rng(3)
    x = t.pos + rng.normal(0, 0.05, t.pos.shape)
    kb = 7.0
    f, _ = BO.forces_and_bead_energies(x, qs, beta0, kb)
    h = 1e-6
    for i in range(len(x)):
        for d in range(3):
            xp, xm = x.copy(), x.copy()
            xp[i, d] += h
            xm[i, d] -= h
            fd = -(BO.energy(xp, qs, beta0, kb) - BO.energy(xm, qs, beta0, kb)) / (2 * h)
            assert abs(fd - f[i, d]) < 1e-6 * max(1.0, abs(fd)), (i, d, fd, f[i, d])


def test_zero_rest_angle_is_the_reference_energy():
    """beta0 = 0: kb (1 - cos beta) = kb (1 - |n0 . n1|), the reference's bending energy."""
    t, qs = _curved_patch()
    rng = np.random.default_rng(4)
    x = t.pos + rng.normal(0, 0.05, t.pos.shape)
    faces = [tuple(f) for f in t.faces]
    for q in qs:
        b0, b1, a0, a1 = q
        f0 = [f for f in faces if b0 in f and b1 in f]
        n = [np.cross(x[f[1]] - x[f[0]], x[f[2]] - x[f[1]]) for f in f0[:2]]
        c = abs(n[0] @ n[1]) / (np.linalg.norm(n[0]) * np.linalg.norm(n[1]))
        assert abs(np.cos(BO.bend_angle(x, q)) - c) < 1e-12
    flat = BO.rest_angles(geometry_flat_positions(), qs)
    assert np.all(np.abs(flat) < 1e-9)


def geometry_flat_positions():
    from souffle_gb300 import geometry
    return geometry.patch_n3(0.0).pos
