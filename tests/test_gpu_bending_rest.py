"""The rest-dihedral bending option on the GPU (souffle_template.bend_rest_pos; no reference
counterpart): bending forces and energies against the FP64 restatement in oracle/bending_oracle.py,
zero bending force in the rest shape, and the reference's bending exactly when the rest shape is
flat."""
import os
import sys

import numpy as np
import pytest

from conftest import REPO, rms_rel

pytestmark = pytest.mark.gpu
sys.path.insert(0, os.path.join(REPO, "oracle"))
import bending_oracle as BO  # noqa: E402


def _system(t, n_sub=20, seed=5, noise=0.05):
    from souffle_gb300 import gpu, workloads
    w = workloads.make(t, n_sub, seed=seed)
    p = gpu.system_params(w.opt, w.derived, n_sub, w.center_local)
    s = gpu.GpuSystem(t, [p])
    pos = w.state.pos + np.random.default_rng(seed).normal(0, noise, w.state.pos.shape) if noise else w.state.pos
    s.set_state(pos, w.state.vel)
    return w, s, pos


@pytest.mark.parametrize("name", ["patch_n3", "bilayer_n5"])
def test_rest_bending_matches_oracle(name):
    from souffle_gb300 import geometry
    t = geometry.with_rest_dihedral(geometry.template_by_name(name, 6.0))
    w, s, pos = _system(t)
    _, _, bf = s.forces(rebuild=True, parts=True)
    _, pb = s.energies(per_bead=True)
    qs = BO.quads(t.edges, t.edge_type, [tuple(f) for f in t.faces])
    beta0 = BO.rest_angles(t.bend_rest, qs)
    assert np.abs(beta0).max() > 0.05
    np_ = t.n_beads
    L = float(w.derived.box)
    ref_f = np.zeros_like(pos)
    ref_e = np.zeros(len(pos))
    for k in range(len(pos) // np_):
        x = pos[k * np_:(k + 1) * np_]
        x = x[0] + ((x - x[0]) - L * np.round((x - x[0]) / L))   # unwrap the subunit
        f, e = BO.forces_and_bead_energies(x, qs, beta0, float(w.opt.b))
        ref_f[k * np_:(k + 1) * np_] = f
        ref_e[k * np_:(k + 1) * np_] = e
    assert rms_rel(bf, ref_f) <= 1e-5, rms_rel(bf, ref_f)
    np.testing.assert_allclose(pb["be"], ref_e, rtol=1e-7, atol=1e-9 * np.abs(ref_e).max())


def test_rest_shape_has_no_bending_force_and_flat_rest_is_the_reference():
    from souffle_gb300 import geometry
    t = geometry.with_rest_dihedral(geometry.patch_n3(6.0))
    w, s, pos = _system(t, noise=0.0)
    _, _, bf = s.forces(rebuild=True, parts=True)
    assert np.abs(bf).max() < 1e-4 * float(w.opt.b)
    plain = geometry.patch_n3(6.0)
    flat = geometry.dataclasses.replace(plain, bend_rest=geometry.patch_n3(0.0).pos)
    _, s1, p1 = _system(plain)
    _, s2, p2 = _system(flat)
    r1, r2 = s1.forces(rebuild=True, parts=True), s2.forces(rebuild=True, parts=True)
    assert all(np.array_equal(a, b) for a, b in zip(r1, r2))


def test_md_with_rest_dihedrals_is_stable():
    from souffle_gb300 import geometry
    t = geometry.with_rest_dihedral(geometry.bilayer_n5(6.0))
    w, s, pos = _system(t, n_sub=40, noise=0.0)
    s.md_begin()
    s.md_steps(0, 300)
    e = s.energies()
    assert np.isfinite(e["bending"]) and 0.3 < e["temperature"] < 3.0
