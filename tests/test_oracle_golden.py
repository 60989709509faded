"""The oracle (C restatement) against fixtures produced by the reference itself.

On x86-64 the oracle and the reference share the x87 long double, so results
must be identical; on hosts with a different long double (aarch64: IEEE
binary128) they agree to the precision of the wider type's rounding of double
inputs.
"""
import ctypes
import os
import shutil

import numpy as np
import pytest

from conftest import golden_workload, load_golden, GOLDEN_CASES

pyoracle = pytest.importorskip("pyoracle")


def _same_platform(g):
    import platform
    return int(g["ld_mant_dig"]) == 64 and platform.machine() in ("x86_64", "AMD64")


def _oracle(g):
    t, opt, d = golden_workload(g)
    o = pyoracle.Oracle(t, int(g["n_sub"]), d, opt.s, opt.b, opt.E, int(g["center"]))
    o.set_state(g["pos"], g["vel"])
    return o, t, opt, d


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_derived_parameters_match_reference(name):
    g = load_golden(name)
    t, opt, d = golden_workload(g)
    assert d.box == float(g["box"])
    assert d.kappa == float(g["kappa"])
    assert d.ecut_el == float(g["ecut_el"])
    assert d.nlist_cutoff == float(g["nlist_cutoff"])
    assert d.nlist_capacity == int(g["nlist_capacity"])


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_center_bead_matches_reference(name):
    from souffle_gb300 import workloads
    g = load_golden(name)
    t, _, d = golden_workload(g)
    assert workloads.center_bead(g["pos"][:t.n_beads], d.box) == int(g["center"])
    assert pyoracle.Oracle.center_bead(t.n_beads, g["pos"], d.box) == int(g["center"])


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_oracle_forces_pairlist_energies(name):
    g = load_golden(name)
    o, t, opt, d = _oracle(g)
    tf, sf, bf, over = o.forces(True)
    assert over == 0
    counts, ids = o.pairlist()
    assert np.array_equal(counts, g["nl_counts"])
    w = g["nl_ids"].shape[1]
    assert np.array_equal(ids[:, :w], g["nl_ids"])
    e = o.energies()
    if _same_platform(g):
        for k, a in (("tforce", tf), ("sforce", sf), ("bforce", bf)):
            assert np.array_equal(a, g[k]), k
        for k in ("se", "ke", "be", "ne", "ce"):
            assert np.array_equal(e[k], g[k]), k
    else:
        for k, a in (("tforce", tf), ("sforce", sf), ("bforce", bf)):
            np.testing.assert_allclose(a, g[k], rtol=1e-9, atol=1e-9 * np.abs(g[k]).max())
        for k in ("se", "ke", "be", "ne", "ce"):
            np.testing.assert_allclose(e[k], g[k], rtol=1e-9, atol=1e-12)


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_oracle_md_matches_reference_run(name):
    g = load_golden(name)
    o, t, opt, d = _oracle(g)
    o.forces(True)
    ke = o.kinetic_energy()
    o.nhc_init(int(opt.q), opt.Q, opt.K)
    end = o.loop_end(int(g["md_steps"]), opt.t)
    assert end == int(g["md_steps"]) + 1
    for a in range(end):
        ke, vcom, over = o.md_step(a, opt.t, int(opt.B), ke)
    pos, vel = o.get_state()
    # the reference restart file carries 12 significant digits
    np.testing.assert_allclose(pos, g["md_pos"], rtol=0, atol=1e-10 * max(1.0, np.abs(g["md_pos"]).max()))
    np.testing.assert_allclose(vel, g["md_vel"], rtol=0, atol=1e-9 * max(1.0, np.abs(g["md_vel"]).max()))


def test_oracle_detects_overflow():
    """A capacity below the longest list is reported, not written out of bounds."""
    g = load_golden("bilayer_dense")
    t, opt, d = golden_workload(g)
    o = pyoracle.Oracle(t, int(g["n_sub"]), d, opt.s, opt.b, opt.E, int(g["center"]), capacity=20)
    o.set_state(g["pos"], g["vel"])
    _, _, _, over = o.forces(True)
    assert over > 0


def test_oracle_rejects_bending_edge_without_faces():
    from souffle_gb300 import geometry
    t = geometry.patch_n3()
    t.faces = t.faces[:1]
    g = load_golden("plain_small")
    _, opt, d = golden_workload(g)
    with pytest.raises(ValueError):
        pyoracle.Oracle(t, 20, d, opt.s, opt.b, opt.E, 5)


def test_oracle_big_beads_match_reference():
    """Encapsulation: forceCalculation_bigbead and update_LJ_ES_energies_bigbeads
    (src/forces.cpp:174-236, src/energies.cpp:96-137) restated, against the reference's own
    forces and energies with three big beads among the subunits."""
    g = load_golden("bigbead")
    o, t, opt, d = _oracle(g)
    assert np.array_equal(g["big_pos"], g["big_pos_in"])
    o.set_big_beads(g["big_pos"], float(g["big_sigma"]), float(g["big_charge"]), float(g["big_shc"]))
    tf, _, _, over = o.forces(True)
    assert over == 0
    e = o.energies()
    big_ne, big_ce = o.big_bead_energies()
    assert big_ne > 0 and big_ce != 0   # beads inside both ranges
    if _same_platform(g):
        assert np.array_equal(tf, g["tforce"])
        assert np.array_equal(e["ne"], g["ne"]) and np.array_equal(e["ce"], g["ce"])
        assert big_ne == float(g["big_ne"]) and big_ce == float(g["big_ce"])
    else:
        np.testing.assert_allclose(tf, g["tforce"], rtol=1e-9, atol=1e-9 * np.abs(g["tforce"]).max())
        np.testing.assert_allclose(e["ne"], g["ne"], rtol=1e-9, atol=1e-12)
        np.testing.assert_allclose(e["ce"], g["ce"], rtol=1e-9, atol=1e-12)
        assert big_ne == pytest.approx(float(g["big_ne"]), rel=1e-9)
        assert big_ce == pytest.approx(float(g["big_ce"]), rel=1e-9)
    # without the big beads the forces differ
    o.set_big_beads(np.zeros((0, 3)), 6.0, -78.0, 3.5)
    tf0, _, _, _ = o.forces(True)
    assert np.abs(tf0 - g["tforce"]).max() > 1.0
