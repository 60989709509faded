"""Encapsulation big beads (-p) on the GPU, through the C ABI (souffle_gpu_set_big_beads),
against the reference's own forces, energies and 20-step MD and Brownian runs with three big
beads among 20 capsomeres (tests/golden/bigbead.npz, made by tests/golden/make_golden.py).

Tolerances as for the plain path: per-bead force RMS relative error <= 1e-5 (FP32 terms,
fixed-point sums); energies FP64 (relative 1e-9 of the scale); trajectories to the reference
restart file's 12 digits and the FP32 force error."""
import dataclasses

import numpy as np
import pytest

from conftest import golden_workload, load_golden, rms_rel

pytestmark = pytest.mark.gpu
FORCE_RMS_TOL = 1e-5


def _gpu(g, **opt_over):
    from souffle_gb300 import gpu
    t, opt, d = golden_workload(g)
    if opt_over:
        opt = dataclasses.replace(opt, **opt_over)
    s = gpu.GpuSystem(t, [gpu.system_params(opt, d, int(g["n_sub"]), int(g["center"]))])
    s.set_state(g["pos"], g["vel"])
    s.set_big_beads(g["big_pos"], float(g["big_sigma"]), float(g["big_charge"]), float(g["big_shc"]))
    return s, t, opt, d


def test_big_bead_forces_match_reference():
    g = load_golden("bigbead")
    s, t, opt, d = _gpu(g)
    f = s.forces(rebuild=True)
    err = rms_rel(f, g["tforce"])
    print(f"force RMS relative error with big beads: {err:.2e}")
    assert err <= FORCE_RMS_TOL
    # the big beads matter: without them the forces differ by far more than the tolerance
    s.set_big_beads(np.zeros((0, 3)), 6.0, -78.0, 3.5)
    f0 = s.forces(rebuild=True)
    assert rms_rel(f0, g["tforce"]) > 100 * FORCE_RMS_TOL


def test_big_bead_energies_match_reference():
    g = load_golden("bigbead")
    s, t, opt, d = _gpu(g)
    tot, per = s.energies(per_bead=True)
    scale = max(np.abs(g["ne"]).max(), np.abs(g["ce"]).max())
    np.testing.assert_allclose(per["ne"], g["ne"], rtol=1e-9, atol=1e-9 * scale)
    np.testing.assert_allclose(per["ce"], g["ce"], rtol=1e-9, atol=1e-9 * scale)
    assert tot["bigbead_lj"] == pytest.approx(float(g["big_ne"]), rel=1e-9)
    assert tot["bigbead_electrostatic"] == pytest.approx(float(g["big_ce"]), rel=1e-9)
    assert tot["lj"] == pytest.approx(float(np.sum(g["ne"])), rel=1e-9)


@pytest.mark.parametrize("mode", ["md", "bd"])
def test_big_bead_runs_match_reference_run(mode):
    """20 MD (Nose-Hoover) or Brownian steps with the big beads against the reference's own run
    from the same state; the Brownian run also checks the noise sequence, which draws three
    uniforms per big bead after the subunit beads' every step (src/md.cpp:482-487)."""
    from souffle_gb300.workloads import base_options
    g = load_golden("bigbead")
    over = {"D": "b", "d": 100.0} if mode == "bd" else {}
    s, t, opt, d = _gpu(g, **over)
    s.md_begin()
    s.md_steps(0, int(g["md_steps"]) + 1)      # T+1 iterations (src/md.cpp:387)
    pos, vel = s.get_state()
    L = float(g["box"])
    dp = pos - g[f"{mode}_pos"]
    dp -= L * np.round(dp / L)
    assert np.abs(dp).max() < 1e-6
    assert np.abs(vel - g[f"{mode}_vel"]).max() < 1e-5 * max(1.0, np.abs(g[f"{mode}_vel"]).max())
    e = s.energies()
    row = g[f"{mode}_energy_rows"][-1]
    assert e["temperature"] == pytest.approx(row[8], rel=2e-5)
    n = pos.shape[0]
    assert e["lj"] / n == pytest.approx(row[4], rel=2e-5, abs=1e-6)
    assert base_options().B == 10


def test_big_beads_of_one_system_leave_the_others_alone():
    """Big beads in the second system of a handle: the first system's forces are bitwise those
    of the same system alone, the second's those of a handle holding it alone."""
    from souffle_gb300 import gpu
    g = load_golden("bigbead")
    t, opt, d = golden_workload(g)
    p = gpu.system_params(opt, d, int(g["n_sub"]), int(g["center"]))
    two = gpu.GpuSystem(t, [p, p])
    two.set_state(np.concatenate([g["pos"], g["pos"]]), np.concatenate([g["vel"], g["vel"]]))
    two.set_big_beads(g["big_pos"], float(g["big_sigma"]), float(g["big_charge"]), float(g["big_shc"]), system=1)
    f2 = two.forces(rebuild=True)
    plain = gpu.GpuSystem(t, [p])
    plain.set_state(g["pos"], g["vel"])
    fp = plain.forces(rebuild=True)
    s, _, _, _ = _gpu(g)
    fb = s.forces(rebuild=True)
    n = g["pos"].shape[0]
    assert np.array_equal(f2[:n], fp)
    assert np.array_equal(f2[n:], fb)


def test_bad_big_beads_are_rejected():
    from souffle_gb300 import gpu
    g = load_golden("bigbead")
    s, t, opt, d = _gpu(g)
    with pytest.raises(gpu.SouffleError):
        s.set_big_beads(g["big_pos"], -1.0, -78.0, 3.5)
    with pytest.raises(gpu.SouffleError):
        s.set_big_beads(g["big_pos"] + 10 * float(g["box"]), 6.0, -78.0, 3.5)
    with pytest.raises(gpu.SouffleError):
        s.set_big_beads(g["big_pos"], 6.0, -78.0, 3.5, system=5)
