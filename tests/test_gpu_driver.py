"""The C++ MD driver (reference command line, infile, restart port, outfiles) on the GPU.

The same infile, injected restart_0.out and command line as the reference run stored in the
golden fixture; energy.out and restart_<T>.out must have the reference's layout (header,
rows, columns) and agree to the digits the reference prints (6 significant digits in
energy.out, 12 in restart files) within FP32-force tolerances.
"""
import os
import subprocess

import numpy as np
import pytest

from conftest import REPO, load_golden

pytestmark = pytest.mark.gpu
DRIVER = os.path.join(REPO, "capsid-souffle_gb300", "_build", "souffle_gb300")


def _run_driver(tmp_path, g, key="md_args"):
    from souffle_gb300 import geometry, state
    t = geometry.template_by_name(str(g["template"]))
    os.makedirs(tmp_path / "infiles")
    os.makedirs(tmp_path / "outfiles")
    geometry.write_infile(t, str(tmp_path / "infiles" / t.name))
    state.write_restart(state.State(g["pos"], g["vel"], float(g["box"])), str(tmp_path / "outfiles"),
                        big_bead_pos=g["big_pos_in"] if "big_pos_in" in g else None)
    args = [str(x) for x in g[key]]
    r = subprocess.run([DRIVER] + args, cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    return args


def _rows(text):
    lines = text.strip().splitlines()
    return lines[0], [[float(x) for x in ln.split()] for ln in lines[1:]]


@pytest.mark.parametrize("name", ["plain_small", "bilayer_dense"])
def test_driver_outfiles_match_reference_run(tmp_path, name):
    g = load_golden(name)
    _run_driver(tmp_path, g)
    head_r, rows_r = _rows(str(g["md_energy_text"]))
    head_g, rows_g = _rows(open(tmp_path / "outfiles" / "energy.out").read())
    assert head_g == head_r
    assert len(rows_g) == len(rows_r)
    for rr, rg in zip(rows_r, rows_g):
        assert len(rg) == len(rr)
        assert rg[0] == rr[0]                       # step
        for k in range(1, len(rr)):
            if k == 11:
                # |v_com| removed per step: round-off of the net force, ~1e-16 in long double,
                # ~1e-8 with FP32 forces; both remove it every step
                assert abs(rg[k]) < 1e-6 and abs(rr[k]) < 1e-6
                continue
            assert rg[k] == pytest.approx(rr[k], rel=5e-5, abs=5e-6), (rr[0], k)
    T = int(g["md_steps"])
    ref_lines = str(g["md_restart_text"]).strip().splitlines()
    our_lines = open(tmp_path / "outfiles" / f"restart_{T}.out").read().strip().splitlines()
    assert our_lines[0] == ref_lines[0]
    assert len(our_lines) == len(ref_lines)
    a = np.array([[float(x) for x in ln.split()] for ln in our_lines[1:]])
    b = np.array([[float(x) for x in ln.split()] for ln in ref_lines[1:]])
    assert np.array_equal(a[:, 0], b[:, 0])
    np.testing.assert_allclose(a[:, 1:], b[:, 1:], rtol=0, atol=2e-6 * max(1.0, np.abs(b).max()))


@pytest.mark.parametrize("name", ["plain_small", "bilayer_dense"])
def test_driver_brownian_run_matches_reference_run(tmp_path, name):
    """-D b through the driver: energy.out rows and the final restart file against the
    reference's own Brownian run from the same state (noise sequence included)."""
    g = load_golden(name)
    _run_driver(tmp_path, g, "bd_args")
    params = open(tmp_path / "outfiles" / "model.parameters.out").read()
    assert params.splitlines()[0] == "Running brownian dynamics."
    rows_r = np.asarray(g["bd_energy_rows"])
    _, rows_g = _rows(open(tmp_path / "outfiles" / "energy.out").read())
    rows_g = np.array([r[:11] for r in rows_g])
    assert rows_g.shape == rows_r.shape
    assert np.array_equal(rows_g[:, 0], rows_r[:, 0])
    np.testing.assert_allclose(rows_g[:, 1:], rows_r[:, 1:], rtol=5e-5, atol=5e-6)
    assert np.all(rows_g[:, 9:11] == 0)             # no thermostat in Brownian runs
    from souffle_gb300 import state
    T = int(g["md_steps"])
    _, vel, pos = state.read_restart(str(tmp_path / "outfiles" / f"restart_{T}.out"))
    L = float(g["box"])
    dp = pos - g["bd_pos"]
    dp -= L * np.round(dp / L)
    assert np.abs(dp).max() < 1e-6
    assert np.abs(vel - g["bd_vel"]).max() < 1e-5 * max(1.0, np.abs(g["bd_vel"]).max())


def test_driver_restart_resume_continues_the_run(tmp_path):
    """Resuming from the last restart file (-R) continues at its step, like the reference."""
    g = load_golden("plain_small")
    args = _run_driver(tmp_path, g)
    T = int(g["md_steps"])
    args2 = list(args)
    args2[args2.index("-T") + 1] = str(2 * T)
    r = subprocess.run([DRIVER] + args2, cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert f"Restarting from: restart_{T}.out" in r.stdout
    assert (tmp_path / "outfiles" / f"restart_{2 * T}.out").exists()


def test_driver_rejects_missing_infile(tmp_path):
    os.makedirs(tmp_path / "outfiles")
    r = subprocess.run([DRIVER, "-f", "nonexistent", "-S", "2"], cwd=tmp_path, capture_output=True,
                       text=True, timeout=60)
    assert r.returncode == 1
    assert "NOT OPENED" in r.stderr


@pytest.mark.parametrize("mode", ["md", "bd"])
def test_driver_encapsulation_run_matches_reference_run(tmp_path, mode):
    """-p true with three big beads read from outfiles/rb_0.out: energy.out and capenergy.out
    rows and the final restart file against the reference's own run from the same state."""
    g = load_golden("bigbead")
    _run_driver(tmp_path, g, f"{mode}_args")
    rows_r = np.asarray(g[f"{mode}_energy_rows"])
    _, rows_g = _rows(open(tmp_path / "outfiles" / "energy.out").read())
    rows_g = np.array([r[:11] for r in rows_g])
    assert rows_g.shape == rows_r.shape
    np.testing.assert_allclose(rows_g[:, 1:], rows_r[:, 1:], rtol=5e-5, atol=5e-6)
    cap_r = np.array([[float(x) for x in ln.split()] for ln in str(g[f"{mode}_cap_text"]).strip().splitlines()])
    cap_g = np.array([[float(x) for x in ln.split()]
                      for ln in open(tmp_path / "outfiles" / "capenergy.out").read().strip().splitlines()])
    assert cap_g.shape == cap_r.shape and cap_r.shape[1] == 6
    assert np.array_equal(cap_g[:, 0], cap_r[:, 0])
    np.testing.assert_allclose(cap_g[:, 1:], cap_r[:, 1:], rtol=5e-5, atol=5e-6)
    from souffle_gb300 import state
    T = int(g["md_steps"])
    _, vel, pos = state.read_restart(str(tmp_path / "outfiles" / f"restart_{T}.out"))
    L = float(g["box"])
    dp = pos - g[f"{mode}_pos"]
    dp -= L * np.round(dp / L)
    assert np.abs(dp).max() < 1e-6
    assert (tmp_path / "outfiles" / f"rb_{T}.out").exists()
    rb = np.loadtxt(str(tmp_path / "outfiles" / f"rb_{T}.out"))
    np.testing.assert_allclose(rb[:, 3:6], g["big_pos_in"], rtol=1e-11, atol=1e-11)
