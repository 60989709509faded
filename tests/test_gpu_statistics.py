"""Statistical parity of long MD runs: GPU path vs the oracle (the reference algorithm in long
double), from the same injected state of the 20-capsomere workload.

Trajectories decorrelate after a few hundred steps (FP32 forces differ from the reference at
~1e-7), so the comparison is on statistics over 2000 steps: the temperature mean and spread,
the potential energy, the mean subunit radius of gyration, and the drift of the extended
(thermostat-including) energy, which both integrators should hold to the same order.
"""
import numpy as np
import pytest

from conftest import golden_workload, load_golden

pytestmark = pytest.mark.gpu
STEPS, EVERY = 2000, 20


def _rg(pos, np_, box):
    p = pos.reshape(-1, np_, 3)
    d = p - p[:, :1, :]
    d -= box * np.round(d / box)              # unwrap each subunit around its first bead
    c = d.mean(axis=1, keepdims=True)
    return float(np.sqrt(((d - c) ** 2).sum(axis=2).mean(axis=1)).mean())


def _series_gpu(g):
    from souffle_gb300 import gpu
    t, opt, d = golden_workload(g)
    s = gpu.GpuSystem(t, [gpu.system_params(opt, d, int(g["n_sub"]), int(g["center"]))])
    s.set_state(g["pos"], g["vel"])
    s.md_begin()
    rows = []
    for a in range(0, STEPS, EVERY):
        s.md_steps(a, EVERY)
        e = s.energies()
        pos, _ = s.get_state()
        pot = e["stretching"] + e["bending"] + e["lj"] + e["electrostatic"]
        rows.append((e["temperature"], pot, pot + e["kinetic"] + e["thermo_pe"] + e["thermo_ke"],
                     _rg(pos, t.n_beads, float(g["box"]))))
    return np.array(rows), t


def _series_oracle(g):
    import pyoracle
    t, opt, d = golden_workload(g)
    o = pyoracle.Oracle(t, int(g["n_sub"]), d, opt.s, opt.b, opt.E, int(g["center"]))
    o.set_state(g["pos"], g["vel"])
    o.forces(True)
    ke = o.kinetic_energy()
    o.nhc_init(int(opt.q), opt.Q, opt.K)
    n = t.n_beads * int(g["n_sub"])
    rows = []
    for a in range(STEPS):
        ke, _, _ = o.md_step(a, opt.t, int(opt.B), ke)
        if (a + 1) % EVERY == 0:
            e = o.energies()
            pos, _ = o.get_state()
            c = o.nhc
            tpe = sum(c.dof[j] * c.t[j] * c.eta[j] for j in range(c.m))
            tke = sum(0.5 * c.q[j] * c.xi[j] ** 2 for j in range(c.m))
            kin = e["ke"].sum()
            pot = e["se"].sum() + e["be"].sum() + e["ne"].sum() + e["ce"].sum()
            rows.append((2 * kin / (3 * n), pot, pot + kin + tpe + tke, _rg(pos, t.n_beads, float(g["box"]))))
    return np.array(rows)


def test_long_run_statistics_match_oracle():
    g = load_golden("plain_small")
    G, t = _series_gpu(g)
    O = _series_oracle(g)
    n = t.n_beads * int(g["n_sub"])
    half = len(G) // 2   # equilibrated second half

    def same_mean(k, rel):
        a, b = G[half:, k], O[half:, k]
        se = np.sqrt(a.var() / len(a) + b.var() / len(b))
        return abs(a.mean() - b.mean()) < 4 * se + rel * abs(b.mean())

    tg, to = G[half:, 0], O[half:, 0]
    assert same_mean(0, 0.02)                        # temperature
    assert 0.5 < tg.std() / max(to.std(), 1e-12) < 2.0
    assert same_mean(1, 0.02)                        # potential energy
    assert same_mean(3, 0.01)                        # subunit radius of gyration
    # extended-energy drift per bead over the run, per 10^4 steps
    slope_g = np.polyfit(np.arange(len(G)) * EVERY, G[:, 2], 1)[0] * 1e4 / n
    slope_o = np.polyfit(np.arange(len(O)) * EVERY, O[:, 2], 1)[0] * 1e4 / n
    print(f"T gpu {tg.mean():.4f}+-{tg.std():.4f} oracle {to.mean():.4f}+-{to.std():.4f}; "
          f"Rg gpu {G[half:, 3].mean():.5f} oracle {O[half:, 3].mean():.5f}; "
          f"extended-energy drift per bead per 1e4 steps gpu {slope_g:.3e} oracle {slope_o:.3e}")
    assert abs(slope_g) < 5 * abs(slope_o) + 1e-3
