"""GPU path (through the C ABI) against the reference's fixtures and the oracle.

Tolerances: forces are FP32 with 64-bit fixed-point accumulation, so the per-bead
force RMS relative error against the FP64/long-double reference must be <= 1e-5;
pair sets are integer results and must be identical; energies are FP64 sums of
exact-difference terms (relative 1e-9 of the total scale).
"""
import numpy as np
import pytest

from conftest import GOLDEN_CASES, golden_workload, load_golden, rms_rel

pytestmark = pytest.mark.gpu
FORCE_RMS_TOL = 1e-5


def _gpu(g, **kw):
    from souffle_gb300 import gpu
    t, opt, d = golden_workload(g)
    p = gpu.system_params(opt, d, int(g["n_sub"]), int(g["center"]))
    s = gpu.GpuSystem(t, [p], **kw)
    s.set_state(g["pos"], g["vel"])
    return s, t, opt, d


def _ref_sets(g):
    c, ids = g["nl_counts"], g["nl_ids"]
    return [set(ids[i, :c[i]].tolist()) for i in range(len(c))]


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_forces_match_reference(name):
    g = load_golden(name)
    s, t, opt, d = _gpu(g)
    tf, sf, bf = s.forces(rebuild=True, parts=True)
    assert rms_rel(tf, g["tforce"]) <= FORCE_RMS_TOL, rms_rel(tf, g["tforce"])
    assert rms_rel(bf, g["bforce"]) <= FORCE_RMS_TOL
    # stretching forces are tiny at rest length; compare against the total force scale
    assert np.sqrt(((sf - g["sforce"]) ** 2).sum() / (g["tforce"] ** 2).sum()) <= FORCE_RMS_TOL


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_pairlist_identical_to_reference(name):
    g = load_golden(name)
    s, t, opt, d = _gpu(g)
    s.forces(rebuild=True)
    cap = int(g["nlist_capacity"])
    counts, ids = s.pairlist(cap)
    assert np.array_equal(counts, g["nl_counts"])
    w = g["nl_ids"].shape[1]
    assert np.array_equal(ids[:, :w], g["nl_ids"])   # same entries in the same (ascending) order
    st = s.pairlist_stats()
    assert st["mean_length"] == pytest.approx(g["nl_counts"].mean())
    assert st["max_length"] == g["nl_counts"].max()


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_energies_match_reference(name):
    g = load_golden(name)
    s, t, opt, d = _gpu(g)
    tot, pb = s.energies(per_bead=True)
    scale = max(1.0, sum(abs(g[k]).sum() for k in ("se", "be", "ne", "ce", "ke")))
    for k in ("se", "be", "ne", "ce", "ke"):
        np.testing.assert_allclose(pb[k], g[k], rtol=1e-7, atol=1e-9 * scale / len(g[k]))
    # velocities are held in 2^-40 fixed point: 1e-12 of a unit velocity
    assert tot["kinetic"] == pytest.approx(g["ke"].sum(), rel=1e-10)
    assert tot["lj"] == pytest.approx(g["ne"].sum(), rel=1e-9, abs=1e-9)
    assert tot["electrostatic"] == pytest.approx(g["ce"].sum(), rel=1e-9, abs=1e-9)


# patch_crowded starts from overlapping subunits and blows up within 20 steps in the reference
# itself (|v| ~ 1e9), so it pins forces, lists and energies but not a trajectory.
@pytest.mark.parametrize("name", ["plain_small", "bilayer_dense"])
def test_md_steps_match_reference_run(name):
    g = load_golden(name)
    s, t, opt, d = _gpu(g)
    s.md_begin()
    n = int(g["md_steps"]) + 1        # loop runs T+1 iterations (src/md.cpp:387)
    s.md_steps(0, n)
    pos, vel = s.get_state()
    L = float(g["box"])
    dp = pos - g["md_pos"]
    dp -= L * np.round(dp / L)
    assert np.abs(dp).max() < 1e-6
    assert np.abs(vel - g["md_vel"]).max() < 1e-5 * max(1.0, np.abs(g["md_vel"]).max())
    # temperature column of energy.out (6 significant digits in the reference file)
    tot = s.energies()
    assert tot["temperature"] == pytest.approx(g["md_energy_rows"][-1, 8], rel=2e-5)


# KE tolerance per fixture over 100 steps: FP32 force differences (~1e-7 relative) grow
# chaotically, fastest in the dense overlapping bilayer state (forces up to ~4e3).
@pytest.mark.parametrize("name,tol", [("plain_small", 1e-5), ("bilayer_dense", 5e-5)])
def test_md_long_run_tracks_oracle(name, tol):
    """100 steps: the kinetic-energy trajectory against the oracle, step by step."""
    import pyoracle
    g = load_golden(name)
    s, t, opt, d = _gpu(g)
    o = pyoracle.Oracle(t, int(g["n_sub"]), d, opt.s, opt.b, opt.E, int(g["center"]))
    o.set_state(g["pos"], g["vel"])
    o.forces(True)
    ke_o = o.kinetic_energy()
    o.nhc_init(int(opt.q), opt.Q, opt.K)
    s.md_begin()
    for a in range(100):
        ke_o, vc_o, _ = o.md_step(a, opt.t, int(opt.B), ke_o)
        s.md_steps(a, 1)
        ke_g, xi_g, vc_g = s.md_scalars()
        assert ke_g == pytest.approx(ke_o, rel=tol), a
    po, vo = o.get_state()
    pg, vg = s.get_state()
    L = float(g["box"])
    dp = pg - po
    dp -= L * np.round(dp / L)
    assert np.abs(dp).max() < 100 * tol


def test_runs_are_bitwise_deterministic():
    g = load_golden("bilayer_dense")
    out = []
    for _ in range(2):
        s, *_ = _gpu(g)
        s.md_begin()
        s.md_steps(0, 25)
        out.append(s.get_state())
        s.close()
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])


def test_graph_windows_equal_single_steps():
    g = load_golden("plain_small")
    s1, *_ = _gpu(g)
    s1.md_begin()
    s1.md_steps(0, 30)           # three 10-step graph windows
    s2, *_ = _gpu(g)
    s2.md_begin()
    for a in range(30):
        s2.md_steps(a, 1)        # direct launches
    p1, v1 = s1.get_state()
    p2, v2 = s2.get_state()
    assert np.array_equal(p1, p2) and np.array_equal(v1, v2)


def test_async_snapshots_equal_synchronous_state():
    """souffle_gpu_snapshot_enqueue behind queued steps returns the state get_state returns after
    the same steps run synchronously, in both slots, with windows queued between the snapshots."""
    g = load_golden("bilayer_dense")
    s1, *_ = _gpu(g)
    s1.md_begin()
    n = s1.n
    p0, v0 = np.full((n, 3), np.nan), np.full((n, 3), np.nan)
    p1, v1 = np.full((n, 3), np.nan), np.full((n, 3), np.nan)
    s1.md_enqueue(0, 7)
    s1.snapshot_enqueue(0, p0, v0)
    s1.md_enqueue(7, 16)
    s1.snapshot_enqueue(1, p1, None)
    s1.snapshot_wait(0)
    s1.snapshot_wait(1)
    s2, *_ = _gpu(g)
    s2.md_begin()
    s2.md_steps(0, 7)
    q0, w0 = s2.get_state()
    s2.md_steps(7, 16)
    q1, _ = s2.get_state()
    assert np.array_equal(p0, q0) and np.array_equal(v0, w0) and np.array_equal(p1, q1)
    assert np.isnan(v1).all()                        # no velocities asked for in slot 1
    # a slot holds one snapshot at a time
    s1.snapshot_enqueue(0, p0, None)
    with pytest.raises(RuntimeError):
        s1.snapshot_enqueue(0, p0, None)
    s1.snapshot_wait(0)


def test_batched_systems_equal_separate_runs():
    """Replicas in one handle give bitwise the same trajectories as separate handles."""
    from souffle_gb300 import gpu, workloads
    reps = workloads.replicas(3, seed=11, sub_range=(20, 40))
    params = [gpu.system_params(w.opt, w.derived, int(w.opt.S), w.center_local) for w in reps]
    batch = gpu.GpuSystem(reps[0].template, params)
    batch.set_state(np.concatenate([w.state.pos for w in reps]), np.concatenate([w.state.vel for w in reps]))
    batch.md_begin()
    batch.md_steps(0, 20)
    pb, vb = batch.get_state()
    off = 0
    for w, p in zip(reps, params):
        one = gpu.GpuSystem(w.template, [p])
        one.set_state(w.state.pos, w.state.vel)
        one.md_begin()
        one.md_steps(0, 20)
        po, vo = one.get_state()
        n = po.shape[0]
        assert np.array_equal(pb[off:off + n], po)
        assert np.array_equal(vb[off:off + n], vo)
        off += n


def test_inter_capacity_overflow_is_reported():
    from souffle_gb300 import gpu
    g = load_golden("bilayer_dense")
    s, *_ = _gpu(g, inter_capacity=4)
    with pytest.raises(gpu.SouffleError) as e:
        s.forces(rebuild=True)
    assert e.value.code == 3


def test_bad_template_is_rejected():
    from souffle_gb300 import gpu, geometry
    g = load_golden("plain_small")
    t, opt, d = golden_workload(g)
    t.faces = t.faces[:2]
    with pytest.raises(gpu.SouffleError) as e:
        gpu.GpuSystem(t, [gpu.system_params(opt, d, 20, 5)])
    assert e.value.code == 1


def test_thermostat_chain_bitwise_equals_host_double_float(tmp_path):
    """The device chain (one lane per link) against the same double-float arithmetic run serially
    on the host, fed the kinetic energies the GPU produced: every step's xi_0 is bitwise equal."""
    from conftest import build_thermostat_lib, chain_of, run_host_chain
    lib = build_thermostat_lib(tmp_path)
    g = load_golden("plain_small")
    s, t, opt, d = _gpu(g)
    s.md_begin()
    ke0, _, _ = s.md_scalars()
    kes, xis = [ke0], []
    for a in range(60):
        s.md_steps(a, 1)
        ke, xi0, _ = s.md_scalars()
        kes.append(ke)
        xis.append(xi0)
    n3 = 3.0 * t.n_beads * int(g["n_sub"])
    q, temp, dof = chain_of(int(opt.q), opt.Q, d.T_reduced, n3)
    rc, rows = run_host_chain(lib, q, temp, dof, opt.t, kes)
    assert rc == 60
    assert np.array_equal(rows[:, 0], np.array(xis)), np.abs(rows[:, 0] - np.array(xis)).max()
    assert np.abs(np.array(xis)).max() > 0


def test_cta_shapes_and_autotuner_give_identical_results():
    """Every force-kernel CTA shape gives bitwise the same forces and trajectory (sums are exact
    fixed point); the autotuner keeps the fastest shape it measured."""
    g = load_golden("bilayer_dense")
    ref, *_ = _gpu(g)
    f0 = ref.forces(rebuild=True)
    ref.md_begin()
    ref.md_steps(0, 15)
    p0, v0 = ref.get_state()
    for subs, thr in [(1, 128), (2, 192), (4, 256), (6, 128)]:
        s, *_ = _gpu(g, threads_per_cta=thr, subunits_per_cta=subs)
        assert np.array_equal(s.forces(rebuild=True), f0), (subs, thr)
        s.md_begin()
        s.md_steps(0, 15)
        p, v = s.get_state()
        assert np.array_equal(p, p0) and np.array_equal(v, v0), (subs, thr)
    s, *_ = _gpu(g)
    t = s.autotune(trials=5)
    assert t["candidates"] >= 3 and 0 < t["forces_us"] <= t["default_forces_us"]
    assert np.array_equal(s.forces(rebuild=True), f0)
    s.md_begin()
    s.md_steps(0, 15)
    p, v = s.get_state()
    assert np.array_equal(p, p0) and np.array_equal(v, v0)


def test_bad_cta_shape_is_rejected():
    from souffle_gb300 import gpu
    g = load_golden("plain_small")
    with pytest.raises(gpu.SouffleError) as e:
        _gpu(g, threads_per_cta=100)
    assert e.value.code == 1


@pytest.mark.parametrize("name", ["plain_small", "bilayer_dense"])
def test_brownian_steps_match_reference_run(name):
    """-D b: the reference's Brownian dynamics, including its noise sequence (minstd_rand0 seeded
    69521, uniform in [-0.5, 0.5) through libstdc++'s generate_canonical), against the
    reference's own 20-step run from the same state."""
    import dataclasses
    from souffle_gb300 import gpu
    g = load_golden(name)
    t, opt, d = golden_workload(g)
    opt = dataclasses.replace(opt, D="b", d=float(g["bd_damp"]))
    s = gpu.GpuSystem(t, [gpu.system_params(opt, d, int(g["n_sub"]), int(g["center"]))])
    s.set_state(g["pos"], g["vel"])
    s.md_begin()
    s.md_steps(0, int(g["md_steps"]) + 1)      # T+1 iterations (src/md.cpp:387)
    pos, vel = s.get_state()
    L = float(g["box"])
    dp = pos - g["bd_pos"]
    dp -= L * np.round(dp / L)
    assert np.abs(dp).max() < 1e-6
    assert np.abs(vel - g["bd_vel"]).max() < 1e-5 * max(1.0, np.abs(g["bd_vel"]).max())
    e = s.energies()
    assert e["temperature"] == pytest.approx(g["bd_energy_rows"][-1, 8], rel=2e-5)
    assert e["thermo_pe"] == 0 and e["thermo_ke"] == 0      # no thermostat in Brownian runs


def test_fp64_chain_variant_tracks_oracle_and_double_float_chain():
    """The FP64 thermostat chain (souffle_options.chain_fp64, one thread, the reference's double
    arithmetic) against the oracle over 100 steps, and against the default double-float chain at
    the same step: the two chains differ by their rounding (2^-53 against ~2^-46 per operation),
    which the trajectory amplifies about a hundredfold per hundred steps on this system."""
    import pyoracle
    g = load_golden("plain_small")
    s64, t, opt, d = _gpu(g, chain_fp64=True)
    o = pyoracle.Oracle(t, int(g["n_sub"]), d, opt.s, opt.b, opt.E, int(g["center"]))
    o.set_state(g["pos"], g["vel"])
    o.forces(True)
    ke_o = o.kinetic_energy()
    o.nhc_init(int(opt.q), opt.Q, opt.K)
    s64.md_begin()
    for a in range(100):
        ke_o, _, _ = o.md_step(a, opt.t, int(opt.B), ke_o)
        s64.md_steps(a, 1)
        ke_g, xi_g, _ = s64.md_scalars()
        assert ke_g == pytest.approx(ke_o, rel=1e-5), a
    assert xi_g == pytest.approx(o.nhc.xi[0], rel=1e-5, abs=1e-9)
    sdf, *_ = _gpu(g)
    sdf.md_begin()
    sdf.md_steps(0, 100)
    k64, x64, _ = s64.md_scalars()
    kdf, xdf, _ = sdf.md_scalars()
    assert k64 == pytest.approx(kdf, rel=1e-9) and x64 == pytest.approx(xdf, rel=1e-9, abs=1e-12)
    e64, edf = s64.energies(), sdf.energies()
    assert e64["thermo_pe"] == pytest.approx(edf["thermo_pe"], rel=1e-9, abs=1e-9)
