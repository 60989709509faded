"""GPU path (through the C ABI) against the oracle at the sizes the throughput figures are
quoted on.

The golden fixtures pin the path against the compiled reference on systems of at most 1,260
beads.  These tests pin it against the oracle -- the C restatement of the reference algorithm in
the reference's own long double types, itself pinned bit for bit to the compiled reference by
tests/test_oracle_golden.py -- on:

* the 84,000-bead workload (2000 two-layer 42-bead capsomeres, seed 12345, 800 uM,
  -e 5 -L 0.3 -B 10): pair-list radius 5.3 sigma, centre prefilter 1.5 x 5.3 = 7.95 sigma
  (src/functions.cpp:80-91), which drops real far Debye-Hueckel pairs between 42-bead patches,
  and the reference's list capacity ceil((5.3 + 0.5)^3) = 196 (src/md.cpp:229-239);
* four systems of the replica sweep at its parameter extremes (Debye length 0.5 and 2 sigma,
  200 and 1600 uM, 200-500 subunits, attraction 1.5 and 3 kT) in one batched handle;
* the 840,000-bead single system: forces and pair lists (the reference's energy block visits
  all N^2/2 bead pairs, src/energies.cpp:24-93, too slow for the oracle at this size).

Tolerances as for the fixtures: per-bead force RMS relative error <= 1e-5 (total and bending
forces; stretching forces against the total-force scale, since they vanish at rest length);
pair lists identical in content and order; per-bead energies relative 1e-7; after 20 MD steps
the kinetic energy and the first chain variable relative 1e-6 and positions within 1e-5 sigma.
"""
import numpy as np
import pytest

from conftest import rms_rel

pytestmark = pytest.mark.gpu
FORCE_RMS_TOL = 1e-5
MD_STEPS = 20


def _oracle(w, capacity=None):
    import pyoracle
    o = pyoracle.Oracle(w.template, int(w.opt.S), w.derived, w.opt.s, w.opt.b, w.opt.E, w.center_local,
                        capacity=capacity)
    o.set_state(w.state.pos, w.state.vel)
    return o


def _params(w):
    from souffle_gb300 import gpu
    return gpu.system_params(w.opt, w.derived, int(w.opt.S), w.center_local)


def _check_forces(gf, of):
    """gf, of: (total, stretching, bending) of the GPU and the oracle for one system."""
    tf, sf, bf = gf
    otf, osf, obf = of
    e_t, e_b = rms_rel(tf, otf), rms_rel(bf, obf)
    e_s = float(np.sqrt(((sf - osf) ** 2).sum() / (otf ** 2).sum()))
    assert e_t <= FORCE_RMS_TOL, e_t
    assert e_b <= FORCE_RMS_TOL, e_b
    assert e_s <= FORCE_RMS_TOL, e_s
    return e_t, e_s, e_b


def _check_pairlist(g_counts, g_ids, o_counts, o_ids, offset):
    """The GPU's rows of one system (global ids, -1 padded) against the oracle's (system ids)."""
    assert np.array_equal(g_counts, o_counts)
    w = o_ids.shape[1]
    g = g_ids[:, :w].astype(np.int64)
    g = np.where(g >= 0, g - offset, -1)
    o = np.where(np.arange(w)[None, :] < o_counts[:, None], o_ids, -1)
    assert np.array_equal(g, o)


def _check_energies(pb, oe):
    scale = max(1.0, sum(abs(oe[k]).sum() for k in ("se", "be", "ne", "ce", "ke")))
    for k in ("se", "be", "ne", "ce", "ke"):
        np.testing.assert_allclose(pb[k], oe[k], rtol=1e-7, atol=1e-9 * scale / len(oe[k]), err_msg=k)


def _wrapped_max(a, b, box):
    d = a - b
    d -= box * np.round(d / box)
    return float(np.abs(d).max())


def test_84k_forces_pairlists_energies():
    from souffle_gb300 import gpu, workloads
    w = workloads.plain_large()
    assert w.n_beads == 84000 and w.derived.nlist_capacity == 196
    s = gpu.GpuSystem(w.template, [_params(w)])
    s.set_state(w.state.pos, w.state.vel)
    gf = s.forces(rebuild=True, parts=True)
    o = _oracle(w)
    otf, osf, obf, over = o.forces(True)
    assert over == 0
    errs = _check_forces(gf, (otf, osf, obf))
    print(f"84k force RMS rel err: total {errs[0]:.2e} stretching {errs[1]:.2e} bending {errs[2]:.2e}")
    oc, oi = o.pairlist()
    gc, gi = s.pairlist(o.cap)
    _check_pairlist(gc, gi, oc, oi, 0)
    st = s.pairlist_stats()
    assert st["max_length"] == oc.max() and st["mean_length"] == pytest.approx(oc.mean())
    tot, pb = s.energies(per_bead=True)
    _check_energies(pb, o.energies())


def test_84k_md_steps_track_oracle():
    from souffle_gb300 import gpu, workloads
    w = workloads.plain_large()
    s = gpu.GpuSystem(w.template, [_params(w)])
    s.set_state(w.state.pos, w.state.vel)
    s.md_begin()
    s.md_steps(0, MD_STEPS)
    ke_g, xi_g, _ = s.md_scalars()
    o = _oracle(w)
    o.forces(True)
    ke_o = o.kinetic_energy()
    o.nhc_init(int(w.opt.q), w.opt.Q, w.opt.K)
    for a in range(MD_STEPS):
        ke_o, _, _ = o.md_step(a, w.opt.t, int(w.opt.B), ke_o)
    xi_o = o.nhc.xi[0]
    print(f"84k after {MD_STEPS} steps: KE {ke_g!r} vs {ke_o!r}, xi0 {xi_g!r} vs {xi_o!r}")
    assert ke_g == pytest.approx(ke_o, rel=1e-6)
    assert xi_g == pytest.approx(xi_o, rel=1e-6, abs=1e-12)
    pg, _ = s.get_state()
    po, _ = o.get_state()
    dmax = _wrapped_max(pg, po, w.derived.box)
    print(f"84k after {MD_STEPS} steps: max position deviation {dmax:.2e}")
    assert dmax < 1e-5


def _extreme_replicas():
    """Four systems of the replica sweep at the corners of its parameter ranges."""
    from souffle_gb300 import geometry, state, workloads
    t = geometry.bilayer_n5()
    corners = [(0.5, 200.0, 500, 1.5), (2.0, 1600.0, 500, 3.0), (0.5, 1600.0, 300, 3.0), (2.0, 200.0, 200, 1.5)]
    return [workloads.make(t, S, seed=9100 + k, name=f"extreme{k}", E=eps, c=state.salt_for_debye_length(lam), C=conc)
            for k, (lam, conc, S, eps) in enumerate(corners)]


def test_replica_sweep_extremes_batched():
    """At a Debye length of 0.5 sigma the pair-list radius is 2.8 sigma and the reference's list
    capacity ceil(3.3^3) = 36 (src/md.cpp:229-239) is shorter than the longest lists: the reference
    itself would write past its lists (src/functions.cpp:108-113).  The GPU grows its rows and
    reports those beads (over_reference_capacity); the oracle runs with room for every entry, so
    the comparison is against the complete lists the reference's rule defines."""
    from souffle_gb300 import gpu
    reps = _extreme_replicas()
    s = gpu.GpuSystem(reps[0].template, [_params(w) for w in reps])
    s.set_state(np.concatenate([w.state.pos for w in reps]), np.concatenate([w.state.vel for w in reps]))
    tf, sf, bf = s.forces(rebuild=True, parts=True)
    oracles = [_oracle(w, capacity=min(w.n_beads, max(256, 4 * w.derived.nlist_capacity))) for w in reps]
    cap = max(o.cap for o in oracles)
    gc, gi = s.pairlist(cap)
    off = 0
    for k, (w, o) in enumerate(zip(reps, oracles)):
        n = w.n_beads
        otf, osf, obf, over = o.forces(True)
        assert over == 0
        errs = _check_forces((tf[off:off + n], sf[off:off + n], bf[off:off + n]), (otf, osf, obf))
        oc, oi = o.pairlist()
        _check_pairlist(gc[off:off + n], gi[off:off + n], oc, oi, off)
        st = s.pairlist_stats(system=k)
        ref_cap = w.derived.nlist_capacity
        assert st["over_reference_capacity"] == int((oc > ref_cap).sum())
        assert st["max_length"] == oc.max()
        _, pb = s.energies(system=k, per_bead=True)
        _check_energies(pb, o.energies())
        print(f"system {k}: {n} beads, Debye length {1 / w.derived.kappa:.2f}, {w.opt.C:g} uM, mean list "
              f"{oc.mean():.1f}, max {oc.max()} (reference capacity {ref_cap}, "
              f"{st['over_reference_capacity']} beads over it); force RMS rel err {errs[0]:.2e}")
        off += n
    # the same systems stepped together: per-system thermostat chains against separate oracle runs
    s.md_begin()
    s.md_steps(0, MD_STEPS)
    for k, (w, o) in enumerate(zip(reps, oracles)):
        o.set_state(w.state.pos, w.state.vel)
        o.forces(True)
        ke_o = o.kinetic_energy()
        o.nhc_init(int(w.opt.q), w.opt.Q, w.opt.K)
        for a in range(MD_STEPS):
            ke_o, _, _ = o.md_step(a, w.opt.t, int(w.opt.B), ke_o)
        ke_g, xi_g, _ = s.md_scalars(system=k)
        assert ke_g == pytest.approx(ke_o, rel=1e-6), k
        assert xi_g == pytest.approx(o.nhc.xi[0], rel=1e-6, abs=1e-12), k


def test_840k_forces_and_pairlists():
    from souffle_gb300 import gpu, workloads
    w = workloads.plain_large(20000)
    assert w.n_beads == 840000
    s = gpu.GpuSystem(w.template, [_params(w)])
    s.set_state(w.state.pos, w.state.vel)
    gf = s.forces(rebuild=True, parts=True)
    o = _oracle(w)
    otf, osf, obf, over = o.forces(True)
    assert over == 0
    errs = _check_forces(gf, (otf, osf, obf))
    print(f"840k force RMS rel err: total {errs[0]:.2e} stretching {errs[1]:.2e} bending {errs[2]:.2e}")
    oc, oi = o.pairlist()
    gc, gi = s.pairlist(o.cap)
    _check_pairlist(gc, gi, oc, oi, 0)
