"""The learned far-field surrogate on the GPU, through the C ABI (include/souffle_surrogate.h):
far-pair classification, descriptors and exact training targets against the CPU restatement in
oracle/surrogate_oracle.py; training on the GPU; force accuracy with the surrogate in the force
path; what the network gains over dropping the far pairs; the exact judge."""
import os
import sys

import numpy as np
import pytest

from conftest import REPO

pytestmark = pytest.mark.gpu
sys.path.insert(0, os.path.join(REPO, "oracle"))
import surrogate_oracle as SO  # noqa: E402

CAP = 8192


def _torch():
    return pytest.importorskip("torch")


def _system(n_sub=300, conc=2000, seed=21):
    from souffle_gb300 import geometry, gpu, workloads
    w = workloads.make(geometry.bilayer_n5(), n_sub, seed=seed, C=conc)
    p = gpu.system_params(w.opt, w.derived, n_sub, w.center_local)
    s = gpu.GpuSystem(w.template, [p])
    s.set_state(w.state.pos, w.state.vel)
    return w, s, p


def _net_and_buffers(w, s, width=256, switch_radius=3.5):
    torch = _torch()
    from souffle_gb300 import gpu
    n_out = 6 + 3 * w.template.n_beads
    net = gpu.Mlp(64, n_out, max_batch=CAP, seed=3, width=width)
    gpu.surrogate_attach(s, net, w.template.pos, far_capacity=CAP, switch_radius=switch_radius)
    x = torch.zeros(CAP, 64, device="cuda")
    t = torch.zeros(CAP, n_out, device="cuda")
    return torch, net, x, t, n_out


def test_collect_matches_oracle():
    from souffle_gb300 import gpu
    w, s, p = _system()
    torch, net, x, t, n_out = _net_and_buffers(w, s)
    n = gpu.surrogate_collect(s, x.data_ptr(), t.data_ptr(), CAP)
    np_ = w.template.n_beads
    L = float(w.derived.box)
    ref = SO.far_pairs(w.state.pos, int(w.opt.S), np_, w.center_local, L, w.derived.nlist_cutoff, 3.5,
                       reach=max(w.derived.ecut_el, w.derived.ecut))
    assert n == len(ref) and n > 20
    b1, b2 = SO.anchors(w.template.pos, w.center_local)
    wts = SO.dh_weights(w.template.charge, w.template.diameter, w.derived.kappa, w.derived.lb)
    pos = w.state.pos.reshape(-1, np_, 3)
    X, T = x[:n].cpu().numpy(), t[:n].cpu().numpy()
    for k, (a, b, dmin) in enumerate(ref):
        fa, fb = SO.frame(pos[a], w.center_local, b1, b2, L), SO.frame(pos[b], w.center_local, b1, b2, L)
        R = SO.min_image(pos[b][w.center_local] - pos[a][w.center_local], L) + fb[3] - fa[3]
        RA = np.array([fa[0] @ R, fa[1] @ R, fa[2] @ R])
        np.testing.assert_allclose(X[k, 0:3], RA, rtol=1e-4, atol=1e-4)
        assert X[k, 3] == pytest.approx(np.linalg.norm(R), rel=1e-5)
        assert X[k, 39] == pytest.approx(dmin, rel=1e-5)
        assert X[k, 37] == pytest.approx(1 / w.derived.kappa, rel=1e-6)
        f = SO.exact_far_forces(pos[a], pos[b], L, wts, w.derived.kappa, w.derived.ecut_el, w.derived.nlist_cutoff)
        tr, g, db, J = SO.targets(f, fa)
        scale = np.abs(g).max() + 1e-30
        # targets reconstruct the exact forces, and agree with the oracle's decomposition
        np.testing.assert_allclose(SO.reconstruct(T[k], db, J), g, atol=2e-4 * scale, rtol=0)
        np.testing.assert_allclose(T[k, :3], tr[:3], atol=2e-4 * np.abs(tr[:3]).max() + 1e-12, rtol=0)


def test_collect_spans_the_systems_of_one_handle():
    """Two systems with different screening lengths (1 and 2 sigma) in one handle: the far list
    is the union of each system's far pairs, pairs beyond every cut-off left out, and each row's
    descriptor carries its own system's screening length."""
    from souffle_gb300 import geometry, gpu, state, workloads
    torch = _torch()
    t = geometry.bilayer_n5()
    ws = [workloads.make(t, 150, seed=31, C=2000),
          workloads.make(t, 120, seed=32, C=1500, c=state.salt_for_debye_length(2.0))]
    ps = [gpu.system_params(w.opt, w.derived, int(w.opt.S), w.center_local) for w in ws]
    s = gpu.GpuSystem(t, ps)
    s.set_state(np.concatenate([w.state.pos for w in ws]), np.concatenate([w.state.vel for w in ws]))
    n_out = 6 + 3 * t.n_beads
    net = gpu.Mlp(64, n_out, max_batch=CAP, seed=3)
    gpu.surrogate_attach(s, net, t.pos, far_capacity=CAP)
    x = torch.zeros(CAP, 64, device="cuda")
    y = torch.zeros(CAP, n_out, device="cuda")
    n = gpu.surrogate_collect(s, x.data_ptr(), y.data_ptr(), CAP)
    counts = []
    for w in ws:
        ref = SO.far_pairs(w.state.pos, int(w.opt.S), t.n_beads, w.center_local, float(w.derived.box),
                           w.derived.nlist_cutoff, 3.5, reach=max(w.derived.ecut_el, w.derived.ecut))
        allp = SO.far_pairs(w.state.pos, int(w.opt.S), t.n_beads, w.center_local, float(w.derived.box),
                            w.derived.nlist_cutoff, 3.5)
        counts.append(len(ref))
        if w is ws[0]:
            assert len(allp) > len(ref)       # at 1 sigma some candidates lie beyond the cut-off
    assert counts[1] > 0 and n == sum(counts)
    lam = x[:n, 37].cpu().numpy()
    assert np.sum(np.isclose(lam, 1 / ws[0].derived.kappa, rtol=1e-6)) == counts[0]
    assert np.sum(np.isclose(lam, 1 / ws[1].derived.kappa, rtol=1e-6)) == counts[1]


def _train(w, s, torch, x, t, frames=12, stride=20, epochs=60):
    from souffle_gb300 import gpu
    n_out = t.shape[1]
    X = torch.zeros(CAP * frames, 64, device="cuda")
    T = torch.zeros(CAP * frames, n_out, device="cuda")
    total = 0
    s.md_begin()
    for f in range(frames):
        n = gpu.surrogate_collect(s, x.data_ptr(), t.data_ptr(), CAP)
        X[total:total + n] = x[:n]
        T[total:total + n] = t[:n]
        total += n
        s.md_steps(f * stride, stride)
    loss = gpu.surrogate_fit(s, X.data_ptr(), T.data_ptr(), total, epochs, 256, 1e-3, seed=5)
    return total, loss


@pytest.mark.parametrize("width,switch_radius", [(256, 3.5), (128, 3.5), (128, 3.0)])
def test_training_and_force_accuracy(width, switch_radius):
    """Trained on exact far-pair data from a short run, the surrogate's far-field forces stay
    within 1e-3 of the exact total force (RMS, relative), and it removes most of the error that
    dropping the far pairs would leave; both hidden widths, and the 3.0 sigma switch radius."""
    from souffle_gb300 import gpu
    w, s, p = _system()
    torch, net, x, t, n_out = _net_and_buffers(w, s, width, switch_radius)
    total, loss = _train(w, s, torch, x, t)
    assert total > 500 and loss < 0.5, (total, loss)
    # exact forces and the exact far-field part at the current state
    exact = s.forces(rebuild=True)
    n = gpu.surrogate_collect(s, x.data_ptr(), t.data_ptr(), CAP)
    np_ = w.template.n_beads
    pos, _ = s.get_state()
    L = float(w.derived.box)
    ref = SO.far_pairs(pos, int(w.opt.S), np_, w.center_local, L, w.derived.nlist_cutoff, switch_radius,
                       reach=max(w.derived.ecut_el, w.derived.ecut))
    assert n == len(ref)
    wts = SO.dh_weights(w.template.charge, w.template.diameter, w.derived.kappa, w.derived.lb)
    P = pos.reshape(-1, np_, 3)
    far = np.zeros_like(pos).reshape(-1, np_, 3)
    for a, b, _ in ref:
        far[a] += SO.exact_far_forces(P[a], P[b], L, wts, w.derived.kappa, w.derived.ecut_el, w.derived.nlist_cutoff)
    far = far.reshape(-1, 3)
    gpu.surrogate_enable(s, True)
    sur = s.forces(rebuild=True)
    st = gpu.surrogate_stats(s)
    assert st["far_pairs"] == n
    err = sur - exact                                   # = surrogate far forces - exact far forces
    rms_total = np.sqrt((err ** 2).sum() / (exact ** 2).sum())
    trunc = np.sqrt((far ** 2).sum())                   # error left by dropping the far pairs
    gain = trunc / max(np.sqrt((err ** 2).sum()), 1e-30)
    print(f"far pairs {n}, train rows {total}, loss {loss:.4f}; total-force RMS rel error {rms_total:.2e}; "
          f"far-field error vs truncation: {1 / gain:.3f} (gain {gain:.1f}x)")
    assert rms_total <= 1e-3
    assert gain > 2.0


def test_judge_reverts_classes_above_tolerance():
    from souffle_gb300 import gpu
    torch = _torch()
    w, s, p = _system(n_sub=200, conc=1500, seed=22)
    n_out = 6 + 3 * w.template.n_beads
    net = gpu.Mlp(64, n_out, max_batch=CAP, seed=3)
    # judged every step, against a tolerance no network meets
    gpu.surrogate_attach(s, net, w.template.pos, far_capacity=CAP, judge_every=1, judge_stride=1,
                         judge_tolerance=1e-9)
    x = torch.zeros(CAP, 64, device="cuda")
    t = torch.zeros(CAP, n_out, device="cuda")
    s.md_begin()
    n = gpu.surrogate_collect(s, x.data_ptr(), t.data_ptr(), CAP)
    assert n > 0
    gpu.surrogate_fit(s, x.data_ptr(), t.data_ptr(), n, 2, 256, 1e-3)
    gpu.surrogate_enable(s, True)
    s.forces(rebuild=True)
    before = gpu.surrogate_stats(s)["far_pairs"]
    assert before > 0
    s.md_steps(0, int(p.build_freq) + 1)              # judged every step, then a rebuild
    st = gpu.surrogate_stats(s)
    assert st["judged"] > 0 and st["classes_off"] != 0
    for k in range(4):
        if st["classes_off"] >> k & 1:
            assert st["last_error"][k] > 1e-9
    assert st["far_pairs"] < before                   # reverted classes are exact again


def test_judge_estimate_matches_measured_total_force_error():
    """With every far pair judged (stride 1), the judge's per-class shares of the total-force RMS
    relative error, added in quadrature, agree with the error measured directly from exact and
    surrogate forces at the same state (within a factor of 3: the judge treats the pairs acting on
    one subunit as independent)."""
    from souffle_gb300 import gpu
    torch = _torch()
    w, s, p = _system()
    n_out = 6 + 3 * w.template.n_beads
    net = gpu.Mlp(64, n_out, max_batch=CAP, seed=3)
    gpu.surrogate_attach(s, net, w.template.pos, far_capacity=CAP, judge_every=1, judge_stride=1,
                         judge_tolerance=1.0)
    x = torch.zeros(CAP, 64, device="cuda")
    t = torch.zeros(CAP, n_out, device="cuda")
    _train(w, s, torch, x, t)
    gpu.surrogate_enable(s, True)
    s.md_begin()
    s.md_steps(0, 1)                                    # one judged step
    st = gpu.surrogate_stats(s)
    assert st["judged"] > 0 and st["classes_off"] == 0
    est = float(np.sqrt(sum(e * e for e in st["last_error"] if e >= 0)))
    pos, vel = s.get_state()
    sur = s.forces(rebuild=True)
    gpu.surrogate_enable(s, False)
    exact = s.forces(rebuild=True)
    meas = float(np.sqrt(((sur - exact) ** 2).sum() / (exact ** 2).sum()))
    print(f"judge estimate {est:.3e}, measured total-force RMS rel error {meas:.3e}")
    assert meas / 3 <= est <= 3 * meas


def test_md_with_surrogate_runs_and_holds_temperature():
    from souffle_gb300 import gpu
    w, s, p = _system()
    torch, net, x, t, n_out = _net_and_buffers(w, s)
    _train(w, s, torch, x, t, frames=6, epochs=30)
    gpu.surrogate_enable(s, True)
    s.md_begin()
    s.md_steps(0, 200)
    e = s.energies()
    assert np.isfinite(e["temperature"]) and 0.5 < e["temperature"] < 2.0
    st = gpu.surrogate_stats(s)
    assert st["enabled"] and st["judged"] > 0


def test_switch_radius_inside_the_lj_range_is_rejected():
    """A far pair must stay beyond the LJ cut-off (2.5 sigma) until the next rebuild: a switch
    radius below the cut-off plus the pair-list skin (0.3 sigma here: 2.8) is refused at attach."""
    from souffle_gb300 import gpu
    w, s, p = _system()
    n_out = 6 + 3 * w.template.n_beads
    net = gpu.Mlp(64, n_out, max_batch=CAP, seed=3)
    with pytest.raises(RuntimeError):
        gpu.surrogate_attach(s, net, w.template.pos, far_capacity=CAP, switch_radius=2.7)
    gpu.surrogate_attach(s, net, w.template.pos, far_capacity=CAP, switch_radius=2.85)
