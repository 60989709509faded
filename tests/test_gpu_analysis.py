"""GPU trajectory analysis (include/souffle_analysis.h) against the analysis oracle and the
reference's own analysis files.

Per frame the GPU gives pcf bin counts, the oligomer size histogram and the sub-oligomer
histogram; they must equal the oracle's integers exactly (oracle/analysis_oracle.py, itself
pinned to the reference's analyze_output by tests/test_analysis_oracle.py).  The driver's
analysis mode must write the reference's five files byte for byte.
"""
import os
import subprocess

import numpy as np
import pytest

import analysis_oracle as ao
from conftest import REPO, load_golden

pytestmark = pytest.mark.gpu

DRIVER = os.path.join(REPO, "capsid-souffle_gb300", "_build", "souffle_gb300")
CASES = ["contacts", "no_equilibrium", "aligned_energy"]
FILES = ["analysis.rdat", "analysis.gr", "analysis.so", "analysis.ms", "info.gr"]


def _analysis(n, np_, L, image, **kw):
    from souffle_gb300.analysis import Analysis
    return Analysis(n, np_, L, image=image, **kw)


def _oracle_frame(types, pos, L, np_, image, pcf_type=5, so_type=0, contact=2.0, bins=100):
    S = len(pos) // np_
    gr, olig, so = ao.frame_analysis(types, pos, L, np_, image, pcf_type, bins, so_type, contact)
    ms = np.zeros(S, dtype=np.int64)
    np.add.at(ms, olig - 1, 1)
    sob = np.zeros(2 * S, dtype=np.int64)
    np.add.at(sob, (so - 1) // 3, 1)
    return gr, ms, sob


def _check_frames(frames, L, np_, image, **kw):
    n = len(frames[0][1])
    a = _analysis(n, np_, L, image, **kw)
    pos = np.stack([f[1] for f in frames])
    types = np.stack([f[0] for f in frames])
    r = a.frames(pos, types)
    okw = {k: kw[k] for k in ("pcf_type", "so_type", "contact") if k in kw}
    if "pcf_bins" in kw:
        okw["bins"] = kw["pcf_bins"]
    for k, (t, p) in enumerate(frames):
        gr, ms, sob = _oracle_frame(t, p, L, np_, image, **okw)
        np.testing.assert_array_equal(r["pcf"][k], gr)
        np.testing.assert_array_equal(r["oligomers"][k], ms)
        np.testing.assert_array_equal(r["so_bins"][k], sob)
        # labels: the smallest subunit index of each oligomer
        lab = r["labels"][k]
        assert (lab <= np.arange(len(lab))).all() and (lab[lab] == lab).all()
        sizes = np.bincount(lab, minlength=len(lab))
        np.testing.assert_array_equal(np.bincount(sizes[sizes > 0] - 1, minlength=len(lab)), ms)
    a.close()
    return r


def _golden_frames(name):
    g = load_golden(f"analysis_{name}")
    fr = ao.read_trajectory(str(g["trajectory"]))
    return [(t, p) for _s, _h, t, p in fr], 2 * fr[0][1], int(g["np_"])


@pytest.mark.parametrize("image", [ao.IMAGE_REFERENCE, ao.IMAGE_MINIMUM])
@pytest.mark.parametrize("name", CASES)
def test_frames_match_oracle_on_reference_fixtures(name, image):
    frames, L, np_ = _golden_frames(name)
    _check_frames(frames, L, np_, image)


def _synthetic(seed, S, np_, L, grid=None, cluster_frac=0.5, so_per=6, pcf_per=4):
    """Subunits of np_ beads within ~1.6 of their centre; half of them packed in clusters so that
    contacts, sub-oligomers across subunits and ties with the contact distance occur."""
    rng = np.random.default_rng(seed)
    off = rng.uniform(-1.6, 1.6, (np_, 3))
    off[0] = 0
    types = np.ones(np_, dtype=np.int32)
    types[1:1 + so_per] = 0
    types[1 + so_per:1 + so_per + pcf_per] = 5
    n_cl = int(S * cluster_frac)
    centres = []
    while len(centres) < n_cl:
        base = rng.uniform(-L / 2, L / 2, 3)
        for k in range(min(6, n_cl - len(centres))):
            centres.append(base + rng.normal(0, 2.2, 3))
    centres += list(rng.uniform(-L / 2, L / 2, (S - n_cl, 3)))
    centres = np.array(centres)
    rot = [np.linalg.qr(rng.normal(size=(3, 3)))[0] for _ in range(S)]
    pos = np.concatenate([centres[s] + off @ rot[s].T for s in range(S)])
    if grid:
        pos = np.round(pos / grid) * grid
    pos = (pos + L / 2) % L - L / 2
    return np.tile(types, S), pos


@pytest.mark.parametrize("image", [ao.IMAGE_REFERENCE, ao.IMAGE_MINIMUM])
@pytest.mark.parametrize("grid", [None, 1.0 / 16])
def test_random_frames_match_oracle(image, grid):
    """Seeded clustered frames, with coordinates on a 1/16 grid (exact ties with the contact
    distance, with bin edges and with zero differences) or unrounded."""
    S, np_, L = 120, 43, 40.0
    frames = [_synthetic(11 + k, S, np_, L, grid) for k in range(2)]
    r = _check_frames(frames, L, np_, image)
    # under the reference's rule a contact needs every nonzero coordinate difference within 2 of a
    # full box, which unrounded coordinates practically never give
    if image == ao.IMAGE_MINIMUM or grid:
        assert (r["oligomers"][:, 1:] > 0).any()
    if image == ao.IMAGE_MINIMUM:
        assert (r["so_bins"][:, 1:] > 0).any()


def test_other_subunit_sizes_types_and_bins():
    """42-bead subunits (which the reference's analysis cannot size), another pcf type, 37 bins,
    a smaller contact distance."""
    S, np_, L = 90, 42, 36.0
    frames = [_synthetic(5, S, np_, L, so_per=9, pcf_per=7)]
    _check_frames(frames, L, np_, ao.IMAGE_MINIMUM, pcf_type=1, pcf_bins=37, so_type=0, contact=1.5)
    _check_frames(frames, L, np_, ao.IMAGE_REFERENCE, pcf_type=0, pcf_bins=7, so_type=5, contact=2.5)


@pytest.mark.parametrize("np_", [1, 3, 10, 32, 33, 100])
def test_subunit_sizes_around_the_warp_width(np_):
    """The contact kernel walks np x np bead pairs 32 at a time; sizes below, at and above the
    warp width, with random types, against the oracle under both rules."""
    rng = np.random.default_rng(np_)
    S, L = max(6, 2400 // np_), 24.0
    off = rng.uniform(-1.2, 1.2, (np_, 3))
    t = rng.choice(np.array([0, 1, 5], dtype=np.int32), size=np_, p=[0.1, 0.7, 0.2] if np_ > 10 else None)
    centres = rng.uniform(-L / 2, L / 2, (S, 3))
    centres[1::2] = centres[0::2][: len(centres[1::2])] + rng.normal(0, 1.5, (len(centres[1::2]), 3))
    p = (centres[:, None, :] + off[None]).reshape(-1, 3)
    p = (p + L / 2) % L - L / 2
    types = np.tile(t, S)
    for image in (ao.IMAGE_REFERENCE, ao.IMAGE_MINIMUM):
        _check_frames([(types, p)], L, np_, image)


def test_edge_cases():
    from souffle_gb300.gpu import SouffleError

    L = 30.0
    # one subunit, no pcf beads, no so beads
    t, p = _synthetic(1, 1, 43, L, so_per=0, pcf_per=0)
    r = _check_frames([(t, p)], L, 43, ao.IMAGE_MINIMUM)
    assert r["pcf"].sum() == 0 and r["oligomers"][0, 0] == 1 and r["so_bins"].sum() == 0
    # every bead of two touching subunits is an so bead: a sub-oligomer of 86 beads needs bin 28
    # of 4, past the reference's histogram -> reported
    t = np.zeros(86, dtype=np.int32)
    p = np.concatenate([np.zeros((43, 3)), np.zeros((43, 3))]) + np.linspace(0, 2, 86)[:, None] * [1, 0, 0]
    a = _analysis(86, 43, L, ao.IMAGE_MINIMUM)
    with pytest.raises(SouffleError, match="BAD_INPUT"):
        a.frames(p[None], t)
    # coordinates far outside the box are reported, not guessed at
    with pytest.raises(SouffleError, match="BAD_INPUT"):
        a.frames((p + 40.0)[None], t)
    # bad arguments
    with pytest.raises(SouffleError):
        _analysis(86, 0, L, 0)
    with pytest.raises(SouffleError):
        _analysis(85, 43, L, 0)
    with pytest.raises(SouffleError):
        _analysis(86, 43, L, 0, pcf_bins=0)


def test_candidate_list_grows():
    """150 subunits inside a few sigma: all 11,175 subunit pairs are candidates, more than the
    initial list holds; the frame is run again with a larger list and everything is one oligomer."""
    rng = np.random.default_rng(8)
    S, np_, L = 150, 43, 60.0
    off = rng.uniform(-1.5, 1.5, (np_, 3))
    pos = np.concatenate([c + off for c in rng.uniform(-1.5, 1.5, (S, 3))])
    t = np.ones(np_ * S, dtype=np.int32)
    a = _analysis(S * np_, np_, L, ao.IMAGE_MINIMUM)
    r = a.frames(pos[None], t)
    assert r["oligomers"][0, S - 1] == 1 and r["oligomers"][0].sum() == 1
    assert a.last_counts()[0] == S * (S - 1) // 2


def test_enqueue_on_device_buffers_matches_frames():
    torch = pytest.importorskip("torch")
    S, np_, L = 200, 43, 50.0
    frames = [_synthetic(40 + k, S, np_, L) for k in range(2)]
    a = _analysis(S * np_, np_, L, ao.IMAGE_REFERENCE)
    ref = a.frames(np.stack([f[1] for f in frames]), np.stack([f[0] for f in frames]))
    dev = torch.device("cuda:0")
    for k, (t, p) in enumerate(frames):
        pd = torch.tensor(p, dtype=torch.float64, device=dev)
        td = torch.tensor(t, dtype=torch.int32, device=dev)
        gr = torch.full((100,), -1, dtype=torch.int64, device=dev)
        ol = torch.full((S,), -1, dtype=torch.int64, device=dev)
        so = torch.full((2 * S,), -1, dtype=torch.int64, device=dev)
        torch.cuda.synchronize()
        a.enqueue(pd.data_ptr(), td.data_ptr(), gr.data_ptr(), ol.data_ptr(), so.data_ptr())
        a.synchronize()
        np.testing.assert_array_equal(gr.cpu().numpy(), ref["pcf"][k])
        np.testing.assert_array_equal(ol.cpu().numpy(), ref["oligomers"][k])
        np.testing.assert_array_equal(so.cpu().numpy(), ref["so_bins"][k])


def test_full_size_frame_against_periodic_kd_tree():
    """84,000 beads (2000 subunits of 42) at the MD workload's density: oligomers under the
    minimum image must be the connected components of a periodic k-d tree's contact pairs, and
    the pcf total the number of pcf pairs closer than half a box."""
    spatial = pytest.importorskip("scipy.spatial")
    csgraph = pytest.importorskip("scipy.sparse.csgraph")
    sparse = pytest.importorskip("scipy.sparse")
    S, np_ = 2000, 42
    L = (S * 1000 / (800 * 1e-27 * 6.022e23)) ** (1 / 3)  # 800 uM, sigma = 1 nm
    t, p = _synthetic(2024, S, np_, L, cluster_frac=0.6, so_per=6, pcf_per=2)
    a = _analysis(S * np_, np_, L, ao.IMAGE_MINIMUM)
    r = a.frames(p[None], t)
    ms = r["oligomers"][0]
    assert (ms * np.arange(1, S + 1)).sum() == S
    q = p + L / 2
    q[q >= L] -= L
    tree = spatial.cKDTree(q, boxsize=L)
    pairs = tree.query_pairs(2.0, output_type="ndarray")
    sub = np.arange(S * np_) // np_
    inter = pairs[sub[pairs[:, 0]] != sub[pairs[:, 1]]]
    g = sparse.coo_matrix((np.ones(len(inter)), (sub[inter[:, 0]], sub[inter[:, 1]])), shape=(S, S))
    _n, lab = csgraph.connected_components(g, directed=False)
    # same partition: map each kd-tree component to its smallest member
    first = np.full(lab.max() + 1, S)
    np.minimum.at(first, lab, np.arange(S))
    np.testing.assert_array_equal(r["labels"][0], first[lab])
    pcf_idx = np.nonzero(t == 5)[0]
    tp = spatial.cKDTree(q[pcf_idx], boxsize=L)
    n_half = len(tp.query_pairs(L / 2 * (1 - 1e-12)))
    assert abs(int(r["pcf"][0].sum()) - n_half) <= 2
    assert ms[1:].sum() > 0


@pytest.mark.parametrize("name", CASES)
def test_driver_analysis_writes_the_reference_files(tmp_path, name):
    g = load_golden(f"analysis_{name}")
    out = tmp_path / "outfiles"
    out.mkdir()
    (out / "energy.out").write_text(str(g["energy"]))
    (out / "ovito.lammpstrj").write_text(str(g["trajectory"]))
    r = subprocess.run([DRIVER, "-A", "o"], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    for fn in FILES:
        assert (out / fn).read_text() == str(g["out_" + fn.replace(".", "_")]), fn
    assert r.stdout == str(g["ref_stdout"])
