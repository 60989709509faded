"""The post-run analysis oracle (oracle/analysis_oracle.py) against the reference's own outputs.

The fixtures in tests/golden/analysis_*.npz hold synthetic energy.out and ovito.lammpstrj files and
the five files the reference's analyze_output wrote for them (tests/golden/make_golden_analysis.py,
reference compiled unmodified by oracle/ref.mk).  CPU only.
"""
import numpy as np
import pytest

import analysis_oracle as ao
from conftest import load_golden

CASES = ["contacts", "no_equilibrium", "aligned_energy"]
FILES = ["analysis.rdat", "analysis.gr", "analysis.so", "analysis.ms", "info.gr"]


@pytest.mark.parametrize("name", CASES)
def test_oracle_reproduces_reference_analysis_files(name):
    g = load_golden(f"analysis_{name}")
    r = ao.analyze(str(g["energy"]), str(g["trajectory"]))
    for fn in FILES:
        assert r[fn] == str(g["out_" + fn.replace(".", "_")]), fn


def test_fixtures_exercise_every_branch():
    """Contacts, sub-oligomers and pcf counts are all nonzero somewhere, the equilibrium search
    finds a later start in one case, and one energy file has misaligned (skipped) groups."""
    seen = {"olig>1": False, "so>1": False, "pcf": False}
    starts = []
    for name in CASES:
        g = load_golden(f"analysis_{name}")
        tf = ao.trust_factor(str(g["energy"]))
        starts.append(tf["hiteqm"])
        for step, _h, types, pos in ao.read_trajectory(str(g["trajectory"])):
            L = 2 * _h
            gr, olig, so = ao.frame_analysis(types, pos, L, int(g["np_"]))
            seen["olig>1"] |= bool((olig > 1).any())
            seen["so>1"] |= bool((so > 1).any())
            seen["pcf"] |= bool(gr.sum() > 0)
    assert all(seen.values()), seen
    assert max(starts) > 0


def test_components_are_connected_components():
    """The union-find helper against a breadth-first search on random graphs."""
    rng = np.random.default_rng(3)
    for _ in range(20):
        n = int(rng.integers(1, 40))
        edges = [tuple(rng.integers(0, n, 2)) for _ in range(int(rng.integers(0, 2 * n)))]
        lab = ao._components(n, edges)
        adj = {i: set() for i in range(n)}
        for a, b in edges:
            adj[a].add(b)
            adj[b].add(a)
        for s in range(n):
            seen, todo = {s}, [s]
            while todo:
                x = todo.pop()
                for y in adj[x] - seen:
                    seen.add(y)
                    todo.append(y)
            assert lab[s] == min(seen)
            assert all(lab[x] == lab[s] for x in seen)


def test_reference_image_rule_takes_the_long_way_round():
    """dist() with the half-box vector left at zero: nonzero differences shift by a full box."""
    L = 10.0
    a = np.array([[0.0, 0.0, 0.0]])
    b = np.array([[1.0, 0.0, 0.0]])
    assert ao.separation(a, b, L, ao.IMAGE_REFERENCE)[0] == pytest.approx(9.0)
    assert ao.separation(a, b, L, ao.IMAGE_MINIMUM)[0] == pytest.approx(1.0)
    c = np.array([[4.5, 0.0, 0.0]])
    d = np.array([[-4.5, 0.0, 0.0]])
    assert ao.separation(c, d, L, ao.IMAGE_REFERENCE)[0] == pytest.approx(1.0)
    assert ao.separation(c, d, L, ao.IMAGE_MINIMUM)[0] == pytest.approx(1.0)


def test_subunit_size_rule():
    assert ao.subunit_size(43 * 7) == 43
    assert ao.subunit_size(41 * 43) == 43   # the last matching size wins (src/analysis.cpp:81-83)
    assert ao.subunit_size(78 * 2) == 78
    assert ao.subunit_size(42 * 2000) == 0  # the reference divides by zero next


@pytest.mark.parametrize("name", CASES)
def test_c_port_agrees_with_the_oracle(name):
    """oracle/analysis_port.c (the reference's loop structure in long double, used as the CPU
    baseline) gives the oracle's integers on the reference fixtures, both image rules."""
    g = load_golden(f"analysis_{name}")
    for _s, half, types, pos in ao.read_trajectory(str(g["trajectory"])):
        for image in (ao.IMAGE_REFERENCE, ao.IMAGE_MINIMUM):
            gr, olig, so = ao.frame_analysis(types, pos, 2 * half, int(g["np_"]), image)
            S = len(pos) // int(g["np_"])
            pg, pm, ps = ao.port_frame(types, pos, 2 * half, int(g["np_"]), image)
            np.testing.assert_array_equal(pg, gr)
            np.testing.assert_array_equal(pm, np.bincount(olig - 1, minlength=S))
            np.testing.assert_array_equal(ps, np.bincount((so - 1) // 3, minlength=2 * S))
