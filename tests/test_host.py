"""Host-side logic and the C-ABI library, without GPU compute."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import REPO, load_golden, golden_workload


def _header_symbols():
    syms = set()
    for name in sorted(os.listdir(os.path.join(REPO, "include"))):
        if name.endswith(".h"):
            text = open(os.path.join(REPO, "include", name)).read()
            syms |= set(re.findall(r"\b(souffle_(?:gpu|mlp|gemm|surrogate|analysis)_\w+)\s*\(", text))
    return sorted(syms)


def test_library_exports_every_declared_symbol():
    from souffle_gb300 import gpu
    lib = gpu.load()
    syms = _header_symbols()
    assert len(syms) >= 14
    for s in syms:
        assert hasattr(lib, s), s
    assert sorted(gpu.EXPORTED) == syms


def test_create_rejects_bad_arguments_without_crashing():
    from souffle_gb300 import gpu
    lib = gpu.load()
    h = ctypes.c_void_p()
    rc = lib.souffle_gpu_create(None, None, 0, None, ctypes.byref(h))
    assert rc in (1, 5)  # BAD_INPUT, or NO_DEVICE on a host without a GPU
    assert not h.value
    assert lib.souffle_gpu_create(None, None, 1, None, None) == 1
    assert lib.souffle_gpu_last_error()


def test_infile_round_trip(tmp_path):
    from souffle_gb300 import geometry
    for t in (geometry.patch_n3(), geometry.bilayer_n5()):
        p = tmp_path / t.name
        geometry.write_infile(t, str(p))
        t2, bl, m, s = geometry.read_infile(str(p))
        assert np.array_equal(t2.pos, t.pos)
        assert np.array_equal(t2.edges, t.edges)
        assert np.array_equal(t2.faces, t.faces)
        assert np.array_equal(t2.edge_len0, t.edge_len0)
        assert t2.lj_attract == t.lj_attract
        assert s == 1e-9


def test_template_shapes():
    from souffle_gb300 import geometry
    a = geometry.patch_n3()
    assert (a.n_beads, len(a.edges), len(a.faces), int((a.edge_type != 0).sum())) == (10, 18, 9, 9)
    b = geometry.bilayer_n5()
    assert (b.n_beads, len(b.faces), int((b.edge_type != 0).sum())) == (42, 50, 60)
    assert len(b.edges) == 2 * 45 + 21 + 45


def test_restart_round_trip_is_exact(tmp_path):
    from souffle_gb300 import geometry, state
    t = geometry.patch_n3()
    s = state.random_state(t, 20, state.box_length(20, 800), seed=3)
    state.write_restart(s, str(tmp_path))
    step, vel, pos = state.read_restart(str(tmp_path / "restart_0.out"))
    assert step == 0
    assert np.array_equal(pos, s.pos)
    assert np.array_equal(vel, s.vel)
    assert (tmp_path / "rb_0.out").exists()
    assert np.abs(pos).max() <= s.box / 2


def test_random_state_has_zero_momentum_and_no_overlap():
    from souffle_gb300 import geometry, state
    t = geometry.bilayer_n5()
    L = state.box_length(200, 800)
    s = state.random_state(t, 200, L, seed=9)
    assert np.abs(s.vel.mean(axis=0)).max() < 1e-12
    com = s.pos.reshape(200, 42, 3)
    # bead sets of different subunits are separated by at least ~1 sigma
    from scipy.spatial import cKDTree
    tree = cKDTree(s.pos + L / 2, boxsize=L * (1 + 1e-12))
    pairs = tree.query_pairs(0.9)
    sub = np.arange(s.pos.shape[0]) // 42
    assert all(sub[i] == sub[j] for i, j in pairs)


def test_salt_for_debye_length_inverts_kappa():
    from souffle_gb300 import state
    for lam in (0.5, 1.0, 2.0):
        c = state.salt_for_debye_length(lam)
        assert abs(1 / state.debye_kappa(c) - lam) < 1e-12


def test_thermostat_exponentials_match_libm(tmp_path):
    """exp_small / expm1_small (truncated Taylor series, Estrin) agree with libm to ~2 ulp."""
    import math
    import random
    import shutil
    import subprocess
    nvcc = shutil.which("nvcc")
    if not nvcc:
        pytest.skip("nvcc not available")
    src = tmp_path / "es.cu"
    src.write_text('#include <cmath>\n#include "souffle_dev.cuh"\n'
                   'extern "C" double e1(double x) { return souffle::exp_small(x); }\n'
                   'extern "C" double e2(double x) { return souffle::expm1_small(x); }\n'
                   'extern "C" double e3(double x) { return souffle::exp_reduced(x); }\n')
    so = tmp_path / "es.so"
    subprocess.run([nvcc, "-shared", "-Xcompiler", "-fPIC", "-I",
                    os.path.join(REPO, "capsid-souffle_gb300", "csrc"), str(src), "-o", str(so)], check=True)
    lib = ctypes.CDLL(str(so))
    for f in (lib.e1, lib.e2, lib.e3):
        f.restype = ctypes.c_double
        f.argtypes = [ctypes.c_double]
    rng = random.Random(1)
    xs = ([rng.uniform(-0.0625, 0.0625) for _ in range(10000)] + [rng.uniform(-1, 1) for _ in range(10000)]
          + [rng.uniform(-700, 700) for _ in range(10000)]
          + [-0.0625, 0.0625, 1e-12, -3e-5, 0.2, -1.5, 0.3466, -0.3466, 707.0, -707.0])
    ulp = 2.220446049250313e-16
    for x in xs:
        ex = math.exp(x)
        assert abs(lib.e1(x) - ex) <= 2 * ulp * ex
        assert abs(lib.e3(x) - ex) <= 2 * ulp * ex
        if x != 0:
            assert abs(lib.e2(x) - math.expm1(x)) <= 4 * ulp * abs(math.expm1(x)) + 1e-300


def test_replica_draws_are_seeded_and_in_range():
    from souffle_gb300 import workloads
    a = workloads.replicas(4, seed=5)
    b = workloads.replicas(4, seed=5)
    for x, y in zip(a, b):
        assert x.opt.S == y.opt.S and x.opt.E == y.opt.E and np.array_equal(x.state.pos, y.state.pos)
        assert 20 <= x.opt.S <= 500 and 1.5 <= x.opt.E <= 3.0 and 200 <= x.opt.C <= 1600


def test_big_bead_placement_keeps_its_distances():
    """Bench placement of encapsulation big beads: inside the box, at least sigma_bead/2 + radius
    from every subunit bead and 2 radius from each other (the rule of generate_big_beads)."""
    from souffle_gb300 import workloads
    w = workloads.plain_small(seed=7)
    big = workloads.place_big_beads(w, 5, radius=3.0, seed=3)
    L = float(w.derived.box)
    assert big.shape == (5, 3) and np.all(np.abs(big) <= L / 2)
    for i, p in enumerate(big):
        d = w.state.pos - p
        d -= L * np.floor(d / L + 0.5)
        assert np.sqrt((d * d).sum(axis=1)).min() >= 0.5 + 3.0
        for q in big[:i]:
            e = q - p
            e -= L * np.floor(e / L + 0.5)
            assert np.sqrt((e * e).sum()) >= 6.0
    assert np.array_equal(big, workloads.place_big_beads(w, 5, radius=3.0, seed=3))


def test_uniform_replicas_are_independent_copies():
    from souffle_gb300 import workloads
    reps = workloads.uniform_replicas(3, 12)
    assert [int(r.opt.S) for r in reps] == [12, 12, 12]
    assert reps[0].derived.box == reps[2].derived.box
    assert not np.array_equal(reps[0].state.pos, reps[1].state.pos)
