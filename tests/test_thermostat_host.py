"""The double-float thermostat arithmetic of the force kernel, compiled for the host and checked
against plain FP64 (the chain recurrences of src/functions.cpp:33-58 and src/md.cpp:401-406,
457-460) and against exact integer arithmetic (the fixed-point conversions)."""
import ctypes
import math
import random
from fractions import Fraction

import pytest

from conftest import build_thermostat_lib, chain_of, run_host_chain

@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    return build_thermostat_lib(tmp_path_factory.mktemp("thermo"))


def test_double_float_exponential(lib):
    # below e^-60 the low word of a double-float turns subnormal and precision falls off; the
    # thermostat's arguments are -dt xi / 4, of order one
    rng = random.Random(3)
    xs = ([rng.uniform(-0.125, 0.125) for _ in range(4000)] + [rng.uniform(-4, 4) for _ in range(4000)]
          + [rng.uniform(-60, 80) for _ in range(2000)] + [0.0, 1e-9, -0.125, 0.125, 0.12500001, 87.0])
    for x in xs:
        x = float(ctypes.c_double(x).value)
        hi = float(ctypes.c_float(x).value)
        x = hi + float(ctypes.c_float(x - hi).value)     # exactly representable as double-float
        ex = math.exp(x)
        tol = 4e-14 if abs(x) <= 0.125 else (2e-12 if abs(x) <= 4 else 3e-11)
        assert abs(lib.t_exp(x) - ex) <= tol * ex, x
        if x != 0:
            em = math.expm1(x)
            assert abs(lib.t_expm1(x) - em) <= max(tol, 4e-14) * max(abs(em), abs(ex) if abs(x) > 0.125 else 0), x


def test_fixed_point_conversions_are_exact(lib):
    rng = random.Random(5)
    for _ in range(20000):
        e = rng.randint(-30, 61)
        hi = float(ctypes.c_float(rng.choice([-1, 1]) * rng.uniform(1, 2) * 2.0 ** e).value)
        ulp = 2.0 ** (math.frexp(hi)[1] - 24)
        lo = float(ctypes.c_float(rng.uniform(-0.5, 0.5) * ulp).value)
        scale = 2.0 ** rng.choice([0, 0, -8, 1])
        if abs((hi + lo) * scale) >= 2.0 ** 62:
            continue
        exact = (Fraction(hi) + Fraction(lo)) * Fraction(scale)
        assert lib.t_to_fixed(hi, lo, scale) == round(exact), (hi, lo, scale)   # ties to even
    out = (ctypes.c_float * 2)()
    for k in [0, 1, -1, 2 ** 63 - 1, -2 ** 63, 2 ** 40 + 12345, -(2 ** 52) - 7] + \
             [rng.randint(-2 ** 63, 2 ** 63 - 1) for _ in range(20000)]:
        for sh in (0, -32, -40):
            lib.t_from_fixed(k, 2.0 ** sh, out)
            v = Fraction(out[0]) + Fraction(out[1])
            ref = Fraction(k) * Fraction(2) ** sh
            assert abs(v - ref) <= abs(ref) * Fraction(1, 2 ** 47), (k, sh)
        if abs(k) < 2 ** 62:
            lib.t_from_fixed(k, 1.0, out)
            back = lib.t_to_fixed(out[0], out[1], 1.0)
            assert abs(back - k) <= abs(k) / 2 ** 47 + 1


def _chain_fp64(q, t, dof, dt, ke_seq):
    """The same recurrences in plain FP64 (the reference's own arithmetic type)."""
    m = len(q)
    on = [qq != 0 for qq in q]
    xi, eta = [0.0] * (m + 1), [0.0] * m

    def g(x, j, ke):
        return 2 * ke - dof[0] * t[0] if j == 0 else q[j - 1] * x[j - 1] ** 2 - dof[j] * t[j]

    def backward(xi, eta, ke):
        gs = [g(xi, j, ke) if on[j] else 0.0 for j in range(m)]
        xb, eb = list(xi), list(eta)
        for j in range(m - 1, -1, -1):
            if on[j]:
                e4 = math.exp(-0.25 * dt * xb[j + 1])
                xb[j] = xb[j] * e4 * e4 + 0.5 * dt / q[j] * gs[j] * e4
        for j in range(m):
            if on[j]:
                eb[j] += 0.5 * dt * xb[j]
        u = math.expm1(-0.25 * dt * xb[0])
        return xb, eb, -(u * (u + 2)), 0.5 * dt * (1 + u)

    def forward(xb, eb, ke):
        x, e = list(xb), list(eb)
        e4 = [math.exp(-0.25 * dt * xb[j + 1]) if on[j] else 1.0 for j in range(m)]
        for j in range(m):
            if on[j]:
                e[j] = eb[j] + 0.5 * dt * xb[j]
        for j in range(m):
            if on[j]:
                x[j] = x[j] * e4[j] ** 2 + 0.5 * dt / q[j] * g(x, j, ke) * e4[j]
        return x, e

    xb, eb, _, _ = backward(xi, eta, ke_seq[0])
    rows = []
    for a in range(len(ke_seq) - 1):
        xi, eta = forward(xb, eb, ke_seq[a + 1])
        xb, eb, delta, c0 = backward(xi, eta, ke_seq[a + 1])
        rows.append((xi[:m], eta, delta, c0))
    return rows


@pytest.mark.parametrize("chain,qmass", [(5, 1.0), (5, 0.05), (3, 10.0), (1, 0.0)])
def test_chain_matches_fp64(lib, chain, qmass):
    n3 = 3.0 * 1200
    temp, dt, steps = 1.0, 0.005, 300
    q, t, dof = chain_of(chain, qmass, temp, n3)
    rng = random.Random(chain * 7 + int(qmass * 100))
    ke = [0.5 * n3 * temp * (1 + 0.2 * math.sin(a / 9.0) + 0.05 * rng.uniform(-1, 1)) for a in range(steps + 1)]
    rc, out = run_host_chain(lib, q, t, dof, dt, ke)
    assert rc == steps
    ref = _chain_fp64(q, t, dof, dt, ke)
    xmax = 0.0
    for a, (xi, eta, delta, c0) in enumerate(ref):
        o = out[a]
        scale = max(1.0, max(abs(v) for v in xi))
        xmax = max(xmax, scale)
        for j in range(chain):
            assert abs(o[j] - xi[j]) <= 1e-10 * scale, (a, j, o[j], xi[j])
            assert abs(o[chain + j] - eta[j]) <= 1e-10 * max(1.0, abs(eta[j])), (a, j)
        assert abs(o[2 * chain] - delta * 2.0 ** 62) <= 1e-10 * 2.0 ** 62 * max(abs(delta), 1e-3) + 2, a
        assert abs(o[2 * chain + 1] - c0) <= 1e-12 * c0, a
    if chain > 1:
        assert xmax > 5.0      # the drive moved the chain well away from rest
