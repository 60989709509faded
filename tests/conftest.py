import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(REPO, "capsid-souffle_gb300"))
sys.path.insert(0, os.path.join(REPO, "oracle"))
GOLDEN = os.path.join(REPO, "tests", "golden")
sys.path.insert(0, GOLDEN)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); parity tests through the C ABI")


def load_golden(name):
    z = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    return {k: z[k] for k in z.files}


GOLDEN_CASES = ["plain_small", "bilayer_dense", "patch_crowded"]


@pytest.fixture(params=GOLDEN_CASES)
def golden(request):
    return request.param, load_golden(request.param)


def golden_workload(g):
    """Template, options and derived parameters of a golden case (as its generator used)."""
    from souffle_gb300 import geometry, params, workloads

    t = geometry.template_by_name(str(g["template"]))
    S = int(g["n_sub"])
    opt = workloads.base_options(S=S, C=float(g["conc"]), f=t.name)
    d = params.derive(opt, 1e-9, 3.9434e-26, S * t.n_beads)
    return t, opt, d


def rms_rel(a, b):
    """Per-bead force RMS relative error: sqrt(sum |a-b|^2 / sum |b|^2)."""
    return float(np.sqrt(((a - b) ** 2).sum() / (b ** 2).sum()))


# The thermostat's double-float arithmetic compiled for the host: exp, the fixed-point
# conversions, and the chain run step by step over a given kinetic-energy sequence.
THERMO_SRC = r'''
#include "thermostat.cuh"
using namespace souffle;
extern "C" {
double t_exp(double x) { return df_to(df_exp(df_from(x))); }
double t_expm1(double x) { return df_to(df_expm1(df_from(x))); }
long long t_to_fixed(float hi, float lo, float scale) { return df_to_fixed(dfloat{hi, lo}, scale); }
void t_from_fixed(long long k, float scale, float* out) {
  const dfloat d = df_from_fixed(k, scale);
  out[0] = d.hi;
  out[1] = d.lo;
}
// As the force kernel runs the chain: the backward half after the initial forces, then per step
// forward + backward with that step's kinetic energy.  Per step writes xi[0..m-1], eta[0..m-1],
// delta_fx, kick_c0 (2 m + 2 doubles).  Returns the steps done (fewer when out of range).
int t_chain(int m, const double* q, const double* t, const double* dof, double dt, int steps,
            const double* ke, double* out) {
  SysState s;
  __builtin_memset(&s, 0, sizeof(s));
  s.m = m;
  for (int j = 0; j < m; j++) { s.q[j] = q[j]; s.t[j] = t[j]; s.dof[j] = dof[j]; }
  nhc_set_constants(s, dt);
  s.ke = df_from(ke[0]);
  if (!nhc_backward(s)) return -1;
  for (int a = 0; a < steps; a++) {
    s.ke = df_from(ke[a + 1]);
    nhc_forward(s);
    if (!nhc_backward(s)) return a;
    double* o = out + (size_t)a * (2 * m + 2);
    for (int j = 0; j < m; j++) { o[j] = df_to(s.xi[j]); o[m + j] = df_to(s.eta[j]); }
    o[2 * m] = (double)s.delta_fx;
    o[2 * m + 1] = df_to(s.kick_c0);
  }
  return steps;
}
}
'''


def build_thermostat_lib(d):
    import ctypes
    import shutil
    import subprocess
    nvcc = shutil.which("nvcc")
    if not nvcc:
        pytest.skip("nvcc not available")
    src, so = os.path.join(str(d), "t.cu"), os.path.join(str(d), "t.so")
    with open(src, "w") as f:
        f.write(THERMO_SRC)
    subprocess.run([nvcc, "-shared", "-Xcompiler", "-fPIC,-ffp-contract=off", "-std=c++17", "-I",
                    os.path.join(REPO, "capsid-souffle_gb300", "csrc"), src, "-o", so], check=True)
    L = ctypes.CDLL(so)
    for fn in (L.t_exp, L.t_expm1):
        fn.restype, fn.argtypes = ctypes.c_double, [ctypes.c_double]
    L.t_to_fixed.restype = ctypes.c_longlong
    L.t_to_fixed.argtypes = [ctypes.c_float, ctypes.c_float, ctypes.c_float]
    L.t_from_fixed.argtypes = [ctypes.c_longlong, ctypes.c_float, ctypes.POINTER(ctypes.c_float)]
    L.t_chain.restype = ctypes.c_int
    return L


def chain_of(length, qmass, temp, n3):
    """The chain's (Q, T, dof) as md_begin builds it (src/md.cpp:187-196)."""
    if length == 1:
        return [0.0], [temp], [n3]
    q = [qmass] + [1.0] * (length - 2) + [0.0]
    dof = [n3] + [1.0] * (length - 2) + [n3]
    return q, [temp] * length, dof


def run_host_chain(lib, q, t, dof, dt, ke):
    """Runs t_chain over ke (len steps + 1); returns per-step rows (xi, eta, delta_fx, kick_c0)."""
    import ctypes
    m, steps = len(q), len(ke) - 1
    arr = lambda v: (ctypes.c_double * len(v))(*v)
    out = (ctypes.c_double * (steps * (2 * m + 2)))()
    rc = lib.t_chain(m, arr(q), arr(t), arr(dof), ctypes.c_double(dt), steps, arr(ke), out)
    rows = np.frombuffer(out, dtype=np.float64).reshape(steps, 2 * m + 2)
    return rc, rows
