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
