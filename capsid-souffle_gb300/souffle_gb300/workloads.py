"""The synthetic workloads: geometry, run options and seeded initial states.

* ``plain_small``  20 single-layer 10-bead capsomeres (patch_n3), 800 uM.
* ``plain_large``  2000 two-layer 42-bead capsomeres (bilayer_n5), 800 uM: 84,000 beads.
* ``replicas``     independent systems of 20-500 bilayer capsomeres with per-system
                   attraction, screening length and concentration drawn from a seed.

Shared options (reference letters): -s 1000 -b 1000 -E 2.1 -e 5 -L 0.3 -B 10 -t 0.005
-q 5 -Q 10 -K 298, salt -c 94.27 mM (Debye length 1 sigma with the reference's constants).
"""
from __future__ import annotations

import dataclasses
from typing import List

import numpy as np

from . import geometry, params, state


@dataclasses.dataclass
class Workload:
    template: geometry.Template
    opt: params.CliOptions
    derived: params.Derived
    state: state.State
    center_local: int
    name: str

    @property
    def n_beads(self) -> int:
        return int(self.opt.S) * self.template.n_beads


def center_bead(pos_subunit0: np.ndarray, box: float) -> int:
    """Template-local index of the bead closest to subunit 0's centroid.

    generate_lattice (src/initialize.cpp:266-288): the centroid is the plain mean of subunit 0's
    positions; distances use the single-shift minimum image; the first strict minimum wins.
    """
    p = np.asarray(pos_subunit0, dtype=np.float64)
    c = p.mean(axis=0)
    best, idx = 1000.0, 0
    for i in range(p.shape[0]):
        r = p[i] - c
        r = np.where(r > box / 2, r - box, np.where(r < -box / 2, r + box, r))
        d = float(r @ r)
        if d < best:
            best, idx = d, i
    return idx


def base_options(**over) -> params.CliOptions:
    o = params.CliOptions(D="m", C=800.0, c=94.27, s=1000.0, b=1000.0, E=2.1, e=5.0, L=0.3, B=10,
                          t=0.005, q=5, Q=10.0, K=298.0)
    for k, v in over.items():
        setattr(o, k, v)
    return o


def make(template: geometry.Template, n_sub: int, seed: int = 12345, name: str = "",
         sigma_si: float = 1e-9, mass_si: float = 3.9434e-26, **over) -> Workload:
    opt = base_options(S=n_sub, f=template.name, **over)
    d = params.derive(opt, sigma_si, mass_si, n_sub * template.n_beads)
    st = state.random_state(template, n_sub, d.box, temperature=d.T_reduced, seed=seed)
    c = center_bead(st.pos[:template.n_beads], d.box)
    return Workload(template, opt, d, st, c, name or template.name)


def plain_small(seed: int = 12345) -> Workload:
    return make(geometry.patch_n3(), 20, seed, name="plain_small")


def plain_large(n_sub: int = 2000, seed: int = 12345) -> Workload:
    return make(geometry.bilayer_n5(), n_sub, seed, name="plain_large")


def replicas(n: int = 256, seed: int = 2024, sub_range=(20, 500)) -> List[Workload]:
    """Independent systems with per-replica parameters drawn from ``seed``."""
    rng = np.random.default_rng(seed)
    t = geometry.bilayer_n5()
    out = []
    for k in range(n):
        S = int(rng.integers(sub_range[0], sub_range[1] + 1))
        eps = float(rng.uniform(1.5, 3.0))
        lam = float(rng.uniform(0.5, 2.0))
        conc = float(rng.uniform(200.0, 1600.0))
        salt = state.salt_for_debye_length(lam)
        out.append(make(t, S, seed=seed * 1000 + k, name=f"replica{k}", E=eps, c=salt, C=conc))
    return out
