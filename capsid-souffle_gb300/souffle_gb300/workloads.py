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


def plain_large(n_sub: int = 2000, seed: int = 12345, debye_length: float = 0.0,
                conc_um: float = 0.0, nhc_mass: float = 0.0) -> Workload:
    """The bilayer workload; ``debye_length`` (sigma), ``conc_um`` (micromolar) and ``nhc_mass``
    (-Q) override the default screening length of 1 sigma, concentration of 800 uM and chain
    mass of 10 when nonzero."""
    over = {}
    if nhc_mass:
        over["Q"] = nhc_mass
    if debye_length:
        over["c"] = state.salt_for_debye_length(debye_length)
    if conc_um:
        over["C"] = conc_um
    return make(geometry.bilayer_n5(), n_sub, seed, name="plain_large", **over)


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


def uniform_replicas(n: int, n_sub: int, seed: int = 4040) -> List[Workload]:
    """``n`` independent copies of the bilayer workload at ``n_sub`` subunits each (800 uM,
    Debye length 1 sigma), each from its own seeded initial state."""
    t = geometry.bilayer_n5()
    return [make(t, n_sub, seed=seed * 1000 + k, name=f"replica{k}") for k in range(n)]


def place_big_beads(w: Workload, n: int, radius: float = 3.0, seed: int = 31) -> np.ndarray:
    """``n`` encapsulation big beads of the given radius at seeded uniform positions in the
    workload's box, each at least (sigma_bead + 2 radius)/2 from every subunit bead and 2 radius
    from the other big beads (the placement rule of generate_big_beads,
    src/initialize.cpp:603-672, with numpy's generator instead of rand())."""
    rng = np.random.default_rng(seed)
    L = float(w.derived.box)
    sig = np.tile(np.asarray(w.template.diameter, dtype=np.float64), int(w.opt.S))
    min_d = sig / 2 + radius
    out = []
    while len(out) < n:
        p = (rng.random(3) - 0.5) * L
        d = w.state.pos - p
        d -= L * np.floor(d / L + 0.5)
        if np.any((d * d).sum(axis=1) < min_d * min_d):
            continue
        if any(np.sum(((q - p) - L * np.floor((q - p) / L + 0.5)) ** 2) < (2 * radius) ** 2 for q in out):
            continue
        out.append(p)
    return np.array(out).reshape(-1, 3)


def analysis_frames(n_sub: int = 2000, n_frames: int = 4, seed: int = 4242, conc_um: float = 800.0,
                    cluster_frac: float = 0.6, sigma_si: float = 1e-9):
    """Frames for the post-run analysis: 43-bead capsomeres (the bilayer patch plus a centre
    bead; the reference's analysis only sizes 41-, 43- and 78-bead subunits), 6 beads of type 0
    (sub-oligomer beads) and 4 of type 5 (pair-correlation beads) per subunit, in the box of
    n_sub subunits at conc_um micromolar (src/md.cpp:159).  A fraction of the subunits sits in
    chains of 2-8 with neighbours 3-5 sigma apart, so that oligomers and sub-oligomers form; later
    frames move every subunit by up to 0.3 sigma.

    Returns (types (N,) int32, frames (F, N, 3) float64, box, beads per subunit)."""
    t = geometry.bilayer_n5()
    local = t.pos - t.pos.mean(axis=0)
    local = np.vstack([local, np.zeros((1, 3))])
    np_ = local.shape[0]
    types = np.ones(np_, dtype=np.int32)
    types[0:6] = 0
    types[6:10] = 5
    box = (n_sub * 1000 / (conc_um * sigma_si ** 3 * 6.022e23)) ** (1.0 / 3.0)
    rng = np.random.default_rng(seed)
    n_cl = int(n_sub * cluster_frac)
    centres = []
    while len(centres) < n_cl:
        c = rng.uniform(-box / 2, box / 2, 3)
        for _ in range(min(int(rng.integers(2, 9)), n_cl - len(centres))):
            centres.append(c.copy())
            d = rng.normal(size=3)
            c = c + d / np.linalg.norm(d) * rng.uniform(3.0, 5.0)
    centres = np.vstack([np.array(centres).reshape(-1, 3), rng.uniform(-box / 2, box / 2, (n_sub - n_cl, 3))])
    rots = state._random_rotations(rng, n_sub)
    frames = []
    for f in range(n_frames):
        shift = rng.uniform(-0.3, 0.3, (n_sub, 3)) if f else np.zeros((n_sub, 3))
        pos = (np.einsum("sij,bj->sbi", rots, local) + (centres + shift)[:, None, :]).reshape(-1, 3)
        pos = pos - box * np.floor(pos / box + 0.5)
        pos = np.where(pos >= box / 2, pos - box, pos)
        frames.append(pos)
    return np.tile(types, n_sub), np.stack(frames), box, np_
