"""Seeded initial states, injected through SOUFFLE's restart-file port.

The reference can only start from a cubic lattice with rigid per-subunit
velocities (src/initialize.cpp:199-264, 422-564).  The synthetic workloads need
random centres of mass, random orientations and Maxwell-Boltzmann velocities,
so they are written as ``outfiles/restart_0.out`` (header
``Velocities & Positions for 0`` then ``i vx vy vz x y z`` rows, the layout of
src/md.cpp:526-536, read back by src/initialize.cpp:179-214) plus a one-line
``outfiles/rb_0.out`` that the reference's restart path opens unconditionally
(src/initialize.cpp:576-583).

Positions are rounded to multiples of 2**-24 sigma and printed exactly, so the
reference (which parses positions into ``long double``) and this package (which
parses ``double``) start from bit-identical coordinates.  Velocities are printed
with 17 significant digits; the reference parses them into ``double`` too.
"""
from __future__ import annotations

import dataclasses
import math
import os
from decimal import Decimal
from typing import Optional

import numpy as np

from .geometry import Template

AVOGADRO = 6.022e23  # the constant of src/md.cpp:45
PI_REF = 3.14159     # the constant of src/md.cpp:49
POS_QUANTUM = 2.0 ** -24


def box_length(n_subunits: int, conc_uM: float, sigma_si: float = 1e-9) -> float:
    """Cubic box edge in sigma units (src/md.cpp:159)."""
    return (n_subunits * 1000.0 / (conc_uM * sigma_si ** 3 * AVOGADRO)) ** (1.0 / 3.0)


def debye_kappa(salt_mM: float, sigma_si: float = 1e-9) -> float:
    """Inverse screening length in 1/sigma (src/md.cpp:165-169)."""
    lb = 0.701e-9 / sigma_si
    ni = salt_mM * AVOGADRO * sigma_si ** 3
    return math.sqrt(8 * PI_REF * ni * lb)


def salt_for_debye_length(lambda_d: float, sigma_si: float = 1e-9) -> float:
    """Salt concentration (mM) that gives screening length ``lambda_d`` sigma."""
    lb = 0.701e-9 / sigma_si
    return 1.0 / (lambda_d ** 2 * 8 * PI_REF * lb * AVOGADRO * sigma_si ** 3)


def _random_rotations(rng: np.random.Generator, n: int) -> np.ndarray:
    """Uniform random rotation matrices from uniform unit quaternions."""
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q.T
    r = np.empty((n, 3, 3))
    r[:, 0, 0] = 1 - 2 * (y * y + z * z)
    r[:, 0, 1] = 2 * (x * y - z * w)
    r[:, 0, 2] = 2 * (x * z + y * w)
    r[:, 1, 0] = 2 * (x * y + z * w)
    r[:, 1, 1] = 1 - 2 * (x * x + z * z)
    r[:, 1, 2] = 2 * (y * z - x * w)
    r[:, 2, 0] = 2 * (x * z - y * w)
    r[:, 2, 1] = 2 * (y * z + x * w)
    r[:, 2, 2] = 1 - 2 * (x * x + y * y)
    return r


def _place_centres(rng: np.random.Generator, n: int, box: float, min_dist: float,
                   max_tries: int = 200000) -> np.ndarray:
    """Non-overlapping uniform random centres in [-box/2, box/2)^3 (cell-grid rejection)."""
    ncell = max(1, int(box // min_dist))
    cell = box / ncell
    grid = {}
    out = np.empty((n, 3))
    placed = 0
    tries = 0
    while placed < n:
        tries += 1
        if tries > max_tries + 50 * n:
            raise RuntimeError("could not place subunits without overlap; lower the concentration")
        p = (rng.random(3) - 0.5) * box
        c = tuple(int((p[d] + box / 2) // cell) % ncell for d in range(3))
        ok = True
        for dx in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dz in (-1, 0, 1):
                    key = ((c[0] + dx) % ncell, (c[1] + dy) % ncell, (c[2] + dz) % ncell)
                    for k in grid.get(key, ()):
                        d = p - out[k]
                        d -= box * np.round(d / box)
                        if d @ d < min_dist * min_dist:
                            ok = False
                            break
                    if not ok:
                        break
                if not ok:
                    break
            if not ok:
                break
        if ok:
            out[placed] = p
            grid.setdefault(c, []).append(placed)
            placed += 1
    return out


@dataclasses.dataclass
class State:
    pos: np.ndarray   # (N, 3) float64, wrapped into [-L/2, L/2)
    vel: np.ndarray   # (N, 3) float64
    box: float


def random_state(t: Template, n_subunits: int, box: float, temperature: float = 1.0,
                 seed: int = 12345, min_gap: float = 1.0) -> State:
    """Random COMs, random orientations, Maxwell-Boltzmann velocities, zero net momentum."""
    rng = np.random.default_rng(seed)
    local = t.pos - t.pos.mean(axis=0)
    diam = 2.0 * float(np.sqrt((local ** 2).sum(axis=1)).max())
    centres = _place_centres(rng, n_subunits, box, diam + min_gap)
    rots = _random_rotations(rng, n_subunits)
    pos = (np.einsum("sij,bj->sbi", rots, local) + centres[:, None, :]).reshape(-1, 3)
    pos = pos - box * np.floor(pos / box + 0.5)            # wrap into [-L/2, L/2)
    pos = np.round(pos / POS_QUANTUM) * POS_QUANTUM
    pos = np.where(pos >= box / 2, pos - box, pos)
    mass = np.tile(t.mass, n_subunits)
    vel = rng.normal(size=pos.shape) * np.sqrt(temperature / mass)[:, None]
    vel -= vel.mean(axis=0)
    return State(pos, vel, box)


def _exact(x: float) -> str:
    """Exact decimal text of a double (finite for multiples of 2**-24)."""
    s = format(Decimal(float(x)), "f")
    return s


def write_restart(state: State, outdir: str, step: int = 0, big_beads: int = 1,
                  big_bead_pos: Optional[np.ndarray] = None) -> None:
    """Write ``restart_<step>.out`` and ``rb_<step>.out`` under ``outdir``.  ``rb`` holds one
    line per big bead (velocity, position: src/md.cpp:537-545); ``big_bead_pos`` [n][3] gives
    their positions (at rest), else ``big_beads`` zero lines."""
    os.makedirs(outdir, exist_ok=True)
    lines = [f"Velocities & Positions for {step}"]
    for i in range(state.pos.shape[0]):
        v = state.vel[i]
        p = state.pos[i]
        lines.append(f"{i}  {v[0]:.17g} {v[1]:.17g} {v[2]:.17g} "
                     f"{_exact(p[0])} {_exact(p[1])} {_exact(p[2])}")
    with open(os.path.join(outdir, f"restart_{step}.out"), "w") as fh:
        fh.write("\n".join(lines) + "\n")
    with open(os.path.join(outdir, f"rb_{step}.out"), "w") as fh:
        if big_bead_pos is not None:
            for p in np.asarray(big_bead_pos, dtype=np.float64).reshape(-1, 3):
                fh.write(f"0 0 0 {_exact(p[0])} {_exact(p[1])} {_exact(p[2])}\n")
        else:
            for _ in range(big_beads):
                fh.write("0 0 0 0 0 0\n")


def read_restart(path: str, n_beads: Optional[int] = None):
    """Read a restart file: returns (step, vel (N,3), pos (N,3))."""
    with open(path) as fh:
        tok = fh.read().split()
    step = int(tok[4])
    rows = np.array(tok[5:], dtype=object).reshape(-1, 7)
    if n_beads is not None:
        rows = rows[:n_beads]
    vel = rows[:, 1:4].astype(np.float64)
    pos = rows[:, 4:7].astype(np.float64)
    return step, vel, pos
