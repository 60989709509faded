"""Oracle test infrastructure -- NOT the product.

ctypes wrapper around the C restatement in ``souffle_oracle.c``.  Only tests,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` import it,
and only as the checker.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")


def build(quiet: bool = True) -> None:
    subprocess.run(["make", "-C", HERE, "-j4"], check=True,
                   stdout=subprocess.DEVNULL if quiet else None)


class _Desc(C.Structure):
    _fields_ = [
        ("n_sub", C.c_int), ("np", C.c_int), ("ne", C.c_int), ("nf", C.c_int), ("n_lj", C.c_int),
        ("b_type", C.POINTER(C.c_int)), ("b_q", C.POINTER(C.c_double)),
        ("b_sigma", C.POINTER(C.c_double)), ("b_mass", C.POINTER(C.c_double)),
        ("e_b", C.POINTER(C.c_int)), ("e_type", C.POINTER(C.c_int)),
        ("e_len0", C.POINTER(C.c_double)), ("f_b", C.POINTER(C.c_int)),
        ("lj_t", C.POINTER(C.c_int)),
        ("box", C.c_double), ("lb", C.c_double), ("kappa", C.c_double), ("ecut", C.c_double),
        ("ecut_el", C.c_double), ("elj_att", C.c_double), ("ks", C.c_double), ("kb", C.c_double),
        ("nlist_cutoff", C.c_double), ("nlist_capacity", C.c_int), ("center_local", C.c_int),
    ]


class _Nhc(C.Structure):
    _fields_ = [("m", C.c_int), ("q", C.c_double * 16), ("xi", C.c_double * 16),
                ("eta", C.c_double * 16), ("t", C.c_double * 16), ("dof", C.c_ulong * 16)]


_libs = {}


def load(variant: str = "ld") -> C.CDLL:
    name = "liboracle.so" if variant == "ld" else "liboracle_f64.so"
    if variant in _libs:
        return _libs[variant]
    path = os.path.join(BUILD, name)
    if not os.path.exists(path):
        build()
    lib = C.CDLL(path)
    vp = C.c_void_p
    dp = C.POINTER(C.c_double)
    ip = C.POINTER(C.c_int)
    lib.oracle_create.restype = vp
    lib.oracle_create.argtypes = [C.POINTER(_Desc)]
    lib.oracle_destroy.argtypes = [vp]
    lib.oracle_set_threads.argtypes = [C.c_int]
    lib.oracle_center_bead.restype = C.c_int
    lib.oracle_center_bead.argtypes = [C.c_int, dp, C.c_double]
    lib.oracle_set_state.argtypes = [vp, dp, dp]
    lib.oracle_get_state.argtypes = [vp, dp, dp]
    lib.oracle_forces.restype = C.c_int
    lib.oracle_forces.argtypes = [vp, C.c_int]
    lib.oracle_get_forces.argtypes = [vp, dp, dp, dp]
    lib.oracle_get_pairlist.argtypes = [vp, ip, ip]
    lib.oracle_energies.argtypes = [vp, dp, dp, dp, dp, dp]
    lib.oracle_kinetic_energy.restype = C.c_double
    lib.oracle_kinetic_energy.argtypes = [vp]
    lib.oracle_set_big_beads.argtypes = [vp, C.c_int, dp, C.c_double, C.c_double, C.c_double]
    lib.oracle_big_bead_energies.argtypes = [vp, dp, dp]
    lib.oracle_nhc_init.argtypes = [C.POINTER(_Nhc), C.c_int, C.c_double, C.c_double, C.c_int]
    lib.oracle_md_step.restype = C.c_int
    lib.oracle_md_step.argtypes = [vp, C.POINTER(_Nhc), C.c_uint, C.c_double, C.c_int, dp, dp]
    lib.oracle_loop_end.restype = C.c_uint
    lib.oracle_loop_end.argtypes = [C.c_double, C.c_double]
    _libs[variant] = lib
    return lib


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


class Oracle:
    """One template-replicated system held by the C restatement."""

    def __init__(self, template, n_sub: int, derived, ks: float, kb: float, elj_att: float,
                 center_local: int, variant: str = "ld", capacity: int | None = None):
        self.lib = load(variant)
        t = template
        self.np = t.n_beads
        self.n = n_sub * self.np
        self.cap = int(capacity if capacity is not None else derived.nlist_capacity)
        self._keep = dict(
            b_type=np.ascontiguousarray(t.types, dtype=np.int32),
            b_q=np.ascontiguousarray(t.charge, dtype=np.float64),
            b_sigma=np.ascontiguousarray(t.diameter, dtype=np.float64),
            b_mass=np.ascontiguousarray(t.mass, dtype=np.float64),
            e_b=np.ascontiguousarray(t.edges, dtype=np.int32).reshape(-1),
            e_type=np.ascontiguousarray(t.edge_type, dtype=np.int32),
            e_len0=np.ascontiguousarray(t.edge_len0, dtype=np.float64),
            f_b=np.ascontiguousarray(t.faces, dtype=np.int32).reshape(-1),
            lj_t=np.ascontiguousarray(np.array(t.lj_attract, dtype=np.int32).reshape(-1)),
        )
        k = self._keep
        d = _Desc(n_sub, self.np, len(t.edges), len(t.faces), len(t.lj_attract),
                  _p(k["b_type"], C.c_int), _p(k["b_q"], C.c_double), _p(k["b_sigma"], C.c_double),
                  _p(k["b_mass"], C.c_double), _p(k["e_b"], C.c_int), _p(k["e_type"], C.c_int),
                  _p(k["e_len0"], C.c_double), _p(k["f_b"], C.c_int), _p(k["lj_t"], C.c_int),
                  derived.box, derived.lb, derived.kappa, derived.ecut, derived.ecut_el,
                  elj_att, ks, kb, derived.nlist_cutoff, self.cap, center_local)
        self.h = self.lib.oracle_create(C.byref(d))
        if not self.h:
            raise ValueError("inconsistent template: a bending edge lacks two faces")
        self.nhc = _Nhc()

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.oracle_destroy(self.h)
            self.h = None

    @staticmethod
    def center_bead(np_: int, pos0: np.ndarray, box: float, variant: str = "ld") -> int:
        lib = load(variant)
        p = np.ascontiguousarray(pos0[:np_], dtype=np.float64)
        return lib.oracle_center_bead(np_, _p(p, C.c_double), box)

    def set_threads(self, n: int) -> None:
        self.lib.oracle_set_threads(n)

    def set_state(self, pos, vel=None):
        pos = np.ascontiguousarray(pos, dtype=np.float64)
        v = None if vel is None else np.ascontiguousarray(vel, dtype=np.float64)
        self.lib.oracle_set_state(self.h, _p(pos, C.c_double),
                                  None if v is None else _p(v, C.c_double))

    def get_state(self):
        pos = np.empty((self.n, 3))
        vel = np.empty((self.n, 3))
        self.lib.oracle_get_state(self.h, _p(pos, C.c_double), _p(vel, C.c_double))
        return pos, vel

    def forces(self, rebuild: bool = True):
        over = self.lib.oracle_forces(self.h, int(rebuild))
        tf, sf, bf = (np.empty((self.n, 3)) for _ in range(3))
        self.lib.oracle_get_forces(self.h, _p(tf, C.c_double), _p(sf, C.c_double),
                                   _p(bf, C.c_double))
        return tf, sf, bf, over

    def pairlist(self):
        counts = np.empty(self.n, dtype=np.int32)
        ids = np.empty((self.n, self.cap), dtype=np.int32)
        self.lib.oracle_get_pairlist(self.h, _p(counts, C.c_int), _p(ids, C.c_int))
        return counts, ids

    def energies(self):
        out = [np.empty(self.n) for _ in range(5)]
        self.lib.oracle_energies(self.h, *[_p(o, C.c_double) for o in out])
        return dict(zip(["se", "ke", "be", "ne", "ce"], out))

    def set_big_beads(self, pos, sigma: float, charge: float, shc: float) -> None:
        """Encapsulation big beads (src/forces.cpp:174-236, src/energies.cpp:96-137)."""
        self._bb = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1)
        self.lib.oracle_set_big_beads(self.h, self._bb.size // 3, _p(self._bb, C.c_double) if self._bb.size else None,
                                      sigma, charge, shc)

    def big_bead_energies(self):
        """(lj, electrostatic) sums over big beads of the last energies() call."""
        ne, ce = C.c_double(), C.c_double()
        self.lib.oracle_big_bead_energies(self.h, C.byref(ne), C.byref(ce))
        return ne.value, ce.value

    def kinetic_energy(self) -> float:
        return self.lib.oracle_kinetic_energy(self.h)

    def nhc_init(self, chain_len: int, q_mass: float, temperature_K: float):
        self.lib.oracle_nhc_init(C.byref(self.nhc), chain_len, q_mass, temperature_K, self.n)

    def md_step(self, a: int, dt: float, build_freq: int, ke: float):
        ke_io = C.c_double(ke)
        vcom = C.c_double(0)
        over = self.lib.oracle_md_step(self.h, C.byref(self.nhc), a, dt, build_freq,
                                       C.byref(ke_io), C.byref(vcom))
        return ke_io.value, vcom.value, over

    def loop_end(self, steps: float, dt: float) -> int:
        return self.lib.oracle_loop_end(steps, dt)
