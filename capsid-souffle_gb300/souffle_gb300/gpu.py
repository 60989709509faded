"""ctypes binding of the C ABI in include/souffle_gpu.h.

The library is ``capsid-souffle_gb300/_build/libsouffle_gb300.so`` (built by
``capsid-souffle_gb300/build.py``).  There is no fallback: if the library or a
GPU is missing, every entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional, Sequence

import numpy as np

from .geometry import Template
from .params import CliOptions, Derived

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG, "_build", "libsouffle_gb300.so")

STATUS = {0: "OK", 1: "BAD_INPUT", 2: "CUDA", 3: "NL_OVERFLOW", 4: "NONFINITE", 5: "NO_DEVICE",
          6: "STATE"}

EXPORTED = [
    "souffle_gpu_create", "souffle_gpu_destroy", "souffle_gpu_num_beads", "souffle_gpu_set_state",
    "souffle_gpu_set_big_beads",
    "souffle_gpu_get_state", "souffle_gpu_forces", "souffle_gpu_get_pairlist",
    "souffle_gpu_pairlist_stats", "souffle_gpu_energies", "souffle_gpu_kinetic_energy",
    "souffle_gpu_md_begin", "souffle_gpu_md_steps", "souffle_gpu_md_enqueue", "souffle_gpu_md_scalars",
    "souffle_gpu_synchronize", "souffle_gpu_last_error", "souffle_gpu_stream",
    "souffle_gpu_md_profile", "souffle_gpu_kinetic_energy_noalloc", "souffle_gpu_autotune",
    "souffle_gpu_snapshot_enqueue", "souffle_gpu_snapshot_wait", "souffle_gpu_host_alloc", "souffle_gpu_host_free",
    # include/souffle_surrogate.h
    "souffle_mlp_create", "souffle_mlp_destroy", "souffle_mlp_stream", "souffle_mlp_param_count", "souffle_mlp_get_params",
    "souffle_mlp_set_params", "souffle_mlp_forward", "souffle_mlp_forward_layered", "souffle_mlp_profile_forward", "souffle_mlp_gradients", "souffle_mlp_train_step",
    "souffle_gemm_bf16", "souffle_surrogate_attach", "souffle_surrogate_collect", "souffle_surrogate_fit",
    "souffle_surrogate_enable", "souffle_surrogate_get_stats",
    # include/souffle_analysis.h
    "souffle_analysis_default_options", "souffle_analysis_create", "souffle_analysis_destroy",
    "souffle_analysis_frames", "souffle_analysis_enqueue", "souffle_analysis_synchronize",
    "souffle_analysis_stream", "souffle_analysis_last_counts",
]


class SurrogateOptions_(C.Structure):
    _fields_ = [("switch_radius", C.c_double), ("far_capacity", C.c_int32), ("judge_every", C.c_int32),
                ("judge_stride", C.c_int32), ("judge_tolerance", C.c_double)]


class SurrogateStats_(C.Structure):
    _fields_ = [("enabled", C.c_int32), ("far_pairs", C.c_int32), ("far_found", C.c_int32),
                ("classes_off", C.c_int32), ("judged", C.c_int64), ("last_error", C.c_double * 4)]


class SouffleError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


class Template_(C.Structure):
    _fields_ = [("np", C.c_int32), ("ne", C.c_int32), ("nf", C.c_int32), ("n_lj", C.c_int32),
                ("bead_type", C.POINTER(C.c_int32)), ("bead_charge", C.POINTER(C.c_double)),
                ("bead_sigma", C.POINTER(C.c_double)), ("bead_mass", C.POINTER(C.c_double)),
                ("edge_beads", C.POINTER(C.c_int32)), ("edge_type", C.POINTER(C.c_int32)),
                ("edge_len0", C.POINTER(C.c_double)), ("face_beads", C.POINTER(C.c_int32)),
                ("lj_types", C.POINTER(C.c_int32)), ("bend_rest_pos", C.POINTER(C.c_double))]


class Params_(C.Structure):
    _fields_ = [("n_subunits", C.c_int32), ("box", C.c_double), ("ks", C.c_double),
                ("kb", C.c_double), ("elj_att", C.c_double), ("lb", C.c_double),
                ("kappa", C.c_double), ("ecut", C.c_double), ("ecut_el", C.c_double),
                ("nlist_cutoff", C.c_double), ("nlist_capacity", C.c_int32),
                ("center_local", C.c_int32), ("dt", C.c_double), ("chain_length", C.c_int32),
                ("nhc_mass", C.c_double), ("temperature", C.c_double), ("build_freq", C.c_int32),
                ("brownian", C.c_int32), ("damp", C.c_double)]


class Options_(C.Structure):
    _fields_ = [("inter_capacity", C.c_int32), ("cand_capacity", C.c_int32),
                ("compat_quirks", C.c_int32), ("device", C.c_int32),
                ("threads_per_cta", C.c_int32), ("subunits_per_cta", C.c_int32), ("chain_fp64", C.c_int32)]


class Tuning_(C.Structure):
    _fields_ = [("subunits_per_cta", C.c_int32), ("threads_per_cta", C.c_int32), ("forces_us", C.c_double),
                ("default_forces_us", C.c_double), ("candidates", C.c_int32)]


class Energies_(C.Structure):
    _fields_ = [(n, C.c_double) for n in ["kinetic", "stretching", "bending", "lj", "electrostatic",
                                           "thermo_pe", "thermo_ke", "temperature",
                                           "vcom_magnitude", "bigbead_lj", "bigbead_electrostatic"]]


class PairStats_(C.Structure):
    _fields_ = [("mean_length", C.c_double), ("max_length", C.c_int32), ("max_inter", C.c_int32),
                ("over_reference_capacity", C.c_int32)]


class KernelTimes_(C.Structure):
    _fields_ = [("drift_ms", C.c_double), ("rebuild_ms", C.c_double), ("forces_ms", C.c_double),
                ("steps", C.c_int32), ("rebuilds", C.c_int32)]


_lib = None


def load() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: build it with capsid-souffle_gb300/build.py")
    lib = C.CDLL(LIB_PATH)
    vp, dp, ip = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int32)
    lib.souffle_gpu_create.argtypes = [C.POINTER(Template_), C.POINTER(Params_), C.c_int32,
                                       C.POINTER(Options_), C.POINTER(vp)]
    lib.souffle_gpu_destroy.argtypes = [vp]
    lib.souffle_gpu_num_beads.restype = C.c_int64
    lib.souffle_gpu_num_beads.argtypes = [vp]
    lib.souffle_gpu_set_state.argtypes = [vp, dp, dp]
    lib.souffle_gpu_set_big_beads.argtypes = [vp, C.c_int32, C.c_int32, dp, C.c_double, C.c_double, C.c_double]
    lib.souffle_gpu_get_state.argtypes = [vp, dp, dp]
    lib.souffle_gpu_forces.argtypes = [vp, C.c_int32, dp, dp, dp]
    lib.souffle_gpu_get_pairlist.argtypes = [vp, C.c_int32, ip, ip]
    lib.souffle_gpu_pairlist_stats.argtypes = [vp, C.c_int32, C.POINTER(PairStats_)]
    lib.souffle_gpu_energies.argtypes = [vp, C.c_int32, C.POINTER(Energies_), dp, dp, dp, dp, dp]
    lib.souffle_gpu_kinetic_energy.argtypes = [vp, C.c_int32, dp]
    lib.souffle_gpu_md_begin.argtypes = [vp]
    lib.souffle_gpu_md_steps.argtypes = [vp, C.c_int64, C.c_int32]
    lib.souffle_gpu_md_enqueue.argtypes = [vp, C.c_int64, C.c_int32]
    lib.souffle_gpu_md_scalars.argtypes = [vp, C.c_int32, dp, dp, dp]
    lib.souffle_gpu_synchronize.argtypes = [vp]
    lib.souffle_gpu_snapshot_enqueue.argtypes = [vp, C.c_int32, vp, vp]
    lib.souffle_gpu_snapshot_wait.argtypes = [vp, C.c_int32]
    lib.souffle_gpu_host_alloc.argtypes = [C.c_int64]
    lib.souffle_gpu_host_alloc.restype = vp
    lib.souffle_gpu_host_free.argtypes = [vp]
    lib.souffle_gpu_host_free.restype = None
    lib.souffle_gpu_last_error.restype = C.c_char_p
    lib.souffle_gpu_stream.restype = C.c_void_p
    lib.souffle_gpu_stream.argtypes = [vp]
    lib.souffle_gpu_md_profile.argtypes = [vp, C.c_int64, C.c_int32, C.POINTER(KernelTimes_)]
    lib.souffle_gpu_autotune.argtypes = [vp, C.c_int32, C.POINTER(Tuning_)]
    lib.souffle_gpu_kinetic_energy_noalloc.argtypes = [dp, dp, C.c_int64, dp, vp]
    fp = C.POINTER(C.c_float)
    lib.souffle_mlp_create.argtypes = [C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_uint64, C.c_int32,
                                       C.POINTER(vp)]
    lib.souffle_mlp_destroy.argtypes = [vp]
    lib.souffle_mlp_stream.restype = C.c_void_p
    lib.souffle_mlp_stream.argtypes = [vp]
    lib.souffle_mlp_param_count.restype = C.c_int64
    lib.souffle_mlp_param_count.argtypes = [vp]
    lib.souffle_mlp_get_params.argtypes = [vp, fp, C.c_int64]
    lib.souffle_mlp_set_params.argtypes = [vp, fp, C.c_int64]
    lib.souffle_mlp_forward.argtypes = [vp, vp, C.c_int32, vp]
    lib.souffle_mlp_forward_layered.argtypes = [vp, vp, C.c_int32, vp]
    lib.souffle_mlp_profile_forward.argtypes = [vp, C.c_int32, C.c_int32, C.c_int32, C.POINTER(C.c_double)]
    lib.souffle_mlp_gradients.argtypes = [vp, vp, vp, C.c_int32, fp, fp]
    lib.souffle_mlp_train_step.argtypes = [vp, vp, vp, C.c_int32, C.c_float, fp]
    lib.souffle_gemm_bf16.argtypes = [vp, vp, C.c_int32, C.c_int32, C.c_int32, vp, C.c_int32]
    lib.souffle_surrogate_attach.argtypes = [vp, vp, dp, C.POINTER(SurrogateOptions_)]
    lib.souffle_surrogate_collect.argtypes = [vp, vp, vp, C.c_int32, C.POINTER(C.c_int32)]
    lib.souffle_surrogate_fit.argtypes = [vp, vp, vp, C.c_int32, C.c_int32, C.c_int32, C.c_float, C.c_uint64,
                                          C.POINTER(C.c_float)]
    lib.souffle_surrogate_enable.argtypes = [vp, C.c_int32]
    lib.souffle_surrogate_get_stats.argtypes = [vp, C.POINTER(SurrogateStats_)]
    for name in EXPORTED:
        if name not in ("souffle_gpu_last_error", "souffle_gpu_num_beads", "souffle_gpu_stream",
                        "souffle_mlp_param_count", "souffle_mlp_stream"):
            getattr(lib, name).restype = C.c_int
    _lib = lib
    return lib


def _check(code: int) -> None:
    if code != 0:
        msg = load().souffle_gpu_last_error().decode(errors="replace")
        raise SouffleError(code, msg)


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


def system_params(opt: CliOptions, d: Derived, n_sub: int, center_local: int) -> Params_:
    """Reduced-unit parameters of one system, as run_simulation derives them."""
    return Params_(int(n_sub), d.box, opt.s, opt.b, opt.E, d.lb, d.kappa, d.ecut, d.ecut_el,
                   d.nlist_cutoff, d.nlist_capacity, int(center_local), opt.t, int(opt.q), opt.Q,
                   d.T_reduced, int(opt.B), 1 if opt.D == "b" else 0, float(opt.d))


class GpuSystem:
    """A handle over one or more systems sharing one template."""

    def __init__(self, t: Template, params: Sequence[Params_], inter_capacity: int = 0,
                 cand_capacity: int = 0, quirks: bool = True, device: int = 0, threads_per_cta: int = 0,
                 subunits_per_cta: int = 0, chain_fp64: bool = False):
        self.lib = load()
        self.t = t
        self._arrs = dict(
            type=np.ascontiguousarray(t.types, dtype=np.int32),
            q=np.ascontiguousarray(t.charge, dtype=np.float64),
            sig=np.ascontiguousarray(t.diameter, dtype=np.float64),
            m=np.ascontiguousarray(t.mass, dtype=np.float64),
            eb=np.ascontiguousarray(t.edges, dtype=np.int32).reshape(-1),
            et=np.ascontiguousarray(t.edge_type, dtype=np.int32),
            l0=np.ascontiguousarray(t.edge_len0, dtype=np.float64),
            fb=np.ascontiguousarray(t.faces, dtype=np.int32).reshape(-1),
            lj=np.ascontiguousarray(np.array(t.lj_attract, dtype=np.int32).reshape(-1)),
        )
        a = self._arrs
        if t.bend_rest is not None:
            a["rest"] = np.ascontiguousarray(t.bend_rest, dtype=np.float64).reshape(-1)
        tpl = Template_(t.n_beads, len(t.edges), len(t.faces), len(t.lj_attract), _ip(a["type"]),
                        _dp(a["q"]), _dp(a["sig"]), _dp(a["m"]), _ip(a["eb"]), _ip(a["et"]),
                        _dp(a["l0"]), _ip(a["fb"]),
                        _ip(a["lj"]) if a["lj"].size else None,
                        _dp(a["rest"]) if t.bend_rest is not None else None)
        self.params = list(params)
        arr = (Params_ * len(self.params))(*self.params)
        opts = Options_(inter_capacity, cand_capacity, 1 if quirks else -1, device, threads_per_cta,
                        subunits_per_cta, 1 if chain_fp64 else 0)
        h = C.c_void_p()
        _check(self.lib.souffle_gpu_create(C.byref(tpl), arr, len(self.params), C.byref(opts),
                                           C.byref(h)))
        self.h = h
        self.n = int(self.lib.souffle_gpu_num_beads(self.h))
        self.np = t.n_beads
        self.sys_beads = [p.n_subunits * self.np for p in self.params]

    def close(self):
        if getattr(self, "h", None):
            self.lib.souffle_gpu_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def set_state(self, pos, vel=None):
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1)
        assert pos.size == 3 * self.n
        v = None if vel is None else np.ascontiguousarray(vel, dtype=np.float64).reshape(-1)
        _check(self.lib.souffle_gpu_set_state(self.h, _dp(pos), None if v is None else _dp(v)))

    def set_big_beads(self, pos, sigma: float, charge: float, shc: float, system: int = 0):
        """Encapsulation big beads of one system (include/souffle_gpu.h souffle_gpu_set_big_beads):
        pos [n][3] in box coordinates; an empty array removes them."""
        p = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1)
        assert p.size % 3 == 0
        _check(self.lib.souffle_gpu_set_big_beads(self.h, int(system), p.size // 3, _dp(p) if p.size else None,
                                                  float(sigma), float(charge), float(shc)))

    def get_state(self):
        pos = np.empty((self.n, 3))
        vel = np.empty((self.n, 3))
        _check(self.lib.souffle_gpu_get_state(self.h, _dp(pos), _dp(vel)))
        return pos, vel

    def snapshot_enqueue(self, slot: int, pos: np.ndarray, vel: np.ndarray) -> None:
        """Queue a read-back of the state into pos / vel ([n][3] float64, C order; either may be
        None) behind the queued work; the arrays must stay alive until snapshot_wait(slot)."""
        for arr in (pos, vel):
            if arr is not None and (arr.dtype != np.float64 or not arr.flags.c_contiguous or arr.size != 3 * self.n):
                raise ValueError("snapshot buffers: [n][3] C-contiguous float64")
        _check(self.lib.souffle_gpu_snapshot_enqueue(self.h, slot, pos.ctypes.data if pos is not None else None,
                                                     vel.ctypes.data if vel is not None else None))

    def snapshot_wait(self, slot: int) -> None:
        _check(self.lib.souffle_gpu_snapshot_wait(self.h, slot))

    def forces(self, rebuild: bool = True, parts: bool = False):
        tf = np.empty((self.n, 3))
        sf = np.empty((self.n, 3)) if parts else None
        bf = np.empty((self.n, 3)) if parts else None
        _check(self.lib.souffle_gpu_forces(self.h, int(rebuild), _dp(tf),
                                           None if sf is None else _dp(sf),
                                           None if bf is None else _dp(bf)))
        return (tf, sf, bf) if parts else tf

    def autotune(self, trials: int = 20) -> dict:
        """Measure the force kernel at every candidate CTA shape and keep the fastest."""
        t = Tuning_()
        _check(self.lib.souffle_gpu_autotune(self.h, trials, C.byref(t)))
        return {f: getattr(t, f) for f, _ in Tuning_._fields_}

    def pairlist(self, cap: int):
        counts = np.empty(self.n, dtype=np.int32)
        ids = np.empty((self.n, cap), dtype=np.int32)
        _check(self.lib.souffle_gpu_get_pairlist(self.h, cap, _ip(counts), _ip(ids)))
        return counts, ids

    def pairlist_stats(self, system: int = 0) -> dict:
        s = PairStats_()
        _check(self.lib.souffle_gpu_pairlist_stats(self.h, system, C.byref(s)))
        return {f: getattr(s, f) for f, _ in PairStats_._fields_}

    def energies(self, system: int = 0, per_bead: bool = False):
        e = Energies_()
        n = self.sys_beads[system]
        arrs = [np.empty(n) for _ in range(5)] if per_bead else [None] * 5
        _check(self.lib.souffle_gpu_energies(self.h, system, C.byref(e),
                                             *[None if x is None else _dp(x) for x in arrs]))
        tot = {f: getattr(e, f) for f, _ in Energies_._fields_}
        if per_bead:
            return tot, dict(zip(["se", "be", "ne", "ce", "ke"], arrs))
        return tot

    def md_begin(self):
        _check(self.lib.souffle_gpu_md_begin(self.h))

    def md_steps(self, first_step: int, n_steps: int):
        _check(self.lib.souffle_gpu_md_steps(self.h, int(first_step), int(n_steps)))

    def md_enqueue(self, first_step: int, n_steps: int):
        """md_steps without waiting; errors surface at the next md_steps or synchronize."""
        _check(self.lib.souffle_gpu_md_enqueue(self.h, int(first_step), int(n_steps)))

    def md_scalars(self, system: int = 0):
        ke, xi0, vc = C.c_double(), C.c_double(), C.c_double()
        _check(self.lib.souffle_gpu_md_scalars(self.h, system, C.byref(ke), C.byref(xi0),
                                               C.byref(vc)))
        return ke.value, xi0.value, vc.value

    def synchronize(self):
        _check(self.lib.souffle_gpu_synchronize(self.h))

    def stream(self) -> int:
        """The handle's cudaStream_t as an integer."""
        return int(self.lib.souffle_gpu_stream(self.h) or 0)

    def md_profile(self, first_step: int, n_steps: int) -> dict:
        k = KernelTimes_()
        _check(self.lib.souffle_gpu_md_profile(self.h, int(first_step), int(n_steps), C.byref(k)))
        return {f: getattr(k, f) for f, _ in KernelTimes_._fields_}


class Mlp:
    """The surrogate network (include/souffle_surrogate.h).  Device arrays are passed as raw
    pointers (integers), e.g. ``tensor.data_ptr()`` of a contiguous float32 CUDA tensor."""

    def __init__(self, n_in: int, n_out: int, max_batch: int, seed: int = 1, width: int = 256, device: int = 0):
        self.lib = load()
        self.h = C.c_void_p()
        _check(self.lib.souffle_mlp_create(n_in, width, n_out, max_batch, seed, device, C.byref(self.h)))
        self.n_in, self.n_out, self.width = n_in, n_out, width
        self.n_params = int(self.lib.souffle_mlp_param_count(self.h))

    def close(self):
        if self.h:
            self.lib.souffle_mlp_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def stream(self) -> int:
        """The network's cudaStream_t as an integer."""
        return int(self.lib.souffle_mlp_stream(self.h) or 0)

    def profile_forward(self, m: int, iters: int, fused: bool = True) -> float:
        """Mean device microseconds per forward over the rows of the last forward's input."""
        us = C.c_double()
        _check(self.lib.souffle_mlp_profile_forward(self.h, m, iters, 1 if fused else 0, C.byref(us)))
        return us.value

    def get_params(self) -> np.ndarray:
        out = np.empty(self.n_params, dtype=np.float32)
        _check(self.lib.souffle_mlp_get_params(self.h, out.ctypes.data_as(C.POINTER(C.c_float)), self.n_params))
        return out

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, dtype=np.float32)
        _check(self.lib.souffle_mlp_set_params(self.h, p.ctypes.data_as(C.POINTER(C.c_float)), self.n_params))

    def forward(self, x_ptr: int, m: int, y_ptr: int) -> None:
        _check(self.lib.souffle_mlp_forward(self.h, C.c_void_p(x_ptr), m, C.c_void_p(y_ptr)))

    def forward_layered(self, x_ptr: int, m: int, y_ptr: int) -> None:
        """The per-layer GEMM forward (the training path's forward)."""
        _check(self.lib.souffle_mlp_forward_layered(self.h, C.c_void_p(x_ptr), m, C.c_void_p(y_ptr)))

    def gradients(self, x_ptr: int, t_ptr: int, m: int):
        g = np.empty(self.n_params, dtype=np.float32)
        loss = C.c_float()
        _check(self.lib.souffle_mlp_gradients(self.h, C.c_void_p(x_ptr), C.c_void_p(t_ptr), m, C.byref(loss),
                                              g.ctypes.data_as(C.POINTER(C.c_float))))
        return float(loss.value), g

    def train_step(self, x_ptr: int, t_ptr: int, m: int, lr: float) -> float:
        loss = C.c_float()
        _check(self.lib.souffle_mlp_train_step(self.h, C.c_void_p(x_ptr), C.c_void_p(t_ptr), m, lr, C.byref(loss)))
        return float(loss.value)


def gemm_bf16(a_ptr: int, b_ptr: int, m: int, n: int, k: int, c_ptr: int, device: int = 0) -> None:
    """C [m][n] = A [m][k] B [n][k]^T on the tensor cores (device pointers)."""
    _check(load().souffle_gemm_bf16(C.c_void_p(a_ptr), C.c_void_p(b_ptr), m, n, k, C.c_void_p(c_ptr), device))


def surrogate_attach(system: "GpuSystem", net: Mlp, rest_pos: np.ndarray, switch_radius: float = 3.5,
                     far_capacity: int = 0, judge_every: int = 100, judge_stride: int = 100,
                     judge_tolerance: float = 1e-3) -> None:
    """Attach a trained-or-not network to a system (include/souffle_surrogate.h)."""
    rp = np.ascontiguousarray(rest_pos, dtype=np.float64).reshape(-1)
    o = SurrogateOptions_(switch_radius, far_capacity, judge_every, judge_stride, judge_tolerance)
    _check(load().souffle_surrogate_attach(system.h, net.h, _dp(rp), C.byref(o)))
    system._surrogate_net = net


def surrogate_collect(system: "GpuSystem", x_ptr: int, t_ptr: int, capacity: int) -> int:
    n = C.c_int32()
    _check(load().souffle_surrogate_collect(system.h, C.c_void_p(x_ptr), C.c_void_p(t_ptr), capacity, C.byref(n)))
    return int(n.value)


def surrogate_fit(system: "GpuSystem", x_ptr: int, t_ptr: int, n: int, epochs: int, batch: int, lr: float,
                  seed: int = 1) -> float:
    loss = C.c_float()
    _check(load().souffle_surrogate_fit(system.h, C.c_void_p(x_ptr), C.c_void_p(t_ptr), n, epochs, batch, lr, seed,
                                        C.byref(loss)))
    return float(loss.value)


def surrogate_enable(system: "GpuSystem", on: bool) -> None:
    _check(load().souffle_surrogate_enable(system.h, 1 if on else 0))


def surrogate_stats(system: "GpuSystem") -> dict:
    st = SurrogateStats_()
    _check(load().souffle_surrogate_get_stats(system.h, C.byref(st)))
    return {"enabled": bool(st.enabled), "far_pairs": st.far_pairs, "far_found": st.far_found,
            "classes_off": st.classes_off, "judged": int(st.judged), "last_error": list(st.last_error)}
