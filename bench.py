"""Benchmark: MD bead-steps/s of the SOUFFLE force-and-integrate path on one GB300.

Workload (default): 2000 two-layer 42-bead capsomeres (84,000 beads) at 800 uM, reference
options -s 1000 -b 1000 -E 2.1 -e 5 -L 0.3 -B 10 -t 0.005 -q 5 -Q 10 -K 298 -c 94.27, FP32
forces with 64-bit fixed-point accumulation, integer fixed-point integration, double-float
thermostat.  A step is one
iteration of the reference MD loop (src/md.cpp:400-514): thermostat half steps, velocity
Verlet, the pair-list rebuild every 10th step, forces, centre-of-mass velocity removal.

  value  device time of K single steps with inputs resident in HBM; the working set (~30 MB)
         fits in L2, so L2 is flushed (a 256 MB write) before every timed step, outside the
         timed region.
  e2e    the same K steps through the C ABI from host buffers: state uploaded from pinned host
         memory, run in rebuild windows with the thermostat scalars read back after each
         window, final state downloaded.
  cpu_baseline / --impl reference: the oracle port of the reference algorithm (long double,
         OpenMP over subunits, all host cores) on a bounded sample of the same workload.

  surrogate_batched (default run, N = 1): the replica sweep (256 systems of 20-500 capsomeres,
         per-system attraction, screening length 0.5-2 sigma and concentration) with the
         learned far-field surrogate, trained on the GPU from exact far-pair data of the same
         run, against the plain GPU path (each replica alone, exact forces): throughput gain,
         total-force RMS error, temperature and potential-energy statistics.

--surrogate: the learned far-field surrogate (include/souffle_surrogate.h) against the plain
path on one system (--debye-length, --concentration set its parameters); --replicas N: a batch
of N uneven systems in one handle (--replica-subunits S: N systems of S subunits at the plain
workload's parameters; with --surrogate: the surrogate+batched measurement alone);
--gemm: the surrogate network's forward pass at several row counts against the tensor peak;
--drift-steps K: extended-energy drift per 10^4 steps, temperature, potential and radius of
gyration over K steps of the default workload;
--big-beads M: the default workload with M encapsulation big beads (-p true -a 3 -G -78 -H 3.5);
--profile: a few steps without autotuning or timing, for a profiler (plain, --replicas, or
--replicas --surrogate after training);
--analysis: the post-run trajectory analysis (include/souffle_analysis.h), frames/s on frames of
2000 43-bead capsomeres (86,000 beads).

Multi-GPU (torchrun): every rank runs an independent replica of the workload (replicas only;
the path has no exchange step), value = total bead-steps / max rank time.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "capsid-souffle_gb300"))

PROFILE_SUMMARY = os.path.join(REPO, "profiles", "k_forces_plain_large.txt")


def _clock_sampler():
    """Sample SM clocks and throttle reasons with nvidia-smi during the timed region."""
    q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")
    samples, stop = [], threading.Event()

    def run():
        while not stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", "0", f"--query-gpu={q}",
                                      "--format=csv,noheader,nounits"], capture_output=True,
                                     text=True, timeout=5).stdout.strip().splitlines()
                if out:
                    samples.append([x.strip() for x in out[0].split(",")])
            except Exception:
                pass
            stop.wait(0.2)

    th = threading.Thread(target=run, daemon=True)
    return samples, stop, th


def _summarize_clocks(samples):
    if not samples:
        return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
    import statistics
    sm = [float(s[0]) for s in samples if s[0].replace(".", "").isdigit()]
    mx = [float(s[1]) for s in samples if s[1].replace(".", "").isdigit()]
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    reasons = sorted({names[k] for s in samples for k in range(4) if len(s) > 2 + k and
                      s[2 + k].lower().startswith("active")})
    return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
            "reasons": reasons, "samples": len(samples)}


def _profile_traffic():
    """DRAM bytes per k_forces launch from the committed ncu summary, if present."""
    try:
        for line in open(PROFILE_SUMMARY):
            if line.startswith("dram_bytes_per_launch_full_size:"):
                return float(line.split(":")[1].split()[0])
    except OSError:
        pass
    return None


def _profile_instructions():
    """Warp instructions issued per k_forces launch (smsp__inst_executed.sum) from the committed
    ncu summary, if present."""
    try:
        for line in open(PROFILE_SUMMARY):
            if line.startswith("smsp__inst_executed.sum"):
                v, unit = line.split()[1:3]
                return float(v) * {"M": 1e6, "K": 1e3, "G": 1e9}.get(unit, 1.0)
    except (OSError, ValueError, IndexError):
        pass
    return None


def rank_aggregate(total_ms: float, beads_per_rank: int, steps: int, world: int, dist=None):
    """Whole-job figures of a weak-scaling run (every rank an independent replica of the
    workload): the slowest rank's timed region (max over ranks, ms) and the total bead-steps/s
    of all ranks over it."""
    if dist is not None and world > 1:
        import torch
        t = torch.tensor([total_ms], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    return total_ms, world * beads_per_rank * steps / (total_ms / 1e3)


BIG_BEAD = dict(sigma=6.0, charge=-78.0, shc=3.5)  # the reference's defaults -a 3 -G -78 -H 3.5


def cpu_reference(w, seconds: float = 10.0, max_steps: int = 30, threads: int = 0, big_beads=None,
                  steps: int = 0, warmup: int = 1, variant: str = "ld"):
    """Time the oracle port (OpenMP over subunits) on the workload: bead-steps/s.

    With ``steps`` > 0, exactly ``warmup`` untimed steps (the first with a pair-list rebuild)
    then exactly ``steps`` timed steps; otherwise one warm-up step and a bounded sample of
    3..max_steps steps or about ``seconds``.  ``variant`` "ld" is the restatement in the
    reference's long double; "f64" the same algorithm with long double replaced by double (a
    labelled variant, not the reference)."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import platform

    import pyoracle
    threads = threads or os.cpu_count()
    o = pyoracle.Oracle(w.template, int(w.opt.S), w.derived, w.opt.s, w.opt.b, w.opt.E,
                        w.center_local, variant=variant)
    o.set_threads(threads)
    o.set_state(w.state.pos, w.state.vel)
    if big_beads is not None and len(big_beads):
        o.set_big_beads(big_beads, BIG_BEAD["sigma"], BIG_BEAD["charge"], BIG_BEAD["shc"])
    o.forces(True)
    ke = o.kinetic_energy()
    o.nhc_init(int(w.opt.q), w.opt.Q, w.opt.K)
    n_warm = max(1, warmup) if steps > 0 else 1
    for a in range(n_warm):  # the first warm-up step rebuilds the pair list (a % B == 0)
        ke, _, _ = o.md_step(a, w.opt.t, int(w.opt.B), ke)
    t0 = time.perf_counter()
    done = 0
    while (done < steps) if steps > 0 else (done < max_steps and (done < 3 or time.perf_counter() - t0 < seconds)):
        ke, _, _ = o.md_step(n_warm + done, w.opt.t, int(w.opt.B), ke)
        done += 1
    dt = time.perf_counter() - t0
    if variant == "ld":
        arith = ("long double = " + ("x87 80-bit" if platform.machine() in ("x86_64", "AMD64")
                                     else "IEEE binary128 (software)") + f" on {platform.machine()}")
    else:
        arith = f"long double replaced by double (FP64-patched variant, not the reference) on {platform.machine()}"
    return {"value": w.n_beads * done / dt, "unit": "bead-steps/s", "cores": threads,
            "kind": "port", "steps": done, "warmup": n_warm,
            "sample": f"{done} MD steps (rebuild every {int(w.opt.B)}) of the {w.n_beads}-bead "
                      f"workload after {n_warm} warm-up step{'s' if n_warm > 1 else ''}; {arith}"}


def oracle_parity(w, s):
    """Forces and pair lists of the handle ``s`` (state just set, before any step) against the
    oracle in long double on the same state: per-bead force RMS relative errors and whether the
    pair lists are identical in content and order."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import numpy as np

    import pyoracle
    tf, sf, bf = s.forces(rebuild=True, parts=True)
    o = pyoracle.Oracle(w.template, int(w.opt.S), w.derived, w.opt.s, w.opt.b, w.opt.E, w.center_local)
    o.set_threads(os.cpu_count())
    o.set_state(w.state.pos, w.state.vel)
    otf, osf, obf, over = o.forces(True)
    oc, oi = o.pairlist()
    gc, gi = s.pairlist(o.cap)
    wdt = oi.shape[1]
    o_pad = np.where(np.arange(wdt)[None, :] < oc[:, None], oi, -1)
    same = bool(over == 0 and np.array_equal(gc, oc) and np.array_equal(gi[:, :wdt], o_pad))
    tot2 = float((otf ** 2).sum())
    return {"force_rms_rel_error": float(np.sqrt(((tf - otf) ** 2).sum() / tot2)),
            "bending_rms_rel_error": float(np.sqrt(((bf - obf) ** 2).sum() / (obf ** 2).sum())),
            "stretching_rms_error_vs_total": float(np.sqrt(((sf - osf) ** 2).sum() / tot2)),
            "pairlist_identical": same, "pairs": int(oc.sum()),
            "against": "oracle (C restatement in long double, pinned bit for bit to the compiled reference "
                       "on x86-64), same seeded initial state, one rebuild + forces"}


def bench_replicas(args):
    """Batched replicas: one handle, every kernel launch covers all systems."""
    import numpy as np
    import torch
    from souffle_gb300 import gpu, workloads
    t0 = time.perf_counter()
    if args.replica_subunits:
        reps = workloads.uniform_replicas(args.replicas, args.replica_subunits)
    else:
        reps = workloads.replicas(args.replicas, seed=2024)
    gen_s = time.perf_counter() - t0
    params = [gpu.system_params(w.opt, w.derived, int(w.opt.S), w.center_local) for w in reps]
    s = gpu.GpuSystem(reps[0].template, params)
    s.set_state(np.concatenate([w.state.pos for w in reps]), np.concatenate([w.state.vel for w in reps]))
    if args.profile:  # a few plain steps for a profiler, no autotuning
        s.md_begin()
        print(json.dumps(s.md_profile(0, args.steps)))
        return
    tuning = s.autotune(trials=20)
    s.md_begin()
    n = s.n
    B = int(reps[0].opt.B)
    ext = torch.cuda.ExternalStream(s.stream())
    s.md_steps(0, args.warmup)
    a = ((args.warmup + B - 1) // B) * B
    if a > args.warmup:
        s.md_steps(args.warmup, a - args.warmup)
    k = max(B, (args.steps // B) * B)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(ext)
    s.md_enqueue(a, k)
    e1.record(ext)
    s.synchronize()
    ms = e0.elapsed_time(e1)
    a += k
    prof = s.md_profile(a, 20)
    sizes = [int(w.opt.S) for w in reps]
    lens = [s.pairlist_stats(i)["mean_length"] for i in range(0, len(reps), max(1, len(reps) // 16))]
    n_bar = float(np.mean(lens))
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(REPO, "MEASURED_PEAKS.json")))
    except OSError:
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    value = n * k / (ms / 1e3)
    forces_ms = prof["forces_ms"] / prof["steps"]
    kern_gbs = (16 + 4 * n_bar + 24 + 48 + 16) * n / (forces_ms / 1e3) / 1e9
    step_b = 112 + 4 * n_bar + (4 * n_bar + 16) / B
    print(json.dumps({
        "metric": "bead-steps/s", "value": n * k / (ms / 1e3), "unit": "bead-steps/s", "n_gpus": 1,
        "steps": k, "warmup": args.warmup, "ms_per_step": ms / k, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+i64 fixed / f64",
        "data": "synthetic (seeded replicas)",
        "config": {"workload": f"replicas: {len(reps)} systems of bilayer capsomeres, {sum(sizes)} "
                               f"subunits, {n} beads, subunits per system {min(sizes)}-{max(sizes)}",
                   "l2": "working set larger than L2" if n * 300 > 129e6 else "warm L2, whole windows"},
        "pairlist_mean_length_sampled": n_bar, "generation_s": gen_s,
        "kernels_ms": {"k_forces": forces_ms, "k_drift": prof["drift_ms"] / prof["steps"],
                       "rebuild": prof["rebuild_ms"] / max(1, prof["rebuilds"])},
        "roofline": {"bound": "hbm", "kernel": "k_forces", "achieved": kern_gbs, "peak": peak,
                     "unit": "GB/s", "frac": kern_gbs / peak, "traffic": None,
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)" if peaks else "fallback 6800"},
        "roofline_step": {"achieved": step_b * value / 1e9, "peak": peak, "unit": "GB/s",
                          "frac": step_b * value / 1e9 / peak, "bytes_per_bead_step": step_b},
        "autotune": tuning}))


def _flushed_steps(s, ext, flush, a, k):
    """K single MD steps, L2 flushed before each, CUDA events on the handle's stream: total ms."""
    import torch
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(k)]
    torch.cuda.synchronize()
    for i in range(k):
        with torch.cuda.stream(ext):
            flush.zero_()
        evs[i][0].record(ext)
        s.md_enqueue(a + i, 1)
        evs[i][1].record(ext)
    s.synchronize()
    torch.cuda.synchronize()
    return float(sum(e0.elapsed_time(e1) for e0, e1 in evs))


def bench_surrogate(args):
    """Learned far-field surrogate on the 2000-subunit workload: trained on exact far-pair data
    from the plain run, then plain and surrogate throughput from the same state (same timing
    protocol as the main line), force error, the judge's per-class errors, and temperature and
    potential-energy statistics of both runs."""
    import numpy as np
    import torch
    from souffle_gb300 import gpu, workloads
    torch.cuda.set_device(0)
    w = workloads.plain_large(args.subunits, debye_length=args.debye_length, conc_um=args.concentration,
                              nhc_mass=args.nhc_mass)
    p = gpu.system_params(w.opt, w.derived, int(w.opt.S), w.center_local)
    s = gpu.GpuSystem(w.template, [p])
    s.set_state(w.state.pos, w.state.vel)
    np_ = w.template.n_beads
    n_out = 6 + 3 * np_
    far_cap = max(4096, args.far_per_subunit * int(w.opt.S))
    batch = 4096
    net = gpu.Mlp(64, n_out, max_batch=max(far_cap, batch), seed=7, width=getattr(args, "net_width", 128))
    gpu.surrogate_attach(s, net, w.template.pos, far_capacity=far_cap,
                         switch_radius=getattr(args, "switch_radius", 3.0))
    B = int(w.opt.B)
    # training data: exact far-pair forces along the plain trajectory, one frame per rebuild window
    rows = args.train_rows
    X = torch.empty(rows, 64, device="cuda")
    T = torch.empty(rows, n_out, device="cuda")
    xb = torch.empty(far_cap, 64, device="cuda")
    tb = torch.empty(far_cap, n_out, device="cuda")
    s.md_begin()
    t0 = time.perf_counter()
    total, frames, a = 0, 0, 0
    while total < rows and frames < args.max_frames:
        n = gpu.surrogate_collect(s, xb.data_ptr(), tb.data_ptr(), far_cap)
        m = min(n, rows - total)
        X[total:total + m] = xb[:m]
        T[total:total + m] = tb[:m]
        total += m
        frames += 1
        s.md_steps(a, B)
        a += B
    torch.cuda.synchronize()
    gen_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    loss = gpu.surrogate_fit(s, X.data_ptr(), T.data_ptr(), total, args.epochs, batch, 1e-3, seed=11)
    fit_s = time.perf_counter() - t0
    del X, T
    # force accuracy at the end state of the training run
    exact = s.forces(rebuild=True)
    gpu.surrogate_enable(s, True)
    sur = s.forces(rebuild=True)
    far_pairs = gpu.surrogate_stats(s)["far_pairs"]
    rms = float(np.sqrt(((sur - exact) ** 2).sum() / (exact ** 2).sum()))
    pos, vel = s.get_state()
    ext = torch.cuda.ExternalStream(s.stream())
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def run(enabled):
        gpu.surrogate_enable(s, enabled)
        s.set_state(pos, vel)
        s.md_begin()
        s.md_steps(0, args.warmup)
        a0 = ((args.warmup + B - 1) // B) * B
        s.md_steps(args.warmup, a0 - args.warmup)
        ms = _flushed_steps(s, ext, flush, a0, args.steps)
        a1 = ((a0 + args.steps + B - 1) // B) * B
        s.md_steps(a0 + args.steps, a1 - (a0 + args.steps))
        kw = max(B, (args.steps // B) * B)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        s.md_enqueue(a1, kw)
        e1.record(ext)
        s.synchronize()
        warm = w.n_beads * kw / (e0.elapsed_time(e1) / 1e3)
        # statistics over a longer run from the same state
        temps, pots, ext_e = [], [], []
        a2 = a1 + kw
        windows = args.stat_steps // 20
        sample = max(1, windows // 10)  # about ten energy evaluations (all pairs, FP64) per run
        for k in range(windows):
            s.md_steps(a2, 20)
            a2 += 20
            ke, _, _ = s.md_scalars()
            temps.append(2 * ke / (3 * w.n_beads))
            if k % sample == 0:
                e = s.energies()
                pot = e["stretching"] + e["bending"] + e["lj"] + e["electrostatic"]
                pots.append(pot)
                ext_e.append((a2, (pot + e["kinetic"] + e["thermo_pe"] + e["thermo_ke"]) / w.n_beads))
        st = gpu.surrogate_stats(s)
        x = np.array(ext_e)
        drift = float(np.polyfit(x[:, 0], x[:, 1], 1)[0] * 1e4) if len(x) > 1 else None
        return {"value": w.n_beads * args.steps / (ms / 1e3), "ms_per_step": ms / args.steps,
                "warm_l2_value": warm, "T_mean": float(np.mean(temps)), "T_std": float(np.std(temps)),
                "potential_mean": float(np.mean(pots)), "potential_std": float(np.std(pots)),
                "extended_energy_drift_per_bead_per_1e4_steps": drift,
                "judge": {"judged": st["judged"], "classes_off": st["classes_off"],
                          "last_error": st["last_error"]} if enabled else None}

    plain = run(False)
    surr = run(True)
    print(json.dumps({
        "metric": "bead-steps/s on 1 GB300: surrogate vs plain GPU at <=1e-3 force RMS err",
        "value": surr["value"], "unit": "bead-steps/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "bf16 network (fp32 accumulate) + f32/i64 exact path", "data": "synthetic",
        "config": {"workload": f"plain_large: {args.subunits} bilayer capsomeres x 42 beads = {w.n_beads} "
                               f"beads, {w.opt.C:g} uM, Debye length {1 / w.derived.kappa:.3g} sigma (-c {w.opt.c:.4g}), "
                               f"switch radius {getattr(args, 'switch_radius', 3.0):g} sigma (closest bead pair), judge 1 % "
                               f"of far pairs every 100 steps",
                   "l2": "flushed (256 MB write) before every timed step"},
        "plain": plain, "surrogate": surr, "gain": surr["value"] / plain["value"],
        "gain_warm_l2": surr["warm_l2_value"] / plain["warm_l2_value"],
        "force_rms_rel_error": rms, "far_pairs": far_pairs,
        "training": {"rows": total, "frames": frames, "epochs": args.epochs, "batch": batch,
                     "final_loss_normalised": loss, "generation_s": gen_s, "fit_s": fit_s}}))


def bench_surrogate_batched(args):
    print(json.dumps(surrogate_batched(args)))


def _series_stats(temps, pots, ext, t_every, e_every, n_beads):
    """Mean and standard error (8 block means) of temperature and potential energy over the last
    three quarters of a run, and the extended energy's drift per bead per 10^4 steps (linear
    fit over the whole run)."""
    import numpy as np

    def mean_se(x):
        x = np.asarray(x[len(x) // 4:], dtype=np.float64)
        blocks = np.array_split(x, 8)
        bm = np.array([b.mean() for b in blocks if len(b)])
        return float(x.mean()), float(bm.std(ddof=1) / np.sqrt(len(bm))) if len(bm) > 1 else 0.0

    tm, tse = mean_se(temps)
    pm, pse = mean_se(pots)
    steps = e_every * (np.arange(len(ext)) + 1)
    drift = float(np.polyfit(steps, np.asarray(ext) / n_beads, 1)[0] * 1e4) if len(ext) > 1 else None
    return {"T_mean": tm, "T_se": tse, "potential_mean": pm, "potential_se": pse,
            "drift_per_bead_per_1e4_steps": drift, "samples": len(temps)}


def _compare_stats(a, b):
    """Differences between two runs' statistics in units of their combined standard error."""
    import math
    out = {}
    for key in a:
        x, y = a[key], b[key]
        zt = (y["T_mean"] - x["T_mean"]) / max(math.hypot(x["T_se"], y["T_se"]), 1e-30)
        zp = (y["potential_mean"] - x["potential_mean"]) / max(math.hypot(x["potential_se"], y["potential_se"]), 1e-30)
        zd = (y["drift_per_bead_per_1e4_steps"] - x["drift_per_bead_per_1e4_steps"]) / max(
            math.hypot(x.get("drift_se", 0.0), y.get("drift_se", 0.0)), 1e-30)
        out[key] = {"T_z": zt, "potential_z": zp, "drift_z": zd}
    zs = [abs(z) for v in out.values() for z in v.values()]
    out["max_abs_z"] = max(zs)
    out["beyond_2se"] = sum(z > 2 for z in zs)
    out["compared"] = len(zs)
    return out


def surrogate_batched(args):
    """Surrogate + batching against the plain GPU path on the replica sweep: 256 independent
    systems of 20-500 bilayer capsomeres with per-system attraction, screening length (0.5-2
    sigma) and concentration (200-1600 uM).  One network is trained on exact far-pair data from
    the batched run (the descriptor carries the screening length and attraction), then:
      plain     every replica alone in its own handle with exact forces (the plain GPU path, one
                system per run), L2 flushed before each replica's timed window;
      batched   all replicas in one handle, exact forces;
      surrogate all replicas in one handle, far subunit pairs from the network.
    Batched windows run whole rebuild windows as CUDA graphs; their working set is larger than
    L2.  Also reported: total-force RMS error of the surrogate batch against exact forces at the
    same state, and, for the four systems with the longest screening lengths in a handle of their
    own with the same network, temperature, potential energy and extended-energy drift over
    stat_steps steps, exact against surrogate, each from six independent velocity draws, with
    standard errors from the run-to-run spread.  (Systems near the
    short end of the screening range can blow up after ~10^3 steps with the reference's
    pair-list rule at -L 0.3: its centre prefilter misses contacts between 42-bead patches.)"""
    import numpy as np
    import torch
    from souffle_gb300 import gpu, workloads
    torch.cuda.set_device(0)
    t0 = time.perf_counter()
    if getattr(args, "replica_subunits", 0):
        reps = workloads.uniform_replicas(args.replicas, args.replica_subunits)
    else:
        reps = workloads.replicas(args.replicas, seed=2024)
    gen_s = time.perf_counter() - t0
    params = [gpu.system_params(w.opt, w.derived, int(w.opt.S), w.center_local) for w in reps]
    tpl = reps[0].template
    s = gpu.GpuSystem(tpl, params)
    pos0 = np.concatenate([w.state.pos for w in reps])
    vel0 = np.concatenate([w.state.vel for w in reps])
    s.set_state(pos0, vel0)
    n = s.n
    S_tot = sum(int(w.opt.S) for w in reps)
    B = int(reps[0].opt.B)
    np_ = tpl.n_beads
    n_out = 6 + 3 * np_
    far_cap = max(4096, args.far_per_subunit * S_tot)
    batch = 4096
    net = gpu.Mlp(64, n_out, max_batch=max(far_cap, batch), seed=7, width=getattr(args, "net_width", 128))
    gpu.surrogate_attach(s, net, tpl.pos, far_capacity=far_cap,
                         switch_radius=getattr(args, "switch_radius", 3.0))
    ext = torch.cuda.ExternalStream(s.stream())

    rows = args.train_rows
    X = torch.empty(rows, 64, device="cuda")
    T = torch.empty(rows, n_out, device="cuda")
    xb = torch.empty(far_cap, 64, device="cuda")
    tb = torch.empty(far_cap, n_out, device="cuda")
    s.md_begin()
    t0 = time.perf_counter()
    total, frames, a = 0, 0, 0
    while total < rows and frames < args.max_frames:
        m = gpu.surrogate_collect(s, xb.data_ptr(), tb.data_ptr(), far_cap)
        # a sample of each frame's pairs, so that the data set spans more of the trajectory
        keep = min(m, rows - total, max(1, rows // 20))
        idx = torch.randperm(m, device="cuda")[:keep] if m > keep else torch.arange(m, device="cuda")
        X[total:total + keep] = xb[idx]
        T[total:total + keep] = tb[idx]
        total += keep
        frames += 1
        s.md_steps(a, B)
        a += B
    torch.cuda.synchronize()
    collect_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    loss = gpu.surrogate_fit(s, X.data_ptr(), T.data_ptr(), total, args.epochs, batch, 1e-3, seed=11)
    fit_s = time.perf_counter() - t0
    del X, T, xb, tb
    torch.cuda.empty_cache()
    pos, vel = s.get_state()
    exact = s.forces(rebuild=True)
    gpu.surrogate_enable(s, True)
    sur = s.forces(rebuild=True)
    far_pairs = gpu.surrogate_stats(s)["far_pairs"]
    rms = float(np.sqrt(((sur - exact) ** 2).sum() / (exact ** 2).sum()))
    # per system: the worst replica's error
    offs = np.cumsum([0] + [w.n_beads for w in reps])
    per_sys = [float(np.sqrt(((sur[offs[i]:offs[i + 1]] - exact[offs[i]:offs[i + 1]]) ** 2).sum()
                             / (exact[offs[i]:offs[i + 1]] ** 2).sum())) for i in range(len(reps))]
    lam = [1.0 / w.derived.kappa for w in reps]
    watch = [int(i) for i in np.argsort(lam)[-4:]]  # the longest screening lengths
    k = max(B, (args.steps // B) * B)

    def run_batch(enabled):
        gpu.surrogate_enable(s, enabled)
        s.set_state(pos, vel)
        s.md_begin()
        s.md_steps(0, 2 * B)
        a0 = 2 * B
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(ext)
        s.md_enqueue(a0, k)
        e1.record(ext)
        s.synchronize()
        ms = e0.elapsed_time(e1)
        st = gpu.surrogate_stats(s) if enabled else None
        return {"value": n * k / (ms / 1e3), "ms_per_step": ms / k,
                "judge": {"judged": st["judged"], "classes_off": st["classes_off"],
                          "last_error": st["last_error"]} if st else None}

    def run_stats(enabled, seed0, n_seeds=6):
        """The watched systems in a handle of their own with the same trained network, each run
        n_seeds times from the post-training configuration with independent Maxwell-Boltzmann
        velocity draws (seeds seed0 ..; other draws for the exact and the surrogate run):
        stat_steps steps, temperature every 20 steps, potential and extended energy every 40.
        Per run the means over the last three quarters; per watched system their mean over the
        runs with the standard error from the run-to-run spread (the runs are independent
        trajectories, so slow relaxation of the potential is in the spread)."""
        sysl = [i for i in watch for _ in range(n_seeds)]
        sw = gpu.GpuSystem(tpl, [params[i] for i in sysl])
        gpu.surrogate_attach(sw, net, tpl.pos, far_capacity=max(4096, args.far_per_subunit *
                                                                 sum(int(reps[i].opt.S) for i in sysl)),
                             switch_radius=getattr(args, "switch_radius", 3.0))
        gpu.surrogate_enable(sw, enabled)
        rng = np.random.default_rng(seed0)
        vels = []
        for i in sysl:
            m = np.tile(np.asarray(tpl.mass, dtype=np.float64), int(reps[i].opt.S))
            v = rng.normal(size=(reps[i].n_beads, 3)) * np.sqrt(reps[i].derived.T_reduced / m)[:, None]
            vels.append(v - v.mean(axis=0))
        sw.set_state(np.concatenate([pos[offs[i]:offs[i + 1]] for i in sysl]), np.concatenate(vels))
        sw.md_begin()
        temps = [[] for _ in sysl]
        pots = [[] for _ in sysl]
        e_ext = [[] for _ in sysl]
        a1 = 0
        for q in range(args.stat_steps // 20):
            sw.md_steps(a1, 20)
            a1 += 20
            for j, i in enumerate(sysl):
                ke, _, _ = sw.md_scalars(j)
                temps[j].append(2 * ke / (3 * reps[i].n_beads))
                if q % 2 == 1:
                    e = sw.energies(j)
                    pot = e["stretching"] + e["bending"] + e["lj"] + e["electrostatic"]
                    pots[j].append(pot)
                    e_ext[j].append(pot + e["kinetic"] + e["thermo_pe"] + e["thermo_ke"])
        st = gpu.surrogate_stats(sw) if enabled else None
        sw.close()
        runs = [_series_stats(temps[j], pots[j], e_ext[j], 20, 40, reps[i].n_beads) for j, i in enumerate(sysl)]
        out = {}
        for i in watch:
            rs = [r for r, k in zip(runs, sysl) if k == i]
            tm = np.array([r["T_mean"] for r in rs])
            pm = np.array([r["potential_mean"] for r in rs])
            dr = np.array([r["drift_per_bead_per_1e4_steps"] for r in rs])
            out[str(i)] = {"T_mean": float(tm.mean()), "T_se": float(tm.std(ddof=1) / np.sqrt(len(tm))),
                           "potential_mean": float(pm.mean()), "potential_se": float(pm.std(ddof=1) / np.sqrt(len(pm))),
                           "drift_per_bead_per_1e4_steps": float(dr.mean()),
                           "drift_se": float(dr.std(ddof=1) / np.sqrt(len(dr))), "runs": len(rs)}
        return {"statistics": out,
                "judge": {"judged": st["judged"], "classes_off": st["classes_off"],
                          "last_error": st["last_error"]} if st else None}

    if getattr(args, "profile", False):  # surrogate steps only, for a profiler's launch list
        gpu.surrogate_enable(s, True)
        s.set_state(pos, vel)
        s.md_begin()
        s.md_steps(0, args.steps)
        return {"profile_steps": args.steps, "far_pairs": gpu.surrogate_stats(s)["far_pairs"]}
    batched = run_batch(False)
    surr = run_batch(True)
    s.close()
    stats_exact = run_stats(False, 101) if args.stat_steps > 0 else None
    stats_surr = run_stats(True, 202) if args.stat_steps > 0 else None
    net.close()

    # the plain GPU path: each replica alone, exact
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    sample = list(range(0, len(reps), max(1, len(reps) // max(1, args.plain_sample))))
    plain_ms, plain_beads = 0.0, 0
    for i in sample:
        w = reps[i]
        si = gpu.GpuSystem(tpl, [params[i]])
        si.set_state(pos[offs[i]:offs[i + 1]], vel[offs[i]:offs[i + 1]])
        si.md_begin()
        si.md_steps(0, 2 * B)
        exi = torch.cuda.ExternalStream(si.stream())
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        with torch.cuda.stream(exi):
            flush.zero_()
        e0.record(exi)
        si.md_enqueue(2 * B, k)
        e1.record(exi)
        si.synchronize()
        plain_ms += e0.elapsed_time(e1)
        plain_beads += w.n_beads
        si.close()
    plain_value = plain_beads * k / (plain_ms / 1e3)
    sizes = [int(w.opt.S) for w in reps]
    return {
        "metric": "bead-steps/s on 1 GB300: surrogate+batched vs plain GPU at <=1e-3 force RMS err",
        "value": surr["value"], "unit": "bead-steps/s", "n_gpus": 1, "steps": k, "warmup": 2 * B,
        "ms_per_step": surr["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "bf16 network (fp32 accumulate) + f32/i64 exact path",
        "data": "synthetic (seeded replicas)",
        "config": {"workload": f"replicas: {len(reps)} systems of bilayer capsomeres, {S_tot} "
                               f"subunits, {n} beads, subunits per system {min(sizes)}-{max(sizes)}, "
                               + ("eps 2.1, Debye length 1 sigma, 800 uM" if getattr(args, "replica_subunits", 0)
                                  else "eps 1.5-3.0, Debye length 0.5-2.0 sigma, 200-1600 uM")
                               + f"; switch radius {getattr(args, 'switch_radius', 3.0):g} "
                               f"sigma (closest bead pair), judge 1 % of far pairs every 100 steps",
                   "l2": "batched: working set larger than L2, whole rebuild windows; plain: L2 "
                         "flushed before each replica's window"},
        "gain": surr["value"] / plain_value,
        "gain_batching": batched["value"] / plain_value,
        "gain_surrogate": surr["value"] / batched["value"],
        "net_width": getattr(args, "net_width", 128),
        "plain": {"value": plain_value, "replicas_timed": len(sample), "beads_timed": plain_beads,
                  "ms_total": plain_ms},
        "batched": batched, "surrogate": surr,
        "statistics": ({"steps": args.stat_steps, "exact": stats_exact["statistics"],
                        "surrogate": stats_surr["statistics"], "surrogate_judge": stats_surr["judge"],
                        "comparison": _compare_stats(stats_exact["statistics"], stats_surr["statistics"])}
                       if stats_exact else None),
        "force_rms_rel_error": rms, "force_rms_rel_error_worst_system": max(per_sys),
        "far_pairs": far_pairs, "far_capacity": far_cap,
        "watched_systems": {str(i): {"subunits": sizes[i], "debye_length": lam[i],
                                     "eps": float(reps[i].opt.E), "conc_um": float(reps[i].opt.C)}
                            for i in watch},
        "training": {"rows": total, "frames": frames, "epochs": args.epochs, "batch": batch,
                     "final_loss_normalised": loss, "collect_s": collect_s, "fit_s": fit_s},
        "generation_s": gen_s}


def bench_gemm(args):
    """The surrogate network's forward pass (64 -> w -> w -> w -> 132, w = --net-width, BF16
    operands, FP32 accumulation) at several row counts through the C ABI: the fused one-kernel forward
    (souffle_mlp_forward) and the per-layer GEMMs (souffle_mlp_forward_layered).  us_per_call:
    CUDA events on the network's stream around the C call (input packing, the forward, output
    unpadding, host gaps between them); us_per_forward: the forward kernels alone, back to back
    (souffle_mlp_profile_forward), the figure against the measured BF16 tensor peak."""
    import torch
    from souffle_gb300 import gpu
    torch.cuda.set_device(0)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(REPO, "MEASURED_PEAKS.json")))
    except OSError:
        pass
    peak = float(peaks.get("bf16_tflops", 1900.0))
    rows = []
    w = args.net_width
    for m in (8192, 32768, 118016, 524288):
        net = gpu.Mlp(64, 132, max_batch=m, seed=1, width=w)
        ext = torch.cuda.ExternalStream(net.stream())
        x = torch.randn(m, 64, device="cuda")
        y = torch.empty(m, 132, device="cuda")
        flop = 2.0 * m * (64 * w + 2 * w * w + w * 144)
        row = {"rows": m}
        for name, fn in (("fused", net.forward), ("layered", net.forward_layered)):
            for _ in range(3):
                fn(x.data_ptr(), m, y.data_ptr())
            torch.cuda.synchronize()
            evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                   for _ in range(args.steps)]
            for e0, e1 in evs:
                e0.record(ext)
                fn(x.data_ptr(), m, y.data_ptr())
                e1.record(ext)
            torch.cuda.synchronize()
            us = sum(e0.elapsed_time(e1) for e0, e1 in evs) / len(evs) * 1e3
            # the forward kernels alone, back to back on pre-packed input
            kus = net.profile_forward(m, args.steps, fused=(name == "fused"))
            row[name] = {"us_per_call": us, "us_per_forward": kus, "tflops": flop / (kus * 1e-6) / 1e12}
        rows.append(row)
        net.close()
    best = rows[2]["fused"]
    print(json.dumps({
        "metric": "surrogate network forward TFLOP/s", "value": best["tflops"], "unit": "TFLOP/s",
        "n_gpus": 1, "steps": args.steps, "warmup": 3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "bf16 (fp32 accumulate)", "data": "synthetic",
        "config": {"workload": f"surrogate MLP 64-{w}-{w}-{w}-132 forward at 118,016 rows, padded output 144"},
        "per_rows": rows,
        "roofline": {"bound": "tensor", "achieved": best["tflops"], "peak": peak, "unit": "TFLOP/s",
                     "frac": best["tflops"] / peak,
                     "peak_source": "MEASURED_PEAKS.json bf16_tflops (measured)" if peaks else "fallback 1900"}}))


def bench_drift(args):
    """Long-run statistics of the plain path on the default workload: extended energy (particle
    kinetic + potential + thermostat energies) per bead sampled every 500 steps over --drift-steps
    MD steps, its linear drift per bead per 10^4 steps, mean temperature and potential energy,
    and the mean subunit radius of gyration (each subunit unwrapped around its first bead)."""
    import numpy as np
    from souffle_gb300 import gpu, workloads
    w = workloads.plain_large(args.subunits, debye_length=args.debye_length, conc_um=args.concentration,
                              nhc_mass=args.nhc_mass)
    p = gpu.system_params(w.opt, w.derived, int(w.opt.S), w.center_local)
    s = gpu.GpuSystem(w.template, [p], chain_fp64=args.chain_fp64)
    s.set_state(w.state.pos, w.state.vel)
    s.md_begin()
    n, np_, L = w.n_beads, w.template.n_beads, float(w.derived.box)
    every, t_every = 500, 50

    def rg():
        pos, _ = s.get_state()
        q = pos.reshape(-1, np_, 3)
        d = q - q[:, :1, :]
        d -= L * np.round(d / L)
        c = d.mean(axis=1, keepdims=True)
        return float(np.sqrt(((d - c) ** 2).sum(axis=2).mean(axis=1)).mean())

    rows, temps = [], []
    t0 = time.perf_counter()
    for a in range(0, args.drift_steps + 1, every):
        if a:
            for b in range(a - every, a, t_every):  # loop steps b .. b + t_every - 1, whole rebuild windows
                s.md_steps(b, t_every)
                temps.append((b + t_every, 2 * s.md_scalars()[0] / (3 * n)))
        e = s.energies()
        pot = e["stretching"] + e["bending"] + e["lj"] + e["electrostatic"]
        rows.append((a, e["temperature"], pot / n, (pot + e["kinetic"] + e["thermo_pe"] + e["thermo_ke"]) / n, rg()))
    wall = time.perf_counter() - t0
    r = np.array(rows)
    half = len(r) // 2
    slope = float(np.polyfit(r[:, 0], r[:, 3], 1)[0] * 1e4)
    tt = np.array([t for step, t in temps if step > args.drift_steps // 2])
    tb = np.array([b.mean() for b in np.array_split(tt, 8)]) if len(tt) >= 8 else tt
    print(json.dumps({
        "metric": "extended-energy drift per bead per 1e4 steps", "value": slope, "unit": "kT per bead",
        "n_gpus": 1, "steps": args.drift_steps, "higher_is_better": False, "dtype": "f32+i64 fixed / f64",
        "data": "synthetic", "config": {"workload": f"plain_large: {args.subunits} bilayer capsomeres x 42 "
                                                    f"beads = {n} beads, {w.opt.C:g} uM, -e 5 -L 0.3 -B 10 "
                                                    f"-t 0.005 -q 5 -Q {w.opt.Q:g}", "sample_every": every},
        "chain": "fp64 (validation variant)" if args.chain_fp64 else "double-float",
        "T_mean_second_half": float(tt.mean()) if len(tt) else None,
        "T_std_second_half": float(tt.std()) if len(tt) else None,
        "T_se_second_half": float(tb.std(ddof=1) / np.sqrt(len(tb))) if len(tb) > 1 else None,
        "potential_per_bead_mean_second_half": float(r[half:, 2].mean()),
        "rg_mean_second_half": float(r[half:, 4].mean()),
        "extended_energy_per_bead_first_last": [float(r[0, 3]), float(r[-1, 3])],
        "wall_s": wall}))


def cpu_analysis_port(n_sub: int, seconds: float = 10.0):
    """Time the C restatement of the reference's analysis loops (oracle/analysis_port.c, long
    double, one thread, as the reference's analyze_output) on frames of the same generator at two
    smaller sizes, and extrapolate to n_sub subunits with the fitted a*S^2 + b*S cost."""
    import numpy as np
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import analysis_oracle as ao
    from souffle_gb300 import workloads
    sizes, times = [], []
    S = 50
    while True:
        ty, fr, L, np_ = workloads.analysis_frames(S, 1)
        t0 = time.perf_counter()
        ao.port_frame(ty, fr[0], L, np_)
        dt = time.perf_counter() - t0
        sizes.append(S)
        times.append(dt)
        if sum(times) > seconds / 3 or S * 2 > n_sub:
            break
        S *= 2
    A = np.array([[s * s, s] for s in sizes], dtype=float)
    coef = np.linalg.lstsq(A, np.array(times), rcond=None)[0]
    t_full = float(coef[0] * n_sub * n_sub + coef[1] * n_sub)
    if n_sub in sizes:
        t_full = times[sizes.index(n_sub)]
    import platform
    return {"value": 1.0 / t_full, "unit": "frames/s", "cores": 1, "kind": "port",
            "sample": f"one frame each at {sizes} subunits ({[round(t, 3) for t in times]} s); "
                      f"full size {n_sub} extrapolated by a*S^2+b*S; long double = "
                      f"{'x87 80-bit' if platform.machine() in ('x86_64', 'AMD64') else 'IEEE binary128 (software)'}"
                      f" on {platform.machine()}"}


def bench_analysis(args):
    """Post-run analysis: frames/s of souffle_analysis on 86,000-bead frames."""
    import numpy as np
    from souffle_gb300 import workloads
    S = args.subunits
    types, frames, box, np_ = workloads.analysis_frames(S, 4)
    N = S * np_
    config = {"workload": f"analysis_large: {S} capsomeres x {np_} beads = {N} beads per frame, "
                          f"800 uM (box {box:.4g}), 60% in chains of 2-8, pcf type 5 (4 per subunit), "
                          f"sub-oligomer type 0 (6 per subunit), 100 bins, contact 2",
              "image": "reference rule (as analyze_output computes dist())",
              "l2": "flushed (256 MB write) before every timed frame",
              "parallelism": "replicas x1"}
    if args.impl == "reference":
        if int(os.environ.get("RANK", "0")) != 0:
            return
        cb = cpu_analysis_port(S, args.cpu_seconds)
        print(json.dumps({
            "impl": "reference", "metric": "frames/s", "value": cb["value"], "unit": "frames/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 / cb["value"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "long double",
            "data": "synthetic (seeded capsomere frames)", "config": config, "cpu_baseline": cb,
            "e2e": {"value": cb["value"], "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))
        return
    import torch
    from souffle_gb300.analysis import Analysis, IMAGE_MINIMUM, IMAGE_REFERENCE
    torch.cuda.set_device(0)
    dev = torch.device("cuda:0")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    pos_d = torch.tensor(frames, dtype=torch.float64, device=dev)
    typ_d = torch.tensor(types, dtype=torch.int32, device=dev)
    out = {}
    for image, key in ((IMAGE_REFERENCE, "reference"), (IMAGE_MINIMUM, "minimum")):
        a = Analysis(N, np_, box, image=image)
        gr = torch.zeros(100, dtype=torch.int64, device=dev)
        ol = torch.zeros(S, dtype=torch.int64, device=dev)
        so = torch.zeros(2 * S, dtype=torch.int64, device=dev)
        ext = torch.cuda.ExternalStream(a.stream())
        for k in range(max(3, args.warmup)):
            a.enqueue(pos_d[k % 4].data_ptr(), typ_d.data_ptr(), gr.data_ptr(), ol.data_ptr(), so.data_ptr())
        a.synchronize()
        torch.cuda.synchronize()
        samples, stop, th = _clock_sampler()
        th.start()
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(args.steps)]
        for k in range(args.steps):
            with torch.cuda.stream(ext):
                flush.zero_()
            evs[k][0].record(ext)
            a.enqueue(pos_d[k % 4].data_ptr(), typ_d.data_ptr(), gr.data_ptr(), ol.data_ptr(), so.data_ptr())
            evs[k][1].record(ext)
        a.synchronize()
        torch.cuda.synchronize()
        stop.set()
        th.join()
        ms = [e0.elapsed_time(e1) for e0, e1 in evs]
        cand, fp64 = a.last_counts()
        olig = ol.cpu().numpy()
        # e2e: frames from host memory through souffle_analysis_frames (H2D of positions and
        # types, results back to the host every frame)
        host = np.ascontiguousarray(np.stack([frames[k % 4] for k in range(args.steps)]))
        host_t = np.ascontiguousarray(np.broadcast_to(types, (args.steps, N)))
        t0 = time.perf_counter()
        a.frames(host, host_t)
        e2e_s = time.perf_counter() - t0
        out[key] = {"ms": float(np.mean(ms)), "value": args.steps / (sum(ms) / 1e3), "e2e": args.steps / e2e_s,
                    "candidate_pairs": cand, "fp64_pairs": fp64, "clocks": _summarize_clocks(samples),
                    "oligomers_gt1": int(olig[1:].sum()), "launches_per_frame": 6}
        a.close()
    r = out["reference"]
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(REPO, "MEASURED_PEAKS.json")))
    except OSError:
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    frame_bytes = (24 + 4) * N  # positions and types read once: the data a frame must move
    n5 = 4 * S
    res = {
        "metric": "frames/s", "value": r["value"], "unit": "frames/s", "n_gpus": 1, "steps": args.steps,
        "warmup": max(3, args.warmup), "ms_per_step": r["ms"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 with f64 tie-breaks", "data": "synthetic (seeded capsomere frames)",
        "config": config,
        "e2e": {"value": r["e2e"], "unit": "frames/s", "h2d_bytes_per_step": frame_bytes,
                "d2h_bytes_per_step": 8 * (100 + 3 * S) + 4 * S,
                "note": "souffle_analysis_frames from host arrays: upload, 6 kernels, results back, per frame"},
        "gpu_launches": 6 * args.steps,
        "minimum_image": out["minimum"],
        "work_per_frame": {"pcf_pairs": n5 * (n5 - 1) // 2, "candidate_subunit_pairs": r["candidate_pairs"],
                           "bead_pair_tests_contacts": r["candidate_pairs"] * np_ * np_,
                           "fp64_decisions": r["fp64_pairs"]},
        "roofline": {"bound": "hbm", "kernel": "whole frame (6 kernels)", "achieved": frame_bytes / (r["ms"] / 1e3) / 1e9,
                     "peak": peak, "unit": "GB/s", "frac": frame_bytes / (r["ms"] / 1e3) / 1e9 / peak,
                     "traffic": None,
                     "note": "the frame's data is 2.4 MB; the work is FP32 pair tests, so the HBM "
                             "fraction is small by construction"},
        "clocks": r["clocks"],
    }
    if not args.no_cpu_baseline:
        res["cpu_baseline"] = cpu_analysis_port(S, args.cpu_seconds)
    print(json.dumps(res))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--subunits", type=int, default=2000)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-parity", action="store_true",
                    help="skip the forces / pair-list check against the oracle on the initial state")
    ap.add_argument("--profile", action="store_true",
                    help="md_begin, then --steps MD steps as direct launches (no graphs); for ncu")
    ap.add_argument("--replicas", type=int, default=0,
                    help="run a batch of this many independent replicas (20-500 subunits each, "
                         "per-replica epsilon, Debye length and concentration) instead")
    ap.add_argument("--replica-subunits", type=int, default=0,
                    help="with --replicas: every replica this many subunits at the plain workload's "
                         "parameters (default: sizes and parameters drawn per replica)")
    ap.add_argument("--surrogate", action="store_true",
                    help="learned far-field surrogate vs the plain path on the same workload")
    ap.add_argument("--analysis", action="store_true",
                    help="post-run trajectory analysis (pcf, oligomers, sub-oligomers), frames/s")
    ap.add_argument("--train-rows", type=int, default=2_000_000)
    ap.add_argument("--max-frames", type=int, default=6000)
    ap.add_argument("--epochs", type=int, default=20)
    ap.add_argument("--stat-steps", type=int, default=2000)
    ap.add_argument("--debye-length", type=float, default=0.0,
                    help="screening length in sigma (default 1: -c 94.27)")
    ap.add_argument("--concentration", type=float, default=0.0, help="subunits in uM (default 800)")
    ap.add_argument("--big-beads", type=int, default=0,
                    help="encapsulation: this many big beads (-a 3 -G -78 -H 3.5) in the workload")
    ap.add_argument("--nhc-mass", type=float, default=0.0, help="-Q for --drift-steps (default 10)")
    ap.add_argument("--chain-fp64", action="store_true",
                    help="--drift-steps with the thermostat chain in FP64 (validation variant)")
    ap.add_argument("--drift-steps", type=int, default=0,
                    help="long-run statistics: extended-energy drift, T, potential, Rg over this many steps")
    ap.add_argument("--gemm", action="store_true",
                    help="the surrogate network's forward pass (tcgen05 GEMMs) at several row counts")
    ap.add_argument("--no-surrogate-batched", action="store_true",
                    help="skip the replica-sweep surrogate+batched measurement in the default run")
    ap.add_argument("--plain-sample", type=int, default=256,
                    help="with --replicas --surrogate: replicas timed alone for the plain path")
    ap.add_argument("--far-per-subunit", type=int, default=4,
                    help="surrogate far-pair list capacity per subunit")
    ap.add_argument("--switch-radius", type=float, default=3.0,
                    help="surrogate: closest bead-pair distance from which a subunit pair is far (3.0: the "
                         "2.5 sigma LJ cut-off plus 0.5 sigma for the motion between pair-list rebuilds, more "
                         "than the reference's own 0.3 sigma list skin; the library default is 3.5)")
    ap.add_argument("--net-width", type=int, default=128, choices=(128, 256),
                    help="hidden width of the surrogate network (128: 65 us per 118k-row forward at a "
                         "force error of ~1.2e-5; 256: 100 us at ~1.1e-5)")
    args = ap.parse_args()
    if args.gemm:
        return bench_gemm(args)
    if args.drift_steps:
        return bench_drift(args)
    if args.replicas and args.surrogate:
        return bench_surrogate_batched(args)
    if args.replicas:
        return bench_replicas(args)
    if args.surrogate:
        return bench_surrogate(args)
    if args.analysis:
        return bench_analysis(args)

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    from souffle_gb300 import workloads
    w = workloads.plain_large(args.subunits, seed=12345 + rank, debye_length=args.debye_length,
                              conc_um=args.concentration)
    big = workloads.place_big_beads(w, args.big_beads) if args.big_beads else None
    config = {"workload": f"plain_large: {args.subunits} bilayer capsomeres x 42 beads = "
                          f"{w.n_beads} beads, {w.opt.C:g} uM, -c {w.opt.c:.4g} (Debye length "
                          f"{1 / w.derived.kappa:.3g} sigma) -e 5 -L 0.3 -B 10 -t 0.005 -q 5" + (
                              f", encapsulation -p true -m {args.big_beads} -a 3 -G -78 -H 3.5"
                              if args.big_beads else ""),
              "l2": "flushed (256 MB write) before every timed step" + (
                  "; working set < L2" if w.n_beads * 400 < 129e6 else "; working set > L2"),
              "parallelism": f"replicas x{world}"}

    if args.impl == "reference":
        if rank != 0:
            return
        # exactly --warmup untimed then --steps timed MD steps of the oracle port
        cb = cpu_reference(w, big_beads=big, steps=args.steps, warmup=args.warmup)
        steps_ms = w.n_beads / cb["value"] * 1e3
        line = {
            "impl": "reference", "metric": "bead-steps/s", "value": cb["value"],
            "unit": "bead-steps/s", "n_gpus": args.gpus, "steps": cb["steps"],
            "warmup": cb["warmup"], "ms_per_step": steps_ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "long double (f80/f128)",
            "data": "synthetic (seeded random capsomere states)", "config": config,
            "cpu_baseline": cb,
            "e2e": {"value": cb["value"], "unit": "bead-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
        if not args.no_cpu_baseline:
            # context only: the same algorithm with long double replaced by double
            line["cpu_baseline_fp64_patched"] = cpu_reference(w, big_beads=big, variant="f64",
                                                              seconds=args.cpu_seconds)
        print(json.dumps(line))
        return

    import numpy as np
    import torch
    from souffle_gb300 import gpu

    torch.cuda.set_device(0)
    dist = None
    if world > 1:
        import torch.distributed as dist_
        dist_.init_process_group("gloo")
        dist = dist_

    p = gpu.system_params(w.opt, w.derived, int(w.opt.S), w.center_local)
    s = gpu.GpuSystem(w.template, [p])
    s.set_state(w.state.pos, w.state.vel)
    if big is not None:
        s.set_big_beads(big, BIG_BEAD["sigma"], BIG_BEAD["charge"], BIG_BEAD["shc"])
    parity = None
    if rank == 0 and not args.profile and not args.no_parity and big is None:
        parity = oracle_parity(w, s)
    tuning = s.autotune(trials=20) if not args.profile else None
    s.md_begin()
    if args.profile:
        print(json.dumps(s.md_profile(0, args.steps)))
        return
    stats = s.pairlist_stats()
    n_bar = stats["mean_length"]
    ext = torch.cuda.ExternalStream(s.stream())
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    B = int(w.opt.B)

    a = 0
    s.md_steps(a, args.warmup)
    a += args.warmup

    # timed region: K single steps, L2 flushed before each, CUDA events on the handle's stream
    samples, stop, th = _clock_sampler()
    th.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(args.steps)]
    launches = 0
    for k in range(args.steps):
        with torch.cuda.stream(ext):
            flush.zero_()
        evs[k][0].record(ext)
        s.md_enqueue(a, 1)  # queued without a host round trip; errors checked after the loop
        evs[k][1].record(ext)
        launches += 2 + (5 if a % B == 0 else 0)
        a += 1
    s.synchronize()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    stop.set()
    th.join()
    step_ms = [e0.elapsed_time(e1) for e0, e1 in evs]
    total_ms = float(sum(step_ms))
    total_ms, value = rank_aggregate(total_ms, w.n_beads, args.steps, world, dist)

    # warm-L2 throughput: the same K steps as whole graph windows, no flush
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a0 = ((a + B - 1) // B) * B
    if a0 > a:
        s.md_steps(a, a0 - a)
    a = a0
    kw = max(B, (args.steps // B) * B)
    start.record(ext)
    s.md_enqueue(a, kw)
    end.record(ext)
    s.synchronize()
    a += kw
    warm_value = w.n_beads * kw / (start.elapsed_time(end) / 1e3)

    # per-kernel times (events between launches, direct launches)
    prof = s.md_profile(a, 20)
    a += 20
    forces_ms = prof["forces_ms"] / prof["steps"]
    drift_ms = prof["drift_ms"] / prof["steps"]
    rebuild_ms = prof["rebuild_ms"] / max(1, prof["rebuilds"])

    # e2e through the C ABI with host buffers
    pos_h = torch.from_numpy(np.ascontiguousarray(w.state.pos)).pin_memory()
    vel_h = torch.from_numpy(np.ascontiguousarray(w.state.vel)).pin_memory()
    pos_o = torch.empty_like(pos_h).pin_memory()
    vel_o = torch.empty_like(vel_h).pin_memory()
    import ctypes as C
    lib = gpu.load()
    dp = C.POINTER(C.c_double)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    gpu._check(lib.souffle_gpu_set_state(s.h, C.cast(pos_h.data_ptr(), dp), C.cast(vel_h.data_ptr(), dp)))
    s.md_begin()
    e2e_steps = max(B, (args.steps // B) * B)
    reads = 0
    for k in range(0, e2e_steps, B):
        s.md_steps(k, B)
        s.md_scalars()
        reads += 1
    gpu._check(lib.souffle_gpu_get_state(s.h, C.cast(pos_o.data_ptr(), dp), C.cast(vel_o.data_ptr(), dp)))
    e2e_s = time.perf_counter() - t0
    e2e = {"value": w.n_beads * e2e_steps / e2e_s, "unit": "bead-steps/s",
           "h2d_bytes_per_step": 48 * w.n_beads / e2e_steps,
           "d2h_bytes_per_step": (48 * w.n_beads + 24 * reads) / e2e_steps,
           "note": "set_state from pinned host + md_begin + steps in rebuild windows with the "
                   "thermostat scalars read after each window + get_state, wall clock"}

    # one energy block (souffle_gpu_energies: every pair j > i in FP64, as the reference's
    # update_LJ_ES_energies_simplified), wall clock around synchronous calls
    s.energies()
    t0 = time.perf_counter()
    for _ in range(3):
        s.energies()
    energies_ms = (time.perf_counter() - t0) / 3 * 1e3

    # roofline of the dominant kernel (k_forces): its share of the algorithmic bytes per bead
    # step: pos32 tile 16 B + neighbour-index stream 4 n_bar + force write 24 B + velocity
    # read/write 48 B + per-bead constants 16 B
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(REPO, "MEASURED_PEAKS.json")))
    except OSError:
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    kern_bytes = (16 + 4 * n_bar + 24 + 48 + 16) * w.n_beads
    achieved = kern_bytes / (forces_ms / 1e3) / 1e9
    step_bytes = (112 + 4 * n_bar + (4 * n_bar + 16) / B) * w.n_beads
    # the committed ncu figure is for the default workload only
    default_workload = args.subunits == 2000 and not args.debye_length and not args.concentration
    traffic = _profile_traffic() if default_workload else None
    inst = _profile_instructions() if default_workload else None
    clk = _summarize_clocks(samples)
    sm_ghz = (clk["sm_mhz"] or 2070.0) / 1e3
    out = {
        "metric": "bead-steps/s", "value": value, "unit": "bead-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+i64 fixed / f64",
        "data": "synthetic (seeded random capsomere states, random orientations, Maxwell-Boltzmann velocities)",
        "config": config,
        "e2e": e2e,
        "gpu_launches": launches,
        "autotune": tuning,
        "warm_l2_value": warm_value,
        "kernels_ms": {"k_forces": forces_ms, "k_drift": drift_ms, "rebuild": rebuild_ms},
        "pairlist": {"mean_length": n_bar, "max_length": stats["max_length"],
                     "max_inter": stats["max_inter"]},
        "roofline": {"bound": "hbm", "kernel": "k_forces", "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)" if peaks else "fallback 6800"},
        # the compute side of the same kernel: ~40 FP32 operations per pair of the reference list
        # (n_bar pairs per bead, the survey's estimate) against the nominal FP32 rate
        "roofline_fp32": {"achieved": 40.0 * n_bar * w.n_beads / (forces_ms / 1e3) / 1e12,
                          "peak": 152 * 128 * 2 * 2.07e9 / 1e12, "unit": "TFLOP/s",
                          "frac": 40.0 * n_bar * w.n_beads / (forces_ms / 1e3) / (152 * 128 * 2 * 2.07e9),
                          "peak_source": "nominal: 152 SMs x 128 FP32 lanes x 2 FLOP x 2.07 GHz"},
        # the bound the kernel actually meets at this size: instruction issue (the working set
        # stays in L2, so HBM is not the limit); instructions per launch from the ncu summary
        "roofline_issue": ({"achieved": inst / (forces_ms / 1e3) / 1e9, "peak": 152 * 4 * sm_ghz,
                            "unit": "G warp instructions/s", "frac": inst / (forces_ms / 1e3) / 1e9 / (152 * 4 * sm_ghz),
                            "instructions_per_launch": inst,
                            "source": "ncu smsp__inst_executed.sum (profiles/k_forces_plain_large.txt); peak 152 SMs x "
                                      "4 schedulers x 1 instruction per cycle at the sampled SM clock"}
                           if inst else None),
        "energies_ms": energies_ms,
        "roofline_step": {"achieved": step_bytes * value / w.n_beads / 1e9, "peak": peak,
                          "unit": "GB/s", "frac": step_bytes * value / w.n_beads / 1e9 / peak,
                          "bytes_per_bead_step": step_bytes / w.n_beads},
        "clocks": clk,
    }
    if parity is not None:
        out["force_rms_rel_error"] = parity["force_rms_rel_error"]
        out["pairlist_identical"] = parity["pairlist_identical"]
        out["parity"] = parity
    if rank == 0 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_reference(w, seconds=args.cpu_seconds, big_beads=big)
        out["cpu_baseline_fp64_patched"] = cpu_reference(w, seconds=args.cpu_seconds, big_beads=big,
                                                         variant="f64")
    if rank == 0 and world == 1 and not args.no_surrogate_batched and not args.big_beads:
        # the replica sweep with the learned surrogate against the plain single-system path
        s.close()
        try:
            sb = surrogate_batched(argparse.Namespace(
                replicas=256, far_per_subunit=16, steps=100, stat_steps=3000, plain_sample=64, profile=False,
                train_rows=args.train_rows, max_frames=args.max_frames, epochs=args.epochs,
                net_width=args.net_width, switch_radius=args.switch_radius))
            out["surrogate_batched"] = {k: sb[k] for k in (
                "metric", "value", "unit", "gain", "gain_batching", "gain_surrogate", "config",
                "force_rms_rel_error", "force_rms_rel_error_worst_system", "far_pairs")}
            out["surrogate_batched"]["plain_value"] = sb["plain"]["value"]
            out["surrogate_batched"]["batched_value"] = sb["batched"]["value"]
            out["surrogate_batched"]["judge"] = sb["surrogate"]["judge"]
            out["surrogate_batched"]["net_width"] = args.net_width
            out["surrogate_batched"]["statistics"] = sb["statistics"]
        except Exception as ex:  # the main line stands on its own
            out["surrogate_batched"] = {"error": f"{type(ex).__name__}: {ex}"}
    if rank == 0:
        print(json.dumps(out))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
