"""Generate the golden fixtures in this folder from the reference itself.

Runs the reference SOUFFLE sources, compiled unmodified by oracle/ref.mk into
oracle/_ref/ (ref_dump: one forceCalculation with a pair-list rebuild plus the
energy block; ref_run: run_simulation), on seeded synthetic states, and stores
inputs and outputs as .npz.  Needs the reference tree (default /root/reference,
or REF=...) only when regenerating; the tests read the committed fixtures.

    python tests/golden/make_golden.py [--bigbead-only]
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "capsid-souffle_gb300"))
sys.path.insert(0, HERE)

from souffle_gb300 import geometry, state, workloads  # noqa: E402
import refdump  # noqa: E402

CASES = [
    # name, template, subunits, concentration (uM), seed, min gap between subunit spheres
    ("plain_small", "patch_n3", 20, 800.0, 12345, 1.0),
    ("bilayer_dense", "bilayer_n5", 30, 6000.0, 777, -1.5),
    ("patch_crowded", "patch_n3", 60, 20000.0, 4242, -1.0),
]
MD_STEPS = 20
BD_DAMP = 100.0   # -d, the reference's default


def cli(name, S, C):
    o = workloads.base_options()
    return ["-f", name, "-S", str(S), "-C", repr(C), "-c", repr(o.c), "-s", repr(o.s), "-b",
            repr(o.b), "-E", repr(o.E), "-e", repr(o.e), "-L", repr(o.L)]


def main():
    ref = os.environ.get("REF", "/root/reference")
    subprocess.run(["make", "-f", os.path.join(REPO, "oracle", "ref.mk"), f"REF={ref}", "-j8"],
                   check=True, stdout=subprocess.DEVNULL)
    for name, tname, S, C, seed, gap in CASES:
        t = geometry.template_by_name(tname)
        L = state.box_length(S, C)
        st = state.random_state(t, S, L, seed=seed, min_gap=gap)
        with tempfile.TemporaryDirectory() as wd:
            os.makedirs(f"{wd}/infiles")
            os.makedirs(f"{wd}/outfiles")
            geometry.write_infile(t, f"{wd}/infiles/{tname}")
            state.write_restart(st, f"{wd}/outfiles")
            # read back exactly what the reference reads
            t2, _, _, _ = geometry.read_infile(f"{wd}/infiles/{tname}")
            _, vel, pos = state.read_restart(f"{wd}/outfiles/restart_0.out")
            d = refdump.run_dump(wd, cli(tname, S, C))
            n = S * t.n_beads
            cap = int(d["params"]["nlist_capacity"])
            counts = np.array([len(x) for x in d["nlist"]], dtype=np.int32)
            ids = np.full((n, max(1, counts.max())), -1, dtype=np.int32)
            for i, lst in enumerate(d["nlist"]):
                ids[i, :len(lst)] = lst
            # MD: run_simulation for MD_STEPS steps from the same state
            md = f"{wd}/md"
            os.makedirs(f"{md}/outfiles")
            shutil.copytree(f"{wd}/infiles", f"{md}/infiles")
            for f in ("restart_0.out", "rb_0.out"):
                shutil.copy(f"{wd}/outfiles/{f}", f"{md}/outfiles/{f}")
            o = workloads.base_options()
            args = cli(tname, S, C) + ["-D", "m", "-B", str(o.B), "-t", repr(o.t), "-q", str(int(o.q)),
                                       "-Q", repr(o.Q), "-K", repr(o.K), "-T", str(MD_STEPS),
                                       "-W", "1", "-M", "1000000", "-w", str(MD_STEPS)]
            subprocess.run([refdump.REF_RUN] + args, cwd=md, check=True, capture_output=True)
            _, vmd, pmd = state.read_restart(f"{md}/outfiles/restart_{MD_STEPS}.out")
            rows = np.loadtxt(f"{md}/outfiles/energy.out", skiprows=1, usecols=range(11))
            energy_text = open(f"{md}/outfiles/energy.out").read()
            restart_text = open(f"{md}/outfiles/restart_{MD_STEPS}.out").read()
            # Brownian dynamics (-D b): the same state and steps
            bd = f"{wd}/bd"
            os.makedirs(f"{bd}/outfiles")
            shutil.copytree(f"{wd}/infiles", f"{bd}/infiles")
            for f in ("restart_0.out", "rb_0.out"):
                shutil.copy(f"{wd}/outfiles/{f}", f"{bd}/outfiles/{f}")
            bd_args = cli(tname, S, C) + ["-D", "b", "-d", repr(BD_DAMP), "-B", str(o.B), "-t", repr(o.t),
                                          "-K", repr(o.K), "-T", str(MD_STEPS), "-W", "1", "-M", "1000000",
                                          "-w", str(MD_STEPS)]
            subprocess.run([refdump.REF_RUN] + bd_args, cwd=bd, check=True, capture_output=True)
            _, vbd, pbd = state.read_restart(f"{bd}/outfiles/restart_{MD_STEPS}.out")
            bd_rows = np.loadtxt(f"{bd}/outfiles/energy.out", skiprows=1, usecols=range(11))
            np.savez_compressed(
                os.path.join(HERE, f"{name}.npz"),
                template=np.array(tname), n_sub=S, conc=C, seed=seed, gap=gap,
                pos=pos, vel=vel, box=d["params"]["box"], center=int(d["params"]["center_bead"]),
                kappa=d["params"]["kappa"], ecut_el=d["params"]["ecut_el"],
                nlist_cutoff=d["params"]["nlist_cutoff"], nlist_capacity=cap,
                ld_mant_dig=int(d["params"]["long_double_mant_dig"]),
                tforce=d["tforce"], sforce=d["sforce"], bforce=d["bforce"],
                nl_counts=counts, nl_ids=ids,
                se=d["se"], ke=d["ke"], be=d["be"], ne=d["ne"], ce=d["ce"], ke_total=d["ke_total"],
                md_steps=MD_STEPS, md_pos=pmd, md_vel=vmd, md_energy_rows=rows,
                md_energy_text=np.array(energy_text), md_restart_text=np.array(restart_text),
                md_args=np.array(args),
                bd_pos=pbd, bd_vel=vbd, bd_energy_rows=bd_rows, bd_args=np.array(bd_args), bd_damp=BD_DAMP,
            )
            print(name, n, "beads; mean list", counts.mean(), "max", counts.max(), "cap", cap)


# Encapsulation (-p): the plain_small state with three big beads (-a 3: diameter 6, -G -78,
# -H 3.5) set 4 sigma from the centroids of subunits 0, 5 and 10, so that subunit beads sit
# inside the shifted WCA range and the DH cut-off of a big bead.
BIG = dict(S=20, C=800.0, seed=12345, gap=1.0, subs=(0, 5, 10), dist=4.0, a=3.0, G=-78.0, H=3.5)


def bigbead_args():
    return ["-p", "1", "-m", str(len(BIG["subs"])), "-a", repr(BIG["a"]), "-G", repr(BIG["G"]), "-H", repr(BIG["H"])]


def run_args_p():
    return ["-p", "true", "-m", str(len(BIG["subs"])), "-a", repr(BIG["a"]), "-G", repr(BIG["G"]), "-H", repr(BIG["H"])]


def make_bigbead():
    t = geometry.template_by_name("patch_n3")
    S, C = BIG["S"], BIG["C"]
    L = state.box_length(S, C)
    st = state.random_state(t, S, L, seed=BIG["seed"], min_gap=BIG["gap"])
    rng = np.random.default_rng(99)
    big = []
    for k in BIG["subs"]:
        c = st.pos[k * t.n_beads:(k + 1) * t.n_beads].mean(axis=0)
        d = rng.normal(size=3)
        p = c + BIG["dist"] * d / np.linalg.norm(d)
        big.append((p + L / 2) % L - L / 2)
    big = np.array(big)
    with tempfile.TemporaryDirectory() as wd:
        os.makedirs(f"{wd}/infiles")
        os.makedirs(f"{wd}/outfiles")
        geometry.write_infile(t, f"{wd}/infiles/patch_n3")
        state.write_restart(st, f"{wd}/outfiles", big_bead_pos=big)
        _, vel, pos = state.read_restart(f"{wd}/outfiles/restart_0.out")
        d = refdump.run_dump(wd, cli("patch_n3", S, C) + bigbead_args())
        o = workloads.base_options()
        runs = {}
        for mode, extra in (("md", ["-D", "m", "-q", str(int(o.q)), "-Q", repr(o.Q)]),
                            ("bd", ["-D", "b", "-d", repr(BD_DAMP)])):
            rd = f"{wd}/{mode}"
            os.makedirs(f"{rd}/outfiles")
            shutil.copytree(f"{wd}/infiles", f"{rd}/infiles")
            for f in ("restart_0.out", "rb_0.out"):
                shutil.copy(f"{wd}/outfiles/{f}", f"{rd}/outfiles/{f}")
            args = cli("patch_n3", S, C) + extra + ["-B", str(o.B), "-t", repr(o.t), "-K", repr(o.K),
                                                  "-T", str(MD_STEPS), "-W", "1", "-M", "1000000",
                                                  "-w", str(MD_STEPS)] + run_args_p()
            subprocess.run([refdump.REF_RUN] + args, cwd=rd, check=True, capture_output=True)
            _, v, p = state.read_restart(f"{rd}/outfiles/restart_{MD_STEPS}.out")
            runs[mode] = dict(pos=p, vel=v, args=np.array(args),
                              energy_rows=np.loadtxt(f"{rd}/outfiles/energy.out", skiprows=1, usecols=range(11)),
                              cap_text=np.array(open(f"{rd}/outfiles/capenergy.out").read()),
                              energy_text=np.array(open(f"{rd}/outfiles/energy.out").read()))
        np.savez_compressed(
            os.path.join(HERE, "bigbead.npz"),
            template=np.array("patch_n3"), n_sub=S, conc=C, seed=BIG["seed"], gap=BIG["gap"],
            pos=pos, vel=vel, big_pos_in=big, big_pos=d["big_pos"], big_sigma=2 * BIG["a"],
            big_charge=BIG["G"], big_shc=BIG["H"], box=d["params"]["box"],
            center=int(d["params"]["center_bead"]), kappa=d["params"]["kappa"],
            ld_mant_dig=int(d["params"]["long_double_mant_dig"]),
            tforce=d["tforce"], ne=d["ne"], ce=d["ce"], big_ne=d["big_energies"][0],
            big_ce=d["big_energies"][1], md_steps=MD_STEPS,
            **{f"{m}_{k}": v for m, r in runs.items() for k, v in r.items()})
        print("bigbead", S * t.n_beads, "beads,", len(big), "big beads; big-bead energies", d["big_energies"])


if __name__ == "__main__":
    if "--bigbead-only" not in sys.argv:
        main()
    make_bigbead()
