#!/usr/bin/env python3
"""Benchmark of the qdyn nonbonded hot path on GB300.

Metric: MD steps/s summed over lambda windows (the headline metric of the reference workflow), mixed form.
Workload: 51 lambda windows (lambda = 0, 0.02, ..., 1) of the seeded 25 A,
2-state sphere (3,000-atom synthetic solute in 3-6-atom charge groups, 12 LJ
types, 20 Q atoms, SPC water filling the sphere), 10 A cut-offs, Rcq 99,
LRF on, pair lists rebuilt every 25 steps.  A step is one nonbonded MD step of
the path: list rebuild (every 25th step), pot_energy_nonbonds (ww, qw, pw,
pp, qp, LRF Taylor), nonbond_qq/qqp, restrain_solvent and watpol.  Inputs
(coordinates, topology) are resident in HBM; every timed step is preceded by
an L2 flush (a 256 MB write) outside its CUDA-event bracket.

--impl reference times the CPU restatement of the reference (oracle/, serial C
FP64) on all host cores, one process per window as the reference's own
lambda-window workflow runs, on the same workload.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NBCYCLE = 25
CUT = dict(Rcq=99.0, RcLRF=99.0, Rcpp=10.0, Rcpw=10.0, Rcww=10.0)
METRIC = "MD steps/s summed over lambda windows (nonbonded hot path, mixed precision)"
DTYPE_MIXED = ("f32 pair math; gradients accumulated in u64 fixed point (a row atom's f32 warp sum converted once "
               "per atom and component); f64 cut-off decisions, group centres, LRF Taylor terms and energy records; "
               "LRF coefficients from f32 terms in double-float sums")
# algorithmic FP32 flops per unit (FMA = 2, rsqrt/rcp = 1)
FLOPS = {"pp_atom_pair": 33, "ww_mol_pair": 209, "pw_atom_water": 77}


def window_lambdas(n):
    return [(w / (n - 1) if n > 1 else 0.5) for w in range(n)]


def max_over_ranks(t_local, world, device="cpu"):
    """The slowest rank's time (ms): every rank runs its own windows (replicas,
    no exchange during the timed steps), so the job takes as long as its
    slowest rank.  NCCL needs a device tensor, gloo a host tensor."""
    if world <= 1:
        return float(t_local)
    import torch
    t = torch.tensor([float(t_local)], device=device, dtype=torch.float64)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    torch.distributed.barrier()
    return float(t.item())


def job_throughput(t_max_ms, world, nwin, steps):
    """Window-steps per second of the whole job: world ranks x nwin windows
    x steps, over the slowest rank's time."""
    return world * nwin * steps / (t_max_ms / 1e3)


def first_rebuild_step(istep):
    """The first step index >= istep at which the lists are rebuilt."""
    return -(-istep // NBCYCLE) * NBCYCLE


def amortised_step_ms(rebuild_ms, plain_ms, nbcycle=NBCYCLE):
    """Mean time of one step of the qdyn cycle (one list rebuild every
    `nbcycle` steps) from steps timed individually: a rebuild step (list
    build + evaluation) once per cycle, a plain step the other nbcycle - 1
    times.  The figure does not depend on how many timed steps fall on a
    rebuild, so any --steps gives the step of the cycle."""
    if not rebuild_ms:
        raise ValueError("no rebuild step timed")
    rb = sum(rebuild_ms) / len(rebuild_ms)
    if not plain_ms:
        return rb
    pl = sum(plain_ms) / len(plain_ms)
    return (rb + (nbcycle - 1) * pl) / nbcycle


def cycle_summary(rebuild_ms, plain_ms):
    return {"list_builds_timed": len(rebuild_ms), "plain_steps_timed": len(plain_ms),
            "rebuild_step_ms": round(sum(rebuild_ms) / len(rebuild_ms), 4) if rebuild_ms else None,
            "plain_step_ms": round(sum(plain_ms) / len(plain_ms), 4) if plain_ms else None,
            "amortisation": f"ms_per_step = (rebuild step + {NBCYCLE - 1} plain steps) / {NBCYCLE}, each step "
                            f"timed on its own; the timed steps start at a rebuild"}


def timed_steps(torch, stream, flush, steps, istep0, step_fn, after=None):
    """`steps` steps from index istep0, each bracketed by CUDA events on the
    engine's stream after an L2 flush (a 256 MB write) outside the bracket.
    Returns (rebuild_ms, plain_ms)."""
    rb, pl = [], []
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    for k in range(steps):
        istep = istep0 + k
        with torch.cuda.stream(stream):
            flush.zero_()
            ev0.record(stream)
        step_fn(istep)
        ev1.record(stream)
        ev1.synchronize()
        (rb if istep % NBCYCLE == 0 else pl).append(ev0.elapsed_time(ev1))
        if after:
            after()
    return rb, pl


def energy_snapshot(eng):
    """Energies of every window after a list build and one evaluation at
    step 1 (no watpol update), for the mixed-versus-FP64 comparison."""
    eng.make_pair_lists_dev(**CUT)
    E, EQ, R = eng.compute_dev(Tfree=300.0, istep=1, sync=True)
    return E, EQ, R


def energy_errors(snap_mixed, snap_fp64, nstates):
    """Largest error of each energy term of the mixed form against the FP64
    form over all windows, on identical coordinates and lists."""
    import numpy as np
    Em, EQm, Rm = snap_mixed
    Ed, EQd, Rd = snap_fp64
    out = {}

    def put(name, a, b):
        a, b = np.asarray(a, float), np.asarray(b, float)
        err = np.abs(a - b)
        out[name] = {"max_abs_kcal": float("%.3g" % err.max()),
                     "max_rel": float("%.3g" % (err / np.maximum(np.abs(b), 1e-300)).max()),
                     "fp64_window0": round(float(b.flat[0]), 6)}
    for k in Em[0]:
        put(k, [e[k] for e in Em], [e[k] for e in Ed])
    qn = ("qq_el", "qq_vdw", "qp_el", "qp_vdw", "qw_el", "qw_vdw")
    for st in range(nstates):
        for j, k in enumerate(qn):
            put(f"EQ{st + 1}.{k}", EQm[:, st, j], EQd[:, st, j])
    put("restraint.solvent_radial", Rm[:, 0], Rd[:, 0])
    put("restraint.water_pol", Rm[:, 1], Rd[:, 1])
    return out


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, device):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(device), f"--query-gpu={q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": []}
        if self.p is None:
            return out
        self.p.terminate()
        self.p.wait()
        self.f.flush()
        rows = [ln.split(",") for ln in open(self.f.name).read().strip().splitlines() if ln.strip()]
        os.unlink(self.f.name)
        sm = [float(r[1]) for r in rows if len(r) >= 9 and r[1].strip().replace(".", "").isdigit()]
        if sm:
            out["sm_mhz"] = statistics.median(sm)
            out["sm_max_mhz"] = float(rows[0][2])
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            if len(r) < 9:
                continue
            for k, nm in enumerate(names):
                if r[5 + k].strip() == "Active" and nm not in out["reasons"]:
                    out["reasons"].append(nm)
        out["samples"] = len(rows)
        return out


def make_window_system(seed=2000):
    from q6_gb300.system import config_window
    return config_window(seed)


def run_ours(args, rank, world, local):
    import numpy as np
    import torch

    from q6_gb300 import build as qbuild
    from q6_gb300.qnb import KERNEL_CLASSES, PREC_FP64, PREC_MIXED, NonbondedEngine
    from q6_gb300.system import default_solvent_params, lambdas_for_window

    qbuild.build()
    torch.cuda.set_device(local)
    if world > 1:
        torch.distributed.init_process_group("nccl")
    s = make_window_system()
    sp = default_solvent_params(s)
    nwin = args.windows
    lams = window_lambdas(nwin)
    rng = np.random.default_rng(1234 + rank)
    prec = PREC_MIXED if args.prec == "mixed" else PREC_FP64
    eng = NonbondedEngine(s, precision=prec, device=local, windows=nwin)
    eng.set_solvent_params(sp)
    for w in range(nwin):
        eng.set_lambda(lambdas_for_window(lams[w], s.nstates), window=w)
    xs = np.stack([s.x + rng.normal(0.0, 0.01, size=s.x.shape) for _ in range(nwin)])  # distinct frames
    eng.set_coordinates_dev(xs)
    eng.make_pair_lists_dev(**CUT)
    if args.tuning:                  # fixed launch geometry (profiling runs, where timing under ncu would mislead)
        from q6_gb300.qnb import TUNE_NAMES
        eng.set_tuning(dict(zip(TUNE_NAMES, [int(v) for v in args.tuning.split(",")])))
        tuning = eng.tuning()
    else:
        tuning = eng.autotune(reps=3)    # launch geometry for this workload (set-up, untimed)
    stream = torch.cuda.ExternalStream(eng.stream())
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def step(istep):
        if istep % NBCYCLE == 0:
            eng.make_pair_lists_dev(**CUT)
        eng.compute_dev(Tfree=300.0, istep=istep, sync=False)

    snap = energy_snapshot(eng)      # mixed-form energies for the per-term error against FP64
    # the dominant per-step class for the roofline: two steps with every class
    # bracketed and the evaluation's branches off, so each class is timed alone
    # (beside the other branches a small kernel's span includes its wait for
    # block slots)
    eng.set_concurrency(False)
    eng.profile(True)
    for i in range(2):
        step(i)
        eng.profile_collect()
    torch.cuda.synchronize()
    kt_warm = eng.kernel_times()
    eng.profile(False)
    eng.set_concurrency(True)
    per_step = [c for c in KERNEL_CLASSES if c not in ("build", "lrf_build") and kt_warm[c][1] > 0]
    dom = max(per_step, key=lambda c: kt_warm[c][0])
    # warm-up in the timed configuration (branches on, the dominant class
    # bracketed): every step graph the timed steps replay is captured here,
    # the watpol-update step's too (every itdis steps)
    istep0 = first_rebuild_step(args.warmup)
    eng.profile_classes([dom])
    for i in range(args.warmup):
        step(i)
        eng.profile_collect()
    itdis = int(round(sp.itdis))
    upd = [k for k in range(istep0, istep0 + args.steps) if itdis > 0 and k > 0 and k % itdis == 0]
    if upd:
        eng.compute_dev(Tfree=300.0, istep=upd[0], sync=False)
        eng.profile_collect()
    torch.cuda.synchronize()
    eng.kernel_times()               # the class totals restart with the timed region
    eng.launches()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks = Clocks(local)
    # timed region: exactly --steps steps as a user runs them (graph replay),
    # starting at a list rebuild, with only the dominant class bracketed by
    # events (two event-record nodes per step)
    rb, pl = timed_steps(torch, stream, flush, args.steps, istep0, step, after=eng.profile_collect)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clk = clocks.stop()
    kt_dom = eng.kernel_times()
    launches = eng.launches()
    # per-class breakdown: a second pass of the same steps with every class
    # bracketed (informational; not part of the timed region)
    nbreak = min(args.steps, 50)
    eng.set_concurrency(False)   # each kernel alone on the device: per-kernel times
    eng.profile(True)
    for k in range(nbreak):
        istep = istep0 + args.steps + k
        with torch.cuda.stream(stream):
            flush.zero_()
        step(istep)
        torch.cuda.synchronize()
        eng.profile_collect()
    ktimes = eng.kernel_times()
    eng.profile(False)
    eng.set_concurrency(True)
    ms_local = amortised_step_ms(rb, pl)
    ms_per_step = max_over_ranks(ms_local, world, device="cuda")
    value = job_throughput(ms_per_step * args.steps, world, nwin, args.steps)
    cycle = cycle_summary(rb, pl)
    cycle["ms_per_step_raw_mean"] = round((sum(rb) + sum(pl)) / args.steps, 4)
    counts = {k: eng.list_size(i) for i, k in enumerate(("pp", "pw", "ww", "qp", "qw", "pp14"))}

    # ---- roofline of the dominant kernel class (live CUDA events) ---------
    dom_ms, dom_n = kt_dom[dom]
    dom_avg_s = dom_ms / 1e3 / max(dom_n, 1)
    bytes_per_unit = 4.0   # list streaming: 4 B per atom pair read once per step
    if args.prec == "mixed":
        # gather rows: the solute-row class evaluates pp and the solute side of
        # pw, the water-row class ww and the water side of pw
        per_win = {"pp": counts["pp"] + counts["pw"], "ww": counts["ww"] + counts["pw"],
                   "qp": counts["qp"] * s.nstates, "qw": counts["qw"] * s.nstates}.get(dom)
        flops_win = {"pp": 33 * counts["pp"] + 77 * counts["pw"] // 3,
                     "ww": 209 * counts["ww"] // 9 + 77 * counts["pw"] // 3,
                     "qp": (22 + 17 * s.nstates) * counts["qp"],
                     "qw": ((22 + 17 * s.nstates) + 2 * (19 + 5 * s.nstates)) * counts["qw"] // 3}.get(dom)
    else:
        per_win = {"pp": counts["pp"], "pw": counts["pw"], "ww": counts["ww"],
                   "qp": counts["qp"] * s.nstates, "qw": counts["qw"] * s.nstates}.get(dom)
        flops_win = None
    units = per_win * nwin if per_win else None   # one launch covers every window
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    ach = bytes_per_unit * units / dom_avg_s / 1e9 if units else None
    roof = {"kernel": dom, "bound": "hbm", "achieved": round(ach, 3) if ach else None, "peak": hbm_peak,
            "unit": "GB/s", "frac": round(ach / hbm_peak, 6) if ach else None, "traffic": read_traffic(dom),
            "peak_source": peak_src, "units_per_launch": units, "bytes_per_unit": bytes_per_unit,
            "avg_launch_us": round(dom_avg_s * 1e6, 2)}
    fp32_peak = sgemm_fp32_peak(torch)
    roof_fp32 = None
    if flops_win:
        fl = flops_win * nwin / dom_avg_s / 1e12
        roof_fp32 = {"kernel": dom, "bound": "fp32", "achieved": round(fl, 3), "peak": fp32_peak, "unit": "TFLOP/s",
                     "frac": round(fl / fp32_peak, 4) if fp32_peak else None,
                     "peak_source": "measured here: cuBLAS SGEMM 8192^3 with TF32 off (FP32 CUDA cores)",
                     "flops_per_launch": flops_win * nwin,
                     "flops_per_unit": "33 per LJ+Coulomb atom pair, 77 per solute atom x SPC water, "
                                       "209 per SPC water pair, 22+17S per Q pair with LJ, 19+5S Coulomb-only"}
    # the same roofline from the breakdown pass, where the kernel ran alone
    iso_ms, iso_n = ktimes[dom]
    iso_s = iso_ms / 1e3 / max(iso_n, 1)
    roof_iso = None
    if units and iso_n:
        a = bytes_per_unit * units / iso_s / 1e9
        roof_iso = {"kernel": dom, "bound": "hbm", "achieved": round(a, 3), "peak": hbm_peak, "unit": "GB/s",
                    "frac": round(a / hbm_peak, 6), "avg_launch_us": round(iso_s * 1e6, 2),
                    "timing": "per-class breakdown pass with the evaluation's branches off (qnb_set_concurrency 0): "
                              "the kernel alone on the device"}
        if flops_win and fp32_peak:
            f = flops_win * nwin / iso_s / 1e12
            roof_iso["fp32_achieved_tflops"] = round(f, 3)
            roof_iso["fp32_frac"] = round(f / fp32_peak, 4)
    roof["timing"] = ("live in the timed region; the kernel shares the device with the step's parallel branches "
                      "(water rows, Q environment, LRF Taylor, restraints and watpol)")
    pair_interactions = counts["pp"] + counts["pw"] + counts["ww"] + (counts["qp"] + counts["qw"]) * s.nstates
    eng.close()
    dg = dg_check(s, sp, lams, local, nwin) if args.dg else None

    e2e = run_e2e(args, s, sp, lams, prec, local, tuning) if args.e2e else None
    out = {
        "metric": METRIC, "value": round(value, 2), "unit": "steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_per_step, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": DTYPE_MIXED if args.prec == "mixed" else "f64",
        "cycle": cycle,
        "data": "synthetic seeded sphere (no dataset)",
        "config": {"workload": f"{nwin} lambda windows x R25 2-state sphere ({s.natom} atoms, "
                               f"{s.nwat} SPC, {s.nat_solute}-atom solute, {s.nqat} Q)",
                   "windows_per_gpu": nwin, "natom": s.natom, "nbcycle": NBCYCLE,
                   "cutoffs": CUT, "precision": args.prec, "l2": "flushed (256 MB write) before every timed step",
                   "step": "list rebuild every 25th step + pot_energy_nonbonds + nonbond_qq/qqp + "
                           "restrain_solvent + watpol (no integrator or bonded terms: outside the path); "
                           "ms_per_step is the step of that cycle (see cycle)",
                   "parallelism": f"replicas: {nwin} windows per GPU in one batched context (each kernel "
                                  f"launch covers all windows), one GPU per rank"},
        "pair_interactions_per_step_per_window": pair_interactions,
        "pair_interactions_per_s": round(pair_interactions * value, 1),
        "list_sizes_window0": counts,
        "kernel_ms_total": {k: round(v[0], 4) for k, v in ktimes.items() if v[1]},
        "kernel_ms_total_steps": nbreak,
        "kernel_breakdown": "second pass of the same step (after the timed region) with every kernel class "
                            "bracketed by CUDA events and the evaluation's branches off (each class alone on the "
                            "device); the timed region brackets only the roofline class",
        "graphs": "each step's evaluation replays a captured CUDA graph (qnb_compute_dev); list rebuilds launch "
                  "kernel by kernel",
        "autotune": tuning,
        "roofline": roof,
        "roofline_isolated": roof_iso,
        "roofline_fp32": roof_fp32,
        "clocks": clk,
        "e2e": e2e,
        "gpu_launches": launches,
        "dg_check": dg,
    }
    if rank == 0:
        if args.cpu:
            out["cpu_baseline"] = cpu_baseline(s, sp, args)
        if args.replicas:
            out["replica_group"] = replica_group(args, local)
        if args.md:
            out["md_step"] = md_step(args, s, sp, lams, local, tuning)
        if args.box:
            out["box_step"] = box_step(args, s, lams, local)
        if args.fp64_compare and args.prec == "mixed":
            fp = fp64_compare(args, s, sp, lams, local, xs)
            out["fp64"] = fp["line"]
            out["fp64_value"] = fp["line"]["value"]
            out["mixed_over_fp64"] = round(value / fp["line"]["value"], 3)
            out["energy_error_vs_fp64"] = energy_errors(snap, fp["snap"], s.nstates)
        print(json.dumps(out))
    if world > 1:
        torch.distributed.destroy_process_group()


def sgemm_fp32_peak(torch):
    """FP32 CUDA-core throughput of this GPU: best of 5 cuBLAS SGEMMs
    (8192^3, TF32 disabled), TFLOP/s."""
    try:
        prev = torch.backends.cuda.matmul.allow_tf32
        torch.backends.cuda.matmul.allow_tf32 = False
        n = 8192
        a = torch.randn(n, n, device="cuda")
        b = torch.randn(n, n, device="cuda")
        best = 1e9
        for _ in range(6):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            torch.matmul(a, b)
            e1.record()
            e1.synchronize()
            best = min(best, e0.elapsed_time(e1))
        torch.backends.cuda.matmul.allow_tf32 = prev
        del a, b
        return round(2.0 * n ** 3 / (best / 1e3) / 1e12, 2)
    except Exception:
        return None


def fp64_md_frames(s, sp, lams, bt, local, nframes, every, equil, minimize_steps):
    """Frames of each window's own FP64 trajectory: the device MD path in
    the plain FP64 form (qnb_md_run: the evaluation, bonded terms, leap-frog
    with Berendsen at 300 K, SHAKE, lists every 25 steps) at the window's
    lambda, after a capped steepest descent of the generated start (in the
    mixed form, set-up only) and `equil` steps.  Returns [nwin][nframes][natom][3]
    and the number of MD steps run per window."""
    import numpy as np
    from q6_gb300.md import MdSetup, maxwell_velocities
    from q6_gb300.qnb import PREC_FP64, PREC_MIXED, NonbondedEngine
    from q6_gb300.system import lambdas_for_window
    nwin = len(lams)
    setup = MdSetup(stepsize=1.0, temp0=300.0, tau_t=10.0, nbcycle=NBCYCLE, cut=dict(CUT))
    with NonbondedEngine(s, precision=PREC_MIXED, device=local, windows=nwin) as e:
        e.set_solvent_params(sp)
        for w in range(nwin):
            e.set_lambda(lambdas_for_window(lams[w], s.nstates), window=w)
        e.set_bonded(bt)
        e.set_coordinates_dev(np.stack([s.x] * nwin))
        e.md_init(setup)
        e.md_minimize(minimize_steps, initial_step=1e-4, force_cutoff=1.0, max_move=0.05)
        x0 = np.stack([e.md_state(w)[0] for w in range(nwin)])
    frames = np.zeros((nwin, nframes, s.natom, 3))
    with NonbondedEngine(s, precision=PREC_FP64, device=local, windows=nwin) as e:
        e.set_solvent_params(sp)
        for w in range(nwin):
            e.set_lambda(lambdas_for_window(lams[w], s.nstates), window=w)
        e.set_bonded(bt)
        e.set_coordinates_dev(x0)
        e.md_init(setup)
        e.md_set_velocities(np.stack([maxwell_velocities(s, 300.0, 300 + w) for w in range(nwin)]))
        e.md_prepare(stop_cm=True)
        e.md_run(equil, 0, records=False)
        for k in range(nframes):
            e.md_run(every, equil + k * every, records=False)
            for w in range(nwin):
                frames[w, k] = e.md_state(w)[0]
    return frames, equil + nframes * every


def dg_check(s, sp, lams, local, nwin, nframes=40, every=10, equil=100):
    """Per-window dG (Qfep exponential averaging) of the mixed form against
    the FP64 form on identical frames: `nframes` frames of each window's own
    FP64 MD trajectory (fp64_md_frames), re-evaluated in both forms with the
    lists rebuilt for every frame.  Every window's per-state energies (Q
    nonbonded and Q bonded terms) go through an energy file in qdyn's layout,
    and dG comes from the Qfep summary of those files."""
    import numpy as np
    from q6_gb300.bonded import remove_shaken, synthetic_bonded
    from q6_gb300.enefile import EnergyFileWriter, qfep_files
    from q6_gb300.fep import BOLTZ, window_increments
    from q6_gb300.qnb import PREC_FP64, PREC_MIXED, NonbondedEngine
    from q6_gb300.system import lambdas_for_window
    bt = remove_shaken(synthetic_bonded(s, seed=21), np.asarray(s.heavy).astype(bool), s.nat_solute)
    t0 = time.perf_counter()
    fr, nsteps = fp64_md_frames(s, sp, lams, bt, local, nframes, every, equil, 3000)
    t_md = time.perf_counter() - t0
    lam = np.array([lambdas_for_window(l, s.nstates) for l in lams])
    out = {}
    tmp = tempfile.mkdtemp(prefix="qnb_dg_")
    for name, prec in (("fp64", PREC_FP64), ("mixed", PREC_MIXED)):
        paths = [os.path.join(tmp, "%s_%03d.en" % (name, w)) for w in range(nwin)]
        files = [EnergyFileWriter(p, s.nstates) for p in paths]
        with NonbondedEngine(s, precision=prec, device=local, windows=nwin) as e:
            e.set_solvent_params(sp)
            e.set_bonded(bt)
            for w in range(nwin):
                e.set_lambda(lam[w], window=w)
            for k in range(nframes):
                e.set_coordinates_dev(fr[:, k])
                e.make_pair_lists_dev(**CUT)
                _, EQ, _ = e.compute_dev(sync=True)
                _, EQb = e.bonded_energies()
                for w in range(nwin):
                    files[w].write_step(lam[w], EQ[w], q_bonded=EQb[w])
        for f in files:
            f.close()
        out[name] = window_increments(qfep_files(paths, s.nstates, rt=BOLTZ * 300.0)[3])
        for p in paths:
            os.remove(p)
    os.rmdir(tmp)
    err = np.abs(out["mixed"] - out["fp64"])
    return {"windows": nwin, "frames_per_window": nframes, "max_abs_err_kcal": float("%.3g" % err.max()),
            "mean_abs_err_kcal": float("%.3g" % err.mean()), "tolerance_kcal": 0.02,
            "total_dG_fp64": round(float(out["fp64"].sum()), 4), "total_dG_mixed": round(float(out["mixed"].sum()), 4),
            "frames": f"FP64 MD trajectory of every window (device FP64 MD path at the window's lambda, 300 K, 1 fs): "
                      f"{equil} steps to equilibrate, then a frame every {every} steps ({nsteps} steps per window), "
                      f"after a capped steepest descent of the generated start",
            "md_seconds": round(t_md, 1),
            "path": "per-window energy files in qdyn's put_ene layout (Q nonbonded and Q bonded terms) -> Qfep "
                    "FEP summary"}


def read_traffic(kernel):
    """dram bytes per launch of `kernel` from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    if not os.path.exists(p):
        return None
    for ln in open(p):
        ln = ln.strip()
        if ln.startswith(kernel + " "):
            try:
                return float(ln.split()[1])
            except ValueError:
                return None
    return None


def run_e2e(args, s, sp, lams, prec, local, tuning=None):
    """Same metric end to end through the public C ABI with host buffers.

    Batched path (the headline): one context holds every window, as a program
    running all lambda windows in one process would; each step is one
    qnb_step_host call: all windows' coordinates in from pinned host memory,
    the lists rebuilt every 25th step, the evaluation, all gradients out to
    pinned memory and the energies read back, with one host synchronisation
    (two on a rebuild step, whose list counts are checked).

    Drop-in path (reported beside it): one context per window, as one qdyn
    process per window holds, through the calls the Fortran shim makes:
    make_pair_lists every 25th step and qnb_pot_energy_step (the nonbonded
    side of pot_energy in one call, one copy of x in and of the gradient out);
    beside it the same with the four separate entry points (pot_energy_nonbonds,
    nonbond_qq, restrain_solvent, watpol), each copying x in and the gradient
    out."""
    import numpy as np
    import torch
    from q6_gb300.qnb import NonbondedEngine
    from q6_gb300.system import lambdas_for_window
    nwin = args.windows
    steps = max(4, min(args.steps, 50))
    eng = NonbondedEngine(s, precision=prec, device=local, windows=nwin)
    eng.set_solvent_params(sp)
    for w in range(nwin):
        eng.set_lambda(lambdas_for_window(lams[w], s.nstates), window=w)
    if tuning:
        eng.set_tuning(tuning)   # the device arm's autotuned geometry (same system and windows)
    shape = (nwin, s.natom, 3)
    x_pin = torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()
    d_pin = torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()
    rng = np.random.default_rng(77)
    x_pin[:] = np.stack([s.x + rng.normal(0.0, 0.01, size=s.x.shape) for _ in range(nwin)])

    def step(k):   # coordinates H2D, lists every 25th step, evaluation, gradients + energies D2H
        eng.step_host(x_pin, out=d_pin, Tfree=300.0, istep=k, rebuild_lists=k % NBCYCLE == 0)

    eng.set_coordinates_dev(x_pin)
    eng.make_pair_lists_dev(**CUT)   # the cut-offs every later rebuild uses
    warm = max(3, args.warmup)
    for k in range(warm):
        step(k)
    rb, pl = [], []
    k0 = first_rebuild_step(warm)
    for k in range(k0, k0 + steps):     # each step ends synchronised (energies and gradients on the host)
        t0 = time.perf_counter()
        step(k)
        (rb if k % NBCYCLE == 0 else pl).append((time.perf_counter() - t0) * 1e3)
    eng.close()
    ms = amortised_step_ms(rb, pl)
    nbytes = s.x.nbytes * nwin
    ebytes = nwin * (7 + 6 * s.nstates + 2) * 8   # E, EQ and restraint records
    out = {"value": round(nwin / (ms / 1e3), 2), "unit": "steps/s", "ms_per_step": round(ms, 4),
           "h2d_bytes_per_step": int(nbytes), "d2h_bytes_per_step": int(nbytes + ebytes), "windows": nwin,
           "steps": steps, "cycle": cycle_summary(rb, pl),
           "path": "qnb_step_host: coordinates in from pinned memory, lists rebuilt every 25th step, "
                   "evaluation, gradients out to pinned memory and energies back in one call, one context "
                   "holding all windows; host clock around each step"}

    # drop-in path: one single-window context per window
    nw1 = min(nwin, 8)
    engs = []
    for w in range(nw1):
        e = NonbondedEngine(s, precision=prec, device=local)
        e.set_solvent_params(sp)
        e.set_lambda(lambdas_for_window(lams[w], s.nstates))
        engs.append(e)
    xs = [s.x.copy() for _ in range(nw1)]
    ds = [np.zeros_like(s.x) for _ in range(nw1)]
    for w, e in enumerate(engs):
        e.make_pair_lists(xs[w], **CUT)
        for k in (k0 - 2, k0 - 1):     # untimed warm-up steps of every context
            d = np.zeros_like(s.x)
            d, E, EQ = e.pot_energy_nonbonds(xs[w], d)
            e.nonbond_qq(xs[w], d, EQ)
            e.restrain_solvent(xs[w], d, 300.0)
            e.watpol(xs[w], d, k)
    def drop_in_steps(fused):
        rb1, pl1 = [], []
        for k in range(k0, k0 + steps):
            t0 = time.perf_counter()
            for w, e1 in enumerate(engs):
                x, d = xs[w], ds[w]
                d[:] = 0.0
                if k % NBCYCLE == 0:
                    e1.make_pair_lists(x, **CUT)
                if fused:
                    e1.pot_energy_step(x, d, Tfree=300.0, istep=k)
                else:
                    d, E, EQ = e1.pot_energy_nonbonds(x, d)
                    d, EQ = e1.nonbond_qq(x, d, EQ)
                    e1.restrain_solvent(x, d, 300.0)
                    e1.watpol(x, d, k)
            (rb1 if k % NBCYCLE == 0 else pl1).append((time.perf_counter() - t0) * 1e3)
        return rb1, pl1

    rb1, pl1 = drop_in_steps(True)
    rb2, pl2 = drop_in_steps(False)
    for e1 in engs:
        e1.close()
    ms1, ms2 = amortised_step_ms(rb1, pl1), amortised_step_ms(rb2, pl2)
    out["drop_in"] = {"value": round(nw1 / (ms1 / 1e3), 2), "unit": "steps/s", "windows": nw1,
                      "cycle": cycle_summary(rb1, pl1),
                      "h2d_bytes_per_step": int(s.x.nbytes * (1 + 1.0 / NBCYCLE)),
                      "d2h_bytes_per_step": int(s.x.nbytes),
                      "path": "qnb_make_pair_lists every 25th step + qnb_pot_energy_step (the nonbonded side of "
                              "pot_energy in one call) with host buffers, one context per window, windows in "
                              "sequence",
                      "separate_calls": {
                          "value": round(nw1 / (ms2 / 1e3), 2), "unit": "steps/s",
                          "cycle": cycle_summary(rb2, pl2),
                          "h2d_bytes_per_step": int(s.x.nbytes * (4 + 1.0 / NBCYCLE)),
                          "d2h_bytes_per_step": int(s.x.nbytes * 4),
                          "path": "qnb_pot_energy_nonbonds/qnb_nonbond_qq/qnb_restrain_solvent/qnb_watpol, each "
                                  "with its own copies and synchronisation"}}
    return out


def replica_group(args, local):
    """Config 3 as one CUDA graph launch per step (qnb_group_compute): the
    51-window context of the R15 system plus 16 single-window replicas with
    radii drawn uniformly from 18-30 A.  Window-steps/s summed over all 67
    windows, L2 flushed before every timed step."""
    import numpy as np
    import torch
    from q6_gb300.qnb import PREC_MIXED, Group, NonbondedEngine
    from q6_gb300.system import config_small, default_solvent_params, lambdas_for_window, make_system
    rng = np.random.default_rng(3016)
    radii = np.sort(rng.uniform(18.0, 30.0, 16))
    systems = [config_small()] + [make_system(R=float(R), n_solute=20, group_sizes=(3, 5), ntypes=6, nq=6,
                                              nstates=2, seed=3100 + i) for i, R in enumerate(radii)]
    nwin = [51] + [1] * 16
    engs = []
    for s, W in zip(systems, nwin):
        e = NonbondedEngine(s, precision=PREC_MIXED, device=local, windows=W)
        e.set_solvent_params(default_solvent_params(s))
        for w in range(W):
            e.set_lambda(lambdas_for_window(w / 50.0 if W == 51 else 0.5, s.nstates), window=w)
        e.set_coordinates_dev(np.stack([s.x] * W))
        e.make_pair_lists_dev(**CUT)
        engs.append(e)
    grp = Group(engs)
    stream = torch.cuda.ExternalStream(engs[0].stream())
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    steps = max(10, min(args.steps, 100))
    for k in range(3):
        grp.compute(Tfree=300.0, istep=k + 1)
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    tot = 0.0
    for k in range(steps):
        with torch.cuda.stream(stream):
            flush.zero_()
            ev0.record(stream)
        grp.compute(Tfree=300.0, istep=k + 4)
        ev1.record(stream)
        ev1.synchronize()
        tot += ev0.elapsed_time(ev1)
    grp.close()
    wins = sum(nwin)
    for e in engs:
        e.close()
    return {"value": round(wins * steps / (tot / 1e3), 1), "unit": "window-steps/s", "ms_per_step": round(tot / steps, 4),
            "windows": wins, "systems": len(systems), "atoms": int(sum(s.natom * w for s, w in zip(systems, nwin))),
            "radii": [15.0] + [round(float(r), 2) for r in radii], "steps": steps,
            "what": "evaluation step (no list rebuild) of 51 windows of the R15 system + 16 replicas of uneven radii, "
                    "one CUDA graph launch per step"}


def md_step(args, s, sp, lams, local, tuning=None):
    """Device-resident MD steps (qnb_md_run) of the same 51 windows: the
    evaluation above plus the solute and Q bonded terms of the generated
    topology, leap-frog with Berendsen coupling (solute and solvent groups),
    SHAKE of the waters and temperature(), lists every 25 steps, 1 fs steps
    at 300 K.  Window-steps/s over the timed run; no host round trip inside
    it (records read back after the run)."""
    import numpy as np
    import torch
    from q6_gb300.bonded import remove_shaken, synthetic_bonded
    from q6_gb300.md import MdSetup, maxwell_velocities
    from q6_gb300.qnb import PREC_MIXED, NonbondedEngine, QnbError
    from q6_gb300.system import lambdas_for_window
    nwin = args.windows
    try:
        e = NonbondedEngine(s, precision=PREC_MIXED, device=local, windows=nwin)
        e.set_solvent_params(sp)
        for w in range(nwin):
            e.set_lambda(lambdas_for_window(lams[w], s.nstates), window=w)
        if tuning:
            e.set_tuning(tuning)
        bt = remove_shaken(synthetic_bonded(s, seed=21), np.asarray(s.heavy).astype(bool), s.nat_solute)
        e.set_bonded(bt)
        e.set_coordinates_dev(np.stack([s.x] * nwin))
        setup = MdSetup(stepsize=1.0, temp0=300.0, tau_t=10.0, nbcycle=25, cut=dict(CUT))
        e.md_init(setup)
        # the generated start structure is strained (random solute tree, lattice
        # water): Qmin-style steepest descent on the device first (untimed)
        t_min = time.perf_counter()
        maxf = e.md_minimize(args.md_minimize, initial_step=1e-4, force_cutoff=1.0, max_move=0.05)
        t_min = time.perf_counter() - t_min
        e.md_set_velocities(np.stack([maxwell_velocities(s, 300.0, 100 + w) for w in range(nwin)]))
        e.md_prepare(stop_cm=True)
        warm = 25
        rec0, _, _ = e.md_run(warm, 0)
        # the generated sphere's MD stays stable for a few hundred steps at
        # the endpoint windows (it is a random solute tree, not an equilibrated
        # structure): 200 timed steps, 8 list builds
        steps = 200
        stream = torch.cuda.ExternalStream(e.stream())
        torch.cuda.synchronize()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        e.md_run(steps, warm, records=False)
        ev1.record(stream)
        ev1.synchronize()
        ms = ev0.elapsed_time(ev1)
        rec, _, Eb = e.md_run(1, warm + steps)
        n = e.launches()
        e.close()
    except QnbError as ex:
        return {"error": str(ex)}
    return {"value": round(nwin * steps / (ms / 1e3), 1), "unit": "window-MD-steps/s",
            "ms_per_step": round(ms / steps, 4), "steps": steps, "windows": nwin,
            "list_builds": steps // 25, "bonded_terms": int((bt.bonds[:, 2] >= 0).sum() + (bt.angles[:, 3] >= 0).sum() +
                                                            (bt.torsions[:, 4] >= 0).sum() +
                                                            (bt.impropers[:, 4] >= 0).sum()),
            "q_bonded_terms": int(len(bt.qbonds) + len(bt.qangles) + len(bt.qtorsions) + len(bt.qimpropers)),
            "tfree_start_end": [round(float(rec0[0]["tfree"].mean()), 2), round(float(rec[0]["tfree"].mean()), 2)],
            "shake_iterations_per_step": round(float(rec[0]["shake_iterations"].mean()), 1),
            "minimisation": {"steps": args.md_minimize, "max_force_after": round(float(maxf.max()), 1),
                             "seconds": round(t_min, 2)},
            "what": "mixed-form evaluation + bonded + leap-frog/Berendsen (tau_T 10 fs) + SHAKE + temperature, "
                    "all windows on the device, after a steepest-descent relaxation of the generated start; timed "
                    "with CUDA events around qnb_md_run (L2 not flushed between steps)"}


def box_step(args, s, lams, local):
    """The periodic-box path (qnb_set_box; the *_box lists and energies) on the
    same 6,060 atoms in a 53 A cubic box (2R + 3 A, so pairs wrap across the
    faces), the sphere's excluded flags cleared and LRF off as the box path
    requires: 51 windows, mixed form, lists every 25th step, Rcq 12 A.
    Window-steps/s, L2 flushed before every timed step."""
    import dataclasses

    import numpy as np
    import torch
    from q6_gb300.qnb import PREC_MIXED, NonbondedEngine, QnbError
    from q6_gb300.system import lambdas_for_window
    nwin = args.windows
    sb = dataclasses.replace(s, excl=np.zeros_like(np.asarray(s.excl)))
    R = float(np.sqrt((np.asarray(s.x) ** 2).sum(1)).max())
    L = 2.0 * round(R) + 3.0
    cut = dict(Rcq=12.0, RcLRF=12.0, Rcpp=10.0, Rcpw=10.0, Rcww=10.0)
    try:
        e = NonbondedEngine(sb, precision=PREC_MIXED, use_lrf=False, device=local, windows=nwin)
        e.set_box([L, L, L])
        for w in range(nwin):
            e.set_lambda(lambdas_for_window(lams[w], sb.nstates), window=w)
        e.set_coordinates_dev(np.stack([sb.x] * nwin))
        stream = torch.cuda.ExternalStream(e.stream())
        flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
        for k in range(3):
            e.make_pair_lists_dev(**cut)
            e.compute_dev(istep=k, sync=True)
        sizes = {k: int(e.list_size(v)) for k, v in (("pp", 0), ("pw", 1), ("ww", 2), ("qp", 3), ("qw", 4))}
        steps = 50
        torch.cuda.synchronize()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        tot = 0.0
        for k in range(steps):
            with torch.cuda.stream(stream):
                flush.zero_()
                ev0.record(stream)
            if k % 25 == 0:
                e.make_pair_lists_dev(**cut)
            e.compute_dev(istep=k, sync=False)
            ev1.record(stream)
            ev1.synchronize()
            tot += ev0.elapsed_time(ev1)
        e.close()
    except QnbError as ex:
        return {"error": str(ex)}
    return {"value": round(nwin * steps / (tot / 1e3), 1), "unit": "window-steps/s",
            "ms_per_step": round(tot / steps, 4), "steps": steps, "windows": nwin, "box_A": L,
            "list_sizes_window0": sizes,
            "what": "periodic box: gather rows built every 25th step by periodic cell binning with minimum-image "
                    "tests; pp/pw/ww on the rows at each unit pair's lattice image, qp/qw box energies, static Q-Q "
                    "(FP32 pair arithmetic, fixed-point sums), all windows per launch"}


def fp64_compare(args, s, sp, lams, local, xs):
    """The plain FP64 form on the same workload, timed exactly as the mixed
    arm: the same coordinates, its own autotuned launch geometry, the same
    warm-up, the same --steps steps from the same rebuild step, an L2 flush
    before every step and CUDA events around each step; the same amortised
    step of the rebuild cycle.  Also returns its energies for the per-term
    error of the mixed form."""
    import torch
    from q6_gb300.qnb import PREC_FP64, NonbondedEngine
    from q6_gb300.system import lambdas_for_window
    nwin = args.windows
    e = NonbondedEngine(s, precision=PREC_FP64, device=local, windows=nwin)
    e.set_solvent_params(sp)
    for w in range(nwin):
        e.set_lambda(lambdas_for_window(lams[w], s.nstates), window=w)
    e.set_coordinates_dev(xs)
    e.make_pair_lists_dev(**CUT)
    tuning = e.autotune(reps=3)
    stream = torch.cuda.ExternalStream(e.stream())
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def step(istep):
        if istep % NBCYCLE == 0:
            e.make_pair_lists_dev(**CUT)
        e.compute_dev(Tfree=300.0, istep=istep, sync=False)

    snap = energy_snapshot(e)
    for i in range(args.warmup):
        step(i)
    torch.cuda.synchronize()
    rb, pl = timed_steps(torch, stream, flush, args.steps, first_rebuild_step(args.warmup), step)
    torch.cuda.synchronize()
    e.close()
    ms = amortised_step_ms(rb, pl)
    line = {"value": round(nwin / (ms / 1e3), 2), "unit": "steps/s", "ms_per_step": round(ms, 4),
            "steps": args.steps, "warmup": args.warmup, "dtype": "f64", "autotune": tuning, "cycle": cycle_summary(rb, pl),
            "timing": "as the mixed arm: CUDA events per step on the engine stream, L2 flushed before each step, "
                      "amortised over the 25-step rebuild cycle"}
    return {"line": line, "snap": snap}


def _oracle_window(payload):
    """One lambda window of the CPU restatement (its -Ofast timing build):
    `warmup` untimed steps, then `steps` steps from the next rebuild step,
    each timed on its own, with a list rebuild every 25th step.  Returns the
    amortised milliseconds per step of the rebuild cycle and the step
    counts."""
    import pickle
    sys.path.insert(0, ROOT)
    from oracle.oracle import Oracle
    s, sp_bytes, lam, steps, warmup = pickle.loads(payload)
    from q6_gb300.system import QnbSolventParams, lambdas_for_window
    sp = QnbSolventParams.from_buffer_copy(sp_bytes)
    o = Oracle(s, timing_build=True)
    o.set_solvent_params(sp)
    o.set_lambda(lambdas_for_window(lam, s.nstates))

    def step(k):
        if k % NBCYCLE == 0:
            o.make_pair_lists(s.x, **CUT)
        d, E, EQ = o.pot_energy_nonbonds(s.x)
        d, EQ = o.nonbond_qq(s.x, d, EQ)
        o.restrain_solvent(s.x, d, 300.0)
        o.watpol(s.x, d, k)

    o.make_pair_lists(s.x, **CUT)
    for k in range(1, warmup + 1):
        step(k)
    rb, pl = [], []
    k0 = first_rebuild_step(warmup + 1)
    for k in range(k0, k0 + steps):
        t0 = time.perf_counter()
        step(k)
        (rb if k % NBCYCLE == 0 else pl).append((time.perf_counter() - t0) * 1e3)
    o.close()
    return amortised_step_ms(rb, pl), len(rb), len(pl)


def _oracle_worker(payloads):
    """The windows one host process runs, one after the other (as one qdyn
    process per window would be queued on a core)."""
    return [_oracle_window(p) for p in payloads]


def cpu_info():
    model = None
    try:
        for ln in open("/proc/cpuinfo"):
            if ln.lower().startswith(("model name", "cpu model")):
                model = ln.split(":", 1)[1].strip()
                break
    except OSError:
        pass
    import platform
    return {"model": model or platform.processor() or platform.machine(), "machine": platform.machine(),
            "logical_cores": os.cpu_count()}


def cpu_baseline(s, sp, args):
    """Serial oracle (1 core, -Ofast timing build) on a bounded sample of one
    window: 2 list builds and 50 steps (about 10-20 s on one core)."""
    import pickle
    from oracle import oracle as orc
    orc.build()
    steps, warmup = 2 * NBCYCLE, 3
    ms, nrb, npl = _oracle_window(pickle.dumps((s, bytes(sp), 0.5, steps, warmup)))
    return {"value": round(1e3 / ms, 4), "unit": "steps/s", "cores": 1, "kind": "port",
            "cpu": cpu_info(),
            "sample": f"1 window x {steps} timed steps ({nrb} list builds) after {warmup} warm-up steps, "
                      f"amortised over the 25-step rebuild cycle; serial C FP64 restatement built with the "
                      f"reference's gcc optimisation flags (-Ofast -funroll-loops -finline-limit=10000000)"}


def run_reference(args, rank, world):
    """CPU reference arm: the oracle on all host cores, one process per core
    running its share of the windows one after the other."""
    if rank != 0:
        return
    import multiprocessing as mp
    import pickle
    from oracle import oracle as orc
    from q6_gb300.system import default_solvent_params
    orc.build()
    s = make_window_system()
    sp = default_solvent_params(s)
    cores = os.cpu_count() or 1
    nwin = args.windows                      # the same windows as the GPU arm
    lams = window_lambdas(nwin)
    # --steps timed steps per window after --warmup untimed ones (an oracle
    # step takes about 30 ms on one core, so K = 100 stays a few seconds)
    steps, warmup = args.steps, args.warmup
    nproc = min(nwin, cores)
    shares = [[pickle.dumps((s, bytes(sp), lams[w], steps, warmup)) for w in range(r, nwin, nproc)]
              for r in range(nproc)]
    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    with ctx.Pool(nproc) as pool:
        res = pool.map(_oracle_worker, shares, chunksize=1)
    wall = time.perf_counter() - t0
    # makespan of the timed work: the busiest process's windows, each
    # --steps steps of the amortised rebuild cycle (process start-up and
    # the untimed warm-up steps left out)
    per_proc_ms = [sum(ms * steps for ms, _, _ in r) for r in res]
    makespan_s = max(per_proc_ms) / 1e3
    value = nwin * steps / makespan_s
    nrb = sum(b for r in res for _, b, _ in r)
    out = {"metric": METRIC, "value": round(value, 4), "unit": "steps/s", "n_gpus": world,
           "steps": steps, "warmup": warmup, "ms_per_step": round(makespan_s * 1e3 / steps, 3),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "impl": "reference",
           "dtype": "f64", "data": "synthetic seeded sphere (no dataset)",
           "config": {"workload": f"{nwin} lambda windows x R25 2-state sphere ({s.natom} atoms)",
                      "windows": nwin, "nbcycle": NBCYCLE, "cutoffs": CUT,
                      "note": "Q6 qdyn (Fortran) cannot be built on this pool (no gfortran); the "
                              "serial C restatement in oracle/ runs each window in its own process, "
                              "as qdyn runs one process per window, on all host cores"},
           "cpu_baseline": {"value": round(value, 4), "unit": "steps/s", "cores": nproc, "kind": "port",
                            "cpu": cpu_info(),
                            "sample": f"{nwin} windows x {steps} timed steps after {warmup} warm-up steps, "
                                      f"{nproc} processes with {-(-nwin // nproc)} windows on the busiest; "
                                      f"value = window-steps over the makespan of the timed work; each step "
                                      f"amortised over the 25-step rebuild cycle ({nrb} rebuild steps timed); "
                                      f"-Ofast timing build"},
           "e2e": {"value": round(value, 4), "unit": "steps/s", "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 0},
           "wall_s": round(wall, 2)}
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--windows", type=int, default=51)
    ap.add_argument("--prec", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--no-fp64-compare", dest="fp64_compare", action="store_false")
    ap.add_argument("--no-e2e", dest="e2e", action="store_false",
                    help="skip the host-buffer arm (profiling runs)")
    ap.add_argument("--no-cpu-baseline", dest="cpu", action="store_false",
                    help="skip the CPU oracle sample (profiling runs)")
    ap.add_argument("--tuning", default="",
                    help="comma-separated launch geometry (autotune order) instead of autotuning")
    ap.add_argument("--no-replicas", dest="replicas", action="store_false",
                    help="skip the 51-window + 16-replica graph group")
    ap.add_argument("--no-dg", dest="dg", action="store_false",
                    help="skip the mixed-vs-FP64 dG check")
    ap.add_argument("--no-box", dest="box", action="store_false",
                    help="skip the periodic-box line (box_step)")
    ap.add_argument("--no-md", dest="md", action="store_false",
                    help="skip the device-resident MD step measurement")
    ap.add_argument("--md-minimize", type=int, default=3000,
                    help="steepest-descent steps before the MD measurement")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    run_ours(args, rank, world, local)


if __name__ == "__main__":
    main()
