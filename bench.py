#!/usr/bin/env python
"""Pair-interaction throughput of the RCB short-range kick on one GB300.

Workload (one "step"): the short-range kick of a 128^3 Zel'dovich particle set
at z = 50 (seeded Gaussian field, n = -2 power law, 2 Mpc/h cells) with
periodic overload ghosts (2.57 M particles), RCB leaves of at most 128
particles, opening angle 0.1, rsm = 0.1, 6th-order polynomial law, monopole
pseudo-particles: every (leaf particle, list entry) pair of every leaf inside
the force box, fused with the velocity kick.

* value      -- pairs/s of the device step with its inputs resident in HBM
                (pair kernel relaunched on the resident lists, L2 flushed
                between launches), max over ranks.
* e2e        -- pairs/s of hsr_rcb_kick through the C ABI with pinned host
                arrays: tree build, lists, host<->device copies and the
                kernels.
* roofline_hbm -- the same kernel's profiled DRAM bytes per launch over its
                time against the measured HBM copy bandwidth (a few percent:
                the kernel is compute-bound).
* roofline   -- the pair kernel against the FP32 FMA peak measured by the
                library's FFMA probe on this device: 31 flops per pair the
                kernel evaluates.  The batched kernel skips list entries
                farther than the cutoff from a particle group's bounding box
                (their contribution is exactly zero), so it evaluates fewer
                pairs than the list holds; `value` counts the list's pairs.
* cpu_baseline -- the CPU restatement of the reference force tree (oracle),
                timed on this host's cores on a bounded slab of the workload.
* treepm     -- the long-range PM kick on the same box (deposit, FFT solve,
                inverse CIC; double and single precision), the short-range
                sub-cycles alone (hsr_subcycle: s/substep), and one whole
                TreePM step (PM half kick, 5 short-range sub-cycles, PM kick)
                end to end from host arrays, with the PM restatement timed on
                the host.

`--impl reference` times that CPU path alone as the reference arm.  Under
torchrun each rank runs an independent replica on its own GPU (the path does
not shard across GPUs); rank 0 prints one JSON line.
"""
from __future__ import annotations

import argparse
import dataclasses
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (os.path.join(ROOT, "hacc-coral_gb300"), os.path.join(ROOT, "oracle"),
           os.path.join(ROOT, "tests")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

import synth  # noqa: E402

FLOPS_PER_PAIR = 31
METRIC = "pair interactions/s"
UNIT = "pairs/s"
L2_NOTE = "L2 flushed (256 MB write) before every timed pair-kernel launch"


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--ng", type=int, default=128)
    ap.add_argument("--nd", type=int, default=128)
    ap.add_argument("--kernel", choices=["auto", "plain", "batched"], default="auto")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--multibox", type=int, default=8,
                    help="boxes of 96^3 in the multi-box line (0: skip)")
    ap.add_argument("--adjoint-boxes", type=int, default=8,
                    help="boxes of 96^3 in the multi-step adjoint line (0: skip)")
    ap.add_argument("--clustered", type=int, default=256,
                    help="side of the clustered set of the leaf size x shape sweep (0: skip)")
    ap.add_argument("--treepm", type=int, default=1,
                    help="time the PM kick and one full TreePM step on the bench box (0: skip)")
    ap.add_argument("--cpu-slab", type=float, default=1.0,
                    help="fraction of the force box (along x) in the CPU sample")
    ap.add_argument("--no-accuracy", action="store_true",
                    help="skip the oracle / FP64 error fields of the results")
    return ap.parse_args()


def workload(ng: int, nd: int, world: int = 1):
    """The bench box and its `config` (the same in both arms)."""
    p = synth.zeldovich_box(ng, z=50.0)
    kp = synth.kick_params(p, nd=nd)
    cfg = {"workload": f"zeldovich{ng}_z50_nd{nd}_monopole", "n_side": ng, "n_particles": p.n,
           "nd": nd, "open_angle": kp.open_angle, "rsm": kp.rsm, "fsrrmax": kp.fsrrmax,
           "tdpts": kp.tdpts, "law": "poly6", "fcoeff": kp.fcoeff, "l2": L2_NOTE,
           "parallelism": f"replicas{world}"}
    return p, kp, cfg


TRAFFIC_NOTE = ("dram__bytes_read.sum + dram__bytes_write.sum of one ncu capture of the pair "
                "kernel on this workload and shape, bytes per launch (profiles/, line "
                "'traffic <workload> <shape>: <bytes>')")


def profiled_traffic(workload: str, shape: dict):
    """DRAM bytes per launch of the pair kernel from the committed ncu
    summaries, or None when no capture of this workload and shape exists."""
    key = (f"traffic {workload} {shape['kernel']}-"
           f"{shape['group'] if shape['kernel'] == 'batched' else shape['leaf_threads']}:")
    pdir = os.path.join(ROOT, "profiles")
    for name in sorted(os.listdir(pdir)) if os.path.isdir(pdir) else []:
        if not name.endswith((".md", ".txt")):
            continue
        with open(os.path.join(pdir, name)) as f:
            for line in f:
                line = line.strip().strip("`")
                if line.startswith(key):
                    try:
                        return int(line[len(key):].split()[0])
                    except ValueError:
                        return None
    return None


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(world, x: float) -> float:
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clock/throttle samples every 200 ms during a timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        self.out = ""
        if self.proc:
            time.sleep(0.3)
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out, _ = self.proc.communicate()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for line in (self.out or "").strip().splitlines():
            f = [v.strip() for v in line.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for nm, v in zip(names, f[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# The reference nests a two-thread OpenMP team per tree split and keeps
# nesting on during the list walk; with nesting capped at one level the same
# code gives the same results 3-4x faster on these hosts.  The CPU timings use
# the faster setting, so they understate the GPU's advantage rather than
# overstate it.
OMP_LEVELS = "1"


def _oracle():
    os.environ["ORA_MAX_ACTIVE_LEVELS"] = OMP_LEVELS
    import oracle
    oracle.build()
    return oracle.Oracle()


def cpu_baseline(p, kp, slab: float, threads: int):
    """Reference force tree (CPU restatement) on a slab of the force box.
    `_out` holds the particles after the run (tree order, kicked)."""
    O = _oracle()
    q = p.copy()
    ks = synth.KickParams(**{**kp.__dict__})
    lo, hi = kp.min_force[0], kp.max_force[0]
    ks.max_force = (lo + slab * (hi - lo), kp.max_force[1], kp.max_force[2])
    t0 = time.perf_counter()
    r = O.rcb_run(q, ks, nthreads=threads)
    dt = time.perf_counter() - t0
    pairs = r.stats["pairs"]
    return {"value": pairs / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": (f"leaves of the force box with x in [{lo:.1f}, {ks.max_force[0]:.1f}] "
                       f"({pairs:.3e} pairs, full tree built), {dt:.2f} s wall, "
                       f"OpenMP nesting capped at {OMP_LEVELS} level"),
            "seconds": dt, "pairs": pairs, "_out": q}


# ---- accuracy of every result: against the oracle and FP64 --------------

EXACT = ("x", "y", "z", "mass", "phi", "id", "mask")
ACC_NOTE = ("rms = sqrt(sum |a - ref|^2 / sum |ref|^2), max = max_i |a_i - ref_i| / rms |ref| "
            "over the particles of the processed leaves; targets rms <= 1e-5, max <= 1e-3")


def _zero_v(p):
    p.vx[:] = 0
    p.vy[:] = 0
    p.vz[:] = 0
    return p


def _vel(p):
    return np.stack([p.vx, p.vy, p.vz], axis=1).astype(np.float64)


def _err(a, ref):
    from hsr_testutil import force_errors
    rms, mx = force_errors(a, ref)
    return {"rms": rms, "max": mx}


def _same_arrays(a, b):
    return all(np.array_equal(getattr(a, k).view(np.uint8), getattr(b, k).view(np.uint8))
               for k in EXACT)


def _oracle_check(O, z, p, kp, threads, oracle_max_x=None):
    """Oracle run on `p` with zero velocities (tree, lists, kick) against the
    GPU's kick `z` of the same input: the permutation bit for bit, the kick
    against the oracle's and against FP64 over the oracle's lists (fcoeff
    times the FP64 acceleration).  With oracle_max_x the oracle processes only
    the leaves of the force box with x below it (the tree is still whole)."""
    zo = _zero_v(p.copy())
    ko = synth.KickParams(**{**kp.__dict__})
    if oracle_max_x is not None:
        ko.max_force = (float(oracle_max_x), kp.max_force[1], kp.max_force[2])
    r = O.rcb_run(zo, ko, keep_lists=True, nthreads=threads)
    off, cnt, _ = r.leaves()
    sel = (np.concatenate([np.arange(o, o + c) for o, c in zip(off, cnt)])
           if len(off) else np.zeros(0, np.int64))
    a64 = r.acc_fp64()[sel] * float(np.float32(kp.fcoeff))
    out = {"permutation_exact": _same_arrays(z, zo), "particles_checked": int(len(sel)),
           "vs_oracle": _err(_vel(z)[sel], _vel(zo)[sel]), "vs_fp64": _err(_vel(z)[sel], a64),
           "oracle_vs_fp64": _err(_vel(zo)[sel], a64)}
    return out, r, sel, a64


def kick_accuracy(ctx, p, kp, threads, oracle_max_x=None, kernel=None):
    """hsr_rcb_kick of `p` with its velocities zeroed -- the output is then
    the kick itself -- checked by _oracle_check."""
    import hsr
    O = _oracle()
    z = _zero_v(p.copy())
    st = ctx.rcb_kick(z, kp, kernel=hsr.KERNEL_AUTO if kernel is None else kernel)
    out, r, sel, a64 = _oracle_check(O, z, p, kp, threads, oracle_max_x)
    if oracle_max_x is None:
        out["pairs_equal"] = st["pairs"] == r.stats["pairs"]
    else:
        out["oracle_leaves"] = f"force box leaves with x < {oracle_max_x:g} (tree whole)"
    return out, sel, a64


def timed_output_check(p0, q_gpu, perm, q_ora, sel, a64):
    """The last timed hsr_rcb_kick (velocities as the workload has them)
    against the oracle's run on the same input (cpu_baseline over the whole
    force box) and against FP64: the ten arrays' permutation bit for bit and
    the velocity change v_out - v_in of the processed leaves' particles
    (input velocities taken in tree order through the kick's permutation)."""
    vin = _vel(p0)[perm]
    dv = _vel(q_gpu) - vin
    return {"permutation_exact": _same_arrays(q_gpu, q_ora),
            "dv_vs_fp64": _err(dv[sel], a64), "dv_vs_oracle": _err(dv[sel], (_vel(q_ora) - vin)[sel]),
            "oracle_dv_vs_fp64": _err((_vel(q_ora) - vin)[sel], a64),
            "note": "v_out = v_in + kick in float: the library rounds once per particle, the "
                    "reference (oracle) once per pair term, so the oracle's dv carries ~sqrt(list "
                    "length) roundings of ulp(|v|) besides the force error"}


def batch_accuracy(ctx, boxes, kps, threads):
    """The multi-box path (hsr_rcb_kick_batch, one persistent launch) on the
    boxes with zeroed velocities, every box checked by _oracle_check; the
    worst box's errors are reported."""
    O = _oracle()
    zs = [_zero_v(b.copy()) for b in boxes]
    ctx.rcb_kick_batch(zs, kps)
    rows = [_oracle_check(O, z, b, k, threads)[0] for z, b, k in zip(zs, boxes, kps)]
    worst = lambda key, f: max(r[key][f] for r in rows)
    return {"boxes_checked": len(rows),
            "permutation_exact": all(r["permutation_exact"] for r in rows),
            "vs_oracle": {"rms": worst("vs_oracle", "rms"), "max": worst("vs_oracle", "max")},
            "vs_fp64": {"rms": worst("vs_fp64", "rms"), "max": worst("vs_fp64", "max")},
            "worst_of": "max over boxes"}


def vjp_accuracy(ctx, p, kp, u, xbar, threads, samples=64):
    """The VJP of the last hsr_force_fwd (tape of `p`) against the FP64 VJP
    over the same lists and FP64 central differences (h = 1e-4) at sampled
    leaf particles (samples with a pair within 2h of the cutoff skipped)."""
    O = _oracle()
    n = p.n
    perm = ctx.last_perm(n)
    idx = ctx.lists_index()
    off, cnt, ptr, e = ctx.lists()
    tree = ctx.tree()
    table = np.zeros((n + len(tree["count"]), 4), np.float32)
    table[:n] = np.stack([p.x, p.y, p.z, p.mass], 1)[perm]
    table[idx] = e.T
    del e
    xt = xbar[perm].astype(np.float64)
    ut = u[perm].astype(np.float64)
    c = float(np.float32(kp.fcoeff))
    ref = O.vjp_tab(n, table, tree["offset"], tree["count"], c, off, cnt, ptr, idx, ut)
    inleaf = np.concatenate([np.arange(o, o + k) for o, k in zip(off, cnt)])
    smp = np.random.default_rng(10).choice(inleaf, samples, replace=False)
    fd, near = O.fd_tab(n, table, tree["offset"], tree["count"], c, off, cnt, ptr, idx, ut, smp,
                        h=1e-4)
    ok = ~near.astype(bool)
    rms_g = np.sqrt((fd[ok] ** 2).sum(1).mean())
    scale = np.maximum(np.linalg.norm(fd[ok], axis=1), rms_g)
    fd_err = np.linalg.norm(xt[smp][ok] - fd[ok], axis=1) / scale
    return {"vs_fp64_vjp": _err(xt, ref), "fd_max_rel": float(fd_err.max()),
            "fd_samples": int(ok.sum()), "fd_h": 1e-4,
            "fd_note": "max over samples of |xbar - fd| / max(|fd|, rms fd); target <= 1e-4"}


def hbm_roofline(traffic, ms):
    """The pair kernel against the measured HBM copy bandwidth (the file the
    pool writes at the repository root), from the profiled DRAM bytes per
    launch: how far the kernel is from being memory-bound."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peak = float(json.load(f)["hbm_gbs"])
        src = "measured (MEASURED_PEAKS.json hbm_gbs)"
    except (OSError, KeyError, ValueError):
        peak, src = 6800.0, "fallback (6.8 TB/s)"
    if not traffic:
        return None
    achieved = traffic / (ms * 1e-3) / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "traffic": traffic, "peak_source": src}


def pinned_copy(p):
    """The particle set in page-locked host memory (torch's pinned allocator,
    seen as numpy arrays)."""
    import torch
    arrs = []
    for k in synth.FIELDS:
        a = getattr(p, k)
        t = torch.empty(a.shape, dtype=getattr(torch, str(a.dtype)) if a.dtype != np.uint16
                        else torch.int16, pin_memory=True)
        v = t.numpy().view(a.dtype)
        v[...] = a
        arrs.append(v)
    q = synth.Particles(*arrs, nglt=p.nglt, meta=dict(p.meta))
    q._pinned = True
    return q


def refill(q, p):
    for k in synth.FIELDS:
        np.copyto(getattr(q, k), getattr(p, k))


def treepm_section(ctx, p0, kp, args, device: int, cpu: bool):
    """The PM kick (hsr_pm_kick) on device-resident arrays of the bench box,
    double and single precision, and one TreePM step (hsr_treepm_step: PM
    half kick, 5 short-range sub-cycles, PM kick) end to end from host
    arrays; with the numpy restatement of the PM kick timed on the host."""
    import torch
    import hsr
    import treepm
    ng, ngo = p0.meta["ng"], p0.meta["ngo"]
    dev = torch.device("cuda", device)
    t = [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in (p0.x, p0.y, p0.z, p0.vx,
                                                                     p0.vy, p0.vz)]
    torch.cuda.synchronize()
    ts = synth.stepper()
    kick = {}
    for name, prec in (("f64", hsr.PM_F64), ("f32", hsr.PM_F32)):
        prm = treepm.pm_params(ts, 0.5, ng, ngo, precision=prec)
        for _ in range(3):
            ctx.pm_kick_device(*t, prm)
        rows = [ctx.pm_kick_device(*t, prm) for _ in range(max(3, args.steps))]
        med = {k: float(np.median([r[k] for r in rows]))
               for k in ("t_deposit_ms", "t_solve_ms", "t_interp_ms")}
        dev_ms = med["t_deposit_ms"] + med["t_solve_ms"] + med["t_interp_ms"]
        v = [a.copy() for a in (p0.vx, p0.vy, p0.vz)]
        ctx.pm_kick(p0.x, p0.y, p0.z, *v, prm)
        e2e = []
        for _ in range(3):
            v = [a.copy() for a in (p0.vx, p0.vy, p0.vz)]
            t0 = time.perf_counter()
            ctx.pm_kick(p0.x, p0.y, p0.z, *v, prm)
            e2e.append(time.perf_counter() - t0)
        hs = ctx.pm_stats()
        kick[name] = {**{k: round(v, 4) for k, v in med.items()}, "device_ms": round(dev_ms, 4),
                      "particles_per_s": p0.n / (dev_ms * 1e-3),
                      "e2e_ms": round(1e3 * min(e2e), 4), "h2d_bytes": hs["h2d_bytes"],
                      "d2h_bytes": hs["d2h_bytes"], "kernel_launches": rows[-1]["kernel_launches"],
                      "fft_execs": rows[-1]["fft_execs"]}
    del t
    # the short-range sub-cycles alone (Particles::subCycle): s/substep
    nsub = 5
    ts_mid = treepm.plan(50.0, 10.0, 10)[0].mid
    kp_sub = dataclasses.replace(kp, fcoeff=float(synth.kick_coefficient(ts_mid, nsub)))
    tau_sub = float(synth.stream_tau(ts_mid, nsub))
    ctx.subcycle(p0.copy(), kp_sub, nsub, p0.nglt, ts_mid.alpha, ts_mid.pp, tau_sub, ts_mid.adot)
    sub_runs = []
    for _ in range(2):
        q = p0.copy()
        t0 = time.perf_counter()
        sst, _ = ctx.subcycle(q, kp_sub, nsub, p0.nglt, ts_mid.alpha, ts_mid.pp, tau_sub,
                              ts_mid.adot)
        sub_runs.append((time.perf_counter() - t0, sst))
    sub_wall, sst = min(sub_runs, key=lambda a: a[0])
    subcycle = {"nsub": nsub, "s_per_substep": sub_wall / nsub, "s_total": sub_wall,
                "pairs_per_substep": sst["pairs"] / nsub,
                "tree_build_ms": sst["t_build_ms"], "lists_ms": sst["t_walk_ms"],
                "force_ms": sst["t_force_ms"],
                "note": "hsr_subcycle from host arrays: 5 x (map1, resort, kick, map1) with the "
                        "arrays resident, copies in and out once"}
    # one step of the loop: the first step of a run has both PM kicks
    sp = treepm.plan(50.0, 10.0, 10)[0]
    T = treepm.step_params(sp, kp, nsub, ng, ngo, p0.nglt)
    treepm.step(ctx, p0.copy(), T)
    steps = []
    for _ in range(2):
        q = p0.copy()
        t0 = time.perf_counter()
        r = treepm.step(ctx, q, T)
        steps.append((time.perf_counter() - t0, r))
    wall, r = min(steps, key=lambda a: a[0])
    out = {"n_side": ng, "n_particles": p0.n, "pm_kick": kick, "subcycle": subcycle,
           "step": {"s_per_step": wall, "sub_cycles": nsub, "pm_kicks": 2,
                    "sr_tree_build_ms": r["sr"]["t_build_ms"], "sr_lists_ms": r["sr"]["t_walk_ms"],
                    "sr_force_ms": r["sr"]["t_force_ms"], "sr_pairs": r["sr"]["pairs"],
                    "pm_deposit_ms": r["pm"]["t_deposit_ms"], "pm_solve_ms": r["pm"]["t_solve_ms"],
                    "pm_interp_ms": r["pm"]["t_interp_ms"],
                    "h2d_bytes": r["sr"]["h2d_bytes"], "d2h_bytes": r["sr"]["d2h_bytes"]},
           "note": "PM kick: deposit + FFT solve + inverse CIC on the whole box; step: "
                   "driver_hires.cxx's loop body (PM half kick, subCycle, PM kick)"}
    if cpu:
        import pm_oracle
        t0 = time.perf_counter()
        pm_oracle.pm_kick(p0.x, p0.y, p0.z, p0.vx, p0.vy, p0.vz, ng, ngo, 1.0, 1.0, 1e-3)
        sec = time.perf_counter() - t0
        out["pm_cpu_baseline"] = {"value": p0.n / sec, "unit": "particles/s", "cores": 1,
                                  "kind": "port", "seconds": sec,
                                  "sample": f"one PM kick of the {ng}^3 box, numpy restatement "
                                            "(float64, one thread; the reference's PM needs FFTW "
                                            "and MPI)"}
    return out


def run_reference_arm(args, world, rank):
    if rank != 0:
        return 0
    p, kp, cfg = workload(args.ng, args.nd, world)
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_baseline(p, kp, args.cpu_slab / 4, threads)
    runs = [cpu_baseline(p, kp, args.cpu_slab / 4, threads) for _ in range(args.steps)]
    pairs = sum(r["pairs"] for r in runs)
    secs = sum(r["seconds"] for r in runs)
    value = pairs / secs
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * secs / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "impl": "reference",
            "data": "synthetic (seeded Zel'dovich lattice with overload ghosts)", "config": cfg,
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": runs[0]["sample"]},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse_args()
    world, rank, local = dist_init()
    if args.impl == "reference":
        return run_reference_arm(args, world, rank)

    import build_ext
    build_ext.build()
    import hsr

    kernel = {"auto": hsr.KERNEL_AUTO, "plain": hsr.KERNEL_PLAIN, "batched": hsr.KERNEL_BATCHED}[args.kernel]
    p0, kp, cfg = workload(args.ng, args.nd, world)
    ctx = hsr.Context(local)
    check = rank == 0 and not args.no_accuracy
    threads = os.cpu_count() or 1

    # ---- launch shape: time every shape on this workload, keep the fastest ----
    tune_rows = None
    if kernel == hsr.KERNEL_AUTO:
        ctx.rcb_kick(p0.copy(), kp, kernel=kernel)
        tune_rows = [{k: (round(v, 4) if k == "ms" else v) for k, v in r.items()}
                     for r in ctx.autotune(iters=3)]
    shape = ctx.get_tune()

    # ---- end to end through the C ABI (pinned host arrays in, host arrays out) ----
    q = pinned_copy(p0)
    for _ in range(max(args.warmup, 3)):
        refill(q, p0)
        ctx.rcb_kick(q, kp, kernel=kernel)
    e2e_secs, st = [], None
    barrier(world)
    for _ in range(args.steps):
        refill(q, p0)  # the step's inputs, outside the timed region
        t0 = time.perf_counter()
        st = ctx.rcb_kick(q, kp, kernel=kernel)
        e2e_secs.append(time.perf_counter() - t0)
    e2e_t = max_over_ranks(world, sum(e2e_secs))
    perm_timed = ctx.last_perm(p0.n)  # tree order of the last timed kick
    pairs = st["pairs"]
    in_cutoff = ctx.pairs_in_cutoff()
    h2d, d2h = st["h2d_bytes"], st["d2h_bytes"]

    evaluated = st["evaluated_pairs"]

    # ---- device-resident step: pair kernel on the resident lists ----
    ctx.bench_pairs(max(args.warmup, 3), kernel=kernel)
    barrier(world)
    with ClockSampler(local) as cs:
        ms = ctx.bench_pairs(args.steps, kernel=kernel)
    ms = max_over_ranks(world, ms)
    value = world * pairs / (ms * 1e-3)
    # the other kernel variant on the same resident lists, for comparison
    other = hsr.KERNEL_PLAIN if kernel != hsr.KERNEL_PLAIN else hsr.KERNEL_AUTO
    ms_plain = ctx.bench_pairs(max(2, args.steps // 2), kernel=hsr.KERNEL_PLAIN) \
        if kernel != hsr.KERNEL_PLAIN else ms

    ms_graph = ctx.bench_pairs_graph(max(2, args.steps // 2))

    # ---- adjoint: forward + VJP of the same workload ----
    ctx.force_fwd(p0.x, p0.y, p0.z, p0.mass, kp)
    u = np.random.default_rng(1).standard_normal((p0.n, 3)).astype(np.float32)
    ctx.force_vjp(u)
    vjp_ms = []
    for _ in range(3):
        xbar = ctx.force_vjp(u)
        vjp_ms.append(ctx.stats()["t_force_ms"])
    vjp_ms = min(vjp_ms)
    vjp_acc = vjp_accuracy(ctx, p0, kp, u, xbar, threads) if check else None
    del xbar

    peak = ctx.fp32_peak_tflops()
    achieved = evaluated * FLOPS_PER_PAIR / (ms * 1e-3) / 1e12

    # ---- several boxes in one persistent launch (8 boxes of 96^3) ----
    multibox = None
    if args.multibox > 0:
        boxes = [synth.zeldovich_box(96, z=50.0, seed=100 + b) for b in range(args.multibox)]
        kpb = [synth.kick_params(b, nd=args.nd) for b in boxes]
        # pinned host arrays, refilled outside the timed calls (as the
        # single-box end-to-end kick)
        qb = [pinned_copy(b) for b in boxes]
        walls = []
        for r in range(3 + max(3, args.steps // 2)):
            for q, b in zip(qb, boxes):
                refill(q, b)
            t0 = time.perf_counter()
            stb = ctx.rcb_kick_batch(qb, kpb)
            if r >= 3:
                walls.append(time.perf_counter() - t0)
        wall_b = float(np.median(walls))
        del qb
        ms_b = ctx.bench_pairs(max(3, args.steps // 2))
        ms_bg = ctx.bench_pairs_graph(max(3, args.steps // 2))
        multibox = {"boxes": args.multibox, "n_side": 96, "pairs": stb["pairs"],
                    "one_launch_ms": ms_b, "one_launch_graph_ms": ms_bg,
                    "pairs_per_s": stb["pairs"] / (ms_b * 1e-3),
                    "e2e_s": wall_b, "e2e_pairs_per_s": stb["pairs"] / wall_b}
        if check:
            multibox["accuracy"] = batch_accuracy(ctx, boxes, kpb, threads)

    # ---- multi-step adjoint: boxes of 96^3, 10 PM steps x 5 sub-cycles ----
    multistep_line = None
    if args.adjoint_boxes > 0:
        import torch
        import multistep
        nsteps, nsub, every = 10, 5, 2
        boxes = [synth.zeldovich_box(96, z=50.0, seed=300 + b) for b in range(args.adjoint_boxes)]
        kps = [synth.kick_params(b, nd=args.nd) for b in boxes]
        sched = multistep.schedule(50.0, 10.0, nsteps, nsub)
        pm = multistep.pm_schedule(50.0, 10.0, nsteps, 96, boxes[0].meta["ngo"])
        msr = multistep.MultiStep(ctx, kps, sched, nsub, checkpoint_every=every, pm=pm)
        states = [multistep.box_state(b, local) for b in boxes]
        targets = [[t.clone() for t in S.x] for S in states]  # L = sum |x_final - x_initial|^2
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        final = msr.forward([S.clone() for S in states])
        torch.cuda.synchronize()
        t_fwd = time.perf_counter() - t0
        xbars, vbars, loss = multistep.position_loss_cotangent(final, targets)
        del final
        k0, q0 = msr.total_kicks()
        c0 = msr.batch_calls
        t0 = time.perf_counter()
        grads = msr.adjoint(states, xbars, vbars)
        torch.cuda.synchronize()
        t_adj = time.perf_counter() - t0
        k1, q1 = msr.total_kicks()
        gnorm = float(sum(float((g.double() ** 2).sum()) for gx, _ in grads for g in gx)) ** 0.5
        nsc = args.adjoint_boxes * nsteps * nsub
        multistep_line = {
            "boxes": args.adjoint_boxes, "n_side": 96, "n_particles_per_box": boxes[0].n,
            "pm_steps": nsteps, "sub_cycles": nsub, "checkpoint_every": every,
            "forward_s": t_fwd, "adjoint_s": t_adj,
            "s_per_substep_forward": t_fwd / nsc, "s_per_substep_adjoint": t_adj / nsc,
            "kicks_in_adjoint": k1 - k0, "pm_kicks_in_adjoint": q1 - q0,
            "multi_box_calls_in_adjoint": msr.batch_calls - c0,
            "loss": loss, "grad_norm": gnorm,
            "note": "all boxes in lockstep: every sub-cycle's kicks of the 8 boxes in one "
                    "persistent launch (hsr_force_kick_batch, replayed as a CUDA graph), the "
                    "reverse pass's tapes and VJPs of the 8 boxes one multi-box call each "
                    "(hsr_force_fwd_batch + hsr_force_vjp_batch); PM kicks (half opening the "
                    "first step, one closing each step) around 5 short-range sub-cycles (map1, "
                    "kick, map1); L = sum |x_final - x_initial|^2, gradient w.r.t. the initial "
                    "positions"}
        del states, grads, xbars, vbars, targets

    # ---- clustered set: leaf size x launch shape sweep ----
    clustered = None
    if args.clustered > 0:
        import autotune
        pc = synth.clustered_box(args.clustered)
        t0 = time.perf_counter()
        sw = autotune.sweep(ctx, pc, nds=(64, 128, 256), iters=2)
        acc_c = None
        if check:
            # the best leaf size and shape (set on the context by the sweep)
            kpc = synth.kick_params(pc, nd=sw["best"]["nd"])
            acc_c = kick_accuracy(ctx, pc, kpc, threads,
                                  oracle_max_x=kpc.min_force[0] + 6.0)[0]
        clustered = {"n_side": args.clustered, "n_particles": pc.n,
                     "halos": pc.meta["nhalo"], "sweep_s": time.perf_counter() - t0,
                     "best": sw["best"], "accuracy": acc_c,
                     "rows": [{"nd": r["nd"], "pairs": r["pairs"],
                               "list_entries": r["list_entries"],
                               "tree_build_ms": round(r["tree_build_ms"], 3),
                               "lists_ms": round(r["lists_ms"], 3),
                               "best_shape": r["best_shape"],
                               "best_kernel_ms": round(r["best_kernel_ms"], 4),
                               "pairs_per_s": r["pairs_per_s"],
                               "shape_ms": {(f"{q['kernel']}-{q['leaf_threads']}"
                                             if q["kernel"] == "plain"
                                             else f"batched-g{q['group']}"): round(q["ms"], 4)
                                            for q in r["shapes"]}}
                              for r in sw["rows"]]}
        del pc

    # ---- long-range PM kick and one whole TreePM step on the bench box ----
    treepm_line = None
    if args.treepm:
        treepm_line = treepm_section(ctx, p0, kp, args, local,
                                     cpu=(rank == 0 and world == 1 and not args.no_cpu_baseline))

    cpu, ora_out = None, None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(p0, kp, args.cpu_slab, os.cpu_count() or 1)
        ora_out = cpu["_out"] if args.cpu_slab >= 1.0 else None
        cpu = {k: v for k, v in cpu.items() if k not in ("seconds", "pairs", "_out")}
        # per-core figure: one thread on a twentieth of the slab
        one = cpu_baseline(p0, kp, args.cpu_slab / 20, 1)
        cpu["per_core"] = {k: one[k] for k in ("value", "unit", "cores", "sample")}

    accuracy = None
    if check:
        accuracy, sel0, a64_0 = kick_accuracy(ctx, p0, kp, threads)
        accuracy["note"] = ("the kick of the bench box with its velocities zeroed (the output is "
                            "then the kick itself) through hsr_rcb_kick, against the oracle "
                            "on the same input and FP64 over the oracle's lists; " + ACC_NOTE)
        if ora_out is not None:
            accuracy["timed_output"] = timed_output_check(p0, q, perm_timed, ora_out, sel0, a64_0)
        del sel0, a64_0
    del ora_out

    if rank == 0:
        clocks = cs.summary()
        sms = fp32_theoretical = None
        try:
            import torch
            sms = torch.cuda.get_device_properties(local).multi_processor_count
            if clocks.get("sm_mhz"):
                # 128 FP32 lanes per SM, one FMA (2 flops) per lane per clock
                fp32_theoretical = sms * 128 * 2 * clocks["sm_mhz"] * 1e6 / 1e12
        except Exception:
            pass
        peak_used = min(v for v in (peak, fp32_theoretical) if v) if (peak or fp32_theoretical) \
            else None
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded Zel'dovich lattice with overload ghosts)",
            "config": cfg,
            "counts": {"pairs_per_step": pairs, "evaluated_pairs_per_step": evaluated,
                       "in_cutoff_pairs_per_step": in_cutoff,
                       "in_cutoff_over_evaluated": in_cutoff / evaluated if evaluated else None,
                       "evaluated_pairs_per_s": world * evaluated / (ms * 1e-3),
                       "processed_leaves": st["processed_leaves"],
                       "list_entries": st["list_entries"], "kernel": args.kernel,
                       "launch_shape": shape,
                       "value_basis": "value counts the listed pairs (what nbody1 iterates); the "
                                      "kernel evaluates evaluated_pairs_per_step of them, the "
                                      "rest are exactly zero by the cutoff"},
            "accuracy": accuracy,
            "plain_vs_batched": {"plain_pairs_per_s": world * pairs / (ms_plain * 1e-3),
                                 "plain_ms": ms_plain, "selected_ms": ms,
                                 "selected_graph_ms": ms_graph,
                                 "speedup": ms_plain / ms},
            "adjoint": {"vjp_ms": vjp_ms, "vjp_pairs_per_s": pairs / (vjp_ms * 1e-3),
                        "vjp_over_forward": vjp_ms / ms, "accuracy": vjp_acc},
            "multibox": multibox,
            "clustered": clustered,
            "multistep_adjoint": multistep_line,
            "treepm": treepm_line,
            "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak_used,
                         "unit": "TFLOP/s",
                         "frac": achieved / peak_used if peak_used else None,
                         "traffic": profiled_traffic(cfg["workload"], shape),
                         "traffic_source": TRAFFIC_NOTE,
                         "peak_probe": peak, "peak_sm_clock_bound": fp32_theoretical, "sms": sms,
                         "peak_source": "the lower of the FFMA-chain probe on this device "
                                        "(hsr_probe_fp32_peak) and SMs x 128 lanes x 2 flops x "
                                        "median SM clock of the timed region",
                         "flops_per_pair": FLOPS_PER_PAIR,
                         "pairs_basis": "evaluated pairs (after the box test)"},
            "roofline_hbm": hbm_roofline(profiled_traffic(cfg["workload"], shape), ms),
            "cpu_baseline": cpu,
            "e2e": {"value": world * pairs * args.steps / e2e_t, "unit": UNIT,
                    "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                    "s_per_kick": e2e_t / args.steps,
                    "tree_build_ms": st["t_build_ms"], "lists_ms": st["t_walk_ms"],
                    "h2d_ms": st["t_h2d_ms"], "force_ms": st["t_force_ms"],
                    "d2h_ms": st["t_d2h_ms"], "kernel_launches": st["kernel_launches"]},
            "autotune": tune_rows,
            "gpu_launches": args.steps,
            "clocks": clocks,
        }
        print(json.dumps(line), flush=True)
    ctx.close()
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
