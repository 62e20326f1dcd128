"""Runs the short-range kick of one synthetic workload a few times through the
C ABI and prints each call's phase statistics as JSON: a fixed, short launch
sequence for profilers (ncu's launch lists and kernel captures).

    python profile_kick.py --workload zeldovich --ng 128 --reps 2
    python profile_kick.py --workload clustered --ng 256 --shape batched-32
    python profile_kick.py --ng 128 --reps 2 --pm f64   # + the PM kick
    python profile_kick.py --ng 128 --reps 3 --vjp      # + force forward and its VJP
"""
from __future__ import annotations

import argparse
import json
import os
import sys

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "hacc-coral_gb300")
if HERE not in sys.path:
    sys.path.insert(0, HERE)

import hsr  # noqa: E402
import synth  # noqa: E402

KEYS = ("t_total_ms", "t_h2d_ms", "t_build_ms", "t_walk_ms", "t_force_ms", "t_d2h_ms",
        "n", "nodes", "processed_leaves", "list_entries", "pairs", "evaluated_pairs",
        "work_items", "cm_fallbacks", "kernel_launches")


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--workload", choices=["zeldovich", "clustered"], default="zeldovich")
    ap.add_argument("--ng", type=int, default=128)
    ap.add_argument("--z", type=float, default=50.0)
    ap.add_argument("--nd", type=int, default=128)
    ap.add_argument("--reps", type=int, default=2)
    ap.add_argument("--shape", default="batched-32",
                    help="plain-32|plain-64|plain-128|batched-16|batched-32")
    ap.add_argument("--pm", choices=["none", "f64", "f32"], default="none",
                    help="also run the long-range PM kick (hsr_pm_kick) after each short-range kick")
    ap.add_argument("--vjp", action="store_true",
                    help="also run the force forward map on the kick's input and its VJP "
                         "(hsr_force_fwd, hsr_force_vjp) with a fixed random cotangent")
    ap.add_argument("--device", type=int, default=0)
    a = ap.parse_args(argv)
    kind, num = a.shape.split("-")
    p = synth.clustered_box(a.ng) if a.workload == "clustered" else synth.zeldovich_box(a.ng, z=a.z)
    kp = synth.kick_params(p, nd=a.nd)
    with hsr.Context(a.device) as ctx:
        if kind == "plain":
            ctx.set_tune("plain", int(num), 32)
        else:
            ctx.set_tune("batched", 128, int(num))
        for r in range(a.reps):
            q = p.copy()
            st = ctx.rcb_kick(q, kp, kernel=hsr.KERNEL_AUTO)
            print(json.dumps({"rep": r, "workload": f"{a.workload}{a.ng}", "shape": a.shape,
                              **{k: st[k] for k in KEYS}}), flush=True)
            if a.vjp:
                import numpy as np
                ctx.force_fwd(p.x, p.y, p.z, p.mass, kp)
                fwd = ctx.stats()["t_force_ms"]
                u = np.random.default_rng(1).standard_normal((p.n, 3)).astype(np.float32)
                ctx.force_vjp(u)
                vjp = ctx.stats()["t_force_ms"]
                print(json.dumps({"rep": r, "forward_ms": fwd, "vjp_ms": vjp,
                                  "vjp_over_forward": vjp / fwd}), flush=True)
            if a.pm != "none":
                prm = hsr.pm_params(a.ng, p.meta["ngo"], 1.0, 1.0, 1e-3,
                                    hsr.PM_F64 if a.pm == "f64" else hsr.PM_F32)
                ps = ctx.pm_kick(q.x, q.y, q.z, q.vx, q.vy, q.vz, prm)
                print(json.dumps({"rep": r, "pm": a.pm, **ps}), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
