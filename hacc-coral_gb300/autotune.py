"""Leaf size x launch shape sweep of the short-range kick, with a per-GPU cache.

For each leaf size nd (RCBForceTree's `nd`, the largest leaf) the sweep kicks
the particle set once through the C ABI (device tree build, lists, kick),
then times every launch shape of the pair kernels on that tree with
hsr_autotune: the plain kernel with 32, 64 and 128 threads per leaf and the
batched kernel with groups of 16 and 32 particles.  The leaf size changes the
tree, the lists and so the pair set (the reference takes it from the caller:
`nd`, src/halo_finder/RCBForceTree.h:96-124); the launch shape changes only
the FP32 summation order.

The best entry (least device time of build + lists + pair kernel) is stored
in a JSON cache keyed by the GPU's name and a workload label, so a later run
can apply it without sweeping (`apply_cached`).

    python hacc-coral_gb300/autotune.py --workload clustered --ng 256
"""
from __future__ import annotations

import argparse
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:
    sys.path.insert(0, HERE)

import hsr  # noqa: E402
import synth  # noqa: E402

DEFAULT_NDS = (64, 128, 256)
CACHE_ENV = "HACC_SR_TUNE_CACHE"


def cache_path() -> str:
    return os.environ.get(CACHE_ENV) or os.path.join(HERE, ".tune", "shapes.json")


def gpu_name(device: int = 0) -> str:
    try:
        import torch
        if torch.cuda.is_available():
            return torch.cuda.get_device_name(device)
    except Exception:  # torch is optional here
        pass
    return f"cuda:{device}"


def sweep(ctx: hsr.Context, p: synth.Particles, nds=DEFAULT_NDS, iters: int = 3,
          flush_l2: bool = True, **kick_kw) -> dict:
    """Runs the sweep on particle set `p` (not modified).  kick_kw goes to
    synth.kick_params (rsm, open_angle, fcoeff, tdpts, ...)."""
    rows = []
    for nd in nds:
        kp = synth.kick_params(p, nd=nd, **kick_kw)
        # the first kick sizes the buffers for this leaf size; the second is timed
        ctx.rcb_kick(p.copy(), kp, kernel=hsr.KERNEL_AUTO)
        st = ctx.rcb_kick(p.copy(), kp, kernel=hsr.KERNEL_AUTO)
        shapes = ctx.autotune(iters=iters, flush_l2=flush_l2)
        best = min(shapes, key=lambda r: r["ms"])
        rows.append({
            "nd": nd, "pairs": st["pairs"], "list_entries": st["list_entries"],
            "processed_leaves": st["processed_leaves"], "tree_build_ms": st["t_build_ms"],
            "lists_ms": st["t_walk_ms"], "shapes": shapes,
            "best_shape": {k: best[k] for k in ("kernel", "leaf_threads", "group")},
            "best_kernel_ms": best["ms"],
            "device_ms": st["t_build_ms"] + st["t_walk_ms"] + best["ms"],
            "pairs_per_s": st["pairs"] / (best["ms"] * 1e-3),
        })
    best = min(rows, key=lambda r: r["device_ms"])
    return {"rows": rows, "best": {"nd": best["nd"], **best["best_shape"],
                                   "device_ms": best["device_ms"]}}


def save(key: str, result: dict, path: str | None = None) -> str:
    path = path or cache_path()
    os.makedirs(os.path.dirname(path), exist_ok=True)
    data = {}
    if os.path.exists(path):
        with open(path) as f:
            try:
                data = json.load(f)
            except json.JSONDecodeError:
                data = {}
    data[key] = result["best"]
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    os.replace(tmp, path)
    return path


def load(key: str, path: str | None = None) -> dict | None:
    path = path or cache_path()
    if not os.path.exists(path):
        return None
    with open(path) as f:
        try:
            return json.load(f).get(key)
        except json.JSONDecodeError:
            return None


def cache_key(workload: str, device: int = 0) -> str:
    return f"{gpu_name(device)}|{workload}"


def apply_cached(ctx: hsr.Context, workload: str, device: int = 0,
                 path: str | None = None) -> dict | None:
    """Sets the context's launch shape from the cache; returns the entry
    (with its leaf size) or None when the workload was never swept."""
    e = load(cache_key(workload, device), path)
    if e:
        ctx.set_tune(e["kernel"], e["leaf_threads"], e["group"])
    return e


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--workload", choices=["zeldovich", "clustered"], default="clustered")
    ap.add_argument("--ng", type=int, default=256)
    ap.add_argument("--nd", type=int, nargs="*", default=list(DEFAULT_NDS))
    ap.add_argument("--iters", type=int, default=3)
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--no-save", action="store_true")
    a = ap.parse_args(argv)
    p = synth.clustered_box(a.ng) if a.workload == "clustered" else synth.zeldovich_box(a.ng)
    label = f"{a.workload}{a.ng}"
    with hsr.Context(a.device) as ctx:
        res = sweep(ctx, p, nds=a.nd, iters=a.iters)
    res["workload"] = label
    if not a.no_save:
        res["cache"] = save(cache_key(label, a.device), res)
    print(json.dumps(res))
    return 0


if __name__ == "__main__":
    sys.exit(main())
