"""Clustered particle sets (60 % uniform, 40 % in NFW halos with a -1.9 mass
function, concentration U[4, 10], virial radius 0.5-4 grid units): the
uneven-list case.  GPU kick vs the oracle at several leaf sizes, the 256^3
set on a slab of its force box (the whole tree built), and the leaf size x
launch shape sweep.
"""
import json

import numpy as np
import pytest

import autotune
import hsr
import synth
from hsr_testutil import MAX_TOL, RMS_TOL, force_errors, same_lists, vel

EXACT = ("x", "y", "z", "mass", "phi", "id", "mask")


def _zero_v(p):
    p.vx[:] = 0
    p.vy[:] = 0
    p.vz[:] = 0
    return p


def _check_vs_oracle(ctx, oracle_lib, p, kp, lists=True):
    q = p.copy()
    st = ctx.rcb_kick(p, kp, kernel=hsr.KERNEL_AUTO)
    r = oracle_lib.rcb_run(q, kp, keep_lists=True, nthreads=0)
    for k in EXACT:
        assert np.array_equal(getattr(p, k).view(np.uint8), getattr(q, k).view(np.uint8)), k
    off, cnt, ptr = r.leaves()
    assert len(off) > 0
    sel = np.concatenate([np.arange(o, o + c) for o, c in zip(off, cnt)])
    rms, mx = force_errors(vel(p)[sel], vel(q)[sel])
    assert rms <= RMS_TOL and mx <= MAX_TOL, (kp.nd, rms, mx)
    if lists:
        goff, gcnt, gptr, ge = ctx.lists()
        assert same_lists(goff, gcnt, gptr, ge, off, cnt, ptr, r.entries())
    assert st["pairs"] == r.stats["pairs"]
    return st, r


def test_cache_roundtrip(tmp_path):
    path = str(tmp_path / "shapes.json")
    res = {"best": {"nd": 128, "kernel": "batched", "leaf_threads": 128, "group": 16,
                    "device_ms": 1.0}}
    autotune.save("GB300|clustered256", res, path)
    autotune.save("GB300|zeldovich128", {"best": dict(res["best"], group=32)}, path)
    assert autotune.load("GB300|clustered256", path)["group"] == 16
    assert autotune.load("GB300|zeldovich128", path)["group"] == 32
    assert autotune.load("other", path) is None
    with open(path) as f:
        assert set(json.load(f)) == {"GB300|clustered256", "GB300|zeldovich128"}


@pytest.mark.gpu
@pytest.mark.parametrize("nd", [64, 128, 256])
def test_clustered48_vs_oracle(ctx, oracle_lib, nd):
    p = _zero_v(synth.clustered_box(48, nhalo=120, seed=9))
    kp = synth.kick_params(p, nd=nd, fcoeff=1.0)
    st, r = _check_vs_oracle(ctx, oracle_lib, p, kp)
    # halo leaves have far longer lists than field leaves
    _, cnt, ptr = r.leaves()
    ln = np.diff(ptr)
    assert ln.max() > 2.5 * np.median(ln)


@pytest.mark.gpu
def test_clustered256_slab_vs_oracle(ctx, oracle_lib, monkeypatch):
    """The full 256^3 clustered set (18.8 M particles with ghosts): the whole
    tree and permutation bit-exact, forces of the leaves in a slab of the
    force box (x in [3.2, 9]) within tolerance of the oracle's.  Halo leaves
    there have lists of ~25 000 entries, past the reference's VMAX of 16384."""
    monkeypatch.setenv("ORA_MAX_ACTIVE_LEVELS", "5")  # the oracle's thread nesting
    p = _zero_v(synth.clustered_box(256))
    kp = synth.kick_params(p, nd=128, fcoeff=1.0)
    kp.max_force = (9.0, kp.max_force[1], kp.max_force[2])
    _check_vs_oracle(ctx, oracle_lib, p, kp, lists=False)


@pytest.mark.gpu
def test_sweep_clustered64(hsr_lib, tmp_path):
    p = synth.clustered_box(64)
    with hsr.Context(0) as c:
        res = autotune.sweep(c, p, nds=(64, 128, 256), iters=1, flush_l2=False)
        assert [r["nd"] for r in res["rows"]] == [64, 128, 256]
        for r in res["rows"]:
            assert len(r["shapes"]) == 5 and all(s["ms"] > 0 for s in r["shapes"])
            assert r["pairs"] > 0
        b = res["best"]
        assert b["nd"] in (64, 128, 256)
        path = str(tmp_path / "s.json")
        autotune.save(autotune.cache_key("clustered64"), res, path)
        c.set_tune("plain", 64, 32)
        e = autotune.apply_cached(c, "clustered64", path=path)
        assert e is not None and e["nd"] == b["nd"]
        t = c.get_tune()
        assert (t["kernel"], t["leaf_threads"], t["group"]) == (b["kernel"], b["leaf_threads"],
                                                               b["group"])
