"""Launch shapes of the pair kernels (hsr_set_tune / hsr_autotune).

Every shape evaluates the same pair set as the reference's nbody1: plain with
32, 64 or 128 threads per leaf, batched with groups of 16 or 32 particles.
Forces are compared with the oracle within RMS_TOL / MAX_TOL; the tree, the
permutation and the lists do not depend on the shape and stay bit-exact.
"""
import numpy as np
import pytest

import hsr
import synth
from hsr_testutil import MAX_TOL, RMS_TOL, force_errors, vel

SHAPES = [("plain", 32, 32), ("plain", 64, 32), ("plain", 128, 32),
          ("batched", 128, 16), ("batched", 128, 32)]
EXACT = ("x", "y", "z", "mass", "phi", "id", "mask")


def _zero_v(p):
    p.vx[:] = 0
    p.vy[:] = 0
    p.vz[:] = 0
    return p


@pytest.fixture(scope="module")
def tctx(hsr_lib):
    c = hsr.Context(0)
    yield c
    c.close()


@pytest.mark.gpu
def test_tune_rejects_bad_shapes(tctx):
    for bad in [("plain", 96, 32), ("batched", 128, 8), ("plain", 128, 24)]:
        with pytest.raises(hsr.HsrError):
            tctx.set_tune(*bad)
    lib = hsr.load()
    t = hsr.HsrTune(hsr.KERNEL_AUTO, 128, 32, 0)
    assert lib.hsr_set_tune(tctx.h, t) == 1  # HSR_ERR_ARG
    assert tctx.get_tune() == {"kernel": "batched", "leaf_threads": 128, "group": 32}


@pytest.mark.gpu
@pytest.mark.parametrize("shape", SHAPES, ids=lambda s: f"{s[0]}-{s[1]}-{s[2]}")
@pytest.mark.parametrize("law", [hsr.LAW_POLY6, hsr.LAW_POLY5_STEP16])
def test_shape_matches_oracle(tctx, oracle_lib, shape, law):
    kernel, threads, group = shape
    p = _zero_v(synth.zeldovich_box(32, z=10.0, seed=11))
    kp = synth.kick_params(p, nd=128, fcoeff=1.0)
    kp.law = law
    q = p.copy()
    tctx.set_tune(kernel, threads, group)
    assert tctx.get_tune() == {"kernel": kernel, "leaf_threads": threads, "group": group}
    st = tctx.rcb_kick(p, kp, kernel=hsr.KERNEL_AUTO)
    r = oracle_lib.rcb_run(q, kp, keep_lists=True, nthreads=0)
    for k in EXACT:
        assert np.array_equal(getattr(p, k).view(np.uint8), getattr(q, k).view(np.uint8)), k
    off, cnt, _ = r.leaves()
    sel = np.concatenate([np.arange(o, o + c) for o, c in zip(off, cnt)])
    rms, mx = force_errors(vel(p)[sel], vel(q)[sel])
    assert rms <= RMS_TOL and mx <= MAX_TOL, (shape, rms, mx)
    assert st["pairs"] == r.stats["pairs"]
    if kernel == "batched":
        assert 0 < st["evaluated_pairs"] <= st["pairs"]
        # groups of `group` particles: one item per group and list chunk
        assert st["work_items"] >= int(np.sum((cnt + group - 1) // group))


@pytest.mark.gpu
def test_group16_uneven_leaves(tctx, oracle_lib):
    """Leaves of odd sizes and odd kept-entry counts (the padding entry of the
    16-particle groups): nd = 23 on a clustered box."""
    p = _zero_v(synth.clustered_box(24, nhalo=40, seed=7))
    kp = synth.kick_params(p, nd=23, fcoeff=1.0)
    q = p.copy()
    tctx.set_tune("batched", 128, 16)
    tctx.rcb_kick(p, kp, kernel=hsr.KERNEL_AUTO)
    r = oracle_lib.rcb_run(q, kp, keep_lists=True, nthreads=0)
    off, cnt, _ = r.leaves()
    sel = np.concatenate([np.arange(o, o + c) for o, c in zip(off, cnt)])
    rms, mx = force_errors(vel(p)[sel], vel(q)[sel])
    assert rms <= RMS_TOL and mx <= MAX_TOL, (rms, mx)


@pytest.mark.gpu
def test_multibox_group16(tctx, oracle_lib):
    boxes = [_zero_v(synth.zeldovich_box(24, seed=40 + b)) for b in range(3)]
    kps = [synth.kick_params(b, nd=nd, fcoeff=1.0) for b, nd in zip(boxes, (32, 64, 128))]
    refs = [b.copy() for b in boxes]
    tctx.set_tune("batched", 128, 16)
    tctx.rcb_kick_batch(boxes, kps)
    for b, q, kp in zip(boxes, refs, kps):
        r = oracle_lib.rcb_run(q, kp, keep_lists=True, nthreads=0)
        off, cnt, _ = r.leaves()
        sel = np.concatenate([np.arange(o, o + c) for o, c in zip(off, cnt)])
        rms, mx = force_errors(vel(b)[sel], vel(q)[sel])
        assert rms <= RMS_TOL and mx <= MAX_TOL, (rms, mx)


@pytest.mark.gpu
def test_autotune_picks_fastest_and_kicks(tctx, oracle_lib):
    p = _zero_v(synth.zeldovich_box(32, seed=21))
    kp = synth.kick_params(p, nd=128, fcoeff=1.0)
    tctx.set_tune("batched", 128, 32)
    tctx.rcb_kick(p.copy(), kp)
    rows = tctx.autotune(iters=2, flush_l2=False)
    assert len(rows) == 5
    assert {(r["kernel"], r["leaf_threads"] if r["kernel"] == "plain" else r["group"])
            for r in rows} == {("plain", 32), ("plain", 64), ("plain", 128), ("batched", 16),
                               ("batched", 32)}
    assert all(r["ms"] > 0 for r in rows)
    best = min(rows, key=lambda r: r["ms"])
    t = tctx.get_tune()
    assert t["kernel"] == best["kernel"]
    # the tuned shape kicks correctly
    q = p.copy()
    tctx.rcb_kick(p, kp, kernel=hsr.KERNEL_AUTO)
    r = oracle_lib.rcb_run(q, kp, keep_lists=True, nthreads=0)
    off, cnt, _ = r.leaves()
    sel = np.concatenate([np.arange(o, o + c) for o, c in zip(off, cnt)])
    rms, mx = force_errors(vel(p)[sel], vel(q)[sel])
    assert rms <= RMS_TOL and mx <= MAX_TOL, (rms, mx)
    tctx.set_tune("batched", 128, 32)


@pytest.mark.gpu
def test_autotune_needs_device_kick(hsr_lib):
    c = hsr.Context(0)
    try:
        with pytest.raises(hsr.HsrError):
            c.autotune(iters=1)
    finally:
        c.close()


@pytest.mark.gpu
def test_adjoint_under_group16_context(tctx, hsr_lib):
    """A context tuned to groups of 16 still runs the forward/VJP pair on its
    own 32-particle items: same dv and xbar as a default context."""
    p = synth.zeldovich_box(24, z=10.0, seed=17)
    kp = synth.kick_params(p, nd=64, fcoeff=1.0)
    u = np.random.default_rng(3).standard_normal((p.n, 3)).astype(np.float32)
    tctx.set_tune("batched", 128, 16)
    dv16 = tctx.force_fwd(p.x, p.y, p.z, p.mass, kp)
    xb16 = tctx.force_vjp(u)
    tctx.set_tune("batched", 128, 32)
    with hsr.Context(0) as c:
        dv = c.force_fwd(p.x, p.y, p.z, p.mass, kp)
        xb = c.force_vjp(u)
    rms, mx = force_errors(dv16.astype(np.float64), dv.astype(np.float64))
    assert rms <= RMS_TOL and mx <= MAX_TOL, (rms, mx)
    rms, mx = force_errors(xb16.astype(np.float64), xb.astype(np.float64))
    assert rms <= RMS_TOL and mx <= MAX_TOL, (rms, mx)
