"""The allocation-free kick (hsr_kick_lists_noalloc) through the C ABI.

It serves callers that cannot allocate device memory while they run; it keeps
its scratch in a fixed device array shared by all calls.  These tests give it
interaction lists built by the library itself and check, on two calls in a
row, that its kick equals hsr_rcb_kick's on the same particles within the
suite's FP32 force tolerance: lists of a few thousand entries, lists longer
than one work item's 8192 entries (split over items that add with atomics),
and the Step16 law.  A caller whose lists need more work items than the fixed
array holds gets HSR_ERR_ARG with its velocities untouched, and the next call
works.  The file is collected last on purpose.
"""
import numpy as np
import pytest

import hsr
import synth
from hsr_testutil import MAX_TOL, RMS_TOL, force_errors

pytestmark = pytest.mark.gpu


def _case():
    p = synth.zeldovich_box(24, z=10.0, seed=77)
    p.vx[:] = 0
    p.vy[:] = 0
    p.vz[:] = 0
    return p, synth.kick_params(p, nd=64, fcoeff=0.5)


def _dense_case():
    """40 000 particles in an 8^3 box: every list holds 9 000 to 37 000 entries."""
    p = synth.random_box(40000, 8.0, 5)
    p.vx[:] = 0
    p.vy[:] = 0
    p.vz[:] = 0
    kp = synth.kick_params(p, nd=64, fcoeff=0.5)
    kp.min_force, kp.max_force = (-1.0,) * 3, (9.0,) * 3
    return p, kp


def _device_lists(torch, p, kp):
    """The tree and lists of `p` (host-built), as device arrays a caller owns:
    table, leaf offsets, counts, list begins and lengths, entry indices; and
    the permuted particles."""
    q = p.copy()
    L = hsr.HostLists(q, kp)
    off, cnt, ptr, e = L.get()
    eidx = L.index()
    ntab = int(max(eidx.max() + 1, q.n))
    table = np.zeros((ntab, 4), np.float32)
    table[: q.n] = np.stack([q.x, q.y, q.z, q.mass], 1)
    table[eidx] = e.T
    dev = "cuda"
    arrs = (torch.from_numpy(table).to(dev), torch.from_numpy(off.astype(np.int32)).to(dev),
            torch.from_numpy(cnt.astype(np.int32)).to(dev),
            torch.from_numpy(ptr[:-1].astype(np.int64)).to(dev),
            torch.from_numpy(np.diff(ptr).astype(np.int32)).to(dev),
            torch.from_numpy(eidx.astype(np.int32)).to(dev))
    return arrs, q, np.diff(ptr)


def _check_twice(ctx, p, kp):
    torch = pytest.importorskip("torch")
    # reference result: the existing entry point (velocities in tree order)
    ref = p.copy()
    ctx.rcb_kick(ref, kp)
    v_ref = np.stack([ref.vx, ref.vy, ref.vz], 1).astype(np.float64)
    (t_table, t_off, t_cnt, t_beg, t_len, t_idx), q, lens = _device_lists(torch, p, kp)
    for call in range(2):
        v = [torch.zeros(q.n, dtype=torch.float32, device="cuda") for _ in range(3)]
        torch.cuda.synchronize()
        hsr.kick_lists_noalloc(t_table, q.n, t_off, t_cnt, t_beg, t_len, t_idx, *v,
                               fcoeff=kp.fcoeff, rsm=kp.rsm, fsrrmax=kp.fsrrmax, law=kp.law)
        got = np.stack([t.cpu().numpy() for t in v], 1).astype(np.float64)
        rms, mx = force_errors(got, v_ref)
        assert rms <= RMS_TOL and mx <= MAX_TOL, (call, rms, mx)
    return lens


def test_noalloc_kick_matches_rcb_kick_twice(ctx):
    p, kp = _case()
    _check_twice(ctx, p, kp)


def test_noalloc_long_lists_split_over_items(ctx):
    """Lists of up to 37 000 entries: each leaf's list runs as several items
    of at most 8192 entries whose sums add with atomics."""
    p, kp = _dense_case()
    lens = _check_twice(ctx, p, kp)
    assert lens.max() > 4 * 8192 and (lens > 8192).mean() > 0.5


def test_noalloc_step16_law(ctx):
    p, kp = _case()
    kp.law = hsr.LAW_POLY5_STEP16
    _check_twice(ctx, p, kp)


def test_noalloc_rejects_too_many_items_and_recovers(ctx):
    """70 000 leaves of 33 particles make 140 000 work items (two groups per
    leaf), more than the 131 064 the fixed array holds: HSR_ERR_ARG, no pair
    evaluated, the caller's velocities unchanged; the next call is unaffected."""
    torch = pytest.importorskip("torch")
    nleaf, per = 70000, 33
    n = nleaf * per
    rng = np.random.default_rng(3)
    table = np.concatenate([rng.uniform(0, 50, (n, 3)), np.ones((n, 1))], 1).astype(np.float32)
    dev = "cuda"
    t_table = torch.from_numpy(table).to(dev)
    t_off = torch.arange(0, n, per, dtype=torch.int32, device=dev)
    t_cnt = torch.full((nleaf,), per, dtype=torch.int32, device=dev)
    t_beg = torch.arange(0, nleaf, dtype=torch.int64, device=dev)
    t_len = torch.ones(nleaf, dtype=torch.int32, device=dev)
    t_idx = t_off.clone()  # each leaf's list: its first particle
    v = [torch.full((n,), 0.25 * (k + 1), dtype=torch.float32, device=dev) for k in range(3)]
    before = [t.clone() for t in v]
    torch.cuda.synchronize()
    with pytest.raises(hsr.HsrError) as e:
        hsr.kick_lists_noalloc(t_table, n, t_off, t_cnt, t_beg, t_len, t_idx, *v, fcoeff=1.0)
    assert e.value.status == hsr.HSR_ERR_ARG
    assert all(torch.equal(a, b) for a, b in zip(v, before))
    p, kp = _case()
    _check_twice(ctx, p, kp)
