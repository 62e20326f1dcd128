"""The allocation-free kick (hsr_kick_lists_noalloc) through the C ABI.

It serves callers that cannot allocate device memory while they run; it keeps
its scratch in a fixed device array shared by all calls.  This test gives it
interaction lists built by the library itself and checks, on two calls in a
row, that its kick equals hsr_rcb_kick's on the same particles within the
suite's FP32 force tolerance.  The file is collected last on purpose.
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


def test_noalloc_kick_matches_rcb_kick_twice(ctx):
    torch = pytest.importorskip("torch")
    p, kp = _case()
    # reference result: the existing entry point (velocities in tree order)
    ref = p.copy()
    ctx.rcb_kick(ref, kp)
    v_ref = np.stack([ref.vx, ref.vy, ref.vz], 1).astype(np.float64)
    # the same tree and lists, host-built, as device arrays the caller owns
    q = p.copy()
    L = hsr.HostLists(q, kp)
    off, cnt, ptr, e = L.get()
    eidx = L.index()
    ntab = int(max(eidx.max() + 1, q.n))
    table = np.zeros((ntab, 4), np.float32)
    table[: q.n] = np.stack([q.x, q.y, q.z, q.mass], 1)
    table[eidx] = e.T
    dev = "cuda"
    t_table = torch.from_numpy(table).to(dev)
    t_off = torch.from_numpy(off.astype(np.int32)).to(dev)
    t_cnt = torch.from_numpy(cnt.astype(np.int32)).to(dev)
    t_beg = torch.from_numpy(ptr[:-1].astype(np.int64)).to(dev)
    t_len = torch.from_numpy(np.diff(ptr).astype(np.int32)).to(dev)
    t_idx = torch.from_numpy(eidx.astype(np.int32)).to(dev)
    for call in range(2):
        v = [torch.zeros(q.n, dtype=torch.float32, device=dev) for _ in range(3)]
        torch.cuda.synchronize()
        hsr.kick_lists_noalloc(t_table, q.n, t_off, t_cnt, t_beg, t_len, t_idx, *v,
                               fcoeff=kp.fcoeff, rsm=kp.rsm, fsrrmax=kp.fsrrmax)
        got = np.stack([t.cpu().numpy() for t in v], 1).astype(np.float64)
        rms, mx = force_errors(got, v_ref)
        assert rms <= RMS_TOL and mx <= MAX_TOL, (call, rms, mx)
