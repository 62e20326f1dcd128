"""The RCO octree variant (RCOForceTree, HACC's -O option): the tree and lists
built on the host, the pairs on the GPU.  Against the oracle's restatement of
RCOForceTree (itself pinned bit for bit to the reference's RCOForceTree with
its octant array sized 8): the permutation of all ten arrays bit-exact, the
lists equal per leaf, the forces within RMS_TOL / MAX_TOL."""
import dataclasses

import numpy as np
import pytest

import hsr
import synth
from hsr_testutil import MAX_TOL, RMS_TOL, force_errors, same_lists, vel

pytestmark = pytest.mark.gpu

EXACT = ("x", "y", "z", "mass", "phi", "id", "mask")


def _zero_v(p):
    p.vx[:] = 0
    p.vy[:] = 0
    p.vz[:] = 0
    return p


@pytest.mark.parametrize("case", ["zeldovich32", "clustered24_quad", "clustered24_oa05"])
@pytest.mark.parametrize("kernel", [hsr.KERNEL_PLAIN, hsr.KERNEL_AUTO])
def test_rco_kick_vs_oracle(ctx, oracle_lib, case, kernel):
    if case == "zeldovich32":
        p = _zero_v(synth.zeldovich_box(32, z=10.0, seed=12))
        kp = synth.kick_params(p, nd=128, fcoeff=1.0)
    elif case == "clustered24_quad":
        p = _zero_v(synth.clustered_box(24, nhalo=40, seed=13))
        kp = synth.kick_params(p, nd=32, tdpts=12, fcoeff=1.0)
    else:
        p = _zero_v(synth.clustered_box(24, nhalo=40, seed=14))
        kp = synth.kick_params(p, nd=16, open_angle=0.5, fcoeff=1.0)
    kp = dataclasses.replace(kp, tree=hsr.TREE_RCO)
    q = p.copy()
    st = ctx.rcb_kick(p, kp, kernel=kernel)
    r = oracle_lib.rcb_run(q, kp, keep_lists=True, nthreads=0)
    for k in EXACT:
        assert np.array_equal(getattr(p, k).view(np.uint8), getattr(q, k).view(np.uint8)), k
    off, cnt, ptr = r.leaves()
    sel = np.concatenate([np.arange(o, o + c) for o, c in zip(off, cnt)])
    rms, mx = force_errors(vel(p)[sel], vel(q)[sel])
    assert rms <= RMS_TOL and mx <= MAX_TOL, (case, rms, mx)
    goff, gcnt, gptr, ge = ctx.lists()
    assert same_lists(goff, gcnt, gptr, ge, off, cnt, ptr, r.entries())
    assert st["pairs"] == r.stats["pairs"]
    assert st["nodes"] == r.stats["nodes"]


def test_rco_differs_from_rcb(ctx):
    """The two tree kinds give different trees and lists.  Their kicks agree
    only roughly: both drop nodes whose centre of mass lies beyond the cutoff
    (RCBForceTree.cxx:1024-1029, RCOForceTree.cxx:865-870) although some of
    their particles may lie within it, and which nodes those are depends on
    the tree's shape."""
    p = _zero_v(synth.zeldovich_box(24, z=10.0, seed=15))
    kp = synth.kick_params(p, nd=64, fcoeff=1.0)
    a, b = p.copy(), p.copy()
    sa = ctx.rcb_kick(a, kp)
    sb = ctx.rcb_kick(b, dataclasses.replace(kp, tree=hsr.TREE_RCO))
    assert sa["nodes"] != sb["nodes"]
    ia, ib = np.argsort(a.id), np.argsort(b.id)
    va, vb = vel(a)[ia], vel(b)[ib]
    # particles kicked by both (the leaves at the force-box edge differ)
    keep = (np.linalg.norm(va, axis=1) > 0) & (np.linalg.norm(vb, axis=1) > 0)
    assert keep.sum() > 0.5 * len(keep)
    rms, _ = force_errors(vb[keep], va[keep])
    assert rms < 0.3, rms


def test_rco_rejected_where_only_rcb_is_built(ctx):
    p = synth.zeldovich_box(12, seed=16)
    kp = dataclasses.replace(synth.kick_params(p, nd=64), tree=hsr.TREE_RCO)
    with pytest.raises(hsr.HsrError):
        ctx.force_fwd(p.x, p.y, p.z, p.mass, kp)
