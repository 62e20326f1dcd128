"""The adjoint pair hsr_force_fwd / hsr_force_vjp against FP64.

The adjoint workload: a 64^3 Zel'dovich lattice at z = 10 with
overload ghosts, opening angle 0.1, monopole pseudo-particles; a seeded N(0,1)
cotangent.  The VJP (FP32 on the GPU) is compared with an FP64 analytic VJP
over the same lists and with FP64 central differences (h = 1e-4 grid units) on
256 sampled particles.  Tolerance: 1e-4 relative to the larger of the sample's
gradient norm and the rms gradient (the adjoint's stated target); samples
with a pair within 2h of the cutoff are skipped (the law steps there).
"""
import numpy as np
import pytest

import hsr
import synth
from hsr_testutil import force_errors

ADJ_TOL = 1e-4


def _tape_arrays(ctx, p_caller, n):
    """Tree-order table, pseudo-particle node ranges and lists of the tape."""
    perm = ctx.last_perm(n)
    idx = ctx.lists_index()
    off, cnt, ptr, e = ctx.lists()
    tree = ctx.tree()
    ntab = n + len(tree["count"])
    table = np.zeros((ntab, 4), np.float32)
    table[:n] = np.stack([p_caller.x, p_caller.y, p_caller.z, p_caller.mass], 1)[perm]
    table[idx] = e.T
    return perm, table, tree["offset"], tree["count"], off, cnt, ptr, idx


def test_vjp_and_fd_oracles_agree_on_cpu(hsr_lib, oracle_lib):
    """The two FP64 references agree with each other (opening angle 0: every
    entry a particle)."""
    p = synth.random_box(3000, 10.0, 5)
    kp = synth.kick_params(p, nd=16, open_angle=0.0, fcoeff=0.7)
    kp.min_force, kp.max_force = (-1.0,) * 3, (11.0,) * 3
    L = hsr.HostLists(p, kp)
    off, cnt, ptr, e = L.get()
    idx = L.index()
    table = np.stack([p.x, p.y, p.z, p.mass], 1).astype(np.float32)
    u = np.random.default_rng(1).standard_normal((p.n, 3))
    none = np.zeros(0, np.int64)
    xb = oracle_lib.vjp_tab(p.n, table, none, none, kp.fcoeff, off, cnt, ptr, idx, u)
    smp = np.random.default_rng(2).choice(p.n, 64, replace=False)
    fd, near = oracle_lib.fd_tab(p.n, table, none, none, kp.fcoeff, off, cnt, ptr, idx, u, smp,
                                 h=1e-5)
    ok = ~near
    err = np.linalg.norm(xb[smp][ok] - fd[ok], axis=1)
    scale = np.maximum(np.linalg.norm(fd[ok], axis=1), np.sqrt((fd[ok] ** 2).sum(1).mean()))
    assert ok.sum() > 40 and np.all(err <= 1e-6 * scale)


@pytest.fixture
def group_tune(ctx, request):
    """The context's batched shape with groups of request.param particles
    (16: the adjoint kernel's half-warp groups), restored afterwards."""
    saved = ctx.get_tune()
    ctx.set_tune("batched", 128, request.param)
    yield request.param
    ctx.set_tune(saved["kernel"], saved["leaf_threads"], saved["group"])


@pytest.mark.gpu
@pytest.mark.parametrize("group_tune", [32, 16], indirect=True)
def test_vjp_matches_fp64_gradient_and_finite_differences(ctx, oracle_lib, group_tune):
    p = synth.zeldovich_box(64, z=10.0, seed=3)
    kp = synth.kick_params(p, nd=64, fcoeff=1.0)
    n = p.n
    dv = ctx.force_fwd(p.x, p.y, p.z, p.mass, kp)
    perm, table, noff, ncnt, off, cnt, ptr, idx = _tape_arrays(ctx, p, n)
    # the forward is the kick from rest
    q = p.copy()
    q.vx[:] = 0
    q.vy[:] = 0
    q.vz[:] = 0
    ctx.rcb_kick(q, kp)
    assert np.array_equal(dv[perm], np.stack([q.vx, q.vy, q.vz], 1))
    u = np.random.default_rng(9).standard_normal((n, 3)).astype(np.float32)
    dv2 = ctx.force_fwd(p.x, p.y, p.z, p.mass, kp)
    assert np.array_equal(dv, dv2)
    xbar = ctx.force_vjp(u)
    xt = xbar[perm].astype(np.float64)
    ut = u[perm].astype(np.float64)
    ref = oracle_lib.vjp_tab(n, table, noff, ncnt, kp.fcoeff, off, cnt, ptr, idx, ut)
    rms, mx = force_errors(xt, ref)
    assert rms <= 1e-5 and mx <= 1e-3, (rms, mx)
    inleaf = np.concatenate([np.arange(o, o + c) for o, c in zip(off, cnt)])
    smp = np.random.default_rng(10).choice(inleaf, 256, replace=False)
    fd, near = oracle_lib.fd_tab(n, table, noff, ncnt, kp.fcoeff, off, cnt, ptr, idx, ut, smp,
                                 h=1e-4)
    ok = ~near
    assert ok.sum() >= 200, ok.sum()
    rms_g = np.sqrt((fd[ok] ** 2).sum(1).mean())
    scale = np.maximum(np.linalg.norm(fd[ok], axis=1), rms_g)
    err = np.linalg.norm(xt[smp][ok] - fd[ok], axis=1) / scale
    assert err.max() <= ADJ_TOL, err.max()


@pytest.mark.gpu
@pytest.mark.parametrize("group_tune", [16, 32], indirect=True)
def test_vjp_through_monopole_pseudo_particles(ctx, oracle_lib, group_tune):
    """Opening angle 1.5 on 16^3 at z = 10: 7 % of the list entries are
    monopole pseudo-particles (at 0.1 the lists hold particles only).  The GPU
    VJP against the FP64 VJP over the same lists with the pseudo-particles'
    chain rule (through each node's centre of mass); without that rule the
    FP64 VJP differs by more than 5x the GPU's error, so it is resolved."""
    p = synth.zeldovich_box(16, z=10.0, seed=4)
    kp = synth.kick_params(p, nd=32, open_angle=1.5, fcoeff=1.0)
    n = p.n
    ctx.force_fwd(p.x, p.y, p.z, p.mass, kp)
    perm, table, noff, ncnt, off, cnt, ptr, idx = _tape_arrays(ctx, p, n)
    assert (idx >= n).sum() > 300
    u = np.random.default_rng(12).standard_normal((n, 3)).astype(np.float32)
    xt = ctx.force_vjp(u)[perm].astype(np.float64)
    ut = u[perm].astype(np.float64)
    ref = oracle_lib.vjp_tab(n, table, noff, ncnt, kp.fcoeff, off, cnt, ptr, idx, ut)
    rms, mx = force_errors(xt, ref)
    assert rms <= 1e-5 and mx <= 1e-3, (rms, mx)
    ref0 = oracle_lib.vjp_tab(n, table, noff, np.zeros_like(ncnt), kp.fcoeff, off, cnt, ptr, idx,
                              ut)
    share, err = np.linalg.norm(ref - ref0), np.linalg.norm(xt - ref)
    assert share >= 5 * err, (share, err)


@pytest.mark.gpu
def test_vjp_is_linear_in_the_cotangent(ctx):
    p = synth.zeldovich_box(24, z=10.0, seed=4)
    kp = synth.kick_params(p, nd=64, fcoeff=1.0)
    ctx.force_fwd(p.x, p.y, p.z, p.mass, kp)
    rng = np.random.default_rng(3)
    u1 = rng.standard_normal((p.n, 3)).astype(np.float32)
    u2 = rng.standard_normal((p.n, 3)).astype(np.float32)
    a = ctx.force_vjp(u1).astype(np.float64)
    b = ctx.force_vjp(u2).astype(np.float64)
    c = ctx.force_vjp(u1 + u2).astype(np.float64)
    rms, mx = force_errors(c, a + b)
    assert rms <= 1e-5 and mx <= 1e-3


@pytest.mark.gpu
def test_vjp_call_order_is_reported():
    """hsr_force_vjp without a forward: HSR_ERR_STATE; after a 12-point
    forward it runs (its accuracy: tests/test_quad_adjoint.py), linear in the
    cotangent (zero for zero)."""
    with hsr.Context(0) as c:
        with pytest.raises(hsr.HsrError) as e:
            c.force_vjp(np.zeros((4, 3), np.float32))
        assert e.value.status == 7
        p = synth.zeldovich_box(12, seed=1)
        kp = synth.kick_params(p, nd=32, tdpts=12)
        c.force_fwd(p.x, p.y, p.z, p.mass, kp)
        xb = c.force_vjp(np.zeros((p.n, 3), np.float32))
        assert np.all(xb == 0)
