"""The adjoint with 12-point (quadrupole) pseudo-particles against FP64.

A 16^3 Zel'dovich lattice at z = 10 with overload ghosts, nd = 32, opening
angle 1.0, fcoeff = 1: 15 % of the 50 600 list entries are 12-point
pseudo-particles (at opening angle 0.5 a node opened within the cutoff holds
fewer than 12 particles at this density, so the lists hold particles only).
The FP64 reference (oracle/quad64.py) restates the kick with its
pseudo-particles in float64 as a function of the particle positions, the tree,
the lists and the cutoff mask
frozen (and the particles that attain each node's box extremes): it must
reproduce the GPU's FP32 forward on the same tape, and its central
differences (h = 1e-4 grid units) check the GPU's VJP along random
directions over all particles and on sampled particles, to 1e-4 of the
gradient's scale, the tolerance of the monopole adjoint's test.
"""
import os
import sys

import numpy as np
import pytest

import synth

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "oracle"))
import quad64  # noqa: E402

ADJ_TOL = 1e-4


def _box():
    p = synth.zeldovich_box(16, z=10.0, seed=4)
    kp = synth.kick_params(p, nd=32, tdpts=12, open_angle=1.0, fcoeff=1.0)
    return p, kp


def test_quad_restatement_matches_oracle_pseudo_particles(oracle_lib):
    """quad64's float64 points and masses against the oracle's (the
    reference's float arithmetic) on the oracle's own tree."""
    p, kp = _box()
    q = p.copy()
    r = oracle_lib.rcb_run(q, kp, keep_lists=True, do_kick=False)
    nodes = r.nodes(12)
    off, cnt, ptr = r.leaves()
    x = np.stack([q.x, q.y, q.z], 1).astype(np.float64)
    M = quad64.QuadMap(nodes, (off, cnt, ptr, np.zeros(int(ptr[-1]), np.int64)), x, q.mass,
                       1.0, kp.ppc, kp.nd)
    tab = M.table(x)
    use = nodes["count"] > 12
    pm = tab[q.n:, 3].reshape(-1, 12)[use]
    ref = nodes["ppm"].astype(np.float64)[use]
    assert np.abs(pm - ref).max() <= 2e-5 * np.abs(ref).max()
    pts = tab[q.n:, :3].reshape(-1, 12, 3)[use]
    xc = nodes["bbox"][:, 6:9].astype(np.float64)[use]
    tdr = nodes["tdr"].astype(np.float64)[use]
    ref_pts = xc[:, None, :] + tdr[:, None, None] * quad64.DESIGN12[None]
    assert np.abs(pts - ref_pts).max() <= 1e-4


@pytest.mark.gpu
def test_quad_vjp_matches_fp64_differences(ctx):
    p, kp = _box()
    n = p.n
    dv = ctx.force_fwd(p.x, p.y, p.z, p.mass, kp)
    perm = ctx.last_perm(n)
    tree = ctx.tree(12)
    off, cnt, ptr, _ = ctx.lists()
    idx = ctx.lists_index()
    x0 = np.stack([p.x, p.y, p.z], 1).astype(np.float64)[perm]
    M = quad64.QuadMap(tree, (off, cnt, ptr, idx), x0, p.mass[perm], kp.fcoeff, kp.ppc, kp.nd,
                       rsm=kp.rsm, fsrrmax=kp.fsrrmax)
    # the float64 map reproduces the GPU's forward on the same tape
    f64 = M.kick(x0)
    dvt = dv[perm].astype(np.float64)
    rel = np.sqrt(((f64 - dvt) ** 2).sum() / (f64 ** 2).sum())
    assert rel <= 1e-5, rel
    rng = np.random.default_rng(9)
    u = rng.standard_normal((n, 3)).astype(np.float32)
    xbar = ctx.force_vjp(u)
    xt = xbar[perm].astype(np.float64)
    ut = u[perm].astype(np.float64)
    h = 1e-4
    gnorm = np.linalg.norm(xt)
    # directional derivatives over all particles; with the pseudo-particles
    # held constant the differences move by several times the VJP's error, so
    # the check resolves their chain rule
    tab0 = M.table(x0)
    miss, errs = 0.0, []
    for _ in range(4):
        D = rng.standard_normal((n, 3))
        D /= np.linalg.norm(D)
        fd = (M.loss(x0 + h * D, ut) - M.loss(x0 - h * D, ut)) / (2 * h)
        errs.append(abs((xt * D).sum() - fd))
        assert errs[-1] <= ADJ_TOL * gnorm, ((xt * D).sum(), fd, gnorm)
        fd0 = (M.loss(x0 + h * D, ut, tab0) - M.loss(x0 - h * D, ut, tab0)) / (2 * h)
        miss = max(miss, abs(fd0 - fd))
    assert miss >= 5 * max(errs), (miss, errs, gnorm)
    # particles, axis by axis
    inleaf = np.concatenate([np.arange(o, o + c) for o, c in zip(off, cnt)])
    smp = rng.choice(inleaf, 8, replace=False)
    fd = np.zeros((len(smp), 3))
    for r, i in enumerate(smp):
        for d in range(3):
            E = np.zeros_like(x0)
            E[i, d] = h
            fd[r, d] = (M.loss(x0 + E, ut) - M.loss(x0 - E, ut)) / (2 * h)
    rms_g = np.sqrt((xt[inleaf] ** 2).sum(1).mean())
    scale = np.maximum(np.linalg.norm(fd, axis=1), rms_g)
    err = np.linalg.norm(xt[smp] - fd, axis=1) / scale
    assert err.max() <= ADJ_TOL, (err, scale)


@pytest.mark.gpu
def test_multibox_vjp_with_a_12_point_box_equals_single_box_vjps(ctx):
    """One multi-box forward and VJP over a 12-point box and a monopole box
    gives each box's single-box VJP (FP32 summation order aside)."""
    torch = pytest.importorskip("torch")
    from hsr_testutil import force_errors
    boxes = [synth.zeldovich_box(16, z=10.0, seed=4), synth.zeldovich_box(12, z=10.0, seed=6)]
    kps = [synth.kick_params(boxes[0], nd=32, tdpts=12, open_angle=1.0, fcoeff=1.0),
           synth.kick_params(boxes[1], nd=32, open_angle=1.5, fcoeff=1.0)]
    rng = np.random.default_rng(21)
    us = [rng.standard_normal((b.n, 3)).astype(np.float32) for b in boxes]
    single = []
    for b, kp, u in zip(boxes, kps, us):
        ctx.force_fwd(b.x, b.y, b.z, b.mass, kp)
        single.append(ctx.force_vjp(u))
    dev = lambda a: torch.tensor(np.ascontiguousarray(a), device="cuda")
    xs = [tuple(dev(getattr(b, k)) for k in ("x", "y", "z")) for b in boxes]
    ms = [dev(b.mass) for b in boxes]
    dvs = [tuple(torch.zeros(b.n, device="cuda") for _ in range(3)) for b in boxes]
    ctx.force_fwd_batch_device(xs, ms, dvs, kps)
    ud = [tuple(dev(u[:, d]) for d in range(3)) for u in us]
    xb = [tuple(torch.zeros(b.n, device="cuda") for _ in range(3)) for b in boxes]
    ctx.force_vjp_batch_device(ud, xb)
    torch.cuda.synchronize()
    for k in range(2):
        got = np.stack([t.cpu().numpy() for t in xb[k]], 1).astype(np.float64)
        rms, mx = force_errors(got, single[k].astype(np.float64))
        assert rms <= 1e-5 and mx <= 1e-3, (k, rms, mx)
