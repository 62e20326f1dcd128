"""Multi-step adjoint of the sub-cycled short-range map (multistep.py).

The benchmark's multi-box adjoint case: boxes of Zel'dovich particles, 10 PM
steps x 5 sub-cycles (map1, kick, map1), checkpoints every 2 PM steps.  The
GPU reverse pass is compared with an FP64 restatement of the same map over
the same frozen trees and lists (oracle.multistep64): its gradient along the
GPU trajectory (rms 1e-5 / max 1e-3 of the rms), and FP64 central differences
(h = 1e-4 grid units) on 64 particles of the first box and 16 of the second
(each sample costs two FP64 runs of the whole map), within 1e-4 of the larger
of the sample's gradient norm and the rms gradient.  The adjoint differentiates
the map with trees, lists and the cutoff mask held fixed (the law steps at
the cutoff, and over 50 sub-cycles some pair of most particles' neighbours
crosses it within h); the differences therefore decide every pair's cutoff
on the unperturbed run's positions.

The GPU gradient is also compared with the FP64 map's gradient at the FP64
map's own trajectory (the one the differences probe).  The FP32 forward
drifts from the FP64 forward over 50 sub-cycles (final positions ~6e-5 grid
units apart in the 12^3 boxes), which moves that gradient by ~1e-4 rms; the
test therefore asks the GPU gradient to be no farther from it than the exact
FP64 adjoint evaluated along the GPU trajectory is (plus 1e-5): the gap is
the forward's drift, not adjoint error.
"""
import dataclasses

import numpy as np
import pytest

import hsr
import multistep
import synth
from hsr_testutil import force_errors

ADJ_TOL = 1e-4


def _host_tape(x, m, kp):
    """Tree and lists of the host build at positions x (no pseudo-particles:
    opening angle 0)."""
    n = len(m)
    f = lambda a: np.ascontiguousarray(a, np.float32)
    p = synth.Particles(x=f(x[:, 0]), y=f(x[:, 1]), z=f(x[:, 2]), vx=np.zeros(n, np.float32),
                        vy=np.zeros(n, np.float32), vz=np.zeros(n, np.float32), mass=f(m),
                        phi=np.zeros(n, np.float32), id=np.arange(n, dtype=np.int64),
                        mask=np.zeros(n, np.uint16))
    L = hsr.HostLists(p, kp)
    off, cnt, ptr, _ = L.get()
    none = np.zeros(0, np.int64)
    return dict(perm=p.id.copy(), noff=none, ncnt=none, off=off, cnt=cnt, ptr=ptr, idx=L.index())


def _fd(O, x0, v0, m, steps, nsub, tapes, xbar, vbar, k, d, h, base):
    """Central difference of L along d at particle k, with every kick's
    cutoff decided on the unperturbed run's positions `base` (the map whose
    derivative the adjoint computes: trees, lists and cutoff mask frozen)."""
    out = []
    for step in (h, -h):
        x = x0.copy()
        x[k] += step * d
        out.append(O.multistep64(x, v0, m, steps, nsub, tapes, cut_pos=base))
    (xp, vp), (xm, vm) = out
    return (float((xbar * (xp - xm)).sum() + (vbar * (vp - vm)).sum())) / (2 * h)


def _check_fd(O, x0, v0, m, steps, nsub, tapes, xbar, vbar, grad, samples, h, rng):
    """Directional differences at the sampled particles against the
    gradient, relative to the larger of the sample's gradient norm and the
    rms gradient; returns the number of samples off by more than ADJ_TOL."""
    base = []
    O.multistep64(x0, v0, m, steps, nsub, tapes, traj_out=base)
    rms = np.sqrt((grad ** 2).sum(1).mean())
    bad = 0
    for k in samples:
        d = rng.standard_normal(3)
        d /= np.linalg.norm(d)
        f = _fd(O, x0, v0, m, steps, nsub, tapes, xbar, vbar, k, d, h, base)
        bad += abs(grad[k] @ d - f) > ADJ_TOL * max(np.linalg.norm(grad[k]), rms)
    return bad


def test_fp64_multistep_gradient_matches_fd(hsr_lib, oracle_lib):
    """The FP64 reference itself: its reverse pass against its own central
    differences (host-built trees, opening angle 0)."""
    O = oracle_lib
    p = synth.random_box(1000, 10.0, 11)
    kp = synth.kick_params(p, nd=16, open_angle=0.0)
    kp.min_force, kp.max_force = (-1.0,) * 3, (10.0,) * 3
    steps = [multistep.StepParams(alpha=1.0, pp=0.5, adot=1.0, tau_sub=0.02, fcoeff=0.03),
             multistep.StepParams(alpha=1.0, pp=0.6, adot=1.0, tau_sub=0.02, fcoeff=0.025)]
    nsub = 2
    x = np.stack([p.x, p.y, p.z], 1).astype(np.float64)
    v = 0.1 * np.stack([p.vx, p.vy, p.vz], 1).astype(np.float64)
    m = p.mass.astype(np.float64)
    # trees and lists along the FP64 trajectory
    tapes = []
    xx, vv = x.copy(), v.copy()
    for st in steps:
        pt = O.stream_factor(st.alpha, st.pp, st.tau_sub, st.adot)
        for _ in range(nsub):
            xx += pt * vv
            t = _host_tape(xx, m, dataclasses.replace(kp, fcoeff=st.fcoeff))
            tapes.append(t)
            vv[t["perm"]] += O.kick64(xx[t["perm"]], m[t["perm"]], t, st.fcoeff)
            xx += pt * vv
    rng = np.random.default_rng(4)
    xbar, vbar = rng.standard_normal(x.shape), rng.standard_normal(v.shape)
    xT, vT, L, gx, gv = O.multistep64(x, v, m, steps, nsub, tapes, xbar, vbar)
    assert np.allclose(xT, xx) and np.allclose(vT, vv)
    smp = rng.choice(len(m), 24, replace=False)
    bad = _check_fd(O, x, v, m, steps, nsub, tapes, xbar, vbar, gx, smp, 1e-4, rng)
    assert bad == 0, bad
    # the velocity gradient: directional differences in v0
    k = int(smp[0])
    d = np.array([0.3, -0.5, 0.8]) / np.linalg.norm([0.3, -0.5, 0.8])
    base = []
    O.multistep64(x, v, m, steps, nsub, tapes, traj_out=base)
    def Sv(step):
        vv0 = v.copy()
        vv0[k] += step * d
        return O.multistep64(x, vv0, m, steps, nsub, tapes, cut_pos=base)
    (xp, vp), (xm, vm) = Sv(1e-4), Sv(-1e-4)
    fdv = float((xbar * (xp - xm)).sum() + (vbar * (vp - vm)).sum()) / 2e-4
    assert abs(fdv - gv[k] @ d) <= ADJ_TOL * max(np.linalg.norm(gv[k]), 1.0)


def _boxes(nbox, ng, seed0):
    return [synth.zeldovich_box(ng, z=50.0, seed=seed0 + b) for b in range(nbox)]


def _tape_of(ctx, n):
    tree = ctx.tree()
    off, cnt, ptr, _ = ctx.lists()
    return dict(perm=ctx.last_perm(n), noff=tree["offset"], ncnt=tree["count"], off=off,
                cnt=cnt, ptr=ptr, idx=ctx.lists_index())


def _tape_hook(torch, boxes, kps, tapes, kick_x):
    """on_tape hook recording each kick's tree and lists and its positions;
    in lockstep (ctx None) the box's tape is rebuilt on a context of its own
    from the kick positions."""
    aux = {}

    def on_tape(b, s, j, c, x1):
        n = boxes[b].n
        if c is None:
            if "ctx" not in aux:
                aux["ctx"] = hsr.Context(0)
            m = torch.ones(n, dtype=torch.float32, device=x1[0].device)
            dv = [torch.empty_like(m) for _ in range(3)]
            aux["ctx"].force_fwd_device(x1[0], x1[1], x1[2], m, *dv, kps[b])
            c = aux["ctx"]
        tapes[(b, s, j)] = _tape_of(c, n)
        kick_x[(b, s, j)] = np.stack([t.cpu().numpy() for t in x1], 1).astype(np.float64)
    return on_tape


@pytest.mark.gpu
@pytest.mark.parametrize("batched", [True, False])
def test_multistep_adjoint_vs_fp64_and_fd(ctx, oracle_lib, batched):
    """2 boxes x 12^3 at z = 50, 10 PM steps x 5 sub-cycles, checkpoints
    every 2 steps, opening angle 0.1 (pseudo-particles on); the boxes in
    lockstep (one multi-box launch per kick) or one after the other."""
    torch = pytest.importorskip("torch")
    O = oracle_lib
    nsteps, nsub = 10, 5
    steps = multistep.schedule(50.0, 10.0, nsteps, nsub)
    boxes = _boxes(2, 12, 70)
    kps = [synth.kick_params(b, nd=64) for b in boxes]
    ms = multistep.MultiStep(ctx, kps, steps, nsub, checkpoint_every=2, batched=batched)
    tapes, kick_x = {}, {}
    ms.on_tape = _tape_hook(torch, boxes, kps, tapes, kick_x)
    rng = np.random.default_rng(8)
    cots = []
    for p in boxes:
        xbar = rng.standard_normal((p.n, 3)).astype(np.float32)
        vbar = rng.standard_normal((p.n, 3)).astype(np.float32)
        cots.append((xbar, vbar))
    dev = lambda a: [torch.from_numpy(np.ascontiguousarray(a[:, d])).cuda() for d in range(3)]
    states = [multistep.box_state(p) for p in boxes]
    grads = ms.adjoint(states, [dev(c[0]) for c in cots], [dev(c[1]) for c in cots])
    for b, p in enumerate(boxes):
        n = p.n
        xbar, vbar = cots[b]
        gx_t, gv_t = grads[b]
        gx = np.stack([t.cpu().numpy() for t in gx_t], 1).astype(np.float64)
        gv = np.stack([t.cpu().numpy() for t in gv_t], 1).astype(np.float64)
        order = [(b, s, j) for s in range(nsteps) for j in range(nsub)]
        tl = [tapes[k] for k in order]
        xl = [kick_x[k] for k in order]
        x0 = np.stack([p.x, p.y, p.z], 1).astype(np.float64)
        v0 = np.stack([p.vx, p.vy, p.vz], 1).astype(np.float64)
        m = p.mass.astype(np.float64)
        # FP64 gradient along the GPU's own trajectory
        _, _, _, rx, rv = O.multistep64(x0, v0, m, steps, nsub, tl, xbar, vbar, kick_pos=xl)
        for g, r in ((gx, rx), (gv, rv)):
            rms, mx = force_errors(g, r)
            assert rms <= 1e-5 and mx <= 1e-3, (b, rms, mx)
        # FP64 differences of the FP64 map (frozen trees) on 64 particles
        inner = np.flatnonzero(p.mask == 0) if np.any(p.mask == 0) else np.arange(n)
        smp = rng.choice(inner, 64 if b == 0 else 16, replace=False)
        _, _, _, fx, _ = O.multistep64(x0, v0, m, steps, nsub, tl, xbar, vbar)
        bad = _check_fd(O, x0, v0, m, steps, nsub, tl, xbar, vbar, fx, smp, 1e-4, rng)
        assert bad == 0, (b, bad)
        # the GPU gradient against the differences' gradient: as close as the
        # FP64 adjoint along the GPU trajectory (the FP32 forward's drift)
        rms, _ = force_errors(gx[smp], fx[smp])
        drift, _ = force_errors(rx[smp], fx[smp])
        assert rms <= drift + 1e-5, (b, rms, drift)
    assert ms.kicks == multistep.kicks_per_box(nsteps, nsub) * 2
    if batched:  # one multi-box call per kick of the forward, the recomputation and the tapes
        assert ms.batch_calls == multistep.kicks_per_box(nsteps, nsub)


@pytest.mark.gpu
def test_kick_and_vjp_batch_equal_single_box_calls(ctx):
    """hsr_force_kick_batch / hsr_force_vjp_batch on three boxes of different
    sizes against hsr_force_kick / hsr_force_vjp box by box (the same pairs;
    FP32 summation order only)."""
    torch = pytest.importorskip("torch")
    boxes = [synth.zeldovich_box(ng, z=20.0, seed=5 + ng) for ng in (12, 20, 16)]
    kps = [synth.kick_params(b, nd=64, fcoeff=0.5 + 0.1 * i) for i, b in enumerate(boxes)]
    Ss = [multistep.box_state(b) for b in boxes]
    rng = np.random.default_rng(3)
    us = [[torch.from_numpy(rng.standard_normal(b.n).astype(np.float32)).cuda() for _ in range(3)]
          for b in boxes]
    vb = [[v.clone() for v in S.v] for S in Ss]
    st = ctx.force_kick_batch_device([S.x for S in Ss], [S.mass for S in Ss], vb, kps)
    assert st["kernel_launches"] == 1 and st["pairs"] > 0
    xb = [[torch.empty_like(S.x[0]) for _ in range(3)] for S in Ss]
    ctx.force_vjp_batch_device(us, xb)
    for b, S in enumerate(Ss):
        v1 = [v.clone() for v in S.v]
        ctx.force_kick_device(*S.x, S.mass, *v1, kps[b])
        x1 = [torch.empty_like(S.x[0]) for _ in range(3)]
        ctx.force_vjp_device(*us[b], *x1)
        dv_b = np.stack([(a - v).double().cpu().numpy() for a, v in zip(vb[b], S.v)], 1)
        dv_1 = np.stack([(a - v).double().cpu().numpy() for a, v in zip(v1, S.v)], 1)
        rms, mx = force_errors(dv_b, dv_1)
        assert rms <= 1e-5 and mx <= 1e-3, (b, rms, mx)
        g_b = np.stack([t.double().cpu().numpy() for t in xb[b]], 1)
        g_1 = np.stack([t.double().cpu().numpy() for t in x1], 1)
        rms, mx = force_errors(g_b, g_1)
        assert rms <= 1e-5 and mx <= 1e-3, (b, rms, mx)
    # the multi-box tape is replaced by any single-box call
    with pytest.raises(hsr.HsrError) as e:
        ctx.force_vjp_batch_device(us, xb)
    assert e.value.status == hsr.HSR_ERR_STATE


@pytest.mark.gpu
def test_lockstep_forward_equals_box_by_box(ctx):
    """The whole multi-step map in lockstep (one multi-box launch per kick)
    and box by box agree to FP32 summation order."""
    torch = pytest.importorskip("torch")
    nsteps, nsub = 3, 5
    steps = multistep.schedule(50.0, 30.0, nsteps, nsub)
    boxes = _boxes(3, 14, 120)
    kps = [synth.kick_params(b, nd=64) for b in boxes]
    a = multistep.MultiStep(ctx, kps, steps, nsub, batched=True)
    b_ = multistep.MultiStep(ctx, kps, steps, nsub, batched=False)
    Sa = a.forward([multistep.box_state(p) for p in boxes])
    Sb = b_.forward([multistep.box_state(p) for p in boxes])
    assert a.batch_calls == nsteps * nsub
    for u, w, p in zip(Sa, Sb, boxes):
        dx = max(float((x - y).abs().max()) for x, y in zip(u.x, w.x))
        assert dx < 1e-4, dx
        v0 = np.stack([p.vx, p.vy, p.vz], 1).astype(np.float64)
        da = np.stack([t.double().cpu().numpy() for t in u.v], 1) - v0
        db = np.stack([t.double().cpu().numpy() for t in w.v], 1) - v0
        rms, mx = force_errors(da, db)
        assert rms <= 1e-5 and mx <= 1e-3, (rms, mx)


@pytest.mark.gpu
def test_checkpointed_equals_stored_and_is_linear(ctx):
    """Checkpointed and fully stored reverse passes agree (the recomputed
    trajectory is the forward one), and the adjoint is linear in the
    cotangent."""
    torch = pytest.importorskip("torch")
    nsteps, nsub = 4, 5
    steps = multistep.schedule(50.0, 30.0, nsteps, nsub)
    p = _boxes(1, 24, 90)[0]
    kp = synth.kick_params(p, nd=128)
    S0 = multistep.box_state(p)
    rng = np.random.default_rng(2)
    cot = lambda: [torch.from_numpy(rng.standard_normal(p.n).astype(np.float32)).cuda()
                   for _ in range(3)]
    xa, va, xb_, vb_ = cot(), cot(), cot(), cot()
    a = multistep.MultiStep(ctx, [kp], steps, nsub, checkpoint_every=1)
    b = multistep.MultiStep(ctx, [kp], steps, nsub, checkpoint_every=None)
    ga = a.adjoint_box(0, S0, xa, va)
    gb = b.adjoint_box(0, S0, xa, va)
    for u, w in zip(ga[0] + ga[1], gb[0] + gb[1]):
        rms, mx = force_errors(u.double().cpu().numpy()[:, None], w.double().cpu().numpy()[:, None])
        assert rms <= 1e-6, rms
    # linearity: adj(2 u + w) = 2 adj(u) + adj(w)
    g1 = b.adjoint_box(0, S0, xb_, vb_)
    comb = b.adjoint_box(0, S0, [2 * s + t for s, t in zip(xa, xb_)],
                         [2 * s + t for s, t in zip(va, vb_)])
    for c_, u, w in zip(comb[0] + comb[1], gb[0] + gb[1], g1[0] + g1[1]):
        ref = (2 * u.double() + w.double()).cpu().numpy()[:, None]
        rms, _ = force_errors(c_.double().cpu().numpy()[:, None], ref)
        assert rms <= 1e-5, rms
    # the forward map alone reproduces the state the reverse pass started from
    S = S0.clone()
    a.forward_box(0, S)
    S2 = S0.clone()
    a.forward_box(0, S2)
    for u, w in zip(S.x + S.v, S2.x + S2.v):
        assert torch.equal(u, w)


# ---------------------------------------------------------------------------
# the map with PM kicks (the whole TreePM step)
# ---------------------------------------------------------------------------

def _pm_dicts(pm):
    return [tuple(None if q is None else dict(ng=q.ng, ngo=q.ngo, gpscal=q.gpscal, fscal=q.fscal,
                                              tau=q.tau) for q in pair) for pair in pm]


def _fd_pm(O, x0, v0, m, steps, nsub, tapes, pm, xbar, vbar, k, d, h, base, pm_base):
    out = []
    for step in (h, -h):
        x = x0.copy()
        x[k] += step * d
        out.append(O.multistep64(x, v0, m, steps, nsub, tapes, cut_pos=base, pm=pm,
                                 pm_cut=pm_base))
    (xp, vp), (xm, vm) = out
    return (float((xbar * (xp - xm)).sum() + (vbar * (vp - vm)).sum())) / (2 * h)


def _check_fd_pm(O, x0, v0, m, steps, nsub, tapes, pm, xbar, vbar, grad, samples, h, rng):
    """_check_fd for the map with PM kicks: cutoffs and CIC cells decided on
    the unperturbed run (the weights are piecewise linear in the positions)."""
    base, pm_base = [], []
    O.multistep64(x0, v0, m, steps, nsub, tapes, pm=pm, traj_out=base, pm_traj_out=pm_base)
    rms = np.sqrt((grad ** 2).sum(1).mean())
    bad = 0
    for k in samples:
        d = rng.standard_normal(3)
        d /= np.linalg.norm(d)
        f = _fd_pm(O, x0, v0, m, steps, nsub, tapes, pm, xbar, vbar, k, d, h, base, pm_base)
        bad += abs(grad[k] @ d - f) > ADJ_TOL * max(np.linalg.norm(grad[k]), rms)
    return bad


def test_fp64_multistep_with_pm_gradient_matches_fd(hsr_lib, oracle_lib):
    """The FP64 reference with PM kicks opening and closing each step (8^3 PM
    grid): its reverse pass against its own central differences."""
    O = oracle_lib
    p = synth.random_box(600, 8.0, 21)
    kp = synth.kick_params(p, nd=16, open_angle=0.0)
    kp.min_force, kp.max_force = (-1.0,) * 3, (9.0,) * 3
    steps = [multistep.StepParams(alpha=1.0, pp=0.5, adot=1.0, tau_sub=0.02, fcoeff=0.03),
             multistep.StepParams(alpha=1.0, pp=0.6, adot=1.0, tau_sub=0.02, fcoeff=0.025)]
    pm = [(dict(ng=8, ngo=0, gpscal=1.0, fscal=2.0, tau=0.05),
           dict(ng=8, ngo=0, gpscal=1.0, fscal=2.2, tau=0.1)),
          (None, dict(ng=8, ngo=0, gpscal=1.0, fscal=2.4, tau=0.05))]
    nsub = 2
    x = np.stack([p.x, p.y, p.z], 1).astype(np.float64)
    v = 0.1 * np.stack([p.vx, p.vy, p.vz], 1).astype(np.float64)
    m = p.mass.astype(np.float64)
    tapes = []
    xx, vv = x.copy(), v.copy()
    import pm_oracle
    for s, st in enumerate(steps):
        pt = O.stream_factor(st.alpha, st.pp, st.tau_sub, st.adot)
        for half in (0, 1):
            if half == 1:
                for _ in range(nsub):
                    xx += pt * vv
                    t = _host_tape(xx, m, dataclasses.replace(kp, fcoeff=st.fcoeff))
                    tapes.append(t)
                    vv[t["perm"]] += O.kick64(xx[t["perm"]], m[t["perm"]], t, st.fcoeff)
                    xx += pt * vv
            q = pm[s][half]
            if q is not None:
                vv += q["fscal"] * q["tau"] * pm_oracle.force64(xx[:, 0], xx[:, 1], xx[:, 2], 8,
                                                                 0, 1.0)
    rng = np.random.default_rng(5)
    xbar, vbar = rng.standard_normal(x.shape), rng.standard_normal(v.shape)
    xT, vT, L, gx, gv = O.multistep64(x, v, m, steps, nsub, tapes, xbar, vbar, pm=pm)
    assert np.allclose(xT, xx) and np.allclose(vT, vv)
    smp = rng.choice(len(m), 16, replace=False)
    bad = _check_fd_pm(O, x, v, m, steps, nsub, tapes, pm, xbar, vbar, gx, smp, 1e-5, rng)
    assert bad == 0, bad


@pytest.mark.gpu
def test_multistep_with_pm_adjoint_vs_fp64_and_fd(ctx, oracle_lib):
    """One 12^3 box with overload ghosts, 3 PM steps x 2 sub-cycles with the
    driver's PM kicks (half kick opening the first step, a kick closing every
    step), checkpoints every 2 steps: the GPU reverse pass against the FP64
    gradient along the GPU trajectory and FP64 differences of the map."""
    torch = pytest.importorskip("torch")
    O = oracle_lib
    nsteps, nsub = 3, 2
    steps = multistep.schedule(50.0, 30.0, nsteps, nsub)
    p = _boxes(1, 12, 130)[0]
    ng, ngo = p.meta["ng"], p.meta["ngo"]
    pm = multistep.pm_schedule(50.0, 30.0, nsteps, ng, ngo)
    kp = synth.kick_params(p, nd=64)
    ms = multistep.MultiStep(ctx, [kp], steps, nsub, checkpoint_every=2, pm=pm)
    tapes, kick_x = {}, {}

    def on_tape(b, s, j, c, x1):
        tapes[(s, j)] = _tape_of(c, p.n)
        kick_x[(s, j)] = np.stack([t.cpu().numpy() for t in x1], 1).astype(np.float64)
    ms.on_tape = on_tape
    rng = np.random.default_rng(9)
    n = p.n
    xbar = rng.standard_normal((n, 3)).astype(np.float32)
    vbar = rng.standard_normal((n, 3)).astype(np.float32)
    tx = [torch.from_numpy(np.ascontiguousarray(xbar[:, d])).cuda() for d in range(3)]
    tv = [torch.from_numpy(np.ascontiguousarray(vbar[:, d])).cuda() for d in range(3)]
    S0 = multistep.box_state(p)
    # PM kick positions of the GPU trajectory (forward pass, stored)
    rec = []
    ms._run(0, S0.clone(), 0, nsteps, record=rec)
    pm_x = [np.stack([t.cpu().numpy() for t in r[2]], 1).astype(np.float64)
            for r in rec if r[0] == "pm"]
    gx_t, gv_t = ms.adjoint_box(0, S0, tx, tv)
    gx = np.stack([t.cpu().numpy() for t in gx_t], 1).astype(np.float64)
    gv = np.stack([t.cpu().numpy() for t in gv_t], 1).astype(np.float64)
    order = [(s, j) for s in range(nsteps) for j in range(nsub)]
    tl = [tapes[k] for k in order]
    xl = [kick_x[k] for k in order]
    pmd = _pm_dicts(pm)
    x0 = np.stack([p.x, p.y, p.z], 1).astype(np.float64)
    v0 = np.stack([p.vx, p.vy, p.vz], 1).astype(np.float64)
    m = p.mass.astype(np.float64)
    _, _, _, rx, rv = O.multistep64(x0, v0, m, steps, nsub, tl, xbar, vbar, kick_pos=xl, pm=pmd,
                                    pm_pos=pm_x)
    for g, r in ((gx, rx), (gv, rv)):
        rms, mx = force_errors(g, r)
        assert rms <= 2e-5 and mx <= 2e-3, (rms, mx)
    inner = np.flatnonzero(p.mask == 0)
    smp = rng.choice(inner, 24, replace=False)
    _, _, _, fx, _ = O.multistep64(x0, v0, m, steps, nsub, tl, xbar, vbar, pm=pmd)
    bad = _check_fd_pm(O, x0, v0, m, steps, nsub, tl, pmd, xbar, vbar, fx, smp, 1e-4, rng)
    assert bad == 0, bad
    rms, _ = force_errors(gx[smp], fx[smp])
    drift, _ = force_errors(rx[smp], fx[smp])
    assert rms <= drift + 1e-5, (rms, drift)
    assert ms.pm_kicks == 3 * (nsteps + 1)  # forward, recomputation, stored run


@pytest.mark.gpu
def test_boxes_on_two_host_threads_match_one(ctx):
    """Several boxes processed two at a time (two host threads, a context
    each) give the adjoint of the one-at-a-time run."""
    torch = pytest.importorskip("torch")
    nsteps, nsub = 2, 2
    steps = multistep.schedule(50.0, 40.0, nsteps, nsub)
    boxes = _boxes(3, 12, 150)
    kps = [synth.kick_params(b, nd=64) for b in boxes]
    pm = multistep.pm_schedule(50.0, 40.0, nsteps, 12, boxes[0].meta["ngo"])
    ms = multistep.MultiStep(ctx, kps, steps, nsub, checkpoint_every=1, pm=pm, batched=False)
    states = [multistep.box_state(b) for b in boxes]
    rng = np.random.default_rng(6)
    cot = [[torch.from_numpy(rng.standard_normal(b.n).astype(np.float32)).cuda()
            for _ in range(6)] for b in boxes]
    one = ms.adjoint(states, [c[:3] for c in cot], [c[3:] for c in cot], workers=1)
    two = ms.adjoint(states, [c[:3] for c in cot], [c[3:] for c in cot], workers=2)
    for (ax, av), (bx, bv) in zip(one, two):
        for u, w in zip(ax + av, bx + bv):
            rms, _ = force_errors(u.double().cpu().numpy()[:, None], w.double().cpu().numpy()[:, None])
            assert rms <= 1e-5, rms
    fwd1 = ms.forward([S.clone() for S in states], workers=1)
    fwd2 = ms.forward([S.clone() for S in states], workers=2)
    for a, b in zip(fwd1, fwd2):
        for u, w in zip(a.x + a.v, b.x + b.v):
            assert torch.allclose(u, w, rtol=0, atol=1e-4)
    k, q = ms.total_kicks()
    assert k > 0 and q > 0
