"""The multi-step driver's host logic on the CPU (no GPU).

multistep.MultiStep orders the half-streams, kicks and PM kicks of every
sub-cycle, keeps checkpoints, recomputes each segment in the reverse pass and
chains the VJPs; in lockstep it sends every box's kick through one multi-box
call.  Here it drives a float64 stand-in for the library context whose stream
is x += c v, whose kick is v += fcoeff m_i sum_j m_j exp(-r_ij^2 / s^2) d_ij
over all pairs and whose PM kick is a smooth external field; the VJPs come
from torch's autograd on the same float64 functions.  The driver's gradient
must then equal central differences of its own forward map, every checkpoint
interval must give the same gradient, and lockstep must equal box by box.
The library's own kernels are checked against FP64 in the GPU tests; this
file checks the orchestration around them.
"""
import dataclasses

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import multistep  # noqa: E402
import synth  # noqa: E402

SIGMA2 = 4.0


def _kick_field(x, m):
    """a_i = sum_j m_j exp(-|x_j - x_i|^2 / s^2) (x_j - x_i) (n x 3)."""
    d = x[None, :, :] - x[:, None, :]
    w = torch.exp(-(d * d).sum(2) / SIGMA2) * m[None, :]
    return (w[:, :, None] * d).sum(1)


def _pm_field(x, q):
    """A smooth external field of strength q (stands in for the PM kick)."""
    return q * torch.stack([torch.sin(0.3 * x[:, 1]), torch.cos(0.2 * x[:, 2]),
                            torch.sin(0.25 * x[:, 0] + 0.1 * x[:, 1])], 1)


class FakeContext:
    """The context methods the driver calls, in float64 on the CPU."""

    device = 0

    def __init__(self):
        self.tape = None
        self.batch_tape = None
        self.calls = {"kick": 0, "kick_batch": 0, "fwd": 0, "fwd_batch": 0, "pm": 0}

    @staticmethod
    def _xs(x, y, z):
        return torch.stack([x, y, z], 1)

    def stream_device(self, x, y, z, vx, vy, vz, alpha, pp, tau, adot):
        c = tau * (1.0 + 0.1 * alpha) / (pp * adot) * 50.0
        x.add_(c * vx)
        y.add_(c * vy)
        z.add_(c * vz)

    def _dv(self, X, m, kp):
        return kp.fcoeff * m[:, None] * _kick_field(X, m)

    def force_kick_device(self, x, y, z, mass, vx, vy, vz, kp):
        dv = self._dv(self._xs(x, y, z), mass, kp)
        for t, d in zip((vx, vy, vz), dv.unbind(1)):
            t.add_(d)
        self.calls["kick"] += 1

    def force_fwd_device(self, x, y, z, mass, dvx, dvy, dvz, kp):
        X = self._xs(x, y, z).clone()
        dv = self._dv(X, mass, kp)
        for t, d in zip((dvx, dvy, dvz), dv.unbind(1)):
            t.copy_(d)
        self.tape = (X, mass, kp)
        self.calls["fwd"] += 1

    def _vjp(self, tape, u):
        X, m, kp = tape
        X = X.clone().requires_grad_(True)
        (g,) = torch.autograd.grad((self._dv(X, m, kp) * u).sum(), X)
        return g

    def force_vjp_device(self, ux, uy, uz, xbx, xby, xbz):
        g = self._vjp(self.tape, self._xs(ux, uy, uz))
        for t, d in zip((xbx, xby, xbz), g.unbind(1)):
            t.copy_(d)

    def force_kick_batch_device(self, xs, masses, vs, kps):
        for x, m, v, kp in zip(xs, masses, vs, kps):
            dv = self._dv(self._xs(*x), m, kp)
            for t, d in zip(v, dv.unbind(1)):
                t.add_(d)
        self.calls["kick_batch"] += 1
        return {}

    def force_fwd_batch_device(self, xs, masses, dvs, kps):
        self.batch_tape = []
        for x, m, out, kp in zip(xs, masses, dvs, kps):
            X = self._xs(*x).clone()
            dv = self._dv(X, m, kp)
            for t, d in zip(out, dv.unbind(1)):
                t.copy_(d)
            self.batch_tape.append((X, m, kp))
        self.calls["fwd_batch"] += 1
        return {}

    def force_vjp_batch_device(self, us, xbars):
        assert len(us) == len(self.batch_tape)
        for tape, u, xb in zip(self.batch_tape, us, xbars):
            g = self._vjp(tape, self._xs(*u))
            for t, d in zip(xb, g.unbind(1)):
                t.copy_(d)

    def pm_kick_device(self, x, y, z, vx, vy, vz, q):
        dv = _pm_field(self._xs(x, y, z), q)
        for t, d in zip((vx, vy, vz), dv.unbind(1)):
            t.add_(d)
        self.calls["pm"] += 1
        return {}

    def pm_vjp_device(self, x, y, z, ux, uy, uz, xbx, xby, xbz, q):
        X = self._xs(x, y, z).clone().requires_grad_(True)
        (g,) = torch.autograd.grad((_pm_field(X, q) * self._xs(ux, uy, uz)).sum(), X)
        for t, d in zip((xbx, xby, xbz), g.unbind(1)):
            t.copy_(d)


@pytest.fixture(autouse=True)
def _no_device_sync(monkeypatch):
    # the stand-in works on CPU tensors: nothing to wait for
    monkeypatch.setattr(multistep, "_torch_done", lambda: None)


def _states(nbox, n, seed):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(nbox):
        f = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.float64))
        x = rng.random((3, n)) * 6.0
        v = rng.standard_normal((3, n)) * 0.5
        m = 1.0 + 0.2 * rng.random(n)
        out.append(multistep.BoxState([f(a) for a in x], [f(a) for a in v], f(m)))
    return out


def _driver(nbox, every, pm=True, batched=True, nsteps=4, nsub=2):
    steps = multistep.schedule(50.0, 30.0, nsteps, nsub)
    # fcoeff scaled so the kicks move the particles visibly over the run
    steps = [dataclasses.replace(s, fcoeff=0.02 * (1 + i)) for i, s in enumerate(steps)]
    kps = [_kp() for _ in range(nbox)]
    pmk = ([(0.05 if s == 0 else None, 0.1 + 0.01 * s) for s in range(nsteps)] if pm else None)
    return multistep.MultiStep(FakeContext(), kps, steps, nsub, checkpoint_every=every, pm=pmk,
                               batched=batched)


def _kp():
    """Kick parameters (the stand-in reads fcoeff only; the driver sets it
    per step)."""
    p = synth.random_box(8, 4.0, 1)
    return synth.kick_params(p, nd=8)


def _cot(states, seed):
    rng = np.random.default_rng(seed)
    f = lambda: torch.from_numpy(rng.standard_normal(states[0].x[0].shape[0]))
    return [[f() for _ in range(3)] for _ in states], [[f() for _ in range(3)] for _ in states]


def _flat(xb, vb):
    return torch.cat([t.reshape(-1) for t in list(xb) + list(vb)])


@pytest.mark.parametrize("pm", [False, True])
def test_gradient_matches_central_differences(pm):
    """<(xbar_0, vbar_0), (dx_0, dv_0)> equals the central difference of
    <(xbar_T, vbar_T), forward(x_0 + h dx_0, v_0 + h dv_0)>."""
    S0 = _states(1, 20, 3)
    xbars, vbars = _cot(S0, 4)
    M = _driver(1, every=2, pm=pm, batched=False)
    gx, gv = M.adjoint_box(0, S0[0], xbars[0], vbars[0])
    rng = np.random.default_rng(5)
    h = 1e-5
    for _ in range(3):
        dx = [torch.from_numpy(rng.standard_normal(20)) for _ in range(3)]
        dv = [torch.from_numpy(rng.standard_normal(20)) for _ in range(3)]
        vals = []
        for s in (h, -h):
            S = multistep.BoxState([a + s * b for a, b in zip(S0[0].x, dx)],
                                   [a + s * b for a, b in zip(S0[0].v, dv)], S0[0].mass)
            M.forward_box(0, S)
            vals.append(float(_flat(xbars[0], vbars[0]) @ _flat(S.x, S.v)))
        fd = (vals[0] - vals[1]) / (2 * h)
        got = float(_flat(gx, gv) @ _flat(dx, dv))
        assert abs(got - fd) <= 1e-7 * max(1.0, abs(fd)), (got, fd)


def test_every_checkpoint_interval_gives_the_same_gradient():
    S0 = _states(1, 16, 6)
    xbars, vbars = _cot(S0, 7)
    ref = None
    for every in (None, 1, 2, 3, 4, 5):
        M = _driver(1, every=every, batched=False, nsteps=5)
        g = _flat(*M.adjoint_box(0, S0[0], xbars[0], vbars[0]))
        if ref is None:
            ref = g
        assert torch.allclose(g, ref, rtol=1e-12, atol=1e-12), every
        # the forward, the recomputed segments and the reverse pass's tapes
        if every is not None:
            assert M.kicks == multistep.kicks_per_box(5, 2, checkpointed=True)
    # the inputs are not modified
    assert all(torch.equal(a, b) for a, b in zip(S0[0].x, _states(1, 16, 6)[0].x))


def test_lockstep_equals_box_by_box():
    """forward_all / adjoint_all (one multi-box call per sub-cycle's kicks)
    against forward_box / adjoint_box of every box."""
    S0 = _states(3, 12, 8)
    xbars, vbars = _cot(S0, 9)
    A = _driver(3, every=2, batched=True)
    B = _driver(3, every=2, batched=False)
    ga = A.adjoint(S0, xbars, vbars)
    gb = B.adjoint(S0, xbars, vbars)
    for (xa, va), (xb, vb) in zip(ga, gb):
        assert torch.allclose(_flat(xa, va), _flat(xb, vb), rtol=1e-12, atol=1e-12)
    Fa = A.forward([S.clone() for S in S0])
    Fb = B.forward([S.clone() for S in S0])
    for Sa, Sb in zip(Fa, Fb):
        assert torch.allclose(_flat(Sa.x, Sa.v), _flat(Sb.x, Sb.v), rtol=1e-14, atol=1e-14)
    # one multi-box call per sub-cycle in the forward and per kick in the
    # reverse pass's recomputation and tapes: 3 x 4 steps x 2 sub-cycles
    ctx = A.ctx
    assert ctx.calls["kick"] == 0 and ctx.calls["fwd"] == 0
    assert ctx.calls["kick_batch"] == 2 * 4 * 2 + 4 * 2
    assert ctx.calls["fwd_batch"] == 4 * 2
    assert A.total_kicks()[0] == 3 * (3 * 4 * 2) + 3 * 4 * 2


def test_pm_kicks_open_the_first_step_and_close_every_step():
    """A PM kick before the first step's sub-cycles (half kick) and one after
    every step's: the forward runs 1 + nsteps of them per box."""
    S0 = _states(2, 10, 10)
    M = _driver(2, every=None, pm=True, batched=True, nsteps=3)
    M.forward([S.clone() for S in S0])
    assert M.pm_kicks == 2 * (1 + 3)
    N = _driver(2, every=None, pm=False, batched=True, nsteps=3)
    N.forward([S.clone() for S in S0])
    assert N.pm_kicks == 0


def test_bad_arguments_are_rejected():
    steps = multistep.schedule(50.0, 30.0, 2, 2)
    with pytest.raises(ValueError):
        multistep.MultiStep(FakeContext(), [_kp()], steps, 2, checkpoint_every=0)
    with pytest.raises(ValueError):
        multistep.MultiStep(FakeContext(), [_kp()], steps, 2, pm=[(None, 0.1)])
