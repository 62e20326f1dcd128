"""The device sub-cycle (hsr_subcycle) against the oracle's restatement of
Particles::subCycle: map1, resortParticles, masses = 1, the RCB kick, map1
(src/cpu/Particles.cxx:1176-1201)."""
import numpy as np
import pytest

import synth
from hsr_testutil import MAX_TOL, RMS_TOL, force_errors, vel

pytestmark = pytest.mark.gpu

NSUB = 5


def _state(ng=24, z=50.0, seed=17):
    p = synth.zeldovich_box(ng, z=z, seed=seed)
    p.id[:] = np.arange(p.n)  # unique ids to match particles across orders
    ts = synth.stepper(z_in=z)
    return p, ts


def _view(p, m):
    return synth.Particles(*(getattr(p, k)[:m] for k in synth.FIELDS), nglt=p.nglt)


def _oracle_subcycle(O, p, kp, ts, nsub, stream=True, kick=True):
    """Particles::subCycle with the oracle (the reference's arithmetic)."""
    tau = np.float32(ts.tau2 / nsub)
    for _ in range(nsub):
        if stream:
            O.map1(p, 1.0, ts.pp, float(tau), ts.adot)
        if kick:
            nin = O.resort(p)
            p.mass[:] = 1.0
            O.rcb_run(_view(p, nin), kp, nthreads=0)
        if stream:
            O.map1(p, 1.0, ts.pp, float(tau), ts.adot)


def _gpu_subcycle(ctx, p, kp, ts, nsub, stream=True, kick=True):
    tau = np.float32(ts.tau2 / nsub)
    return ctx.subcycle(p, kp, nsub, p.nglt, 1.0, ts.pp, float(tau), ts.adot,
                        skip_stream=not stream, skip_kick=not kick)


def test_resort_and_tree_permutation_bit_exact(ctx, oracle_lib):
    p, ts = _state()
    # scramble the order and push a few particles out of the box first
    rng = np.random.default_rng(3)
    p = p.take(rng.permutation(p.n))
    p.x[:50] += 200.0
    kp = synth.kick_params(p, nd=64, fcoeff=0.0)
    q = p.copy()
    _, nin = _gpu_subcycle(ctx, p, kp, ts, 1, stream=False)
    _oracle_subcycle(oracle_lib, q, kp, ts, 1, stream=False)
    assert nin == p.n - 50
    for k in synth.FIELDS:
        assert np.array_equal(getattr(p, k).view(np.uint8), getattr(q, k).view(np.uint8)), k


def test_one_subcycle_matches_oracle(ctx, oracle_lib):
    p, ts = _state()
    kp = synth.kick_params(p, nd=64, nsub=NSUB)
    q = p.copy()
    _gpu_subcycle(ctx, p, kp, ts, 1)
    _oracle_subcycle(oracle_lib, q, kp, ts, 1)
    for k in ("id", "mask", "mass", "phi"):
        assert np.array_equal(getattr(p, k), getattr(q, k)), k
    # positions after the second half-stream carry the kicks' FP32 differences
    assert np.abs(np.stack([p.x - q.x, p.y - q.y, p.z - q.z])).max() < 1e-5


def test_five_subcycles_match_oracle_by_particle(ctx, oracle_lib):
    p0, ts = _state(seed=23)
    kp = synth.kick_params(p0, nd=64, nsub=NSUB)
    p, q = p0.copy(), p0.copy()
    st, _ = _gpu_subcycle(ctx, p, kp, ts, NSUB)
    _oracle_subcycle(oracle_lib, q, kp, ts, NSUB)
    assert st["pairs"] > 0
    a, b = np.argsort(p.id), np.argsort(q.id)
    dx = np.stack([p.x[a] - q.x[b], p.y[a] - q.y[b], p.z[a] - q.z[b]])
    assert np.abs(dx).max() < 1e-4
    v0 = vel(p0)[np.argsort(p0.id)]
    rms, mx = force_errors(vel(p)[a] - v0, vel(q)[b] - v0)
    assert rms <= 10 * RMS_TOL and mx <= MAX_TOL, (rms, mx)
