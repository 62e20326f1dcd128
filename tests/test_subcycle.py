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
    # the sub-cycles of the first PM step run at its mid point
    ts = synth.stepper(z_in=z, z_fin=10.0, nsteps=10).advanced(1)
    return p, ts


def _oracle_subcycle(O, p, kp, ts, nsub, stream=True, kick=True, fcoeff=None):
    """Particles::subCycle restated by the oracle (pinned bit for bit to the
    reference's own subCycle in the CPU suite); fcoeff overrides map2's c."""
    return O.subcycle(p, ts, nsub, kp, stream=stream, kick=kick, fcoeff=fcoeff)


def _gpu_subcycle(ctx, p, kp, ts, nsub, stream=True, kick=True, fcoeff=None):
    kc = synth.KickParams(**{**kp.__dict__})
    kc.fcoeff = float(synth.kick_coefficient(ts, nsub)) if fcoeff is None else float(fcoeff)
    return ctx.subcycle(p, kc, nsub, p.nglt, ts.alpha, ts.pp, float(synth.stream_tau(ts, nsub)),
                        ts.adot, skip_stream=not stream, skip_kick=not kick)


def test_resort_and_tree_permutation_bit_exact(ctx, oracle_lib):
    p, ts = _state()
    # scramble the order and push a few particles out of the box first
    rng = np.random.default_rng(3)
    p = p.take(rng.permutation(p.n))
    p.x[:50] += 200.0
    kp = synth.kick_params(p, nd=64, fcoeff=0.0)
    q = p.copy()
    # a zero kick coefficient: the velocities are only permuted
    _, nin = _gpu_subcycle(ctx, p, kp, ts, 1, stream=False, fcoeff=0.0)
    _oracle_subcycle(oracle_lib, q, kp, ts, 1, stream=False, fcoeff=0.0)
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
    """The one-PM-step workload: 32^3 at z = 50 with ghosts, 5 sub-cycles,
    starting from rest.  The GPU's kicks differ from the reference's by FP32
    summation order only, and positions by the resulting map1 differences:
    the velocity changes stay within the single-kick tolerance.  (From rest
    because the reference adds every pair term into v: with the box's own
    velocities its kicks carry ~sqrt(list length) roundings of ulp(|v|) each,
    which is not force error.)"""
    p0, ts = _state(ng=32, seed=23)
    p0.vx[:] = 0
    p0.vy[:] = 0
    p0.vz[:] = 0
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
    assert rms <= RMS_TOL and mx <= MAX_TOL, (rms, mx)
