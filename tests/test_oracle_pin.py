"""The CPU oracle against the reference: golden fixtures written by the
reference build, and (when the reference tree is present) live runs."""
import numpy as np
import pytest

import oracle
import synth
from hsr_testutil import golden_names, load_golden


@pytest.mark.parametrize("name", golden_names())
def test_oracle_reproduces_golden(oracle_lib, name):
    p, kp, out = load_golden(name)
    oracle_lib.rcb_run(p, kp, nthreads=2)
    for k in synth.FIELDS:
        got = getattr(p, k)
        assert np.array_equal(got.view(np.uint8), out[k].view(np.uint8)), f"{name}: {k} differs"


@pytest.mark.skipif(not oracle.reference_available(), reason="reference build (oracle/_ref) absent")
@pytest.mark.parametrize("nd,tdpts,oa", [(64, 1, 0.1), (32, 12, 0.5)])
def test_oracle_matches_reference_live(oracle_lib, nd, tdpts, oa):
    p = synth.zeldovich_box(16, z=10.0, seed=99)
    kp = synth.kick_params(p, nd=nd, tdpts=tdpts, open_angle=oa)
    q = p.copy()
    oracle_lib.rcb_run(q, kp, nthreads=4)
    ref, _, _ = oracle.run_reference(p, kp, nthreads=4)
    for k in synth.FIELDS:
        assert np.array_equal(getattr(q, k).view(np.uint8), ref[k].view(np.uint8)), k


@pytest.mark.skipif(not oracle.reference_available(), reason="reference build (oracle/_ref) absent")
def test_oracle_matches_reference_on_long_chains(oracle_lib):
    """A node order whose partitions each carry one swap chain through all of
    their left elements: the oracle's tree, permutation and kick against the
    reference's."""
    p = synth.sorted_line(20000)
    kp = synth.kick_params(p, nd=32, fcoeff=1.0)
    kp.min_force, kp.max_force = (1.0, 0.0, 0.0), (39.0, 0.5, 0.5)
    q = p.copy()
    st = oracle_lib.rcb_run(q, kp, nthreads=4).stats
    ref, _, _ = oracle.run_reference(p, kp, nthreads=4)
    for k in synth.FIELDS:
        assert np.array_equal(getattr(q, k).view(np.uint8), ref[k].view(np.uint8)), k
    assert st["processed_leaves"] > 0


@pytest.mark.skipif(not oracle.reference_available(1), reason="RCO reference build absent")
@pytest.mark.parametrize("nd,tdpts,oa", [(64, 1, 0.1), (16, 12, 0.5), (8, 1, 0.1)])
def test_oracle_rco_matches_reference_live(oracle_lib, nd, tdpts, oa):
    """The RCO octree restatement against the reference's RCOForceTree
    (oracle/_ref/rco_ref: its octant array sized 8, otherwise unmodified)."""
    p = synth.clustered_box(16, nhalo=20, seed=98)
    kp = synth.kick_params(p, nd=nd, tdpts=tdpts, open_angle=oa)
    kp.tree = 1
    q = p.copy()
    st = oracle_lib.rcb_run(q, kp, nthreads=4).stats
    ref, _, _ = oracle.run_reference(p, kp, nthreads=4)
    for k in synth.FIELDS:
        assert np.array_equal(getattr(q, k).view(np.uint8), ref[k].view(np.uint8)), k
    assert st["processed_leaves"] > 0


def test_oracle_law_matches_fp64(oracle_lib):
    r2 = np.linspace(0.0, 9.7, 977)
    for x in r2:
        g32 = oracle_lib.law_f32(oracle.LAW_POLY6, 0.1, float(np.float32(x)))
        g64 = oracle_lib.law_f64(oracle.LAW_POLY6, 0.1, float(np.float32(x)))
        # g is a difference of (r2+rsm^2)^-1.5 and a polynomial of size ~0.27:
        # the FP32 error scales with the larger term
        scale = max(float(np.float32(x) + 0.01) ** -1.5, 0.3)
        assert abs(g32 - g64) <= 1e-6 * scale


def test_oracle_list_overflow_reported(oracle_lib):
    p = synth.random_box(3000, 4.0, 1)
    kp = synth.kick_params(p, nd=64)
    kp.min_force, kp.max_force = (0.1,) * 3, (3.9,) * 3
    with pytest.raises(RuntimeError, match="VMAX"):
        oracle_lib.rcb_run(p, kp, vmax=1000)


# ---- the sub-cycle around the kick and its time stepper -------------------

SUBREF = pytest.mark.skipif(not oracle.subcycle_reference_available(),
                            reason="reference sub-cycle build (oracle/_ref/sub_ref) absent")


@SUBREF
@pytest.mark.parametrize("z_in,z_fin,nsteps", [(50.0, 10.0, 10), (200.0, 0.0, 500), (30.0, 20.0, 3)])
def test_stepper_matches_reference(z_in, z_fin, nsteps):
    """synth.stepper / Stepper.advanced against the reference's TimeStepper
    (built from Basedata's float values and advanced half a step at a time):
    pp, aa, adot, fscal, tau and tau2 equal to the last bit."""
    empty = synth.random_box(0, 4.0, 1)
    base = synth.stepper(z_in=z_in, z_fin=z_fin, nsteps=nsteps)
    for half in sorted({0, 1, 2, 3, nsteps, 2 * nsteps - 1, 2 * nsteps}):
        _, info = oracle.run_reference_subcycle(empty, ng=(4, 4, 4), nsub=0, z_in=z_in,
                                                z_fin=z_fin, nsteps=nsteps, half_steps=half)
        ts = base.advanced(half)
        got = {"pp": ts.pp, "aa": ts.aa, "adot": ts.adot, "fscal": ts.fscal, "tau": ts.tau,
               "tau2": ts.tau2}
        for k, v in got.items():
            assert v == info[k], (half, k, v, info[k])


@SUBREF
@pytest.mark.parametrize("ng,nsub,tdpts,half", [(16, 1, 1, 1), (20, 5, 1, 3), (16, 5, 12, 1),
                                                (32, 5, 1, 1)])
def test_subcycle_restatement_matches_reference(oracle_lib, ng, nsub, tdpts, half):
    """Oracle.subcycle (map1, resortParticles, the kick with map2's
    coefficient, map1) against the reference's own Particles::subCycle on a
    Zel'dovich box with ghosts: all ten arrays bit for bit after nsub
    sub-cycles.  The last case is the one-PM-step workload's 32^3 box."""
    p = synth.zeldovich_box(ng, z=50.0, seed=40 + ng)
    q = p.copy()
    z_in, z_fin, nsteps = 50.0, 10.0, 10
    ts = synth.stepper(z_in=z_in, z_fin=z_fin, nsteps=nsteps).advanced(half)
    kp = synth.kick_params(q, nd=64, tdpts=tdpts)
    nin = oracle_lib.subcycle(q, ts, nsub, kp, nthreads=4)
    ref, info = oracle.run_reference_subcycle(
        p, ng=p.nglt, nsub=nsub, z_in=z_in, z_fin=z_fin, nsteps=nsteps, half_steps=half, nd=64,
        ds=kp.ds, tmin=kp.tmin,
        use_rcb_tree=oracle.USE_RCB_MONO if tdpts == 1 else oracle.USE_RCB_QUAD, nthreads=4)
    assert info["np_last"] == nin and info["pp"] == ts.pp
    for k in synth.FIELDS:
        assert np.array_equal(getattr(q, k).view(np.uint8), ref[k].view(np.uint8)), k
    # the kicks did move the velocities
    assert not np.array_equal(q.vx, p.vx)
