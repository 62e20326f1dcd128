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
