"""Parity of the GPU path (through the C ABI) with the reference and the oracle.

Tolerances: FP32 forces within RMS_TOL = 1e-5 rms relative and MAX_TOL = 1e-3
of the rms force (hsr_testutil.force_errors); every integer/index result (the
tree permutation, positions, ids, masks, the list entries) bit-exact.
"""
import numpy as np
import pytest

import hsr
import synth
from hsr_testutil import (MAX_TOL, RMS_TOL, force_errors, golden_names, load_golden,
                          same_lists, same_lists_exact, vel)

pytestmark = pytest.mark.gpu

EXACT = ("x", "y", "z", "mass", "phi", "id", "mask")


@pytest.mark.parametrize("kernel", [hsr.KERNEL_PLAIN, hsr.KERNEL_AUTO])
@pytest.mark.parametrize("name", golden_names())
def test_golden_kick(ctx, name, kernel):
    p, kp, out = load_golden(name)
    v_in = p.copy()
    hsr.HostLists(v_in, kp)  # the input velocities in the tree's order
    st = ctx.rcb_kick(p, kp, kernel=kernel)
    for k in EXACT:
        assert np.array_equal(getattr(p, k).view(np.uint8), out[k].view(np.uint8)), f"{name}: {k}"
    dv = vel(p) - vel(v_in)
    dv_ref = np.stack([out["vx"], out["vy"], out["vz"]], 1).astype(np.float64) - vel(v_in)
    rms, mx = force_errors(dv, dv_ref)
    # The reference adds every pair term straight into v, so its kick carries
    # FP32 rounding of |v| per term; allow for that where v_in is not zero.
    vscale = np.abs(vel(v_in)).max(initial=0.0)
    dscale = np.sqrt((dv_ref ** 2).sum(1).mean()) if p.n else 1.0
    slack = 0.0 if vscale == 0 else 64 * 2.0 ** -24 * vscale / dscale
    assert rms <= RMS_TOL + slack, (name, rms, slack)
    assert mx <= MAX_TOL + slack, (name, mx, slack)
    assert st["kernel_launches"] >= (1 if st["processed_leaves"] else 0)


def _zero_v(p):
    p.vx[:] = 0
    p.vy[:] = 0
    p.vz[:] = 0
    return p


@pytest.mark.parametrize("nd,tdpts", [(64, 1), (128, 1), (32, 12)])
def test_zeldovich32_forces_vs_oracle(ctx, oracle_lib, nd, tdpts):
    """32^3 lattice at z=50 with overload ghosts (the one-PM-step case): GPU
    forces vs the oracle's (the reference's arithmetic) and vs FP64 over the
    same lists; lists bit-exact."""
    p = _zero_v(synth.zeldovich_box(32))
    kp = synth.kick_params(p, nd=nd, tdpts=tdpts, fcoeff=1.0)
    q = p.copy()
    ctx.rcb_kick(p, kp, kernel=hsr.KERNEL_AUTO)
    r = oracle_lib.rcb_run(q, kp, keep_lists=True, nthreads=0)
    for k in EXACT:
        assert np.array_equal(getattr(p, k).view(np.uint8), getattr(q, k).view(np.uint8)), k
    off, cnt, ptr = r.leaves()
    sel = np.concatenate([np.arange(o, o + c) for o, c in zip(off, cnt)])
    rms, mx = force_errors(vel(p)[sel], vel(q)[sel])
    assert rms <= RMS_TOL and mx <= MAX_TOL, (rms, mx)
    a64 = r.acc_fp64()[sel]
    rms64, mx64 = force_errors(vel(p)[sel], a64)
    assert rms64 <= RMS_TOL and mx64 <= MAX_TOL, (rms64, mx64)
    goff, gcnt, gptr, ge = ctx.lists()
    assert same_lists(goff, gcnt, gptr, ge, off, cnt, ptr, r.entries())
    assert ctx.stats()["pairs"] == r.stats["pairs"]


def test_plain_and_batched_agree(ctx):
    p = _zero_v(synth.zeldovich_box(32, z=10.0, seed=3))
    kp = synth.kick_params(p, nd=128, fcoeff=1.0)
    q = p.copy()
    ctx.rcb_kick(p, kp, kernel=hsr.KERNEL_PLAIN)
    ctx.rcb_kick(q, kp, kernel=hsr.KERNEL_BATCHED)
    rms, mx = force_errors(vel(q), vel(p))
    assert rms <= RMS_TOL and mx <= MAX_TOL


def test_force_law_on_device(ctx, oracle_lib):
    r2 = np.linspace(0.0, 10.0, 4001).astype(np.float32)
    g = ctx.force_law(r2)
    rmax2 = np.float32(3.116326355) ** 2
    for x, gx in zip(r2, g):
        if x < rmax2:
            g64 = oracle_lib.law_f64(0, 0.1, float(x))
            assert abs(gx - g64) <= 1e-6 * max(float(x + 0.01) ** -1.5, 0.3), (x, gx, g64)
        else:
            assert gx == 0.0
    # the cutoff is strict at fsrrmax^2 and inclusive of the law's own r2max
    g2 = ctx.force_law(np.array([np.nextafter(rmax2, 0, dtype=np.float32), rmax2], np.float32))
    assert g2[0] != 0.0 and g2[1] == 0.0


def test_linear_in_fcoeff(ctx):
    """v_out = fcoeff * m * a: doubling fcoeff doubles the kick bit for bit."""
    p = _zero_v(synth.zeldovich_box(24, z=10.0, seed=8))
    kp = synth.kick_params(p, nd=64, fcoeff=0.375)
    q = p.copy()
    ctx.rcb_kick(p, kp)
    kp.fcoeff = 0.75
    ctx.rcb_kick(q, kp)
    assert np.array_equal(2 * vel(p), vel(q))


def test_momentum_conserved_with_symmetric_lists(ctx):
    """Opening angle 0 opens every node, so every list holds whole leaves whose
    boxes lie within fsrrmax of the target leaf: the pair set is symmetric and
    the pair forces cancel, sum_i m_i a_i = 0 up to FP32 rounding."""
    p = _zero_v(synth.random_box(6000, 14.0, 17))
    kp = synth.kick_params(p, nd=32, open_angle=0.0, fcoeff=1.0)
    kp.min_force, kp.max_force = (-1.0,) * 3, (15.0,) * 3
    ctx.rcb_kick(p, kp)
    a = vel(p)
    total = np.abs((a * p.mass[:, None]).sum(0))
    scale = np.abs(a).sum(0)
    assert np.all(total <= 1e-5 * scale), (total, scale)


@pytest.mark.parametrize("case", ["empty", "one", "coincident", "nd1", "outside"])
def test_edge_cases(ctx, oracle_lib, case):
    if case == "empty":
        p = synth.random_box(0, 4.0, 1)
    elif case == "one":
        p = synth.random_box(1, 4.0, 1)
    elif case == "coincident":  # one split fails: a leaf far above nd
        p = synth.random_box(300, 4.0, 1)
        p.x[:200] = 2.0
        p.y[:200] = 2.0
        p.z[:200] = 2.0
    elif case == "nd1":
        p = synth.random_box(400, 6.0, 2)
    else:  # nothing inside the force box
        p = synth.random_box(500, 6.0, 3)
    p = _zero_v(p)
    kp = synth.kick_params(p, nd=1 if case == "nd1" else 16, fcoeff=1.0)
    if case == "outside":
        kp.min_force, kp.max_force = (20.0,) * 3, (30.0,) * 3
    else:
        kp.min_force, kp.max_force = (-1.0,) * 3, (9.0,) * 3
    q = p.copy()
    st = ctx.rcb_kick(p, kp)
    r = oracle_lib.rcb_run(q, kp, nthreads=2)
    assert st["pairs"] == r.stats["pairs"]
    for k in EXACT:
        assert np.array_equal(getattr(p, k).view(np.uint8), getattr(q, k).view(np.uint8)), k
    if p.n:
        rms, mx = force_errors(vel(p), vel(q))
        assert rms <= RMS_TOL and mx <= MAX_TOL, (rms, mx)


def test_repeated_calls_reuse_buffers(ctx):
    """Shrinking and growing inputs on one context give the same answers as
    fresh calls."""
    big = _zero_v(synth.zeldovich_box(20, seed=1))
    small = _zero_v(synth.zeldovich_box(10, seed=2))
    kb, ks = synth.kick_params(big, nd=64, fcoeff=1.0), synth.kick_params(small, nd=64, fcoeff=1.0)
    outs = []
    for p, kp in ((big, kb), (small, ks), (big, kb)):
        q = p.copy()
        ctx.rcb_kick(q, kp)
        outs.append(vel(q))
    assert np.array_equal(outs[0], outs[2])


def test_full_size_128_sampled_leaves_vs_fp64(ctx):
    """128^3 at z=50 (the plain-vs-batched workload) through the C ABI: the
    permutation keeps every particle, and the forces of a sample of leaves
    match an FP64 evaluation of the exported lists."""
    p = _zero_v(synth.zeldovich_box(128))
    ids_in = np.sort(p.id)
    kp = synth.kick_params(p, nd=128, fcoeff=1.0)
    st = ctx.rcb_kick(p, kp)
    assert np.array_equal(np.sort(p.id), ids_in)
    off, cnt, ptr, e = ctx.lists()
    rng = np.random.default_rng(0)
    a_gpu, a64 = [], []
    for l in rng.choice(len(off), 40, replace=False):
        o, c = off[l], cnt[l]
        E = e[:, ptr[l]:ptr[l + 1]].astype(np.float64)
        xi = np.stack([p.x[o:o + c], p.y[o:o + c], p.z[o:o + c]], 1).astype(np.float64)
        d = E[:3].T[None, :, :] - xi[:, None, :]
        r2 = (d ** 2).sum(-1)
        g = _g64(r2)
        w = g * E[3][None, :] * (r2 < float(np.float32(3.116326355) ** 2))
        a64.append((w[:, :, None] * d).sum(1) * p.mass[o:o + c, None])
        a_gpu.append(vel(p)[o:o + c])
    rms, mx = force_errors(np.concatenate(a_gpu), np.concatenate(a64))
    assert rms <= RMS_TOL and mx <= MAX_TOL, (rms, mx)
    assert st["pairs"] > 1e9


def test_full_size_128_vs_oracle(ctx, oracle_lib, monkeypatch):
    """The bench workload itself -- 128^3 Zel'dovich at z = 50 with overload
    ghosts (2.57 M particles), nd = 128, opening angle 0.1, rsm = 0.1, poly6,
    monopole -- through hsr_rcb_kick against the oracle run on the same input:
    the permutation of x, y, z, mass, phi, id and mask bit for bit, every
    processed leaf's list the same multiset of entries bit for bit, the same
    pair count, and the kick within RMS_TOL / MAX_TOL of the oracle's and of
    FP64 over the same lists."""
    monkeypatch.setenv("ORA_MAX_ACTIVE_LEVELS", "1")  # the oracle's nesting; same results
    p = _zero_v(synth.zeldovich_box(128))
    kp = synth.kick_params(p, nd=128, fcoeff=1.0)
    q = p.copy()
    st = ctx.rcb_kick(p, kp)
    r = oracle_lib.rcb_run(q, kp, keep_lists=True, nthreads=0)
    for k in EXACT:
        assert np.array_equal(getattr(p, k).view(np.uint8), getattr(q, k).view(np.uint8)), k
    assert st["pairs"] == r.stats["pairs"] and st["pairs"] > 5e9
    assert st["list_entries"] == r.stats["list_entries"]
    assert st["processed_leaves"] == r.stats["processed_leaves"]
    off, cnt, ptr = r.leaves()
    goff, gcnt, gptr, ge = ctx.lists()
    assert same_lists_exact(goff, gcnt, gptr, ge, off, cnt, ptr, r.entries())
    del ge
    sel = np.concatenate([np.arange(o, o + c) for o, c in zip(off, cnt)])
    rms, mx = force_errors(vel(p)[sel], vel(q)[sel])
    assert rms <= RMS_TOL and mx <= MAX_TOL, (rms, mx)
    rms64, mx64 = force_errors(vel(p)[sel], r.acc_fp64()[sel])
    assert rms64 <= RMS_TOL and mx64 <= MAX_TOL, (rms64, mx64)


def _g64(r2, rsm=float(np.float32(0.1))):
    a = [0.271431, -0.0783394, 0.0133122, -0.00159485, 0.000132336, -0.00000663394,
         0.000000147305]
    a = [float(np.float32(v)) for v in a]
    p = np.zeros_like(r2)
    for c in a[::-1]:
        p = p * r2 + c
    return (r2 + rsm * rsm) ** -1.5 - p


@pytest.mark.parametrize("case", ["zel32_nd64", "zel24_quad", "blob_oa05", "random_nd4",
                                  "long_chains"])
def test_device_build_equals_host_build(ctx, case):
    """The GPU tree/list build gives the host build's permutation and lists
    bit for bit, and the same kick within the FP32 tolerance."""
    if case == "zel32_nd64":
        p = synth.zeldovich_box(32, seed=21)
        kp = synth.kick_params(p, nd=64)
    elif case == "zel24_quad":
        # opening angle 1.0: the lists hold 12-point pseudo-particles (none at
        # 0.1 on this set), compared bit for bit with the host build's
        p = synth.zeldovich_box(24, z=10.0, seed=22)
        kp = synth.kick_params(p, nd=32, tdpts=12, open_angle=1.0)
    elif case == "blob_oa05":
        p, kp, _ = load_golden("blob3000_nd8_oa05_mono")
    elif case == "long_chains":
        # the chunk partition's run jumps at the top levels, the one-block
        # partition's pointer jumping below 16384 elements
        p = synth.sorted_line(40000)
        kp = synth.kick_params(p, nd=64, fcoeff=1.0)
        kp.min_force, kp.max_force = (1.0, 0.0, 0.0), (39.0, 0.5, 0.5)
    else:
        p = synth.random_box(5000, 10.0, 23)
        kp = synth.kick_params(p, nd=4, fcoeff=1.0)
        kp.min_force, kp.max_force = (0.5,) * 3, (9.5,) * 3
    q = p.copy()
    ctx.rcb_kick(p, kp, build=hsr.BUILD_HOST)
    lh = ctx.lists()
    st = ctx.rcb_kick(q, kp, build=hsr.BUILD_DEVICE)
    ld = ctx.lists()
    for k in EXACT:
        assert np.array_equal(getattr(p, k).view(np.uint8), getattr(q, k).view(np.uint8)), k
    assert same_lists(*lh, *ld)
    rms, mx = force_errors(vel(q), vel(p))
    assert rms <= RMS_TOL and mx <= MAX_TOL, (rms, mx)
    assert st["pairs"] == ctx.stats()["pairs"]


def test_cm_sequential_fallback_path(ctx, monkeypatch):
    """Every node's centre of mass through the sequential fallback gives the
    same tree as the certified parallel sum."""
    p = synth.zeldovich_box(20, seed=31)
    kp = synth.kick_params(p, nd=32)
    q = p.copy()
    ctx.rcb_kick(p, kp)
    lp = ctx.lists()
    monkeypatch.setenv("HSR_FORCE_CM_FALLBACK", "1")
    st = ctx.rcb_kick(q, kp)
    monkeypatch.delenv("HSR_FORCE_CM_FALLBACK")
    assert st["cm_fallbacks"] == st["nodes"]
    for k in EXACT:
        assert np.array_equal(getattr(p, k).view(np.uint8), getattr(q, k).view(np.uint8)), k
    assert same_lists(*lp, *ctx.lists())
    assert np.array_equal(vel(p), vel(q))


@pytest.mark.parametrize("ng,nd", [(20, 32), (48, 64)])
def test_cm_tight_certification_path(ctx, monkeypatch, ng, nd):
    """Every node's centre of mass through the tight certification (up to 64
    nodes per level; the rest sequential) gives the same tree as the loose
    certification: the tight bound never certifies a wrong float."""
    p = synth.clustered_box(ng, nhalo=30, seed=5)
    kp = synth.kick_params(p, nd=nd)
    q = p.copy()
    ctx.rcb_kick(p, kp)
    lp = ctx.lists()
    monkeypatch.setenv("HSR_FORCE_CM_FALLBACK", "2")
    st = ctx.rcb_kick(q, kp)
    monkeypatch.delenv("HSR_FORCE_CM_FALLBACK")
    assert st["cm_fallbacks"] < st["nodes"]  # the tight pass certified some
    for k in EXACT:
        assert np.array_equal(getattr(p, k).view(np.uint8), getattr(q, k).view(np.uint8)), k
    assert same_lists(*lp, *ctx.lists())
    assert np.array_equal(vel(p), vel(q))


def test_device_memory_arrays(ctx):
    """HSR_MEM_DEVICE: the same kick on arrays already in HBM."""
    torch = pytest.importorskip("torch")
    p = synth.zeldovich_box(24, seed=41)
    kp = synth.kick_params(p, nd=64)
    q = p.copy()
    ctx.rcb_kick(p, kp)
    t = {k: torch.from_numpy(getattr(q, k).view(np.int16) if k == "mask" else getattr(q, k)).cuda()
         for k in synth.FIELDS}
    torch.cuda.synchronize()
    ctx.rcb_kick_device(t, q.n, kp)
    for k in EXACT:
        got = t[k].cpu().numpy()
        if k == "mask":
            got = got.view(np.uint16)
        assert np.array_equal(got.view(np.uint8), getattr(p, k).view(np.uint8)), k
    gv = np.stack([t["vx"].cpu().numpy(), t["vy"].cpu().numpy(), t["vz"].cpu().numpy()], 1)
    assert np.array_equal(gv, np.stack([p.vx, p.vy, p.vz], 1))


def test_batch_of_boxes_equals_separate_kicks(ctx):
    """hsr_rcb_kick_batch: boxes of different sizes and kick coefficients in
    one persistent launch give each box's separate kick."""
    boxes = [synth.zeldovich_box(ng, z=z, seed=s) for ng, z, s in ((16, 50.0, 1), (24, 10.0, 2),
                                                                    (20, 30.0, 3))]
    kps = [synth.kick_params(b, nd=nd, fcoeff=f) for b, nd, f in zip(boxes, (32, 64, 128),
                                                                      (0.5, 1.0, 2.0))]
    sep = [b.copy() for b in boxes]
    for b, kp in zip(sep, kps):
        ctx.rcb_kick(b, kp)
    st = ctx.rcb_kick_batch(boxes, kps)
    assert st["kernel_launches"] == 1
    for b, q in zip(boxes, sep):
        for k in EXACT:
            assert np.array_equal(getattr(b, k).view(np.uint8), getattr(q, k).view(np.uint8)), k
        # same kernel, same per-particle summation order as the separate kick
        assert np.array_equal(vel(b), vel(q))
    assert ctx.bench_pairs(2, flush_l2=False) > 0
    assert ctx.bench_pairs_graph(2, flush_l2=False) > 0


def test_batch_of_monopole_and_12_point_boxes_equals_separate_kicks(ctx):
    """Boxes of 12-point and monopole pseudo-particles in one batch (their
    trees built concurrently on their own streams) give each box's separate
    kick bit for bit."""
    boxes = [synth.zeldovich_box(ng, z=10.0, seed=s) for ng, s in ((16, 4), (20, 7), (16, 8),
                                                                   (12, 9))]
    kps = [synth.kick_params(b, nd=32, tdpts=t, open_angle=1.0, fcoeff=1.0)
           for b, t in zip(boxes, (12, 1, 12, 1))]
    sep = [b.copy() for b in boxes]
    for b, kp in zip(sep, kps):
        ctx.rcb_kick(b, kp)
    ctx.rcb_kick_batch(boxes, kps)
    for b, q in zip(boxes, sep):
        for k in EXACT:
            assert np.array_equal(getattr(b, k).view(np.uint8), getattr(q, k).view(np.uint8)), k
        assert np.array_equal(vel(b), vel(q))


def test_graph_replay_of_single_kick(ctx):
    p = synth.zeldovich_box(24, seed=5)
    ctx.rcb_kick(p, synth.kick_params(p, nd=64))
    assert ctx.bench_pairs_graph(3, flush_l2=True) > 0


def test_pairs_in_cutoff_count(ctx):
    """hsr_pairs_in_cutoff against a count over the exported lists (float32
    r2 as the reference rounds it)."""
    p = synth.zeldovich_box(16, z=10.0, seed=31)
    kp = synth.kick_params(p, nd=32)
    q = p.copy()
    st = ctx.rcb_kick(q, kp)
    got = ctx.pairs_in_cutoff()
    off, cnt, ptr, e = ctx.lists()
    fs2 = np.float32(kp.fsrrmax) * np.float32(kp.fsrrmax)
    r2max = np.float32(3.116326355) * np.float32(3.116326355)
    rc2 = min(fs2, np.nextafter(r2max, np.float32(np.inf)))
    want = 0
    for l in range(len(off)):
        xi = np.stack([q.x, q.y, q.z], 1)[off[l]:off[l] + cnt[l]].astype(np.float32)
        ej = e[:3, ptr[l]:ptr[l + 1]].T.astype(np.float32)
        d = ej[None, :, :] - xi[:, None, :]
        r2 = (d[..., 0] * d[..., 0] + d[..., 1] * d[..., 1]) + d[..., 2] * d[..., 2]
        want += int((r2 < rc2).sum())
    assert got == want, (got, want)
    assert 0 < got < st["pairs"]

