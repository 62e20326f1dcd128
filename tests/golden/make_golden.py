"""Writes the golden fixtures of the RCB and RCO short-range kicks.

Each fixture holds a seeded input particle set, the constructor arguments, and
the ten arrays after the reference's own RCBForceTree constructor ran on it
(oracle/_ref/rcb_ref: the reference sources compiled unmodified, single
thread) -- or, for the *_rco fixtures, its RCOForceTree constructor
(oracle/_ref/rco_ref: RCOForceTree.cxx with its octant array sized 8, the one
change it needs to run; see oracle/Makefile).  Run from the repository root in
a checkout that has the reference tree and `make -C oracle ref` built:

    python tests/golden/make_golden.py

The fixtures are small (a few thousand particles) so the CPU tests stay fast.
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(ROOT, "hacc-coral_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle  # noqa: E402
import synth  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def blob_box(n: int, side: float, seed: int) -> synth.Particles:
    """Half uniform, half in a dense Plummer-like clump (uneven leaves)."""
    rng = np.random.default_rng(seed)
    nu = n // 2
    u = rng.random((nu, 3)) * side
    r = 0.8 * rng.random(n - nu) ** (1 / 3) / np.sqrt(1 + rng.random(n - nu))
    v = rng.standard_normal((n - nu, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    c = u[: n - nu] * 0 + side / 2
    pos = np.concatenate([u, c + r[:, None] * v]).astype(np.float32)
    p = synth.random_box(n, side, seed + 1)
    p.x[:], p.y[:], p.z[:] = pos[:, 0], pos[:, 1], pos[:, 2]
    p.vx[:] = 0
    p.vy[:] = 0
    p.vz[:] = 0
    return p


def cases():
    out = []
    # A: uniform random, zero initial velocities (v_out is the kick itself), monopole
    p = synth.random_box(2000, 12.0, 11)
    p.vx[:] = 0
    p.vy[:] = 0
    p.vz[:] = 0
    kp = synth.kick_params(p, nd=16, fcoeff=1.0)
    out.append(("random2000_nd16_mono", p, kp))
    # B: Zel'dovich 8^3 lattice with overload ghosts at z=50, realistic velocities and
    # kick coefficient, quadrupole pseudo-particles
    p = synth.zeldovich_box(8, z=10.0, seed=5009888)
    kp = synth.kick_params(p, nd=32, tdpts=12)
    out.append(("zeldovich8_nd32_quad", p, kp))
    # C: clumped set, wide opening angle (many pseudo-particle entries), small leaves
    p = blob_box(3000, 10.0, 23)
    kp = synth.kick_params(p, nd=8, open_angle=0.5, fcoeff=1.0)
    kp.min_force, kp.max_force = (0.5, 0.5, 0.5), (9.5, 9.5, 9.5)
    out.append(("blob3000_nd8_oa05_mono", p, kp))
    # D: a single leaf (root is the only node): the reference lists the root's
    # particles twice for it
    p = synth.random_box(40, 6.0, 5)
    p.vx[:] = 0
    p.vy[:] = 0
    p.vz[:] = 0
    kp = synth.kick_params(p, nd=64, fcoeff=1.0)
    kp.min_force, kp.max_force = (-1.0, -1.0, -1.0), (7.0, 7.0, 7.0)
    out.append(("single_leaf40", p, kp))
    # E-G: the RCO octree (RCOForceTree): uniform random, Zel'dovich with
    # quadrupole pseudo-particles, and the clumped set with a wide opening angle
    for name, p, kp in list(out[:3]):
        kp2 = synth.KickParams(**{**kp.__dict__, "tree": 1})
        out.append((name + "_rco", p, kp2))
    return out


def main():
    oracle.build(ref=True)
    for name, p, kp in cases():
        res, times, _ = oracle.run_reference(p, kp, nthreads=1)
        arrays = {f"in_{k}": getattr(p, k) for k in synth.FIELDS}
        arrays.update({f"out_{k}": res[k] for k in synth.FIELDS})
        params = np.array([*kp.min, *kp.max, *kp.min_force, *kp.max_force, kp.avg_mass, kp.fsrrmax,
                           kp.rsm, kp.open_angle, kp.nd, kp.ds, kp.tmin, kp.fcoeff, kp.ppc,
                           kp.tdpts, kp.law, kp.tree], dtype=np.float64)
        path = os.path.join(OUT, f"{name}.npz")
        np.savez_compressed(path, params=params, nglt=np.array(p.nglt), **arrays)
        print(f"{name}: n={p.n} -> {path} ({os.path.getsize(path)} bytes, {times[0]:.3f} s)")


if __name__ == "__main__":
    main()
