"""Seeded synthetic particle sets for the short-range force path.

The reference benchmarks full cosmological runs whose inputs cannot be
regenerated here; these generators stand in for them with the same shapes,
sizes and statistics:

* ``zeldovich_box`` -- a lattice of np^3 particles on an ng^3 grid displaced
  with the Zel'dovich (1LPT) field of a seeded Gaussian random field with a
  power-law spectrum P(k) ~ k^n (n = -2), then wrapped into the rank-local
  frame with periodic overload ghosts exactly as HACC sizes the local domain
  (src/simulation/Domain.cxx:53-69: ngo = ceil(oL*ng/L), nglt = ng + 2*ngo + 1)
  and counting-sorted by grid cell as Particles::resortParticles leaves them
  before a kick (src/cpu/Particles.cxx:402-488).
* ``clustered_box`` -- 60 % uniform random particles and 40 % in NFW halos
  with a power-law mass function, for uneven leaf occupancy.

Positions are in local grid units; masses are 1, as Particles::map2 sets them
(src/cpu/Particles.cxx:1256-1257).  ``kick_params`` gives the RCBForceTree
arguments Particles::map2 passes (src/cpu/Particles.cxx:1205-1336), with the
kick coefficient from the TimeStepper scalars (src/simulation/TimeStepper.cxx).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

# FGrid::m_rmax (src/halo_finder/ForceLaw.cxx:32): the short-range cutoff.
RMAX = np.float32(3.116326355)
# indat values used by every reference example (indat:24-25, 36-41).
OMEGA_DM = 0.23387755
DEUT = 0.0226
HUBBLE = 0.7
OMEGA_B = DEUT / HUBBLE ** 2
OVERLOAD_MPC = 8.0
EDGE = 3.2

# rms displacement per axis at z = 50, grid units; linear growth D ~ a scales
# it to other redshifts.
SIGMA_Z50 = 0.15


@dataclass
class Particles:
    """SoA particle arrays in the layout RCBForceTree takes."""

    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    vx: np.ndarray
    vy: np.ndarray
    vz: np.ndarray
    mass: np.ndarray
    phi: np.ndarray
    id: np.ndarray
    mask: np.ndarray
    nglt: tuple = (0, 0, 0)
    meta: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return int(self.x.shape[0])

    def copy(self) -> "Particles":
        return Particles(*(getattr(self, k).copy() for k in FIELDS), nglt=self.nglt,
                         meta=dict(self.meta))

    def arrays(self):
        return [getattr(self, k) for k in FIELDS]

    def take(self, idx) -> "Particles":
        return Particles(*(np.ascontiguousarray(getattr(self, k)[idx]) for k in FIELDS),
                         nglt=self.nglt, meta=dict(self.meta))


FIELDS = ("x", "y", "z", "vx", "vy", "vz", "mass", "phi", "id", "mask")


# ---------------------------------------------------------------------------
# TimeStepper scalars (src/simulation/TimeStepper.cxx:1-88): double members;
# the run's stepper is built from Basedata's float members
# (src/initializer/Basedata.h:133-140, driver_hires.cxx:269-270).
# ---------------------------------------------------------------------------

@dataclass
class Stepper:
    alpha: float
    pp: float
    omegatot: float
    tau: float

    def advanced(self, halves: int = 1) -> "Stepper":
        """The stepper after `halves` calls of advanceHalfStep: pp += tau2
        each time, accumulated in double as the reference does."""
        pp = self.pp
        for _ in range(halves):
            pp += self.tau2
        return Stepper(alpha=self.alpha, pp=pp, omegatot=self.omegatot, tau=self.tau)

    @property
    def aa(self) -> float:
        return self.pp ** (1.0 / self.alpha)

    @property
    def adot(self) -> float:
        pp1 = self.pp ** (3.0 / self.alpha)
        tmp = (self.omegatot + (1.0 - self.omegatot) * pp1) / self.pp ** (1.0 / self.alpha)
        return math.sqrt(tmp)

    @property
    def fscal(self) -> float:
        phiscal = 1.5 * self.omegatot / self.pp ** (1.0 / self.alpha)
        return phiscal / (self.alpha * self.adot * self.pp ** (1.0 - 1.0 / self.alpha))

    @property
    def tau2(self) -> float:
        return 0.5 * self.tau


def stepper(z_in: float = 50.0, z_fin: float = 20.0, nsteps: int = 3, alpha: float = 1.0,
            omegadm: float = OMEGA_DM, deut: float = DEUT, hubble: float = HUBBLE) -> Stepper:
    """TimeStepper at the start of the run, as driver_hires.cxx:269-270 builds
    it from Basedata: the indat values are floats, ain = 1.0 / (1 + zin) and
    omegatot = omegadm + deut / hubble / hubble are rounded to float
    (Basedata.h:133-137); the stepper itself computes in double
    (TimeStepper.cxx:3-38)."""
    f = np.float32
    ain = float(f(1.0 / float(f(1.0) + f(z_in))))
    afin = float(f(1.0 / float(f(1.0) + f(z_fin))))
    omegatot = float(f(f(omegadm) + f(f(deut) / f(hubble)) / f(hubble)))
    a = float(f(alpha))
    pin, pfin = ain ** a, afin ** a
    return Stepper(alpha=a, pp=pin, omegatot=omegatot, tau=(pfin - pin) / (1.0 * nsteps))


def kick_coefficient(ts: Stepper, nsub: int, gpscal: float = 1.0) -> np.float32:
    """map2's c = divscal / 4.0 / pi * fscal * tau * stepFraction
    (Particles.cxx:1229-1233): divscal = gpscal^3 and pi = 4.0 * atanf(1.0)
    are floats, the product runs in double from `/ 4.0` on (stepFraction =
    1.0 / nsub from subCycle, :1179), and c is stored as a float."""
    f = np.float32
    g = f(gpscal)
    divscal = g * g * g
    pi = f(4.0 * float(f(math.atan(1.0))))
    c = float(divscal) / 4.0 / float(pi) * ts.fscal * ts.tau * (1.0 / nsub)
    return f(c)


def stream_tau(ts: Stepper, nsub: int) -> np.float32:
    """map1's tau argument in subCycle: stepFraction * tau2 in double, passed
    as a float (Particles.cxx:1179-1185)."""
    return np.float32((1.0 / nsub) * ts.tau2)


# ---------------------------------------------------------------------------
# Particle sets
# ---------------------------------------------------------------------------

def _overload(ng: int, box_mpc: float) -> int:
    return int(math.ceil(OVERLOAD_MPC * ng / box_mpc))


def _displacement(ng: int, n_index: float, sigma: float, rng) -> np.ndarray:
    """Zel'dovich displacement on the ng^3 lattice: psi(k) = i k / k^2 delta(k)
    with <|delta_k|^2> ~ k^n, normalised to rms `sigma` per axis."""
    noise = rng.standard_normal((ng, ng, ng))
    dk = np.fft.rfftn(noise)
    kx = np.fft.fftfreq(ng) * 2 * np.pi
    kz = np.fft.rfftfreq(ng) * 2 * np.pi
    KX, KY, KZ = np.meshgrid(kx, kx, kz, indexing="ij")
    k2 = KX ** 2 + KY ** 2 + KZ ** 2
    k2[0, 0, 0] = 1.0
    amp = np.sqrt(k2 ** (n_index / 2.0))
    amp[0, 0, 0] = 0.0
    dk = dk * amp
    psi = np.empty((3, ng, ng, ng))
    for a, K in enumerate((KX, KY, KZ)):
        psi[a] = np.fft.irfftn(1j * K / k2 * dk, s=(ng, ng, ng), axes=(0, 1, 2))
    psi *= sigma / max(psi.std(), 1e-30)
    return psi


def _add_ghosts(pos: np.ndarray, vel: np.ndarray, ids: np.ndarray, ng: int, ngo: int):
    """Periodic overload copies into the rank-local frame [0, ng + 2 ngo + 1)."""
    nglt = ng + 2 * ngo + 1
    local = pos + ngo
    mask = np.zeros(len(ids), dtype=np.uint16)
    for d in range(3):
        up = local[:, d] + ng < nglt
        dn = local[:, d] - ng >= 0
        sel_up = np.nonzero(up)[0]
        sel_dn = np.nonzero(dn)[0]
        add_pos = [local[sel_up].copy(), local[sel_dn].copy()]
        add_pos[0][:, d] += ng
        add_pos[1][:, d] -= ng
        local = np.concatenate([local] + add_pos)
        vel = np.concatenate([vel, vel[sel_up], vel[sel_dn]])
        ids = np.concatenate([ids, ids[sel_up], ids[sel_dn]])
        mask = np.concatenate([mask, np.ones(len(sel_up) + len(sel_dn), np.uint16)])
    return local, vel, ids, mask, nglt


def resort(p: Particles) -> int:
    """Stable counting sort by unit grid cell with out-of-box particles last,
    in place (Particles::resortParticles, src/cpu/Particles.cxx:402-488).
    Returns the in-box count."""
    ng = p.nglt
    ix = np.floor(p.x).astype(np.int64)
    iy = np.floor(p.y).astype(np.int64)
    iz = np.floor(p.z).astype(np.int64)
    inb = (ix >= 0) & (ix < ng[0]) & (iy >= 0) & (iy < ng[1]) & (iz >= 0) & (iz < ng[2])
    key = np.where(inb, (ix * ng[1] + iy) * ng[2] + iz, ng[0] * ng[1] * ng[2])
    order = np.argsort(key, kind="stable")
    for k in FIELDS:
        a = getattr(p, k)
        a[:] = a[order]
    return int(inb.sum())


def zeldovich_box(ng: int, z: float = 50.0, seed: int = 5009888, n_index: float = -2.0,
                  box_mpc: float | None = None, sigma50: float = SIGMA_Z50) -> Particles:
    """np = ng particles per side, Zel'dovich-displaced at redshift z."""
    if box_mpc is None:
        box_mpc = 2.0 * ng  # 2 Mpc/h per grid cell, as 32^3 in a 64 Mpc/h box
    rng = np.random.default_rng(seed)
    sigma = sigma50 * (1.0 + 50.0) / (1.0 + z)
    psi = _displacement(ng, n_index, sigma, rng)
    q = np.stack(np.meshgrid(np.arange(ng), np.arange(ng), np.arange(ng), indexing="ij"))
    pos = (q + 0.5 + psi).reshape(3, -1).T % ng
    a = 1.0 / (1.0 + z)
    ts = Stepper(alpha=1.0, pp=a, omegatot=OMEGA_DM + OMEGA_B, tau=0.0)
    vel = psi.reshape(3, -1).T * (a * ts.adot)
    ids = np.arange(ng ** 3, dtype=np.int64)
    ngo = _overload(ng, box_mpc)
    local, vel, ids, mask, nglt = _add_ghosts(pos, vel, ids, ng, ngo)
    n = len(ids)
    p = Particles(
        x=local[:, 0].astype(np.float32), y=local[:, 1].astype(np.float32),
        z=local[:, 2].astype(np.float32), vx=vel[:, 0].astype(np.float32),
        vy=vel[:, 1].astype(np.float32), vz=vel[:, 2].astype(np.float32),
        mass=np.ones(n, np.float32), phi=np.zeros(n, np.float32), id=ids, mask=mask,
        nglt=(nglt, nglt, nglt),
        meta=dict(kind="zeldovich", ng=ng, z=z, seed=seed, n_index=n_index, box_mpc=box_mpc,
                  ngo=ngo, sigma=sigma))
    p.meta["n_inbox"] = resort(p)
    return p


def _nfw_radii(rng, n: int, c: float, rvir: float) -> np.ndarray:
    """Inverse-CDF samples of the NFW enclosed mass truncated at rvir."""
    xs = np.linspace(0.0, c, 2049)
    mu = np.log1p(xs) - xs / (1.0 + xs)
    u = rng.random(n) * mu[-1]
    x = np.interp(u, mu, xs)
    return x * (rvir / c)


def clustered_box(ng: int, nhalo: int = 4000, frac_halo: float = 0.4, slope: float = -1.9,
                  seed: int = 5009888, box_mpc: float | None = None) -> Particles:
    """ng^3 particles: (1-frac_halo) uniform random, frac_halo in NFW halos
    (mass function dN/dM ~ M^slope, concentration U[4,10], virial radius in
    [0.5, 4] grid units growing as M^(1/3))."""
    if box_mpc is None:
        box_mpc = 2.0 * ng
    rng = np.random.default_rng(seed)
    ntot = ng ** 3
    nh = int(frac_halo * ntot)
    nu = ntot - nh
    upos = rng.random((nu, 3)) * ng
    # masses from a truncated power law over two decades
    a1 = slope + 1.0
    u = rng.random(nhalo)
    mlo, mhi = 1.0, 100.0
    m = (mlo ** a1 + u * (mhi ** a1 - mlo ** a1)) ** (1.0 / a1)
    counts = np.floor(m / m.sum() * nh).astype(np.int64)
    counts[: nh - counts.sum()] += 1
    rvir = 0.5 + 3.5 * ((m / mhi) ** (1.0 / 3.0) - (mlo / mhi) ** (1.0 / 3.0)) / (
        1.0 - (mlo / mhi) ** (1.0 / 3.0))
    conc = rng.uniform(4.0, 10.0, nhalo)
    centres = rng.random((nhalo, 3)) * ng
    hpos = []
    for h in range(nhalo):
        k = int(counts[h])
        if k == 0:
            continue
        r = _nfw_radii(rng, k, conc[h], rvir[h])
        v = rng.standard_normal((k, 3))
        v /= np.linalg.norm(v, axis=1, keepdims=True)
        hpos.append(centres[h] + r[:, None] * v)
    pos = np.concatenate([upos] + hpos) % ng
    vel = np.zeros_like(pos)
    ids = np.arange(len(pos), dtype=np.int64)
    ngo = _overload(ng, box_mpc)
    local, vel, ids, mask, nglt = _add_ghosts(pos, vel, ids, ng, ngo)
    n = len(ids)
    p = Particles(
        x=local[:, 0].astype(np.float32), y=local[:, 1].astype(np.float32),
        z=local[:, 2].astype(np.float32), vx=vel[:, 0].astype(np.float32),
        vy=vel[:, 1].astype(np.float32), vz=vel[:, 2].astype(np.float32),
        mass=np.ones(n, np.float32), phi=np.zeros(n, np.float32), id=ids, mask=mask,
        nglt=(nglt, nglt, nglt),
        meta=dict(kind="clustered", ng=ng, seed=seed, nhalo=nhalo, ngo=ngo, box_mpc=box_mpc))
    p.meta["n_inbox"] = resort(p)
    return p


def random_box(n: int, side: float, seed: int) -> Particles:
    """Uniform random particles in [0, side)^3 with random velocities (small
    edge-case and property tests)."""
    rng = np.random.default_rng(seed)
    pos = rng.random((n, 3)).astype(np.float32) * np.float32(side)
    vel = rng.standard_normal((n, 3)).astype(np.float32)
    return Particles(
        x=pos[:, 0].copy(), y=pos[:, 1].copy(), z=pos[:, 2].copy(),
        vx=vel[:, 0].copy(), vy=vel[:, 1].copy(), vz=vel[:, 2].copy(),
        mass=np.ones(n, np.float32), phi=np.zeros(n, np.float32),
        id=np.arange(n, dtype=np.int64), mask=np.zeros(n, np.uint16),
        nglt=(int(math.ceil(side)),) * 3, meta=dict(kind="random", seed=seed))


def sorted_line(n: int, length: float = 40.0, width: float = 0.5, seed: int = 24) -> Particles:
    """n particles along a thin box [0, length) x [0, width)^2, sorted by x
    with the largest x moved to the front: the partitions split along x, and
    every level's last node has one swap chain through all of its left
    elements (an adversarial case for the tree build's partition)."""
    rng = np.random.default_rng(seed)
    x = np.roll(np.sort(rng.random(n).astype(np.float32) * np.float32(length)), 1)
    y = rng.random(n).astype(np.float32) * np.float32(width)
    z = rng.random(n).astype(np.float32) * np.float32(width)
    zero = np.zeros(n, np.float32)
    return Particles(x=x, y=y, z=z, vx=zero.copy(), vy=zero.copy(), vz=zero.copy(),
                     mass=np.ones(n, np.float32), phi=zero.copy(),
                     id=np.arange(n, dtype=np.int64), mask=np.zeros(n, np.uint16),
                     nglt=(int(math.ceil(length)), 1, 1), meta=dict(kind="sorted_line", seed=seed))


@dataclass
class KickParams:
    """RCBForceTree constructor arguments (src/halo_finder/RCBForceTree.h:96-124)."""

    min: tuple = (0.0, 0.0, 0.0)
    max: tuple = (0.0, 0.0, 0.0)
    min_force: tuple = (0.0, 0.0, 0.0)
    max_force: tuple = (0.0, 0.0, 0.0)
    avg_mass: float = 1.0
    fsrrmax: float = float(RMAX)
    rsm: float = 0.1
    open_angle: float = 0.1
    nd: int = 128
    ds: int = 2
    tmin: int = 128
    fcoeff: float = 1.0
    ppc: float = 0.9
    tdpts: int = 1
    law: int = 0
    tree: int = 0  # 0: RCBForceTree, 1: RCOForceTree


def kick_params(p: Particles, nd: int = 128, rsm: float = 0.1, open_angle: float = 0.1,
                fcoeff: float | None = None, tdpts: int = 1, edge: float = EDGE,
                nsub: int = 5) -> KickParams:
    """Arguments as Particles::map2 builds them (Particles.cxx:1205-1336): the
    tree box is [0, max(nglt)]^3 and the force box [edge, nglt - edge]."""
    g = max(p.nglt)
    if fcoeff is None:
        fcoeff = float(kick_coefficient(stepper(), nsub))
    return KickParams(min=(0.0, 0.0, 0.0), max=(float(g),) * 3,
                      min_force=(float(edge),) * 3,
                      max_force=tuple(float(np.float32(n) - np.float32(edge)) for n in p.nglt),
                      rsm=rsm, open_angle=open_angle, nd=nd, fcoeff=fcoeff, tdpts=tdpts)
