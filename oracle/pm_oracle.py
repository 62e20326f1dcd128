"""CPU restatement of HACC's long-range PM kick (numpy, float64).

TEST INFRASTRUCTURE ONLY.  Imported by tests/ and bench.py's CPU-baseline
leg; never by the product package.

It follows the reference step by step, in the reference's own layout: the
rank's local grid of ng + 2 ngo + 1 cells a side with its alive block at
[ngo, ngo + ng), and one rank holding the whole periodic box.

  cic                   Particles::cic           src/cpu/Particles.cxx:589-643
  copy_forward          fft_copy_arr_forward     src/simulation/mc3.cxx:206-225
  quiet_tables, green   SolverQuiet::initialize_greens_function
                                                 src/dfft/solver.hpp:726-820
  gradient_fields       forward_solve, kspace_solve_gradient, backward_solve_
                        gradient (complex FFT of the whole grid, unnormalised
                        both ways as FFTW), fft_copy_arr_backward
                                                 solver.hpp:91-160, 506-547;
                                                 mc3.cxx:228-245
  exchange              GridExchange::exchangeGrid on one rank: every dead
                        cell takes its periodic image in the alive block
                        (dead widths ngo below, ngo + 1 above)
                                                 src/halo_finder/GridExchange.cxx:
                                                 139-470; driver_hires.cxx:258
  inverse_cic           Particles::inverse_cic   Particles.cxx:647-714
  pm_kick               map2_poisson_forward + map2_poisson_backward_gradient
                                                 mc3.cxx:304-374

Parity status: the reference's PM solver needs FFTW and MPI, neither of which
is in this image, so it is not run here and the restatement is not pinned
bit for bit.  It is pinned physically instead: the reference's own fit of
the PM force of a unit point mass (f_grid in src/simulation/force.py:18-37,
the function its short-range force law complements) is reproduced by
`point_mass_force` to the accuracy the tests state.
"""
from __future__ import annotations

import math

import numpy as np


# ---------------------------------------------------------------------------
# the quiet solver's tables and Green's function
# ---------------------------------------------------------------------------

A0, A1, A2, A3 = -21.0 / 8.0, 128.0 / 45.0, -2.0 / 9.0, 1.0 / 360.0
B1, B2 = 4.0 / 3.0, -1.0 / 6.0
SIGMA, NS = 0.8, 3.0
PI = 3.14159265358979323846


def quiet_tables(ng: int):
    """(filter W(k), denominator term d(k), gradient factor g(k)), each ng
    entries by wave index (solver.hpp:726-790)."""
    kstep = 2.0 * PI / float(ng)
    kk = np.arange(ng)
    c1 = np.cos(kk * kstep)
    c2 = np.cos(2 * kk * kstep)
    c3 = np.cos(4 * kk * kstep)
    kp = np.zeros(ng)
    h = ng // 2
    kp[:h] = kk[:h] * kstep
    kp[h:2 * h] = (kk[:h] - h) * kstep
    filt = np.ones(ng)
    grad = np.ones(ng)
    k1 = kp[1:]
    filt[1:] = np.exp(-0.25 * SIGMA * SIGMA * k1 * k1) * (np.sin(0.5 * k1) / (0.5 * k1)) ** NS
    grad[1:] = B1 * np.sin(k1) + B2 * np.sin(2 * k1)
    denom = A0 + A1 * c1 + A2 * c2 + A3 * c3
    return filt, denom, grad


def green(ng: int) -> np.ndarray:
    """The full ng^3 Green's function (solver.hpp:800-819), index [kx, ky, kz]."""
    filt, denom, _ = quiet_tables(ng)
    coeff = 1.0 / float(ng) ** 3
    f = coeff * filt[:, None, None] * filt[None, :, None] * filt[None, None, :]
    d = denom[:, None, None] + denom[None, :, None] + denom[None, None, :]
    with np.errstate(divide="ignore", invalid="ignore"):
        g = f / d
    g[0, 0, 0] = 0.0
    return g


# ---------------------------------------------------------------------------
# CIC and its inverse on the local grid
# ---------------------------------------------------------------------------

def _corners(x, y, z):
    ix, iy, iz = (np.floor(a).astype(np.int64) for a in (x, y, z))
    # ab = 1 + (ix - x) in float, as the reference's POSVEL_T arithmetic
    ab = (np.float32(1.0) + (ix.astype(np.float32) - x)).astype(np.float64)
    de = (np.float32(1.0) + (iy.astype(np.float32) - y)).astype(np.float64)
    gh = (np.float32(1.0) + (iz.astype(np.float32) - z)).astype(np.float64)
    # the eight corners in the reference's order
    out = []
    for a, b, c in ((0, 0, 0), (0, 1, 0), (0, 1, 1), (0, 0, 1),
                    (1, 0, 1), (1, 1, 1), (1, 1, 0), (1, 0, 0)):
        w = (ab if a == 0 else 1.0 - ab) * (de if b == 0 else 1.0 - de) * (gh if c == 0 else 1.0 - gh)
        out.append((ix + a, iy + b, iz + c, w))
    return out


def cic(x, y, z, ng: int, ngo: int, gpscal: float = 1.0) -> np.ndarray:
    """Particles::cic onto the local grid (nglt^3, float64 sums); deposits
    outside [0, nglt) go to the safe slot and are dropped."""
    nglt = ng + 2 * ngo + 1
    x, y, z = (np.asarray(a, np.float32) for a in (x, y, z))
    c = float(np.float32(gpscal) * np.float32(gpscal) * np.float32(gpscal))
    rho = np.zeros(nglt ** 3 + 1)
    safe = nglt ** 3
    ok_any = np.isfinite(x) & np.isfinite(y) & np.isfinite(z)
    for cx, cy, cz, w in _corners(np.where(ok_any, x, -10), np.where(ok_any, y, -10),
                                  np.where(ok_any, z, -10)):
        inb = ((cx >= 0) & (cx < nglt) & (cy >= 0) & (cy < nglt) & (cz >= 0) & (cz < nglt))
        idx = np.where(inb, (cx * nglt + cy) * nglt + cz, safe)
        np.add.at(rho, idx, c * w)
    return rho[:safe].reshape(nglt, nglt, nglt)


def copy_forward(local: np.ndarray, ng: int, ngo: int) -> np.ndarray:
    """The alive block of a local grid (fft_copy_arr_forward), as GRID_T float."""
    return local[ngo:ngo + ng, ngo:ngo + ng, ngo:ngo + ng].astype(np.float32)


def exchange(alive: np.ndarray, ng: int, ngo: int) -> np.ndarray:
    """The local grid after GridExchange::exchangeGrid on one rank."""
    nglt = ng + 2 * ngo + 1
    src = (np.arange(nglt) - ngo) % ng
    return alive[np.ix_(src, src, src)]


def gradient_fields(rho_alive: np.ndarray) -> np.ndarray:
    """The three gradient components of the solved potential on the alive
    block, (3, ng, ng, ng) float32: forward FFT of the density, the
    quiet solver's I * (-g(k_a)) * green * rho_k, unnormalised inverse FFT,
    real part (fft_copy_arr_backward into GRID_T)."""
    ng = rho_alive.shape[0]
    rk = np.fft.fftn(rho_alive.astype(np.complex128))
    G = green(ng)
    _, _, g = quiet_tables(ng)
    out = np.empty((3, ng, ng, ng), np.float32)
    shp = [(ng, 1, 1), (1, ng, 1), (1, 1, ng)]
    for a in range(3):
        spec = 1j * (-g.reshape(shp[a])) * G * rk
        out[a] = (np.fft.ifftn(spec) * float(ng) ** 3).real.astype(np.float32)
    return out


def inverse_cic(x, y, z, local: np.ndarray) -> np.ndarray:
    """Sum over the eight corners of local-grid value * weight (cells outside
    the local grid read 0), per particle."""
    nglt = local.shape[0]
    x, y, z = (np.asarray(a, np.float32) for a in (x, y, z))
    flat = np.concatenate([local.reshape(-1).astype(np.float64), [0.0]])
    safe = nglt ** 3
    f = np.zeros(x.shape[0])
    ok = np.isfinite(x) & np.isfinite(y) & np.isfinite(z)
    for cx, cy, cz, w in _corners(np.where(ok, x, -10), np.where(ok, y, -10), np.where(ok, z, -10)):
        inb = ((cx >= 0) & (cx < nglt) & (cy >= 0) & (cy < nglt) & (cz >= 0) & (cz < nglt))
        idx = np.where(inb, (cx * nglt + cy) * nglt + cz, safe)
        f += flat[idx] * w
    return f


def fields(x, y, z, ng: int, ngo: int, gpscal: float = 1.0):
    """(density of the alive block (ng^3 float32), gradient fields (3, ng^3))."""
    rho = copy_forward(cic(x, y, z, ng, ngo, gpscal), ng, ngo)
    return rho, gradient_fields(rho)


def pm_kick(x, y, z, vx, vy, vz, ng: int, ngo: int, gpscal: float, fscal: float, tau: float):
    """map2_poisson_forward + map2_poisson_backward_gradient: returns the
    kicked velocities (float32 copies; inputs unchanged)."""
    _, grad = fields(x, y, z, ng, ngo, gpscal)
    out = []
    for a, v in enumerate((vx, vy, vz)):
        f = inverse_cic(x, y, z, exchange(grad[a], ng, ngo))
        out.append((np.asarray(v, np.float64) + f * float(fscal) * float(tau)).astype(np.float32))
    return out


# ---------------------------------------------------------------------------
# the reference's fit of the PM force of a point mass
# ---------------------------------------------------------------------------

def f_grid_fit(r):
    """The reference's fit of the PM force of a unit point mass in grid units
    (ShortRangeForce.f_grid, src/simulation/force.py:5-37, default
    parameters); 1 / r^2 - f_grid is the short-range force its polynomial
    force law approximates."""
    b, c, d, e, f, g, h, l = 0.72, 0.01, 0.27, 0.0001, 360.0, 100.0, 0.67, 17.0
    r = np.asarray(r, np.float64)
    return (np.tanh(b * r) / r ** 2 - b / r / np.cosh(b * r) ** 2
            + c * r * (1.0 + d * r ** 2) * np.exp(-d * r ** 2)
            + e * (f * r ** 2 + g * r ** 4 + l * r ** 6) * np.exp(-h * r ** 2))


def point_mass_force(ng: int, src, targets) -> np.ndarray:
    """Radial PM force on unit test masses at `targets` (k, 3) from a unit
    point mass at `src` (alive-block grid coordinates, ngo = 0), normalised as
    force.py's f_grid: the solved gradient interpolated at each target times
    4 pi (the Poisson equation here is div grad phi = rho, so a unit mass
    pulls with 1 / (4 pi r^2)), projected on the direction to the source
    (positive = attractive)."""
    src = np.asarray(src, np.float64)
    t = np.asarray(targets, np.float64)
    rho = copy_forward(cic([src[0]], [src[1]], [src[2]], ng, 0), ng, 0)
    grad = gradient_fields(rho)
    acc = np.stack([inverse_cic(t[:, 0], t[:, 1], t[:, 2], exchange(grad[a], ng, 0))
                    for a in range(3)], axis=1)
    dvec = src[None, :] - t
    dvec -= ng * np.round(dvec / ng)
    r = np.linalg.norm(dvec, axis=1)
    return 4.0 * math.pi * np.sum(acc * dvec, axis=1) / r


# ---------------------------------------------------------------------------
# float64 forward and its vector-Jacobian product (FP64 reference of hsr_pm_vjp)
# ---------------------------------------------------------------------------
#
# The kick is dv_i = fscal tau F(x_i) with F_d(x) = sum_c W(x - c) G_d[img(c)],
# G_d = A_d rho, A_d = Re IFFT(S_d FFT .), S_d = -i g(k_d) green (the solve
# above), rho[c] = gpscal^3 sum_j W(x_j - c) over the alive block.  For a
# cotangent vbar of dv:
#   xbar_i = fscal tau [ sum_c grad W(x_i - c) (vbar_i . G[img(c)])
#                       + gpscal^3 sum_{c alive} grad W(x_i - c) phibar[c] ],
#   phibar = sum_d A_d^T a_d,  A_d^T = Re IFFT(conj(S_d) FFT .),
#   a_d[img(c)] += W(x_i - c) vbar_{i,d}  (the transpose of the interpolation).
# W is the CIC weight, piecewise linear: the product is the derivative away
# from cell faces.

def _corners64(x, y, z, base=None):
    """(cx, cy, cz, w, dw/dx, dw/dy, dw/dz) of the eight corners, float64.
    base (n, 3), if given, fixes each particle's cell (the weights continue
    linearly past the cell faces: the map with its CIC cells frozen)."""
    x, y, z = (np.asarray(a, np.float64) for a in (x, y, z))
    if base is None:
        ix, iy, iz = (np.floor(a).astype(np.int64) for a in (x, y, z))
    else:
        ix, iy, iz = (np.floor(np.asarray(base, np.float64)[:, d]).astype(np.int64)
                      for d in range(3))
    fx, fy, fz = x - ix, y - iy, z - iz
    wx, wy, wz = (1.0 - fx, fx), (1.0 - fy, fy), (1.0 - fz, fz)
    sg = (-1.0, 1.0)
    out = []
    for a, b, c in ((0, 0, 0), (0, 1, 0), (0, 1, 1), (0, 0, 1),
                    (1, 0, 1), (1, 1, 1), (1, 1, 0), (1, 0, 0)):
        out.append((ix + a, iy + b, iz + c, wx[a] * wy[b] * wz[c],
                    sg[a] * wy[b] * wz[c], wx[a] * sg[b] * wz[c], wx[a] * wy[b] * sg[c]))
    return out


def _alive_index(cx, cy, cz, ng, ngo):
    u, v, w = cx - ngo, cy - ngo, cz - ngo
    ok = (u >= 0) & (u < ng) & (v >= 0) & (v < ng) & (w >= 0) & (w < ng)
    return ok, (np.where(ok, u, 0) * ng + np.where(ok, v, 0)) * ng + np.where(ok, w, 0)


def _image_index(cx, cy, cz, ng, ngo):
    nglt = ng + 2 * ngo + 1
    ok = ((cx >= 0) & (cx < nglt) & (cy >= 0) & (cy < nglt) & (cz >= 0) & (cz < nglt))
    u, v, w = ((c - ngo) % ng for c in (cx, cy, cz))
    return ok, (u * ng + v) * ng + w


def _solve_ops(ng):
    G = green(ng)
    _, _, g = quiet_tables(ng)
    shp = [(ng, 1, 1), (1, ng, 1), (1, 1, ng)]
    return [-1j * g.reshape(shp[a]) * G for a in range(3)]


def _deposit64(x, y, z, ng, ngo, c, base=None):
    rho = np.zeros(ng ** 3)
    for cx, cy, cz, w, *_ in _corners64(x, y, z, base):
        ok, k = _alive_index(cx, cy, cz, ng, ngo)
        np.add.at(rho, k[ok], c * w[ok])
    return rho.reshape(ng, ng, ng)


def force64(x, y, z, ng: int, ngo: int, gpscal: float = 1.0, base=None) -> np.ndarray:
    """F (n, 3) in float64: the interpolated gradient fields (dv / (fscal tau)).
    base: see _corners64."""
    S = _solve_ops(ng)
    rk = np.fft.fftn(_deposit64(x, y, z, ng, ngo, gpscal ** 3, base))
    Gd = [(np.fft.ifftn(S[a] * rk) * ng ** 3).real.ravel() for a in range(3)]
    F = np.zeros((len(np.atleast_1d(x)), 3))
    for cx, cy, cz, w, *_ in _corners64(x, y, z, base):
        ok, k = _image_index(cx, cy, cz, ng, ngo)
        for a in range(3):
            F[:, a] += np.where(ok, w * Gd[a][k], 0.0)
    return F


def vjp64(x, y, z, vbar, ng: int, ngo: int, gpscal: float = 1.0) -> np.ndarray:
    """(dF/dx)^T vbar per particle, (n, 3) float64 (multiply by fscal tau for
    the kick's)."""
    vbar = np.asarray(vbar, np.float64)
    c = gpscal ** 3
    S = _solve_ops(ng)
    rk = np.fft.fftn(_deposit64(x, y, z, ng, ngo, c))
    Gd = [(np.fft.ifftn(S[a] * rk) * ng ** 3).real.ravel() for a in range(3)]
    corners = _corners64(x, y, z)
    xbar = np.zeros((vbar.shape[0], 3))
    adj = [np.zeros(ng ** 3) for _ in range(3)]
    for cx, cy, cz, w, gx, gy, gz in corners:
        ok, k = _image_index(cx, cy, cz, ng, ngo)
        dot = sum(vbar[:, a] * np.where(ok, Gd[a][k], 0.0) for a in range(3))
        xbar += np.stack([gx, gy, gz], 1) * dot[:, None]
        for a in range(3):
            np.add.at(adj[a], k[ok], (w * vbar[:, a])[ok])
    spec = sum(np.conj(S[a]) * np.fft.fftn(adj[a].reshape(ng, ng, ng)) for a in range(3))
    phibar = (np.fft.ifftn(spec) * ng ** 3).real.ravel()
    for cx, cy, cz, w, gx, gy, gz in corners:
        ok, k = _alive_index(cx, cy, cz, ng, ngo)
        f = np.where(ok, phibar[k], 0.0) * c
        xbar += np.stack([gx, gy, gz], 1) * f[:, None]
    return xbar
