"""HACC's TreePM time-step loop on one GPU through hsr_treepm_step.

The loop of src/simulation/driver_hires.cxx:320-447 on one rank, with the
whole periodic box on the device:

    for step in steps:
        if doHalfKick: PM kick, stepFraction 0.5        (map2_poisson_*)
        ts.advanceHalfStep()
        Particles::subCycle(ts)                         (nsub short-range kicks)
        ts.advanceHalfStep()
        PM kick, stepFraction 0.5 on the last step, else 1
        doHalfKick = last step

Each PM kick takes TimeStepper::fscal() and tau() * stepFraction of the
stepper at its point in the step (TimeStepper.cxx:45-67); the sub-cycles take
map1's and map2's arguments of the mid-step stepper (Particles.cxx:1176-1233).
Halo finding, analysis and output steps (the "extras") are not part of this
path: the loop never takes their extra half kicks.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
from typing import List

import numpy as np

import hsr
import synth


class HsrTreePMParams(C.Structure):
    """hsr_treepm_params (include/hacc_pm.h)."""
    _fields_ = [("sub", hsr.HsrSubcycleParams), ("pm_open", hsr.HsrPmParams),
                ("pm_close", hsr.HsrPmParams)]


def _lib():
    lib = hsr.load()
    if not getattr(lib, "_treepm_bound", False):
        lib.hsr_treepm_step.argtypes = ([C.c_void_p, C.POINTER(HsrTreePMParams), C.c_int64]
                                        + [C.POINTER(C.c_float)] * 8
                                        + [C.POINTER(C.c_int64), C.POINTER(C.c_uint16), C.c_int32,
                                           C.POINTER(C.c_int64)])
        lib.hsr_treepm_step.restype = C.c_int32
        lib._treepm_bound = True
    return lib


@dataclasses.dataclass
class StepPlan:
    """The three stepper points of one step and the parameters taken there."""
    start: synth.Stepper
    mid: synth.Stepper
    end: synth.Stepper
    open_fraction: float    # 0: no opening half kick
    close_fraction: float


def plan(z_in: float, z_fin: float, nsteps: int) -> List[StepPlan]:
    """The stepper points of driver_hires.cxx's loop (:320-447): each step
    advances half a step before the sub-cycles and half a step after them
    (pp += tau2 each time)."""
    ts = synth.stepper(z_in=z_in, z_fin=z_fin, nsteps=nsteps)
    out = []
    half_kick = True
    for s in range(nsteps):
        mid = ts.advanced(1)
        end = mid.advanced(1)
        last = s == nsteps - 1
        out.append(StepPlan(start=ts, mid=mid, end=end,
                            open_fraction=0.5 if half_kick else 0.0,
                            close_fraction=0.5 if last else 1.0))
        half_kick = last
        ts = end
    return out


def pm_params(ts: synth.Stepper, fraction: float, ng: int, ngo: int, gpscal: float = 1.0,
              precision: int = hsr.PM_F64) -> hsr.HsrPmParams:
    """map2_poisson_backward_gradient's arguments (mc3.cxx:336-374):
    inverse_cic(ts.tau() * stepFraction, ts.fscal(), d), the product taken
    in double and both passed as floats."""
    tau = float(np.float32(ts.tau * fraction))
    return hsr.pm_params(ng, ngo, gpscal, float(np.float32(ts.fscal)), tau, precision)


def step_params(sp: StepPlan, kp: synth.KickParams, nsub: int, ng: int, ngo: int, nglt,
                gpscal: float = 1.0, precision: int = hsr.PM_F64) -> HsrTreePMParams:
    T = HsrTreePMParams()
    S = T.sub
    S.kick = hsr.make_params(dataclasses.replace(
        kp, fcoeff=float(synth.kick_coefficient(sp.mid, nsub, gpscal))), hsr.KERNEL_AUTO,
        hsr.BUILD_DEVICE)
    S.nsub = nsub
    S.ng[:] = [int(v) for v in nglt]
    S.alpha, S.pp, S.adot = sp.mid.alpha, sp.mid.pp, sp.mid.adot
    S.tau = float(synth.stream_tau(sp.mid, nsub))
    S.skip_stream = S.skip_kick = 0
    if sp.open_fraction:
        T.pm_open = pm_params(sp.start, sp.open_fraction, ng, ngo, gpscal, precision)
    else:
        T.pm_open = hsr.pm_params(ng, ngo, gpscal, 0.0, 0.0, precision)
    T.pm_close = pm_params(sp.end, sp.close_fraction, ng, ngo, gpscal, precision)
    return T


def step(ctx: hsr.Context, p: synth.Particles, T: HsrTreePMParams) -> dict:
    """hsr_treepm_step on the host arrays of `p` (modified in place): returns
    {"sr": hsr_stats, "pm": hsr_pm_stats, "n_inbox": ...}."""
    lib = _lib()
    nin = C.c_int64()
    args = [a.ctypes.data_as(C.POINTER(C.c_float)) for a in (p.x, p.y, p.z, p.vx, p.vy, p.vz,
                                                             p.mass, p.phi)]
    st = lib.hsr_treepm_step(ctx.h, C.byref(T), p.n, *args,
                             p.id.ctypes.data_as(C.POINTER(C.c_int64)),
                             p.mask.ctypes.data_as(C.POINTER(C.c_uint16)), hsr.MEM_HOST,
                             C.byref(nin))
    ctx._check(st, "hsr_treepm_step")
    return {"sr": ctx.stats(), "pm": ctx.pm_stats(), "n_inbox": nin.value}


def step_device(ctx: hsr.Context, t: dict, n: int, T: HsrTreePMParams) -> dict:
    """hsr_treepm_step on device arrays: `t` maps the ten field names to CUDA
    tensors (float32 x..phi, int64 id, int16/uint16 mask), modified in place."""
    lib = _lib()
    nin = C.c_int64()
    fp = lambda k: C.cast(C.c_void_p(t[k].data_ptr()), C.POINTER(C.c_float))
    st = lib.hsr_treepm_step(ctx.h, C.byref(T), n,
                             *[fp(k) for k in ("x", "y", "z", "vx", "vy", "vz", "mass", "phi")],
                             C.cast(C.c_void_p(t["id"].data_ptr()), C.POINTER(C.c_int64)),
                             C.cast(C.c_void_p(t["mask"].data_ptr()), C.POINTER(C.c_uint16)),
                             hsr.MEM_DEVICE, C.byref(nin))
    ctx._check(st, "hsr_treepm_step(device arrays)")
    return {"sr": ctx.stats(), "pm": ctx.pm_stats(), "n_inbox": nin.value}


def run(ctx: hsr.Context, p: synth.Particles, z_in: float, z_fin: float, nsteps: int, nsub: int,
        kp: synth.KickParams, precision: int = hsr.PM_F64) -> List[dict]:
    """The whole loop on `p` (in place); per-step statistics."""
    ng, ngo = p.meta["ng"], p.meta["ngo"]
    return [step(ctx, p, step_params(sp, kp, nsub, ng, ngo, p.nglt, precision=precision))
            for sp in plan(z_in, z_fin, nsteps)]
