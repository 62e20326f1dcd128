"""Multi-step adjoint of HACC's short-range sub-cycles, with checkpoints.

The forward map is the sub-cycled short-range part of HACC's time step
(src/simulation/driver_hires.cxx:320-447 around Particles::subCycle,
src/cpu/Particles.cxx:1176-1201): for each PM step s, with the time stepper
advanced half a step (TimeStepper::advanceHalfStep, src/simulation/
TimeStepper.cxx:60-67), nsub times

    x += pt v              Particles::map1 with tau2 / nsub     (hsr_stream)
    v += c K(x)            the RCB short-range kick, c = map2's  (hsr_force_kick)
    x += pt v              map1 again                            (hsr_stream)

on a fixed set of particles kept at fixed indices (the kick does not permute
them; the tree is rebuilt at every kick).  With `pm` set, each PM step is the
whole TreePM step of src/simulation/driver_hires.cxx:320-447: the long-range
PM kick v += dv(x) (hsr_pm_kick) before the sub-cycles where the step opens
with a half kick, and after them.

The reverse pass gives the vector-Jacobian product of the whole map: for
cotangents (xbar_T, vbar_T) of the final state, (xbar_0, vbar_0) of the
initial one.  Per sub-cycle, in reverse:

    vbar += pt xbar                                   (hsr_stream on (vbar, xbar))
    xbar += (dK/dx)^T (c vbar) at the kick positions  (hsr_force_fwd + hsr_force_vjp)
    vbar += pt xbar

and for a PM kick, xbar += (d dv / dx)^T vbar at its positions (hsr_pm_vjp).

The trees and lists are held fixed within each kick (they are piecewise
constant in the positions).  The kick positions are not stored for the whole
run: the state is checkpointed every `checkpoint_every` PM steps and each
segment is recomputed from its checkpoint during the reverse pass.

Boxes are independent.  By default (`batched`) they advance in lockstep:
every sub-cycle's kicks of all boxes run as one call (hsr_force_kick_batch:
each box's tree and lists on the device, one persistent pair launch over
all boxes, replayed as a CUDA graph), and in the reverse pass every kick's
tapes of all boxes are rebuilt by one hsr_force_fwd_batch and differentiated
by one hsr_force_vjp_batch launch.  Otherwise boxes run one after another (or
`workers` at a time on separate contexts), one kick per call.

Buffers are CUDA tensors (torch is used for device memory only); every
arithmetic step on particle data runs in this library's kernels, apart from
the vector sum xbar += (kick VJP), done with torch's add on the device.  The
library works on its context's own stream and returns with it synchronized;
the torch copies and sums run on torch's current stream and are waited for
before the next library call reads their results.
"""
from __future__ import annotations

import dataclasses
from typing import Callable, List, Optional, Sequence, Tuple

import numpy as np

import hsr
import synth


@dataclasses.dataclass
class StepParams:
    """One PM step's sub-cycle parameters (time stepper at mid-step)."""
    alpha: float
    pp: float
    adot: float
    tau_sub: float   # map1's tau: stepFraction * tau2 = tau / (2 nsub)
    fcoeff: float    # map2's kick coefficient with stepFraction 1 / nsub


def schedule(z_in: float, z_fin: float, nsteps: int, nsub: int) -> List[StepParams]:
    """PM steps from z_in to z_fin (the reference's TimeStepper)."""
    ts = synth.stepper(z_in=z_in, z_fin=z_fin, nsteps=nsteps)
    out = []
    for s in range(nsteps):
        mid = ts.advanced(1)  # the sub-cycles run at mid-step (pp += tau2)
        out.append(StepParams(alpha=mid.alpha, pp=mid.pp, adot=mid.adot,
                              tau_sub=float(synth.stream_tau(mid, nsub)),
                              fcoeff=float(synth.kick_coefficient(mid, nsub))))
        ts = mid.advanced(1)
    return out


@dataclasses.dataclass
class BoxState:
    """Device state of one box: positions, velocities (3 float32 CUDA tensors
    each) and masses."""
    x: list
    v: list
    mass: object

    def clone(self) -> "BoxState":
        return BoxState([t.clone() for t in self.x], [t.clone() for t in self.v], self.mass)


def _torch_done():
    import torch
    torch.cuda.current_stream().synchronize()


def box_state(p: synth.Particles, device: int = 0) -> BoxState:
    import torch
    dev = torch.device("cuda", device)
    f = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.float32)).to(dev)
    return BoxState([f(p.x), f(p.y), f(p.z)], [f(p.vx), f(p.vy), f(p.vz)], f(p.mass))


TapeHook = Callable[[int, int, int, hsr.Context, list], None]

# Per PM step: the opening PM kick's parameters (None: no opening kick) and
# the closing one's (None: none), hsr.HsrPmParams each.
PMKicks = Sequence[Tuple[Optional[object], Optional[object]]]


def pm_schedule(z_in: float, z_fin: float, nsteps: int, ng: int, ngo: int,
                gpscal: float = 1.0, precision: int = hsr.PM_F64) -> List[tuple]:
    """The PM kicks of driver_hires' loop for `schedule`'s steps: a half kick
    opening the first step, a kick closing every step (half on the last)."""
    import treepm
    out = []
    for sp in treepm.plan(z_in, z_fin, nsteps):
        open_p = (treepm.pm_params(sp.start, sp.open_fraction, ng, ngo, gpscal, precision)
                  if sp.open_fraction else None)
        out.append((open_p, treepm.pm_params(sp.end, sp.close_fraction, ng, ngo, gpscal,
                                             precision)))
    return out


class MultiStep:
    """Forward map and its checkpointed adjoint for a list of boxes.

    kps: one synth.KickParams per box (fcoeff is replaced per PM step).
    on_tape(box, step, sub, ctx, x), if set, runs in the reverse pass right
    after each kick's tape is recorded at its positions x.  One box at a time,
    `ctx` then holds that kick's tree and lists (the FP64 references in the
    tests read them there); in lockstep `ctx` is None (the tape is the
    multi-box one) and a hook that needs a box's tree builds it on a context
    of its own from x (the tree and lists are a function of the positions).
    """

    def __init__(self, ctx: hsr.Context, kps: Sequence[synth.KickParams],
                 steps: Sequence[StepParams], nsub: int, checkpoint_every: Optional[int] = 2,
                 pm: Optional[PMKicks] = None, batched: bool = True):
        if checkpoint_every is not None and checkpoint_every < 1:
            raise ValueError("checkpoint_every must be >= 1 or None")
        if pm is not None and len(pm) != len(steps):
            raise ValueError("one (open, close) PM pair per step")
        self.ctx = ctx
        self.kps = list(kps)
        self.steps = list(steps)
        self.nsub = nsub
        self.every = checkpoint_every
        self.pm = list(pm) if pm is not None else None
        self.on_tape: Optional[TapeHook] = None
        # on_record(s0, records), if set, runs in the lockstep reverse pass
        # after each segment's recomputation: records[b] lists box b's kicks
        # of steps s0.. in forward order, ("sr", step, x) or ("pm", params, x)
        self.on_record: Optional[Callable[[int, list], None]] = None
        self.batched = batched
        self.kicks = 0
        self.pm_kicks = 0
        self.batch_calls = 0  # multi-box forward calls (one persistent launch each)

    # ---- one box ----------------------------------------------------------
    def _kp(self, b: int, st: StepParams) -> synth.KickParams:
        return dataclasses.replace(self.kps[b], fcoeff=st.fcoeff)

    def _stream(self, x, v, st: StepParams):
        self.ctx.stream_device(x[0], x[1], x[2], v[0], v[1], v[2], st.alpha, st.pp, st.tau_sub,
                               st.adot)

    def _subcycle(self, b: int, s: int, j: int, S: BoxState, record: Optional[list]):
        st = self.steps[s]
        self._stream(S.x, S.v, st)
        if record is not None:
            record.append(("sr", s, [t.clone() for t in S.x]))
            _torch_done()  # the copy is taken before the next half-stream moves x
        self.ctx.force_kick_device(S.x[0], S.x[1], S.x[2], S.mass, S.v[0], S.v[1], S.v[2],
                                   self._kp(b, st))
        self.kicks += 1
        self._stream(S.x, S.v, st)

    def _pm_kick(self, prm, S: BoxState, record: Optional[list]):
        if prm is None:
            return
        if record is not None:
            record.append(("pm", prm, [t.clone() for t in S.x]))
            _torch_done()
        self.ctx.pm_kick_device(S.x[0], S.x[1], S.x[2], S.v[0], S.v[1], S.v[2], prm)
        self.pm_kicks += 1

    def _run(self, b: int, S: BoxState, s0: int, s1: int, record: Optional[list] = None):
        for s in range(s0, s1):
            if self.pm:
                self._pm_kick(self.pm[s][0], S, record)
            for j in range(self.nsub):
                self._subcycle(b, s, j, S, record)
            if self.pm:
                self._pm_kick(self.pm[s][1], S, record)

    def forward_box(self, b: int, S: BoxState) -> BoxState:
        """The whole map on box b's state (in place); returns it."""
        _torch_done()
        self._run(b, S, 0, len(self.steps))
        return S

    def _reverse_segment(self, b: int, s0: int, s1: int, xk: list, mass, xb, vb, scratch):
        """Adjoint of steps s0..s1-1 from their recorded kick positions xk
        (("sr", step, x) per sub-cycle kick, ("pm", params, x) per PM kick,
        in forward order)."""
        sub = {s: self.nsub for s in range(s0, s1)}
        for kind, arg, x1 in reversed(xk):
            if kind == "pm":
                # v += dv(x): vbar passes through, xbar += (d dv / dx)^T vbar
                self.ctx.pm_vjp_device(x1[0], x1[1], x1[2], vb[0], vb[1], vb[2], *scratch, arg)
                for d in range(3):
                    xb[d].add_(scratch[d])
                _torch_done()
                continue
            s = arg
            st = self.steps[s]
            sub[s] -= 1
            j = sub[s]
            self._stream(vb, xb, st)                      # second half-stream
            self.ctx.force_fwd_device(x1[0], x1[1], x1[2], mass, *scratch, self._kp(b, st))
            self.kicks += 1
            if self.on_tape:
                self.on_tape(b, s, j, self.ctx, x1)
            self.ctx.force_vjp_device(vb[0], vb[1], vb[2], *scratch)
            for d in range(3):
                xb[d].add_(scratch[d])                     # kick
            _torch_done()
            self._stream(vb, xb, st)                      # first half-stream

    def adjoint_box(self, b: int, S0: BoxState, xbar, vbar):
        """(xbar_0, vbar_0) for the final-state cotangents (xbar, vbar) (lists
        of 3 CUDA tensors); S0, xbar and vbar are not modified.  With
        checkpoints the forward keeps the state every `checkpoint_every` PM
        steps and the reverse pass recomputes each segment's kick positions;
        without (None) the forward keeps every kick position."""
        import torch
        nst = len(self.steps)
        xb = [t.clone() for t in xbar]
        vb = [t.clone() for t in vbar]
        scratch = [torch.empty_like(S0.x[0]) for _ in range(3)]
        S = S0.clone()
        _torch_done()
        if self.every is None:
            xk: list = []
            self._run(b, S, 0, nst, record=xk)
            self._reverse_segment(b, 0, nst, xk, S0.mass, xb, vb, scratch)
            return xb, vb
        cps = []
        for s0 in range(0, nst, self.every):
            cps.append((s0, S.clone()))
            _torch_done()
            self._run(b, S, s0, min(nst, s0 + self.every))
        for s0, C in reversed(cps):
            s1 = min(nst, s0 + self.every)
            xk = []
            self._run(b, C, s0, s1, record=xk)
            self._reverse_segment(b, s0, s1, xk, S0.mass, xb, vb, scratch)
        return xb, vb

    # ---- all boxes in lockstep: one persistent launch per kick ----------
    def _kps_at(self, st: StepParams, nbox: int) -> List[synth.KickParams]:
        return [dataclasses.replace(self.kps[b], fcoeff=st.fcoeff) for b in range(nbox)]

    def _run_all(self, Ss: Sequence[BoxState], s0: int, s1: int,
                 record: Optional[List[list]] = None):
        """Steps s0..s1-1 of every box, in lockstep (states in place); with
        `record`, each box's kick positions are appended to record[b]."""
        nb = len(Ss)
        for s in range(s0, s1):
            st = self.steps[s]
            if self.pm:
                for b, S in enumerate(Ss):
                    self._pm_kick(self.pm[s][0], S, record[b] if record is not None else None)
            for _ in range(self.nsub):
                for S in Ss:
                    self._stream(S.x, S.v, st)
                if record is not None:
                    for b, S in enumerate(Ss):
                        record[b].append(("sr", s, [t.clone() for t in S.x]))
                    _torch_done()
                self.ctx.force_kick_batch_device([S.x for S in Ss], [S.mass for S in Ss],
                                                 [S.v for S in Ss], self._kps_at(st, nb))
                self.kicks += nb
                self.batch_calls += 1
                for S in Ss:
                    self._stream(S.x, S.v, st)
            if self.pm:
                for b, S in enumerate(Ss):
                    self._pm_kick(self.pm[s][1], S, record[b] if record is not None else None)

    def _reverse_all(self, s0: int, s1: int, xks: List[list], masses, xbs, vbs, scratch):
        """Adjoint of steps s0..s1-1 of every box from their recorded kick
        positions (xks[b] as _reverse_segment's list, the same sequence for
        every box), each kick's tapes rebuilt and differentiated for all boxes
        at once."""
        nb = len(xks)
        sub = {s: self.nsub for s in range(s0, s1)}
        for k in reversed(range(len(xks[0]))):
            kind, arg, _ = xks[0][k]
            if kind == "pm":
                for b in range(nb):
                    _, prm, x1 = xks[b][k]
                    self.ctx.pm_vjp_device(x1[0], x1[1], x1[2], vbs[b][0], vbs[b][1], vbs[b][2],
                                           *scratch[b], prm)
                    for d in range(3):
                        xbs[b][d].add_(scratch[b][d])
                _torch_done()
                continue
            s = arg
            st = self.steps[s]
            sub[s] -= 1
            j = sub[s]
            for b in range(nb):
                self._stream(vbs[b], xbs[b], st)             # second half-stream
            xs = [xks[b][k][2] for b in range(nb)]
            self.ctx.force_fwd_batch_device(xs, masses, scratch, self._kps_at(st, nb))
            self.kicks += nb
            self.batch_calls += 1
            if self.on_tape:
                for b in range(nb):
                    self.on_tape(b, s, j, None, xs[b])
            self.ctx.force_vjp_batch_device(vbs, scratch)
            for b in range(nb):
                for d in range(3):
                    xbs[b][d].add_(scratch[b][d])            # kick
            _torch_done()
            for b in range(nb):
                self._stream(vbs[b], xbs[b], st)             # first half-stream

    def forward_all(self, states: Sequence[BoxState]) -> List[BoxState]:
        """The whole map on every box's state (in place), in lockstep."""
        _torch_done()
        self._run_all(list(states), 0, len(self.steps))
        return list(states)

    def adjoint_all(self, states: Sequence[BoxState], xbars, vbars):
        """adjoint_box of every box, in lockstep: [(xbar_0, vbar_0)] per box."""
        import torch
        nst, nb = len(self.steps), len(states)
        xbs = [[t.clone() for t in xb] for xb in xbars]
        vbs = [[t.clone() for t in vb] for vb in vbars]
        scratch = [[torch.empty_like(S.x[0]) for _ in range(3)] for S in states]
        masses = [S.mass for S in states]
        Ss = [S.clone() for S in states]
        _torch_done()
        every = self.every if self.every is not None else nst
        cps = []
        for s0 in range(0, nst, every):
            cps.append((s0, [S.clone() for S in Ss]))
            _torch_done()
            if self.every is not None:
                self._run_all(Ss, s0, min(nst, s0 + every))
        for s0, C in reversed(cps):
            s1 = min(nst, s0 + every)
            xks = [[] for _ in range(nb)]
            self._run_all(C, s0, s1, record=xks)
            if self.on_record:
                self.on_record(s0, xks)
            self._reverse_all(s0, s1, xks, masses, xbs, vbs, scratch)
        return [(xbs[b], vbs[b]) for b in range(nb)]

    # ---- several boxes ---------------------------------------------------
    def _workers(self, n: int) -> List["MultiStep"]:
        """This driver and n - 1 peers, each on its own context (CUDA stream
        and buffers) of the same device."""
        peers = self.__dict__.setdefault("_peers", [])
        while len(peers) < n - 1:
            m = MultiStep(hsr.Context(self.ctx.device), self.kps, self.steps, self.nsub,
                          self.every, self.pm, batched=False)
            m.on_tape = self.on_tape
            peers.append(m)
        return [self] + peers[:max(0, n - 1)]

    def _map(self, fn, nbox: int, workers: int):
        ws = self._workers(workers)
        if len(ws) == 1:
            return [fn(self, b) for b in range(nbox)]
        # one box per host thread at a time: a box's host-side waits (the
        # tree build's per-level synchronisation) overlap another box's
        # kernels; the library releases the interpreter lock in its calls
        import threading
        from concurrent.futures import ThreadPoolExecutor
        lock = threading.Lock()
        free = list(ws)

        def job(b):
            with lock:
                w = free.pop()
            try:
                return fn(w, b)
            finally:
                with lock:
                    free.append(w)
        with ThreadPoolExecutor(len(ws)) as ex:
            return list(ex.map(job, range(nbox)))

    def total_kicks(self) -> Tuple[int, int]:
        """(short-range kicks, PM kicks) run by this driver and its peers."""
        ws = [self] + self.__dict__.get("_peers", [])
        return sum(w.kicks for w in ws), sum(w.pm_kicks for w in ws)

    def forward(self, states: Sequence[BoxState], workers: int = 1) -> List[BoxState]:
        """The map on every box: in lockstep when batched, else forward_box
        per box (workers > 1: that many boxes at once, each on its own
        context)."""
        if self.batched:
            return self.forward_all(states)
        _torch_done()
        return self._map(lambda w, b: w.forward_box(b, states[b]), len(states), workers)

    def adjoint(self, states: Sequence[BoxState], xbars, vbars, workers: int = 1):
        """The adjoint on every box: in lockstep when batched, else
        adjoint_box per box (workers as forward)."""
        if self.batched:
            return self.adjoint_all(states, xbars, vbars)
        _torch_done()
        return self._map(lambda w, b: w.adjoint_box(b, states[b], xbars[b], vbars[b]),
                         len(states), workers)


def kicks_per_box(nsteps: int, nsub: int, checkpointed: bool = True) -> int:
    """Kicks one box's adjoint runs: the forward, the recomputation of every
    segment (checkpointed only) and the tape of every kick in the reverse
    pass."""
    return (3 if checkpointed else 2) * nsteps * nsub


def position_loss_cotangent(states: Sequence[BoxState], targets):
    """Cotangents of L = sum_b sum_i |x_b,i - t_b,i|^2 at the final states:
    xbar = 2 (x - t), vbar = 0 (targets[b]: 3 CUDA tensors per box); and L
    itself (float64)."""
    import torch
    xbars, vbars, L = [], [], 0.0
    for S, T in zip(states, targets):
        d = [x.double() - t.double() for x, t in zip(S.x, T)]
        L += float(sum((u * u).sum() for u in d))
        xbars.append([(2.0 * u).float() for u in d])
        vbars.append([torch.zeros_like(v) for v in S.v])
    return xbars, vbars, L
