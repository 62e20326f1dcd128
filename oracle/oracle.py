"""Python access to the CPU oracle.

TEST INFRASTRUCTURE ONLY.  Imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg; never by the product package.

* ``Oracle``  -- ctypes binding of this project's C restatement
  (hsr_oracle.c, built by ``make`` into oracle/_build/).
* ``run_reference`` -- runs the reference's own force tree (oracle/_ref/rcb_ref,
  built by ``make ref`` from the reference sources) in a subprocess with the
  unlimited stack it needs.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import resource
import struct
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libhsr_oracle.so")
REF_EXE = os.path.join(HERE, "_ref", "rcb_ref")
# the reference's RCOForceTree, built from a copy with its octant array sized
# 8 (the file as shipped reads past that array; see oracle/Makefile)
REF_RCO_EXE = os.path.join(HERE, "_ref", "rco_ref")
# the reference's Particles::subCycle and TimeStepper (oracle/sub_driver.cpp)
REF_SUB_EXE = os.path.join(HERE, "_ref", "sub_ref")

LAW_POLY6 = 0
LAW_POLY5_STEP16 = 1
ERRORS = {1: "bad argument", 2: "interaction list reached VMAX", 3: "out of memory"}


# Where the reference tree is looked for when HSR_REFERENCE_ROOT is unset.
_REFERENCE_CHECKOUT = "/root/reference"


def reference_root() -> str:
    """Root of the reference tree (the directory holding src/halo_finder):
    $HSR_REFERENCE_ROOT, else the checkout beside this repository when it
    exists, else "" (machines that only receive this repository)."""
    root = os.environ.get("HSR_REFERENCE_ROOT", "")
    if not root and os.path.isfile(os.path.join(_REFERENCE_CHECKOUT, "src", "halo_finder",
                                                "RCBForceTree.cxx")):
        root = _REFERENCE_CHECKOUT
    return root


def build(ref: bool = False, ref_if_present: bool = False) -> None:
    """Compiles the restatement; with `ref` also the reference build (the
    reference tree must exist), with `ref_if_present` the reference build
    where the tree exists."""
    targets = ["all"] + (["ref"] if ref else ["ref-if-present"] if ref_if_present else [])
    subprocess.run(["make", "-s", "-C", HERE, f"REF={reference_root()}"] + targets, check=True)


class OraParams(C.Structure):
    _fields_ = [("min", C.c_float * 3), ("max", C.c_float * 3),
                ("min_force", C.c_float * 3), ("max_force", C.c_float * 3),
                ("avg_mass", C.c_float), ("fsrrmax", C.c_float), ("rsm", C.c_float),
                ("open_angle", C.c_float), ("nd", C.c_int64), ("ds", C.c_int64),
                ("tmin", C.c_int64), ("fcoeff", C.c_float), ("ppc", C.c_float),
                ("tdpts", C.c_int32), ("law", C.c_int32), ("vmax", C.c_int32),
                ("nthreads", C.c_int32), ("tree", C.c_int32)]


class OraStats(C.Structure):
    _fields_ = [("nodes", C.c_int64), ("leaves", C.c_int64), ("empty_leaves", C.c_int64),
                ("max_ppn", C.c_int64), ("processed_leaves", C.c_int64),
                ("list_entries", C.c_int64), ("pairs", C.c_int64), ("t_build", C.c_double),
                ("t_walk", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


def _ptr(a, ct):
    return a.ctypes.data_as(C.POINTER(ct))


def params_struct(kp, nthreads: int = 0, vmax: int = 0) -> OraParams:
    P = OraParams()
    for k in ("min", "max", "min_force", "max_force"):
        getattr(P, k)[:] = [float(v) for v in getattr(kp, k)]
    P.avg_mass, P.fsrrmax, P.rsm, P.open_angle = kp.avg_mass, kp.fsrrmax, kp.rsm, kp.open_angle
    P.nd, P.ds, P.tmin = kp.nd, kp.ds, kp.tmin
    P.fcoeff, P.ppc, P.tdpts, P.law = kp.fcoeff, kp.ppc, kp.tdpts, kp.law
    P.vmax, P.nthreads = vmax, nthreads
    P.tree = getattr(kp, "tree", 0)
    return P


class OracleResult:
    """Tree, lists and statistics of one restatement run."""

    def __init__(self, lib, handle, particles):
        self._lib, self._h, self._p = lib, handle, particles
        st = OraStats()
        lib.ora_result_stats(handle, C.byref(st))
        self.stats = st.as_dict()

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.ora_result_free(self._h)
            self._h = None

    def leaves(self):
        nl = self._lib.ora_result_nleaves(self._h)
        off = np.zeros(nl, np.int64)
        cnt = np.zeros(nl, np.int64)
        ptr = np.zeros(nl + 1, np.int64)
        self._lib.ora_result_leaves(self._h, _ptr(off, C.c_int64), _ptr(cnt, C.c_int64),
                                    _ptr(ptr, C.c_int64))
        return off, cnt, ptr

    def entries(self):
        ne = self._lib.ora_result_nentries(self._h)
        e = np.zeros((4, ne), np.float32)
        self._lib.ora_result_entries(self._h, *[_ptr(e[i], C.c_float) for i in range(4)])
        return e

    def nodes(self, tdpts: int):
        nn = self._lib.ora_result_nnodes(self._h)
        cnt, off, cl, cr = (np.zeros(nn, np.int64) for _ in range(4))
        tdr = np.zeros(nn, np.float32)
        bbox = np.zeros((nn, 9), np.float32)
        ppm = np.zeros((nn, tdpts), np.float32)
        self._lib.ora_result_nodes(self._h, _ptr(cnt, C.c_int64), _ptr(off, C.c_int64),
                                   _ptr(cl, C.c_int64), _ptr(cr, C.c_int64),
                                   _ptr(tdr, C.c_float), _ptr(bbox, C.c_float),
                                   _ptr(ppm, C.c_float))
        return dict(count=cnt, offset=off, cl=cl, cr=cr, tdr=tdr, bbox=bbox, ppm=ppm)

    def acc_fp64(self):
        n = self._p.n
        a = [np.full(n, np.nan) for _ in range(3)]
        self._lib.ora_result_acc_fp64(self._h, *[_ptr(v, C.c_double) for v in a])
        return np.stack(a, axis=1)


class Oracle:
    def __init__(self, path: str = LIB):
        if not os.path.exists(path):
            build()
        lib = C.CDLL(path)
        self.lib = lib
        i64, f32, f64 = C.c_int64, C.c_float, C.c_double
        pf, pd, pi64, pu16 = (C.POINTER(C.c_float), C.POINTER(C.c_double),
                              C.POINTER(C.c_int64), C.POINTER(C.c_uint16))
        lib.ora_rcb_run.restype = C.c_void_p
        lib.ora_rcb_run.argtypes = [C.POINTER(OraParams), i64] + [pf] * 8 + [pi64, pu16, C.c_int,
                                                                             C.c_int, C.POINTER(C.c_int)]
        lib.ora_result_stats.argtypes = [C.c_void_p, C.POINTER(OraStats)]
        lib.ora_result_nleaves.restype = i64
        lib.ora_result_nleaves.argtypes = [C.c_void_p]
        lib.ora_result_nentries.restype = i64
        lib.ora_result_nentries.argtypes = [C.c_void_p]
        lib.ora_result_leaves.argtypes = [C.c_void_p, pi64, pi64, pi64]
        lib.ora_result_entries.argtypes = [C.c_void_p, pf, pf, pf, pf]
        lib.ora_result_nnodes.restype = i64
        lib.ora_result_nnodes.argtypes = [C.c_void_p]
        lib.ora_result_nodes.argtypes = [C.c_void_p, pi64, pi64, pi64, pi64, pf, pf, pf]
        lib.ora_result_acc_fp64.argtypes = [C.c_void_p, pd, pd, pd]
        lib.ora_result_free.argtypes = [C.c_void_p]
        lib.ora_law_f32.restype = f32
        lib.ora_law_f32.argtypes = [C.c_int, f32, f32]
        lib.ora_law_f64.restype = f64
        lib.ora_law_f64.argtypes = [C.c_int, f64, f64]
        lib.ora_law_dg_f64.restype = f64
        lib.ora_law_dg_f64.argtypes = [C.c_int, f64, f64]
        lib.ora_direct_fp64.argtypes = [i64, pf, pf, pf, pf, C.c_int, f32, f32, i64, pi64, pd, pd, pd]
        lib.ora_vjp_fp64.argtypes = [i64, pf, pf, pf, pf, C.c_int, f32, f32, f64, i64, pi64, pi64,
                                     pi64, pi64, pd, pd]
        lib.ora_vjp_fp64_tab.argtypes = [i64, pf, i64, pi64, pi64, C.c_int, f32, f32, f64, i64, pi64,
                                         pi64, pi64, pi64, pd, pd]
        lib.ora_fd_fp64_tab.argtypes = [i64, pf, i64, pi64, pi64, C.c_int, f32, f32, f64, i64, pi64,
                                        pi64, pi64, pi64, pd, i64, pi64, f64, pd,
                                        C.POINTER(C.c_int32)]
        lib.ora_map1.argtypes = [i64, pf, pf, pf, pf, pf, pf, f32, f32, f32, f32]
        kick64 = [i64, pd, pd, i64, pi64, pi64, C.c_int, f64, f64, f64, i64, pi64, pi64, pi64,
                  pi64]
        lib.ora_kick64.argtypes = kick64 + [pd, pd]
        lib.ora_kick64_vjp.argtypes = kick64 + [pd, pd]
        lib.ora_resort.restype = i64
        lib.ora_resort.argtypes = [i64, C.POINTER(C.c_int), pf, pf, pf, pf, pf, pf, pf, pf, pi64, pu16]

    # -- the RCBForceTree constructor -------------------------------------
    def rcb_run(self, p, kp, keep_lists: bool = False, do_kick: bool = True,
                nthreads: int = 0, vmax: int = 0) -> OracleResult:
        """Runs build + walk (+ kick) on `p` in place."""
        P = params_struct(kp, nthreads, vmax)
        err = C.c_int(0)
        arrs = [_ptr(getattr(p, k), C.c_float) for k in ("x", "y", "z", "vx", "vy", "vz", "mass", "phi")]
        h = self.lib.ora_rcb_run(C.byref(P), p.n, *arrs, _ptr(p.id, C.c_int64),
                                 _ptr(p.mask, C.c_uint16), int(keep_lists), int(do_kick),
                                 C.byref(err))
        if not h:
            raise RuntimeError(f"oracle failed: {ERRORS.get(err.value, err.value)}")
        return OracleResult(self.lib, h, p)

    def law_f32(self, law: int, rsm: float, r2: float) -> float:
        return self.lib.ora_law_f32(law, rsm, r2)

    def law_f64(self, law: int, rsm: float, r2: float) -> float:
        return self.lib.ora_law_f64(law, rsm, r2)

    def direct_fp64(self, p, targets, law=LAW_POLY6, rsm=0.1, fsrrmax=3.116326355):
        t = np.ascontiguousarray(targets, dtype=np.int64)
        a = [np.zeros(len(t)) for _ in range(3)]
        self.lib.ora_direct_fp64(p.n, _ptr(p.x, C.c_float), _ptr(p.y, C.c_float),
                                 _ptr(p.z, C.c_float), _ptr(p.mass, C.c_float), law, rsm,
                                 fsrrmax, len(t), _ptr(t, C.c_int64),
                                 *[_ptr(v, C.c_double) for v in a])
        return np.stack(a, axis=1)

    def vjp_fp64(self, p, c, leaf_offset, leaf_count, list_ptr, list_idx, u,
                 law=LAW_POLY6, rsm=0.1, fsrrmax=3.116326355):
        u = np.ascontiguousarray(u, dtype=np.float64)
        xbar = np.zeros((p.n, 3))
        lo, lc, lp, li = (np.ascontiguousarray(a, dtype=np.int64)
                          for a in (leaf_offset, leaf_count, list_ptr, list_idx))
        self.lib.ora_vjp_fp64(p.n, _ptr(p.x, C.c_float), _ptr(p.y, C.c_float),
                              _ptr(p.z, C.c_float), _ptr(p.mass, C.c_float), law, rsm, fsrrmax,
                              c, len(lo), _ptr(lo, C.c_int64), _ptr(lc, C.c_int64),
                              _ptr(lp, C.c_int64), _ptr(li, C.c_int64),
                              _ptr(u, C.c_double), _ptr(xbar, C.c_double))
        return xbar

    def vjp_tab(self, n, tab, pnode_off, pnode_cnt, c, leaf_offset, leaf_count, list_ptr,
                list_idx, u, law=LAW_POLY6, rsm=0.1, fsrrmax=3.116326355):
        """FP64 VJP over table-index lists (monopole pseudo-particles through
        their node's centre of mass); u, result: n x 3."""
        tab = np.ascontiguousarray(tab, np.float32)
        arrs = [np.ascontiguousarray(a, np.int64) for a in (pnode_off, pnode_cnt, leaf_offset,
                                                             leaf_count, list_ptr, list_idx)]
        u = np.ascontiguousarray(u, np.float64)
        xbar = np.zeros((n, 3))
        self.lib.ora_vjp_fp64_tab(n, _ptr(tab, C.c_float), tab.shape[0], _ptr(arrs[0], C.c_int64),
                                  _ptr(arrs[1], C.c_int64), law, rsm, fsrrmax, c, len(arrs[2]),
                                  *[_ptr(a, C.c_int64) for a in arrs[2:]], _ptr(u, C.c_double),
                                  _ptr(xbar, C.c_double))
        return xbar

    def fd_tab(self, n, tab, pnode_off, pnode_cnt, c, leaf_offset, leaf_count, list_ptr,
               list_idx, u, samples, h=1e-4, law=LAW_POLY6, rsm=0.1, fsrrmax=3.116326355):
        """FP64 central differences of sum_i u_i . dv_i at the sampled
        particles; returns (fd: s x 3, near_cutoff: s)."""
        tab = np.ascontiguousarray(tab, np.float32)
        arrs = [np.ascontiguousarray(a, np.int64) for a in (pnode_off, pnode_cnt, leaf_offset,
                                                             leaf_count, list_ptr, list_idx)]
        u = np.ascontiguousarray(u, np.float64)
        smp = np.ascontiguousarray(samples, np.int64)
        fd = np.zeros((len(smp), 3))
        near = np.zeros(len(smp), np.int32)
        self.lib.ora_fd_fp64_tab(n, _ptr(tab, C.c_float), tab.shape[0], _ptr(arrs[0], C.c_int64),
                                 _ptr(arrs[1], C.c_int64), law, rsm, fsrrmax, c, len(arrs[2]),
                                 *[_ptr(a, C.c_int64) for a in arrs[2:]], _ptr(u, C.c_double),
                                 len(smp), _ptr(smp, C.c_int64), h, _ptr(fd, C.c_double),
                                 near.ctypes.data_as(C.POINTER(C.c_int32)))
        return fd, near.astype(bool)

    # -- FP64 multi-step reference ------------------------------------------
    def kick64(self, pos, m, tape, c, law=LAW_POLY6, rsm=0.1, fsrrmax=3.116326355,
               pos_cut=None):
        """FP64 kick over one tape (tree order): dv (n x 3).  pos_cut: the
        cutoff of every pair decided at these positions instead."""
        n = len(m)
        dv = np.zeros((n, 3))
        pc = None if pos_cut is None else np.ascontiguousarray(pos_cut, np.float64)
        self.lib.ora_kick64(n, *self._k64args(pos, m, tape, law, rsm, fsrrmax, c),
                            None if pc is None else _ptr(pc, C.c_double), _ptr(dv, C.c_double))
        return dv

    def kick64_vjp(self, pos, m, tape, c, u, law=LAW_POLY6, rsm=0.1, fsrrmax=3.116326355):
        """(d dv / d pos)^T u for kick64, n x 3 (tree order)."""
        n = len(m)
        u = np.ascontiguousarray(u, np.float64)
        xb = np.zeros((n, 3))
        self.lib.ora_kick64_vjp(n, *self._k64args(pos, m, tape, law, rsm, fsrrmax, c),
                                _ptr(u, C.c_double), _ptr(xb, C.c_double))
        return xb

    def _k64args(self, pos, m, tape, law, rsm, fsrrmax, c):
        self._keep = [np.ascontiguousarray(pos, np.float64), np.ascontiguousarray(m, np.float64)]
        self._keep += [np.ascontiguousarray(tape[k], np.int64)
                       for k in ("noff", "ncnt", "off", "cnt", "ptr", "idx")]
        pos, m, noff, ncnt, off, cnt, ptr, idx = self._keep
        return (_ptr(pos, C.c_double), _ptr(m, C.c_double), len(noff), _ptr(noff, C.c_int64),
                _ptr(ncnt, C.c_int64), law, float(np.float32(rsm)), float(np.float32(fsrrmax)),
                float(c), len(off), _ptr(off, C.c_int64), _ptr(cnt, C.c_int64),
                _ptr(ptr, C.c_int64), _ptr(idx, C.c_int64))

    def stream_factor(self, alpha, pp, tau, adot) -> float:
        """map1's float factor pt (x += pt v), from the restated map1."""
        z = np.zeros(1, np.float32)
        one = np.ones(1, np.float32)
        x, y, zz = z.copy(), z.copy(), z.copy()
        self.lib.ora_map1(1, _ptr(x, C.c_float), _ptr(y, C.c_float), _ptr(zz, C.c_float),
                          _ptr(one, C.c_float), _ptr(one.copy(), C.c_float),
                          _ptr(one.copy(), C.c_float), alpha, pp, tau, adot)
        return float(x[0])

    def multistep64(self, x0, v0, m, steps, nsub, tapes, xbar=None, vbar=None, kick_pos=None,
                    law=LAW_POLY6, rsm=0.1, fsrrmax=3.116326355, cut_pos=None, traj_out=None,
                    pm=None, pm_pos=None, pm_cut=None, pm_traj_out=None):
        """FP64 restatement of the sub-cycled short-range map (map1, kick,
        map1; nsub per PM step) with every kick's tree and lists frozen to
        `tapes` (one per kick in forward order: perm, node ranges, leaves and
        lists in tree order).  Caller-order n x 3 arrays.

        Returns the final (x, v) and, when cotangents (xbar, vbar) are given,
        also L = sum xbar.x_T + vbar.v_T and its FP64 gradient (x0bar, v0bar).
        kick_pos: optional positions of every kick (n x 3 each) at which the
        reverse pass evaluates the kick's VJP (default: this FP64 trajectory).
        cut_pos: optional positions of every kick on which the pairs' cutoff is
        decided (the map with its cutoff mask frozen); traj_out, a list, receives
        this run's kick positions.

        pm: optional PM kicks, one (open, close) pair per step, each None or a
        dict(ng, ngo, gpscal, fscal, tau): v += fscal tau F(x) before the step's
        sub-cycles (open) and after them (close), F from pm_oracle.force64.
        pm_pos / pm_cut / pm_traj_out play the roles of kick_pos / cut_pos /
        traj_out for the PM kicks (pm_cut freezes each particle's CIC cell).
        """
        import pm_oracle

        def pm_kick(q, prm, base):
            return prm["fscal"] * prm["tau"] * pm_oracle.force64(
                q[:, 0], q[:, 1], q[:, 2], prm["ng"], prm["ngo"], prm["gpscal"], base=base)
        pm_traj = []
        x = np.array(x0, np.float64)
        v = np.array(v0, np.float64)
        m = np.asarray(m, np.float64)
        pts = [self.stream_factor(st.alpha, st.pp, st.tau_sub, st.adot) for st in steps]
        traj = []
        k = 0
        q = 0
        for s, st in enumerate(steps):
            for half in (0, 1):
                prm = pm[s][half] if pm is not None else None
                if half == 1:
                    for _ in range(nsub):
                        x += pts[s] * v
                        traj.append(x.copy())
                        t = tapes[k]
                        perm = t["perm"]
                        pc = None if cut_pos is None else np.asarray(cut_pos[k], np.float64)[perm]
                        v[perm] += self.kick64(x[perm], m[perm], t, st.fcoeff, law, rsm, fsrrmax,
                                               pc)
                        x += pts[s] * v
                        k += 1
                if prm is not None:
                    pm_traj.append(x.copy())
                    base = None if pm_cut is None else np.asarray(pm_cut[q], np.float64)
                    v += pm_kick(x, prm, base)
                    q += 1
        if traj_out is not None:
            traj_out.extend(traj)
        if pm_traj_out is not None:
            pm_traj_out.extend(pm_traj)
        if xbar is None:
            return x, v
        L = float((np.asarray(xbar) * x).sum() + (np.asarray(vbar) * v).sum())
        xb = np.array(xbar, np.float64)
        vb = np.array(vbar, np.float64)

        def pm_adj(prm):
            nonlocal q
            q -= 1
            xq = pm_traj[q] if pm_pos is None else np.asarray(pm_pos[q], np.float64)
            return prm["fscal"] * prm["tau"] * pm_oracle.vjp64(
                xq[:, 0], xq[:, 1], xq[:, 2], vb, prm["ng"], prm["ngo"], prm["gpscal"])
        for s in reversed(range(len(steps))):
            st = steps[s]
            if pm is not None and pm[s][1] is not None:
                xb += pm_adj(pm[s][1])
            for _ in range(nsub):
                k -= 1
                vb += pts[s] * xb
                t = tapes[k]
                perm = t["perm"]
                xk = traj[k] if kick_pos is None else np.asarray(kick_pos[k], np.float64)
                xb[perm] += self.kick64_vjp(xk[perm], m[perm], t, st.fcoeff, vb[perm], law, rsm,
                                            fsrrmax)
                vb += pts[s] * xb
            if pm is not None and pm[s][0] is not None:
                xb += pm_adj(pm[s][0])
        return x, v, L, xb, vb

    def map1(self, p, alpha, pp, tau, adot):
        self.lib.ora_map1(p.n, *[_ptr(getattr(p, k), C.c_float) for k in ("x", "y", "z", "vx", "vy", "vz")],
                          alpha, pp, tau, adot)

    def subcycle(self, p, ts, nsub, kp, gpscal=1.0, stream=True, kick=True, nthreads=0,
                 fcoeff=None):
        """Particles::subCycle (Particles.cxx:1176-1201) restated on `p` in
        place: nsub times map1 (tau = stepFraction * tau2 as a float), map2
        (resortParticles, masses = 1, the RCB kick of the in-box particles
        with c from the stepper), map1.  `ts` is the stepper at which the
        sub-cycles run (synth.Stepper), `kp` the tree parameters (its fcoeff
        is replaced by map2's c, or by `fcoeff` when given).  Returns the
        last in-box count."""
        import synth
        tau = float(synth.stream_tau(ts, nsub))
        kc = synth.KickParams(**{**kp.__dict__})
        kc.fcoeff = (float(synth.kick_coefficient(ts, nsub, gpscal)) if fcoeff is None
                     else float(fcoeff))
        nin = p.n
        for _ in range(nsub):
            if stream:
                self.map1(p, ts.alpha, ts.pp, tau, ts.adot)
            if kick:
                nin = self.resort(p)
                p.mass[:] = 1.0
                view = synth.Particles(*(getattr(p, k)[:nin] for k in synth.FIELDS),
                                       nglt=p.nglt)
                self.rcb_run(view, kc, nthreads=nthreads)
            if stream:
                self.map1(p, ts.alpha, ts.pp, tau, ts.adot)
        return nin

    def resort(self, p) -> int:
        ng = (C.c_int * 3)(*p.nglt)
        return self.lib.ora_resort(p.n, ng, *[_ptr(getattr(p, k), C.c_float) for k in
                                             ("x", "y", "z", "vx", "vy", "vz", "phi", "mass")],
                                   _ptr(p.id, C.c_int64), _ptr(p.mask, C.c_uint16))


# ---------------------------------------------------------------------------
# Reference runs (case files for oracle/_ref/rcb_ref)
# ---------------------------------------------------------------------------

CASE_MAGIC = b"HSRCASE1"
_PFMT = "<16f3q2f6i"


def write_case(path: str, p, kp, nthreads: int = 0, reps: int = 1) -> None:
    head = struct.pack(_PFMT, *kp.min, *kp.max, *kp.min_force, *kp.max_force, kp.avg_mass,
                       kp.fsrrmax, kp.rsm, kp.open_angle, kp.nd, kp.ds, kp.tmin, kp.fcoeff,
                       kp.ppc, kp.tdpts, kp.law, 0, nthreads, reps, getattr(kp, "tree", 0))
    with open(path, "wb") as f:
        f.write(CASE_MAGIC)
        f.write(struct.pack("<q", p.n))
        f.write(head)
        for k in ("x", "y", "z", "vx", "vy", "vz", "mass", "phi"):
            f.write(np.ascontiguousarray(getattr(p, k), np.float32).tobytes())
        f.write(np.ascontiguousarray(p.id, np.int64).tobytes())
        f.write(np.ascontiguousarray(p.mask, np.uint16).tobytes())


def read_case_arrays(path: str):
    with open(path, "rb") as f:
        buf = f.read()
    assert buf[:8] == CASE_MAGIC
    n = struct.unpack_from("<q", buf, 8)[0]
    off = 16 + struct.calcsize(_PFMT)
    out = {}
    for k in ("x", "y", "z", "vx", "vy", "vz", "mass", "phi"):
        out[k] = np.frombuffer(buf, np.float32, n, off).copy()
        off += 4 * n
    out["id"] = np.frombuffer(buf, np.int64, n, off).copy()
    off += 8 * n
    out["mask"] = np.frombuffer(buf, np.uint16, n, off).copy()
    return out


def _unlimited_stack():
    resource.setrlimit(resource.RLIMIT_STACK, (resource.RLIM_INFINITY, resource.RLIM_INFINITY))


def reference_available(tree: int = 0) -> bool:
    return os.path.exists(REF_RCO_EXE if tree == 1 else REF_EXE)


def run_reference(p, kp, nthreads: int = 0, reps: int = 1, timeout: float = 3600.0):
    """Runs the reference force tree on a copy of `p`; returns (arrays after the
    last repetition, list of wall times in seconds)."""
    tree = getattr(kp, "tree", 0)
    exe = REF_RCO_EXE if tree == 1 else REF_EXE
    if not reference_available(tree):
        raise FileNotFoundError(exe)
    with tempfile.TemporaryDirectory() as td:
        cin, cout = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        write_case(cin, p, kp, nthreads, reps)
        env = dict(os.environ, OMP_STACKSIZE="256M")
        if nthreads > 0:
            env["OMP_NUM_THREADS"] = str(nthreads)
        r = subprocess.run([exe, cin, cout], env=env, capture_output=True, text=True,
                           preexec_fn=_unlimited_stack, timeout=timeout)
        if r.returncode != 0:
            raise RuntimeError(f"reference run failed ({r.returncode}): {r.stderr[-2000:]}")
        info = json.loads(r.stdout.strip().splitlines()[-1])
        return read_case_arrays(cout), info["times"], info["threads"]


# ---------------------------------------------------------------------------
# Reference sub-cycle runs (oracle/_ref/sub_ref)
# ---------------------------------------------------------------------------

SUB_MAGIC = b"HSRSUBC1"
_SFMT = "<4d3q10i4f"
# Particles::m_useRCBTree values (Particles.cxx:1259-1363)
USE_RCB_MONO, USE_RCB_QUAD, USE_RCO_MONO, USE_RCO_QUAD = 2, 1, 5, 4


def subcycle_reference_available() -> bool:
    return os.path.exists(REF_SUB_EXE)


def run_reference_subcycle(p, *, ng, nsub, z_in, z_fin, nsteps, half_steps, nd=128, ds=1,
                           tmin=128, use_rcb_tree=USE_RCB_MONO, edge=3.2, gpscal=1.0, rsm=0.1,
                           open_angle=0.1, alpha=1.0, omegatot=None, skip_stream=False,
                           skip_kick=False, nthreads=0, timeout=3600.0):
    """Runs the reference's Particles::subCycle on a copy of `p` with a
    TimeStepper(alpha, 1/(1+z_in), 1/(1+z_fin), nsteps, omegatot) advanced
    `half_steps` half steps (ain, afin and omegatot rounded to float as
    Basedata holds them).  Returns (arrays after the sub-cycles, the
    stepper's values and the last in-box count as a dict)."""
    import numpy as np
    f = np.float32
    if omegatot is None:
        omegatot = float(f(f(0.23387755) + f(f(0.0226) / f(0.7)) / f(0.7)))
    ain = float(f(1.0 / float(f(1.0) + f(z_in))))
    afin = float(f(1.0 / float(f(1.0) + f(z_fin))))
    head = struct.pack(_SFMT, float(f(alpha)), ain, afin, float(f(omegatot)), nd, ds, tmin,
                       *[int(v) for v in ng], nsub, nsteps, half_steps, use_rcb_tree,
                       int(skip_stream), int(skip_kick), nthreads, edge, gpscal, rsm, open_angle)
    if not subcycle_reference_available():
        raise FileNotFoundError(REF_SUB_EXE)
    with tempfile.TemporaryDirectory() as td:
        cin, cout = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        with open(cin, "wb") as fh:
            fh.write(SUB_MAGIC)
            fh.write(struct.pack("<q", p.n))
            fh.write(head)
            for k in ("x", "y", "z", "vx", "vy", "vz", "mass", "phi"):
                fh.write(np.ascontiguousarray(getattr(p, k), np.float32).tobytes())
            fh.write(np.ascontiguousarray(p.id, np.int64).tobytes())
            fh.write(np.ascontiguousarray(p.mask, np.uint16).tobytes())
        env = dict(os.environ, OMP_STACKSIZE="256M")
        if nthreads > 0:
            env["OMP_NUM_THREADS"] = str(nthreads)
        r = subprocess.run([REF_SUB_EXE, cin, cout], env=env, capture_output=True, text=True,
                           preexec_fn=_unlimited_stack, timeout=timeout)
        if r.returncode != 0:
            raise RuntimeError(f"reference sub-cycle failed ({r.returncode}): {r.stderr[-2000:]}")
        info = json.loads(r.stdout.strip().splitlines()[-1])
        with open(cout, "rb") as fh:
            if fh.read(8) != SUB_MAGIC:
                raise RuntimeError("bad sub-cycle output")
            n = struct.unpack("<q", fh.read(8))[0]
            fh.read(struct.calcsize(_SFMT))
            out = {}
            for k in ("x", "y", "z", "vx", "vy", "vz", "mass", "phi"):
                out[k] = np.frombuffer(fh.read(4 * n), np.float32).copy()
            out["id"] = np.frombuffer(fh.read(8 * n), np.int64).copy()
            out["mask"] = np.frombuffer(fh.read(2 * n), np.uint16).copy()
        return out, info
