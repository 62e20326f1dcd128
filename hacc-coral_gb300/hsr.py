"""Python binding of the GB300 short-range gravity library (libhacc_sr.so).

Everything goes through the C ABI declared in include/hacc_sr.h.  There is no
CPU fallback: if the library is missing or no CUDA device is present, the
calls raise.

``RCBForceTree`` mirrors the reference constructor
(src/halo_finder/RCBForceTree.h:96-124): the same arguments in the same order,
the same in-place effect on the ten particle arrays (tree permutation plus the
short-range velocity kick).  ``ForceLawSR`` stands for the reference's
ForceLawSR over FGridEvalPoly (src/halo_finder/ForceLaw.h:114-127).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libhacc_sr.so")

HSR_OK = 0
(HSR_ERR_ARG, HSR_ERR_CUDA, HSR_ERR_NOMEM, HSR_ERR_TIMEOUT, HSR_ERR_UNSUPPORTED,
 HSR_ERR_NO_DEVICE, HSR_ERR_STATE) = range(1, 8)
STATUS = {0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "out of memory",
          4: "device wait timed out", 5: "unsupported", 6: "no CUDA device", 7: "bad call order"}
MEM_HOST, MEM_DEVICE = 0, 1
LAW_POLY6, LAW_POLY5_STEP16 = 0, 1
KERNEL_AUTO, KERNEL_PLAIN, KERNEL_BATCHED = 0, 1, 2
TREE_RCB, TREE_RCO = 0, 1
BUILD_DEVICE, BUILD_HOST = 0, 1

# Symbols the library exports (include/hacc_sr.h).
EXPORTS = ("hsr_create", "hsr_destroy", "hsr_last_error", "hsr_version", "hsr_rcb_kick",
           "hsr_get_stats", "hsr_lists_size", "hsr_lists_export", "hsr_build_lists",
           "hsr_lists_info", "hsr_lists_get", "hsr_lists_index", "hsr_lists_free",
           "hsr_force_law", "hsr_bench_pairs", "hsr_probe_fp32_peak", "hsr_kick_lists_noalloc",
           "hsr_force_fwd", "hsr_force_vjp", "hsr_last_perm", "hsr_tree_size", "hsr_tree_export",
           "hsr_lists_export_index", "hsr_rcb_kick_batch", "hsr_bench_pairs_graph",
           "hsr_subcycle", "hsr_set_tune", "hsr_get_tune", "hsr_autotune",
           "hsr_force_kick", "hsr_stream", "hsr_force_fwd_batch", "hsr_force_kick_batch",
           "hsr_force_vjp_batch",
           # include/hacc_pm.h
           "hsr_pm_kick", "hsr_pm_fields", "hsr_pm_get_stats", "hsr_pm_tables",
           "hsr_treepm_step", "hsr_pm_vjp", "hsr_pairs_in_cutoff")

PM_F64, PM_F32 = 0, 1


class HsrError(RuntimeError):
    def __init__(self, status: int, msg: str = ""):
        super().__init__(f"hsr status {status} ({STATUS.get(status, '?')}): {msg}")
        self.status = status


class HsrParams(C.Structure):
    _fields_ = [("min", C.c_float * 3), ("max", C.c_float * 3),
                ("min_force", C.c_float * 3), ("max_force", C.c_float * 3),
                ("avg_mass", C.c_float), ("fsrrmax", C.c_float), ("rsm", C.c_float),
                ("open_angle", C.c_float), ("nd", C.c_int64), ("ds", C.c_int64),
                ("tmin", C.c_int64), ("fcoeff", C.c_float), ("ppc", C.c_float),
                ("tdpts", C.c_int32), ("law", C.c_int32), ("kernel", C.c_int32),
                ("build", C.c_int32), ("tree", C.c_int32), ("reserved", C.c_int32)]


class HsrPmParams(C.Structure):
    """hsr_pm_params (include/hacc_pm.h)."""
    _fields_ = [("ng", C.c_int32), ("ngo", C.c_int32), ("gpscal", C.c_float),
                ("fscal", C.c_float), ("tau", C.c_float), ("precision", C.c_int32)]


class HsrPmStats(C.Structure):
    _fields_ = [("t_total_ms", C.c_double), ("t_h2d_ms", C.c_double),
                ("t_deposit_ms", C.c_double), ("t_solve_ms", C.c_double),
                ("t_interp_ms", C.c_double), ("t_d2h_ms", C.c_double),
                ("h2d_bytes", C.c_int64), ("d2h_bytes", C.c_int64),
                ("kernel_launches", C.c_int64), ("fft_execs", C.c_int64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


def pm_params(ng: int, ngo: int, gpscal: float = 1.0, fscal: float = 1.0, tau: float = 1.0,
              precision: int = PM_F64) -> HsrPmParams:
    P = HsrPmParams()
    P.ng, P.ngo, P.gpscal, P.fscal, P.tau, P.precision = ng, ngo, gpscal, fscal, tau, precision
    return P


class HsrSubcycleParams(C.Structure):
    _fields_ = [("kick", HsrParams), ("nsub", C.c_int32), ("ng", C.c_int32 * 3),
                ("alpha", C.c_float), ("pp", C.c_float), ("tau", C.c_float), ("adot", C.c_float),
                ("skip_stream", C.c_int32), ("skip_kick", C.c_int32)]


class HsrTune(C.Structure):
    _fields_ = [("kernel", C.c_int32), ("leaf_threads", C.c_int32), ("group", C.c_int32),
                ("reserved", C.c_int32)]

    def as_dict(self):
        return {"kernel": {KERNEL_PLAIN: "plain", KERNEL_BATCHED: "batched"}.get(self.kernel, self.kernel),
                "leaf_threads": self.leaf_threads, "group": self.group}


class HsrTuneRow(C.Structure):
    _fields_ = [("tune", HsrTune), ("ms", C.c_double), ("evaluated_pairs", C.c_int64)]


class HsrStats(C.Structure):
    _fields_ = [("n", C.c_int64), ("nodes", C.c_int64), ("leaves", C.c_int64),
                ("processed_leaves", C.c_int64), ("list_entries", C.c_int64),
                ("pairs", C.c_int64), ("kernel_launches", C.c_int64),
                ("t_build_ms", C.c_double), ("t_walk_ms", C.c_double),
                ("t_force_ms", C.c_double), ("t_total_ms", C.c_double),
                ("h2d_bytes", C.c_int64), ("d2h_bytes", C.c_int64),
                ("evaluated_pairs", C.c_int64), ("work_items", C.c_int64),
                ("cm_fallbacks", C.c_int64), ("t_h2d_ms", C.c_double),
                ("t_d2h_ms", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None


def load(path: str = LIB_PATH):
    """Loads libhacc_sr.so (built by build_ext.py); raises if it is absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise FileNotFoundError(
            f"{path} is missing: build it with `python hacc-coral_gb300/build_ext.py` "
            "(there is no CPU fallback)")
    lib = C.CDLL(path)
    vp, i32, i64, f32 = C.c_void_p, C.c_int32, C.c_int64, C.c_float
    pf, pi64, pu16 = C.POINTER(C.c_float), C.POINTER(C.c_int64), C.POINTER(C.c_uint16)
    lib.hsr_create.restype = i32
    lib.hsr_create.argtypes = [C.POINTER(vp), C.c_int]
    lib.hsr_destroy.restype = i32
    lib.hsr_destroy.argtypes = [vp]
    lib.hsr_last_error.restype = C.c_char_p
    lib.hsr_last_error.argtypes = [vp]
    lib.hsr_version.restype = C.c_char_p
    lib.hsr_rcb_kick.restype = i32
    lib.hsr_rcb_kick.argtypes = [vp, C.POINTER(HsrParams), i64] + [pf] * 8 + [pi64, pu16, i32]
    lib.hsr_get_stats.restype = i32
    lib.hsr_get_stats.argtypes = [vp, C.POINTER(HsrStats)]
    lib.hsr_lists_size.restype = i32
    lib.hsr_lists_size.argtypes = [vp, pi64, pi64]
    lib.hsr_lists_export.restype = i32
    lib.hsr_lists_export.argtypes = [vp, pi64, pi64, pi64, pf, pf, pf, pf]
    lib.hsr_build_lists.restype = i32
    lib.hsr_build_lists.argtypes = [C.POINTER(HsrParams), i64] + [pf] * 8 + [pi64, pu16, C.POINTER(vp)]
    lib.hsr_lists_info.restype = i32
    lib.hsr_lists_info.argtypes = [vp, pi64, pi64, C.POINTER(HsrStats)]
    lib.hsr_lists_get.restype = i32
    lib.hsr_lists_get.argtypes = [vp, pi64, pi64, pi64, pf, pf, pf, pf]
    lib.hsr_lists_index.restype = i32
    lib.hsr_lists_index.argtypes = [vp, pi64]
    lib.hsr_lists_free.restype = i32
    lib.hsr_lists_free.argtypes = [vp]
    lib.hsr_force_law.restype = i32
    lib.hsr_force_law.argtypes = [vp, i32, f32, f32, i64, pf, pf]
    lib.hsr_force_fwd.restype = i32
    lib.hsr_force_fwd.argtypes = [vp, C.POINTER(HsrParams), i64, vp, vp, vp, vp, vp, vp, vp, i32]
    lib.hsr_force_vjp.restype = i32
    lib.hsr_force_vjp.argtypes = [vp, vp, vp, vp, vp, vp, vp, i32]
    lib.hsr_last_perm.restype = i32
    lib.hsr_last_perm.argtypes = [vp, pi64]
    lib.hsr_tree_size.restype = i32
    lib.hsr_tree_size.argtypes = [vp, pi64]
    lib.hsr_tree_export.restype = i32
    lib.hsr_tree_export.argtypes = [vp, pi64, pi64, pi64, pi64, pf, pf, pf]
    lib.hsr_lists_export_index.restype = i32
    lib.hsr_lists_export_index.argtypes = [vp, pi64]
    lib.hsr_kick_lists_noalloc.restype = i32
    lib.hsr_kick_lists_noalloc.argtypes = [vp, i64, i64, vp, vp, vp, vp, i64, vp, vp, vp, vp,
                                           f32, f32, f32, i32, vp]
    lib.hsr_subcycle.restype = i32
    lib.hsr_subcycle.argtypes = [vp, C.POINTER(HsrSubcycleParams), i64] + [pf] * 8 + [pi64, pu16, i32,
                                                                                  pi64]
    lib.hsr_rcb_kick_batch.restype = i32
    lib.hsr_rcb_kick_batch.argtypes = [vp, i32, C.POINTER(HsrParams), pi64] + [vp] * 10 + [i32]
    lib.hsr_bench_pairs_graph.restype = i32
    lib.hsr_bench_pairs_graph.argtypes = [vp, i32, i32, C.POINTER(C.c_double)]
    lib.hsr_bench_pairs.restype = i32
    lib.hsr_bench_pairs.argtypes = [vp, i32, i32, i32, C.POINTER(C.c_double)]
    lib.hsr_probe_fp32_peak.restype = i32
    lib.hsr_probe_fp32_peak.argtypes = [vp, C.POINTER(C.c_double)]
    lib.hsr_force_kick.restype = i32
    lib.hsr_force_kick.argtypes = [vp, C.POINTER(HsrParams), i64, vp, vp, vp, vp, vp, vp, vp, i32]
    for nm in ("hsr_force_fwd_batch", "hsr_force_kick_batch"):
        getattr(lib, nm).restype = i32
        getattr(lib, nm).argtypes = [vp, i32, C.POINTER(HsrParams), pi64] + [vp] * 7 + [i32]
    lib.hsr_force_vjp_batch.restype = i32
    lib.hsr_force_vjp_batch.argtypes = [vp, i32] + [vp] * 6 + [i32]
    lib.hsr_stream.restype = i32
    lib.hsr_stream.argtypes = [vp, i64, vp, vp, vp, vp, vp, vp, f32, f32, f32, f32, i32]
    lib.hsr_set_tune.restype = i32
    lib.hsr_set_tune.argtypes = [vp, C.POINTER(HsrTune)]
    lib.hsr_get_tune.restype = i32
    lib.hsr_get_tune.argtypes = [vp, C.POINTER(HsrTune)]
    lib.hsr_autotune.restype = i32
    lib.hsr_autotune.argtypes = [vp, i32, i32, C.POINTER(HsrTuneRow), i32, C.POINTER(C.c_int32)]
    lib.hsr_pm_kick.argtypes = [vp, C.POINTER(HsrPmParams), i64] + [vp] * 6 + [i32]
    lib.hsr_pm_kick.restype = i32
    lib.hsr_pm_fields.argtypes = [vp, C.POINTER(HsrPmParams), i64] + [vp] * 5 + [i32]
    lib.hsr_pm_fields.restype = i32
    lib.hsr_pairs_in_cutoff.argtypes = [vp, pi64]
    lib.hsr_pairs_in_cutoff.restype = i32
    lib.hsr_pm_vjp.argtypes = [vp, C.POINTER(HsrPmParams), i64] + [vp] * 9 + [i32]
    lib.hsr_pm_vjp.restype = i32
    lib.hsr_pm_get_stats.argtypes = [vp, C.POINTER(HsrPmStats)]
    lib.hsr_pm_get_stats.restype = i32
    lib.hsr_pm_tables.argtypes = [i32, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                  C.POINTER(C.c_double)]
    lib.hsr_pm_tables.restype = i32
    _lib = lib
    return lib


def pm_tables(ng: int):
    """hsr_pm_tables: the quiet solver's (filter, denominator, gradient)
    tables as the library computes them (host code, no device)."""
    lib = load()
    out = [np.zeros(ng, np.float64) for _ in range(3)]
    st = lib.hsr_pm_tables(ng, *[_p(a, C.c_double) for a in out])
    if st != HSR_OK:
        raise HsrError(st, "hsr_pm_tables")
    return tuple(out)


def _p(a, ct):
    return a.ctypes.data_as(C.POINTER(ct))


def _check_host(a, dtype, n, name):
    if not isinstance(a, np.ndarray) or a.dtype != dtype or not a.flags.c_contiguous \
            or a.shape[0] < n or not a.flags.writeable:
        raise TypeError(f"{name} must be a writable C-contiguous {np.dtype(dtype)} array of >= {n}")


def make_params(kp, kernel: int = KERNEL_AUTO, build: int = BUILD_DEVICE) -> HsrParams:
    P = HsrParams()
    for k in ("min", "max", "min_force", "max_force"):
        getattr(P, k)[:] = [float(v) for v in getattr(kp, k)]
    P.avg_mass, P.fsrrmax, P.rsm, P.open_angle = kp.avg_mass, kp.fsrrmax, kp.rsm, kp.open_angle
    P.nd, P.ds, P.tmin = kp.nd, kp.ds, kp.tmin
    P.fcoeff, P.ppc, P.tdpts, P.law = kp.fcoeff, kp.ppc, kp.tdpts, kp.law
    P.kernel = kernel
    P.build = build
    P.tree = getattr(kp, "tree", TREE_RCB)
    return P


class Context:
    """One hsr_ctx: a CUDA device, its stream and buffers (one per host thread)."""

    def __init__(self, device: int = 0):
        self.lib = load()
        self.device = device
        h = C.c_void_p()
        st = self.lib.hsr_create(C.byref(h), device)
        if st != HSR_OK:
            raise HsrError(st, f"hsr_create(device={device})")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.hsr_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, st, what):
        if st != HSR_OK:
            raise HsrError(st, f"{what}: {self.lib.hsr_last_error(self.h).decode()}")

    def stats(self) -> dict:
        s = HsrStats()
        self._check(self.lib.hsr_get_stats(self.h, C.byref(s)), "hsr_get_stats")
        return s.as_dict()

    def rcb_kick(self, p, kp, kernel: int = KERNEL_AUTO, build: int = BUILD_DEVICE) -> dict:
        """hsr_rcb_kick on the host arrays of `p` (modified in place)."""
        P = make_params(kp, kernel, build)
        st = self.lib.hsr_rcb_kick(self.h, C.byref(P), p.n, *_particle_args(p), MEM_HOST)
        self._check(st, "hsr_rcb_kick")
        return self.stats()

    def rcb_kick_device(self, t: dict, n: int, kp, kernel: int = KERNEL_AUTO) -> dict:
        """hsr_rcb_kick on device arrays: `t` maps the ten field names to CUDA
        tensors (float32 x..phi, int64 id, int16/uint16 mask) on this context's
        device, modified in place.  The caller synchronizes its own streams
        before the call; the call returns with the results in place."""
        P = make_params(kp, kernel, BUILD_DEVICE)
        ptr = [C.cast(C.c_void_p(t[k].data_ptr()), C.POINTER(C.c_float))
               for k in ("x", "y", "z", "vx", "vy", "vz", "mass", "phi")]
        st = self.lib.hsr_rcb_kick(self.h, C.byref(P), n, *ptr,
                                   C.cast(C.c_void_p(t["id"].data_ptr()), C.POINTER(C.c_int64)),
                                   C.cast(C.c_void_p(t["mask"].data_ptr()), C.POINTER(C.c_uint16)),
                                   MEM_DEVICE)
        self._check(st, "hsr_rcb_kick(device arrays)")
        return self.stats()

    def subcycle(self, p, kp, nsub, ng, alpha, pp, tau, adot, skip_stream=False,
                 skip_kick=False, kernel: int = KERNEL_AUTO):
        """hsr_subcycle on the host arrays of `p` (all n particles, modified in
        place); returns (stats, in-box count of the last resort)."""
        S = HsrSubcycleParams()
        S.kick = make_params(kp, kernel, BUILD_DEVICE)
        S.nsub = nsub
        S.ng[:] = [int(v) for v in ng]
        S.alpha, S.pp, S.tau, S.adot = alpha, pp, tau, adot
        S.skip_stream, S.skip_kick = int(skip_stream), int(skip_kick)
        nin = C.c_int64()
        self._check(self.lib.hsr_subcycle(self.h, C.byref(S), p.n, *_particle_args(p), MEM_HOST,
                                          C.byref(nin)), "hsr_subcycle")
        return self.stats(), nin.value

    def lists(self):
        nl, ne = C.c_int64(), C.c_int64()
        self._check(self.lib.hsr_lists_size(self.h, C.byref(nl), C.byref(ne)), "hsr_lists_size")
        off = np.zeros(nl.value, np.int64)
        cnt = np.zeros(nl.value, np.int64)
        ptr = np.zeros(nl.value + 1, np.int64)
        e = np.zeros((4, ne.value), np.float32)
        self._check(self.lib.hsr_lists_export(self.h, _p(off, C.c_int64), _p(cnt, C.c_int64),
                                              _p(ptr, C.c_int64),
                                              *[_p(e[i], C.c_float) for i in range(4)]),
                    "hsr_lists_export")
        return off, cnt, ptr, e

    def force_fwd(self, x, y, z, mass, kp, kernel: int = KERNEL_AUTO):
        """hsr_force_fwd on host arrays; returns dv (n x 3, caller order)."""
        n = len(x)
        arrs = [np.ascontiguousarray(a, np.float32) for a in (x, y, z, mass)]
        dv = [np.zeros(n, np.float32) for _ in range(3)]
        P = make_params(kp, kernel, BUILD_DEVICE)
        vp = lambda a: a.ctypes.data_as(C.c_void_p)
        self._check(self.lib.hsr_force_fwd(self.h, C.byref(P), n, *[vp(a) for a in arrs],
                                           *[vp(a) for a in dv], MEM_HOST), "hsr_force_fwd")
        return np.stack(dv, 1)

    def force_kick_device(self, x, y, z, mass, vx, vy, vz, kp, kernel: int = KERNEL_AUTO):
        """hsr_force_kick on device buffers (objects with data_ptr(), e.g. CUDA
        tensors of float32): v += dv in the caller's order; records the tape."""
        n = int(x.numel())
        P = make_params(kp, kernel, BUILD_DEVICE)
        ptr = lambda t: C.c_void_p(t.data_ptr())
        self._check(self.lib.hsr_force_kick(self.h, C.byref(P), n, ptr(x), ptr(y), ptr(z),
                                            ptr(mass), ptr(vx), ptr(vy), ptr(vz), MEM_DEVICE),
                    "hsr_force_kick")

    def force_fwd_device(self, x, y, z, mass, dvx, dvy, dvz, kp, kernel: int = KERNEL_AUTO):
        """hsr_force_fwd on device buffers: dv written in the caller's order."""
        n = int(x.numel())
        P = make_params(kp, kernel, BUILD_DEVICE)
        ptr = lambda t: C.c_void_p(t.data_ptr())
        self._check(self.lib.hsr_force_fwd(self.h, C.byref(P), n, ptr(x), ptr(y), ptr(z),
                                           ptr(mass), ptr(dvx), ptr(dvy), ptr(dvz), MEM_DEVICE),
                    "hsr_force_fwd")

    def force_vjp_device(self, ux, uy, uz, xbx, xby, xbz):
        """hsr_force_vjp on device buffers: xbar = (d dv / d x)^T u, caller order."""
        ptr = lambda t: C.c_void_p(t.data_ptr())
        self._check(self.lib.hsr_force_vjp(self.h, ptr(ux), ptr(uy), ptr(uz), ptr(xbx), ptr(xby),
                                           ptr(xbz), MEM_DEVICE), "hsr_force_vjp")

    # ---- several boxes at once, device buffers ---------------------------
    @staticmethod
    def _ptr_tables(groups):
        """One C array of device pointers per group of tensors (kept alive by
        the returned list) and their addresses."""
        arrs = [(C.c_void_p * len(ts))(*[t.data_ptr() for t in ts]) for ts in groups]
        return arrs, [C.cast(a, C.c_void_p) for a in arrs]

    def _batch(self, fn, name, xs, masses, outs, kps, kernel):
        nb = len(kps)
        P = (HsrParams * nb)(*[make_params(k, kernel, BUILD_DEVICE) for k in kps])
        ns = np.array([int(x[0].numel()) for x in xs], np.int64)
        groups = ([[x[d] for x in xs] for d in range(3)] + [list(masses)]
                  + [[o[d] for o in outs] for d in range(3)])
        keep, tabs = self._ptr_tables(groups)
        self._check(fn(self.h, nb, P, _p(ns, C.c_int64), *tabs, MEM_DEVICE), name)
        del keep
        return self.stats()

    def force_kick_batch_device(self, xs, masses, vs, kps, kernel: int = KERNEL_AUTO) -> dict:
        """hsr_force_kick_batch on device buffers: for every box b, v_b +=
        dv_b in its caller's order, all boxes' pairs in one persistent launch;
        xs[b] and vs[b] are (x, y, z) triples of float32 CUDA tensors, masses[b]
        one tensor, kps[b] its KickParams.  Records the multi-box tape."""
        return self._batch(self.lib.hsr_force_kick_batch, "hsr_force_kick_batch", xs, masses, vs,
                           kps, kernel)

    def force_fwd_batch_device(self, xs, masses, dvs, kps, kernel: int = KERNEL_AUTO) -> dict:
        """hsr_force_fwd_batch on device buffers: every box's dv written in
        its caller's order (dvs[b] a triple); records the multi-box tape."""
        return self._batch(self.lib.hsr_force_fwd_batch, "hsr_force_fwd_batch", xs, masses, dvs,
                           kps, kernel)

    def force_vjp_batch_device(self, us, xbars):
        """hsr_force_vjp_batch on device buffers: xbars[b] = (d dv_b / d x_b)^T
        us[b] for the tape of the last multi-box forward (triples per box)."""
        nb = len(us)
        keep, tabs = self._ptr_tables([[u[d] for u in us] for d in range(3)]
                                      + [[o[d] for o in xbars] for d in range(3)])
        self._check(self.lib.hsr_force_vjp_batch(self.h, nb, *tabs, MEM_DEVICE),
                    "hsr_force_vjp_batch")
        del keep

    # ---- long-range PM kick (include/hacc_pm.h) ---------------------------
    def pm_kick(self, x, y, z, vx, vy, vz, params: HsrPmParams) -> dict:
        """hsr_pm_kick on host float32 arrays (velocities kicked in place);
        returns the call's hsr_pm_stats."""
        n = len(x)
        for a, nm in ((x, "x"), (y, "y"), (z, "z"), (vx, "vx"), (vy, "vy"), (vz, "vz")):
            _check_host(a, np.float32, n, nm)
        vp = lambda a: a.ctypes.data_as(C.c_void_p)
        self._check(self.lib.hsr_pm_kick(self.h, C.byref(params), n, vp(x), vp(y), vp(z), vp(vx),
                                         vp(vy), vp(vz), MEM_HOST), "hsr_pm_kick")
        return self.pm_stats()

    def pm_kick_device(self, x, y, z, vx, vy, vz, params: HsrPmParams) -> dict:
        """hsr_pm_kick on device buffers (objects with data_ptr())."""
        ptr = lambda t: C.c_void_p(t.data_ptr())
        self._check(self.lib.hsr_pm_kick(self.h, C.byref(params), int(x.numel()), ptr(x), ptr(y),
                                         ptr(z), ptr(vx), ptr(vy), ptr(vz), MEM_DEVICE),
                    "hsr_pm_kick(device arrays)")
        return self.pm_stats()

    def pm_fields(self, x, y, z, params: HsrPmParams, grad: bool = True):
        """hsr_pm_fields on host positions: (rho (ng,ng,ng), grad (3,ng,ng,ng)
        or None), float32, x the slowest index."""
        ng = params.ng
        xs = [np.ascontiguousarray(a, np.float32) for a in (x, y, z)]
        rho = np.zeros((ng, ng, ng), np.float32)
        g = np.zeros((3, ng, ng, ng), np.float32) if grad else None
        vp = lambda a: a.ctypes.data_as(C.c_void_p) if a is not None else None
        self._check(self.lib.hsr_pm_fields(self.h, C.byref(params), len(xs[0]), *[vp(a) for a in xs],
                                           vp(rho), vp(g), MEM_HOST), "hsr_pm_fields")
        return rho, g

    def pm_vjp(self, x, y, z, vbar, params: HsrPmParams):
        """hsr_pm_vjp on host arrays: xbar (n x 3) for the cotangent vbar
        (n x 3) of the PM kick's velocity change at positions x, y, z."""
        n = len(x)
        xs = [np.ascontiguousarray(a, np.float32) for a in (x, y, z)]
        u = [np.ascontiguousarray(vbar[:, d], np.float32) for d in range(3)]
        xb = [np.zeros(n, np.float32) for _ in range(3)]
        vp = lambda a: a.ctypes.data_as(C.c_void_p)
        self._check(self.lib.hsr_pm_vjp(self.h, C.byref(params), n, *[vp(a) for a in xs],
                                        *[vp(a) for a in u], *[vp(a) for a in xb], MEM_HOST),
                    "hsr_pm_vjp")
        return np.stack(xb, 1)

    def pm_vjp_device(self, x, y, z, ux, uy, uz, xbx, xby, xbz, params: HsrPmParams):
        """hsr_pm_vjp on device buffers (objects with data_ptr())."""
        ptr = lambda t: C.c_void_p(t.data_ptr())
        self._check(self.lib.hsr_pm_vjp(self.h, C.byref(params), int(x.numel()), ptr(x), ptr(y),
                                        ptr(z), ptr(ux), ptr(uy), ptr(uz), ptr(xbx), ptr(xby),
                                        ptr(xbz), MEM_DEVICE), "hsr_pm_vjp(device arrays)")

    def pairs_in_cutoff(self) -> int:
        """hsr_pairs_in_cutoff: pairs of the last device-built kick within the cutoff."""
        c = C.c_int64()
        self._check(self.lib.hsr_pairs_in_cutoff(self.h, C.byref(c)), "hsr_pairs_in_cutoff")
        return c.value

    def pm_stats(self) -> dict:
        s = HsrPmStats()
        self._check(self.lib.hsr_pm_get_stats(self.h, C.byref(s)), "hsr_pm_get_stats")
        return s.as_dict()

    def stream_device(self, x, y, z, vx, vy, vz, alpha, pp, tau, adot):
        """hsr_stream (Particles::map1) on device buffers: x += pt v."""
        ptr = lambda t: C.c_void_p(t.data_ptr())
        self._check(self.lib.hsr_stream(self.h, int(x.numel()), ptr(x), ptr(y), ptr(z), ptr(vx),
                                        ptr(vy), ptr(vz), alpha, pp, tau, adot, MEM_DEVICE),
                    "hsr_stream")

    def force_vjp(self, dvbar):
        """hsr_force_vjp: xbar (n x 3) for the cotangent dvbar (n x 3), caller order."""
        u = [np.ascontiguousarray(dvbar[:, d], np.float32) for d in range(3)]
        xb = [np.zeros(len(u[0]), np.float32) for _ in range(3)]
        vp = lambda a: a.ctypes.data_as(C.c_void_p)
        self._check(self.lib.hsr_force_vjp(self.h, *[vp(a) for a in u], *[vp(a) for a in xb],
                                           MEM_HOST), "hsr_force_vjp")
        return np.stack(xb, 1)

    def last_perm(self, n: int):
        perm = np.zeros(n, np.int64)
        self._check(self.lib.hsr_last_perm(self.h, _p(perm, C.c_int64)), "hsr_last_perm")
        return perm

    def tree(self, tdpts: int = 1):
        nn = C.c_int64()
        self._check(self.lib.hsr_tree_size(self.h, C.byref(nn)), "hsr_tree_size")
        nn = nn.value
        cnt, off, cl, cr = (np.zeros(nn, np.int64) for _ in range(4))
        tdr = np.zeros(nn, np.float32)
        bbox = np.zeros((nn, 9), np.float32)
        ppm = np.zeros((nn, tdpts), np.float32)
        self._check(self.lib.hsr_tree_export(self.h, _p(cnt, C.c_int64), _p(off, C.c_int64),
                                             _p(cl, C.c_int64), _p(cr, C.c_int64),
                                             _p(tdr, C.c_float), _p(bbox, C.c_float),
                                             _p(ppm, C.c_float)), "hsr_tree_export")
        return dict(count=cnt, offset=off, cl=cl, cr=cr, tdr=tdr, bbox=bbox, ppm=ppm)

    def lists_index(self):
        nl, ne = C.c_int64(), C.c_int64()
        self._check(self.lib.hsr_lists_size(self.h, C.byref(nl), C.byref(ne)), "hsr_lists_size")
        idx = np.zeros(ne.value, np.int64)
        self._check(self.lib.hsr_lists_export_index(self.h, _p(idx, C.c_int64)),
                    "hsr_lists_export_index")
        return idx

    def bench_pairs(self, iters: int, kernel: int = KERNEL_AUTO, flush_l2: bool = True) -> float:
        """Mean ms per relaunch of the last kick's pair kernel (hsr_bench_pairs)."""
        ms = C.c_double()
        self._check(self.lib.hsr_bench_pairs(self.h, kernel, iters, int(flush_l2), C.byref(ms)),
                    "hsr_bench_pairs")
        return ms.value

    def bench_pairs_graph(self, iters: int, flush_l2: bool = True) -> float:
        """Mean ms per replay of the batched launch captured as a CUDA graph."""
        ms = C.c_double()
        self._check(self.lib.hsr_bench_pairs_graph(self.h, iters, int(flush_l2), C.byref(ms)),
                    "hsr_bench_pairs_graph")
        return ms.value

    def rcb_kick_batch(self, boxes, kps, kernel: int = KERNEL_AUTO) -> dict:
        """hsr_rcb_kick_batch on a list of particle sets (host arrays, each
        permuted and kicked in place) with one KickParams each."""
        nb = len(boxes)
        P = (HsrParams * nb)(*[make_params(k, kernel, BUILD_DEVICE) for k in kps])
        ns = np.array([b.n for b in boxes], np.int64)
        for b in boxes:
            _particle_args(b)  # type and size checks
        tables = []
        for k in ("x", "y", "z", "vx", "vy", "vz", "mass", "phi", "id", "mask"):
            arr = (C.c_void_p * nb)(*[getattr(b, k).ctypes.data for b in boxes])
            tables.append(arr)
        self._check(self.lib.hsr_rcb_kick_batch(self.h, nb, P, _p(ns, C.c_int64),
                                                *[C.cast(t, C.c_void_p) for t in tables], MEM_HOST),
                    "hsr_rcb_kick_batch")
        return self.stats()

    def set_tune(self, kernel: str = "batched", leaf_threads: int = 128, group: int = 32):
        """Launch shape for HSR_KERNEL_AUTO kicks (hsr_set_tune)."""
        k = {"plain": KERNEL_PLAIN, "batched": KERNEL_BATCHED}[kernel]
        t = HsrTune(k, leaf_threads, group, 0)
        self._check(self.lib.hsr_set_tune(self.h, C.byref(t)), "hsr_set_tune")

    def get_tune(self) -> dict:
        t = HsrTune()
        self._check(self.lib.hsr_get_tune(self.h, C.byref(t)), "hsr_get_tune")
        return t.as_dict()

    def autotune(self, iters: int = 5, flush_l2: bool = True) -> list:
        """Times every launch shape on the last device-built kick and keeps the
        fastest (hsr_autotune); returns one dict per shape."""
        rows = (HsrTuneRow * 16)()
        nr = C.c_int32()
        self._check(self.lib.hsr_autotune(self.h, iters, int(flush_l2), rows, 16, C.byref(nr)),
                    "hsr_autotune")
        return [dict(rows[i].tune.as_dict(), ms=rows[i].ms, evaluated_pairs=rows[i].evaluated_pairs)
                for i in range(nr.value)]

    def fp32_peak_tflops(self) -> float:
        t = C.c_double()
        self._check(self.lib.hsr_probe_fp32_peak(self.h, C.byref(t)), "hsr_probe_fp32_peak")
        return t.value

    def force_law(self, r2, law: int = LAW_POLY6, rsm: float = 0.1,
                  fsrrmax: float = 3.116326355) -> np.ndarray:
        r2 = np.ascontiguousarray(r2, dtype=np.float32)
        g = np.zeros_like(r2)
        self._check(self.lib.hsr_force_law(self.h, law, rsm, fsrrmax, r2.size,
                                           _p(r2, C.c_float), _p(g, C.c_float)), "hsr_force_law")
        return g


def _particle_args(p):
    n = p.n
    for k in ("x", "y", "z", "vx", "vy", "vz", "mass", "phi"):
        _check_host(getattr(p, k), np.float32, n, k)
    _check_host(p.id, np.int64, n, "id")
    _check_host(p.mask, np.uint16, n, "mask")
    return ([_p(getattr(p, k), C.c_float) for k in ("x", "y", "z", "vx", "vy", "vz", "mass", "phi")]
            + [_p(p.id, C.c_int64), _p(p.mask, C.c_uint16)])


class HostLists:
    """hsr_build_lists: the tree and lists built on the host only (no GPU)."""

    def __init__(self, p, kp):
        self.lib = load()
        P = make_params(kp)
        h = C.c_void_p()
        st = self.lib.hsr_build_lists(C.byref(P), p.n, *_particle_args(p), C.byref(h))
        if st != HSR_OK:
            raise HsrError(st, "hsr_build_lists")
        self.h = h
        self.n = p.n
        nl, ne, s = C.c_int64(), C.c_int64(), HsrStats()
        self.lib.hsr_lists_info(self.h, C.byref(nl), C.byref(ne), C.byref(s))
        self.nleaves, self.nentries, self.stats = nl.value, ne.value, s.as_dict()

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.hsr_lists_free(self.h)
            self.h = None

    def get(self):
        off = np.zeros(self.nleaves, np.int64)
        cnt = np.zeros(self.nleaves, np.int64)
        ptr = np.zeros(self.nleaves + 1, np.int64)
        e = np.zeros((4, self.nentries), np.float32)
        st = self.lib.hsr_lists_get(self.h, _p(off, C.c_int64), _p(cnt, C.c_int64),
                                    _p(ptr, C.c_int64), *[_p(e[i], C.c_float) for i in range(4)])
        if st != HSR_OK:
            raise HsrError(st, "hsr_lists_get")
        return off, cnt, ptr, e

    def index(self):
        idx = np.zeros(self.nentries, np.int64)
        st = self.lib.hsr_lists_index(self.h, _p(idx, C.c_int64))
        if st != HSR_OK:
            raise HsrError(st, "hsr_lists_index")
        return idx


def kick_lists_noalloc(table, n, leaf_offset, leaf_count, list_begin, list_len, list_index,
                       vx, vy, vz, fcoeff, rsm=0.1, fsrrmax=3.116326355, law=LAW_POLY6):
    """hsr_kick_lists_noalloc on CUDA tensors (the caller owns every buffer;
    the library allocates nothing).  Raises HsrError on a non-zero status."""
    lib = load()
    ptr = lambda t: C.c_void_p(t.data_ptr())
    st = lib.hsr_kick_lists_noalloc(ptr(table), table.shape[0], n, ptr(leaf_offset),
                                    ptr(leaf_count), ptr(list_begin), ptr(list_len),
                                    leaf_offset.shape[0], ptr(list_index), ptr(vx), ptr(vy),
                                    ptr(vz), fcoeff, rsm, fsrrmax, law, None)
    if st != HSR_OK:
        raise HsrError(st, "hsr_kick_lists_noalloc")


# ---------------------------------------------------------------------------
# Reference-shaped interface
# ---------------------------------------------------------------------------

class ForceLawSR:
    """ForceLawSR(FGridEvalPoly, rsm): the short-range law the tree evaluates
    (src/halo_finder/ForceLaw.h:114-127; POLY_ORDER 6)."""

    def __init__(self, rsm: float, law: int = LAW_POLY6):
        self.rsm = float(rsm)
        self.law = law


_default_ctx = None


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


class _Args:
    pass


def RCBForceTree(minLoc, maxLoc, minForceLoc, maxForceLoc, count, xLoc, yLoc, zLoc, xVel, yVel,
                 zVel, mass, phiLoc, idLoc, maskLoc, avgMass, fsm, r, oa, nd=1, ds=1, tmin=128,
                 fl=None, fcoeff=0.0, ppc=0.9, tdpts=1, ctx: Context | None = None):
    """The RCBForceTree<TDPTS> constructor: builds the tree over `count`
    particles (permuting the ten arrays in place), walks it and kicks the
    velocities.  `fl` must be a ForceLawSR: the reference's default
    (fl = 0 -> ForceLawNewton, fcoeff = 1) is not part of the short-range
    path and raises.  Returns the call's statistics."""
    if fl is None:
        raise HsrError(5, "fl=None selects ForceLawNewton in the reference; pass a ForceLawSR")
    a = _Args()
    a.min, a.max = tuple(minLoc), tuple(maxLoc)
    a.min_force, a.max_force = tuple(minForceLoc), tuple(maxForceLoc)
    a.avg_mass, a.fsrrmax, a.rsm, a.open_angle = avgMass, fsm, fl.rsm, oa
    a.nd, a.ds, a.tmin, a.fcoeff, a.ppc, a.tdpts, a.law = nd, ds, tmin, fcoeff, ppc, tdpts, fl.law
    p = _Args()
    p.n = int(count)
    p.x, p.y, p.z, p.vx, p.vy, p.vz = xLoc, yLoc, zLoc, xVel, yVel, zVel
    p.mass, p.phi, p.id, p.mask = mass, phiLoc, idLoc, maskLoc
    return (ctx or default_context()).rcb_kick(p, a)


def RCOForceTree(minLoc, maxLoc, minForceLoc, maxForceLoc, count, xLoc, yLoc, zLoc, xVel, yVel,
                 zVel, mass, phiLoc, idLoc, maskLoc, avgMass, fsm, oa, nd=1, ds=1, fl=None,
                 fcoeff=0.0, ppc=0.9, tdpts=1, ctx: Context | None = None):
    """The RCOForceTree<TDPTS> constructor (src/halo_finder/RCOForceTree.h:
    95-121, RCOForceTree.cxx:326-412): the octree variant -- every inner node
    split along all three axes at its centre of mass.  The softening comes
    from `fl` (a ForceLawSR), as in the reference."""
    if fl is None:
        raise HsrError(5, "fl=None selects ForceLawNewton in the reference; pass a ForceLawSR")
    a = _Args()
    a.min, a.max = tuple(minLoc), tuple(maxLoc)
    a.min_force, a.max_force = tuple(minForceLoc), tuple(maxForceLoc)
    a.avg_mass, a.fsrrmax, a.rsm, a.open_angle = avgMass, fsm, fl.rsm, oa
    a.nd, a.ds, a.tmin, a.fcoeff, a.ppc, a.tdpts, a.law = nd, ds, 0, fcoeff, ppc, tdpts, fl.law
    a.tree = TREE_RCO
    p = _Args()
    p.n = int(count)
    p.x, p.y, p.z, p.vx, p.vy, p.vz = xLoc, yLoc, zLoc, xVel, yVel, zVel
    p.mass, p.phi, p.id, p.mask = mass, phiLoc, idLoc, maskLoc
    return (ctx or default_context()).rcb_kick(p, a)
