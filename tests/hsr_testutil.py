"""Shared helpers of the test suite: fixtures on disk and error metrics."""
from __future__ import annotations

import glob
import os

import numpy as np

import synth

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

# FP32 force tolerances (rms relative and max relative to the rms force).
RMS_TOL = 1e-5
MAX_TOL = 1e-3


def golden_names():
    return sorted(os.path.splitext(os.path.basename(p))[0]
                  for p in glob.glob(os.path.join(GOLDEN, "*.npz")))


def load_golden(name):
    """Returns (input particles, KickParams, expected output arrays)."""
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    p = synth.Particles(*(d["in_" + k].copy() for k in synth.FIELDS),
                        nglt=tuple(int(v) for v in d["nglt"]))
    v = d["params"]
    kp = synth.KickParams(min=tuple(v[0:3]), max=tuple(v[3:6]), min_force=tuple(v[6:9]),
                          max_force=tuple(v[9:12]), avg_mass=float(v[12]), fsrrmax=float(v[13]),
                          rsm=float(v[14]), open_angle=float(v[15]), nd=int(v[16]), ds=int(v[17]),
                          tmin=int(v[18]), fcoeff=float(v[19]), ppc=float(v[20]),
                          tdpts=int(v[21]), law=int(v[22]),
                          tree=int(v[23]) if len(v) > 23 else 0)
    out = {k: d["out_" + k] for k in synth.FIELDS}
    return p, kp, out


def vel(p):
    return np.stack([p.vx, p.vy, p.vz], axis=1).astype(np.float64)


def force_errors(a, ref):
    """rms relative error sqrt(sum |a - ref|^2 / sum |ref|^2) and max error
    max_i |a_i - ref_i| / rms_i |ref_i|."""
    a = np.asarray(a, np.float64)
    ref = np.asarray(ref, np.float64)
    d = a - ref
    ref2 = (ref ** 2).sum()
    if ref2 == 0:
        return float(np.sqrt((d ** 2).sum())), float(np.abs(d).max(initial=0.0))
    rms = np.sqrt(ref2 / len(ref))
    return float(np.sqrt((d ** 2).sum() / ref2)), float(np.linalg.norm(d, axis=1).max() / rms)


def sorted_rows(e):
    """Entries (4 x m) as a lexicographically sorted array of row tuples."""
    e = np.ascontiguousarray(e.T).view(np.uint32)
    order = np.lexsort(e.T[::-1])
    return e[order]


def same_lists(a_off, a_cnt, a_ptr, a_e, b_off, b_cnt, b_ptr, b_e):
    """True when both sets of lists name the same leaves with the same
    multisets of entries (bitwise)."""
    ka = np.argsort(a_off, kind="stable")
    kb = np.argsort(b_off, kind="stable")
    if not (np.array_equal(a_off[ka], b_off[kb]) and np.array_equal(a_cnt[ka], b_cnt[kb])):
        return False
    for la, lb in zip(ka, kb):
        ea = a_e[:, a_ptr[la]:a_ptr[la + 1]]
        eb = b_e[:, b_ptr[lb]:b_ptr[lb + 1]]
        if ea.shape != eb.shape or not np.array_equal(sorted_rows(ea), sorted_rows(eb)):
            return False
    return True


def _leaf_major(off, ptr, e):
    """Entries (4 x m) regrouped leaf by leaf in order of leaf offset, with
    the leaf rank of every entry."""
    k = np.argsort(off, kind="stable")
    lens = np.diff(ptr)[k]
    starts = ptr[:-1][k]
    total = int(lens.sum())
    first = np.cumsum(lens) - lens
    idx = np.repeat(starts - first, lens) + np.arange(total, dtype=np.int64)
    return k, e[:, idx], np.repeat(np.arange(len(k), dtype=np.int64), lens)


def same_lists_exact(a_off, a_cnt, a_ptr, a_e, b_off, b_cnt, b_ptr, b_e):
    """same_lists for lists of any size (vectorised): True when both sets name
    the same leaves (offset and count) with the same multiset of entries per
    leaf, bit for bit.  Entries in the same order compare directly; otherwise
    each leaf's entries are sorted by their bits first."""
    if len(a_off) != len(b_off) or a_e.shape != b_e.shape:
        return False
    ka, ea, la = _leaf_major(a_off, a_ptr, a_e)
    kb, eb, lb = _leaf_major(b_off, b_ptr, b_e)
    if not (np.array_equal(a_off[ka], b_off[kb]) and np.array_equal(a_cnt[ka], b_cnt[kb])
            and np.array_equal(np.diff(a_ptr)[ka], np.diff(b_ptr)[kb])):
        return False
    ua, ub = ea.view(np.uint32), eb.view(np.uint32)
    if np.array_equal(ua, ub):
        return True

    def by_bits(u, leaf):
        w = u.astype(np.uint64)
        k1 = (w[0] << np.uint64(32)) | w[1]
        k2 = (w[2] << np.uint64(32)) | w[3]
        o = np.lexsort((k2, k1, leaf))
        return k1[o], k2[o]

    a1, a2 = by_bits(ua, la)
    b1, b2 = by_bits(ub, lb)
    return bool(np.array_equal(a1, b1) and np.array_equal(a2, b2))
