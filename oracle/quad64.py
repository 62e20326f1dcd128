"""FP64 restatement of the short-range kick with 12-point (quadrupole)
pseudo-particles as a function of the particle positions, the tree and lists
frozen: the FP64 reference of the quadrupole adjoint.

TEST INFRASTRUCTURE ONLY (the tests import it; the product never does).

It follows the reference's pseudo-particle construction in
src/halo_finder/RCBForceTree.cxx: `pptdr` (:519-523, the smallest distance
from the centre of mass to a face of the node's box, times ppContract,
:790, :858), `pppts` (:525-534, the design points xc + tdr e_a) and `pp`
(:536-568, each source adds m (1/K + (3/K)(r/tdr) cos + (5/K)(r/tdr)^2
(3 cos^2 - 1)/2) to point a, with cos the angle between the source and the
point as seen from xc); leaves of more than TDPTS and at most nDirect
particles take their particles (:786-799), inner nodes take each child's
particles (a child of at most TDPTS) or its pseudo-particles (:861-889).  The
law and the pair sum are the reference's nbody1 with the cutoff of every pair
decided once, at the unperturbed positions (the adjoint differentiates with
the trees, lists and cutoff mask held fixed).  The box extremes and the
argmin of pptdr are frozen to the particles and the face that attain them at
the unperturbed positions, so the map is smooth where the adjoint is taken.

In exact arithmetic r cos = d . e_a (|e_a| = 1, rj = tdr), so a source at d =
y - xc adds m [1/K + (3/K)(d.e_a)/tdr + (5/(2K))(3 (d.e_a)^2 - |d|^2)/tdr^2]
(1/K alone where tdr = 0, as the reference's rj2 == 0 branch).
"""
from __future__ import annotations

import numpy as np

# the design's 12 points as the library stores them (float): the icosahedron's
# vertices (+-a, +-b, 0) cycled, a = 0.525731112119134, b = 0.85065080835204
_IA, _IB = np.float32(0.525731112119134), np.float32(0.85065080835204)
DESIGN12 = np.array([[0, _IB, _IA], [0, _IB, -_IA], [_IA, 0, _IB], [-_IA, 0, _IB],
                     [_IB, _IA, 0], [-_IB, _IA, 0], [0, -_IB, -_IA], [0, -_IB, _IA],
                     [-_IA, 0, -_IB], [_IA, 0, -_IB], [-_IB, -_IA, 0], [_IB, -_IA, 0]],
                    np.float32).astype(np.float64)
K = 12

# the poly6 law's coefficients as the reference stores them (ForceLaw.cxx:98-104)
_POLY6 = [np.float32(c) for c in (0.271431, -0.0783394, 0.0133122, -0.00159485, 0.000132336,
                                  -0.00000663394, 0.000000147305)]


def law_g(r2, rsm):
    """g(r2) = (r2 + rsm^2)^(-3/2) - poly6(r2) in float64."""
    s = r2 + float(np.float32(rsm)) ** 2
    p = np.zeros_like(r2)
    for c in reversed(_POLY6):
        p = p * r2 + float(c)
    return s ** -1.5 - p


class QuadMap:
    """The frozen-structure FP64 kick with quadrupole pseudo-particles.

    tree: dict of tree-order node arrays offset, count, cl, cr (as
    hsr.Context.tree exports them); lists: (off, cnt, ptr, idx) of the
    processed leaves, idx indexing the position table (particles first, then
    node t's 12 points at n + 12 t + a); pos0: the unperturbed positions in
    tree order (n x 3, fixing the cutoff mask and the frozen argmins)."""

    def __init__(self, tree, lists, pos0, mass, fcoeff, ppc, nd, rsm=0.1, fsrrmax=3.116326355):
        self.off = np.asarray(tree["offset"], np.int64)
        self.cnt = np.asarray(tree["count"], np.int64)
        self.cl = np.asarray(tree["cl"], np.int64)
        self.cr = np.asarray(tree["cr"], np.int64)
        self.nn = len(self.off)
        self.m = np.asarray(mass, np.float64)
        self.n = len(self.m)
        self.c, self.ppc, self.nd, self.rsm = float(fcoeff), float(ppc), int(nd), float(rsm)
        loff, lcnt, lptr, idx = lists
        # the pairs (particle i, table entry e) of every processed leaf
        pi, pe = [], []
        for o, c, p0, p1 in zip(loff, lcnt, lptr[:-1], lptr[1:]):
            ent = np.asarray(idx[p0:p1], np.int64)
            ii = np.repeat(np.arange(o, o + c, dtype=np.int64), len(ent))
            pi.append(ii)
            pe.append(np.tile(ent, c))
        self.pi = np.concatenate(pi) if pi else np.zeros(0, np.int64)
        self.pe = np.concatenate(pe) if pe else np.zeros(0, np.int64)
        pos0 = np.asarray(pos0, np.float64)
        self.freeze = self._freeze(pos0)
        tab = self.table(pos0)
        d = tab[self.pe, :3] - pos0[self.pi]
        r2 = (d * d).sum(1)
        self.mask = r2 < float(np.float32(fsrrmax)) ** 2

    def _freeze(self, x):
        """Per node: the particles attaining the box's extremes and the face
        pptdr takes (index 0-2: xmax_d - xc_d, 3-5: xc_d - xmin_d)."""
        fr = []
        for t in range(self.nn):
            o, c = self.off[t], self.cnt[t]
            if c <= 0:
                fr.append(None)
                continue
            xs = x[o:o + c]
            ms = self.m[o:o + c]
            xc = (ms[:, None] * xs).sum(0) / ms.sum()
            amax, amin = o + xs.argmax(0), o + xs.argmin(0)
            cand = np.concatenate([xs.max(0) - xc, xc - xs.min(0)])
            fr.append((amax, amin, int(np.argmin(cand))))
        return fr

    def table(self, x):
        """Position table (n + 12 nnodes) x 4 at positions x (tree order)."""
        n, nn = self.n, self.nn
        tab = np.zeros((n + K * nn, 4))
        tab[:n, :3] = x
        tab[:n, 3] = self.m
        xc = np.zeros((nn, 3))
        tdr = np.zeros(nn)
        for t in range(nn):
            o, c = self.off[t], self.cnt[t]
            if c <= 0:
                continue
            ms = self.m[o:o + c]
            xc[t] = (ms[:, None] * x[o:o + c]).sum(0) / ms.sum()
            amax, amin, face = self.freeze[t]
            d = face % 3
            v = x[amax[d], d] - xc[t, d] if face < 3 else xc[t, d] - x[amin[d], d]
            tdr[t] = self.ppc * v
        # pseudo-particles, children first (children have larger indices)
        for t in range(nn - 1, -1, -1):
            c = self.cnt[t]
            if c <= 0:
                continue
            pts = xc[t] + tdr[t] * DESIGN12
            tab[n + K * t: n + K * t + K, :3] = pts
            leaf = self.cl[t] == 0 and self.cr[t] == 0
            srcs = []
            if leaf:
                if K < c <= self.nd:
                    srcs.append(tab[self.off[t]:self.off[t] + c])
            else:
                for ch in (self.cl[t], self.cr[t]):
                    if ch <= 0 or self.cnt[ch] <= 0:
                        continue
                    if self.cnt[ch] <= K:
                        srcs.append(tab[self.off[ch]:self.off[ch] + self.cnt[ch]])
                    else:
                        srcs.append(tab[n + K * ch: n + K * ch + K])
            ppm = np.zeros(K)
            for S in srcs:
                d = S[:, :3] - xc[t]
                if tdr[t] == 0.0:
                    ppm += S[:, 3].sum() / K
                    continue
                q = d @ DESIGN12.T                     # (s, a)
                dd = (d * d).sum(1)[:, None]
                f = 1.0 / K + (3.0 / K) * q / tdr[t] + (2.5 / K) * (3 * q * q - dd) / tdr[t] ** 2
                ppm += (S[:, 3:4] * f).sum(0)
            tab[n + K * t: n + K * t + K, 3] = ppm
        return tab

    def kick(self, x, points=None):
        """dv (n x 3, tree order) of the frozen map at positions x; with
        `points` (a table), its pseudo-particles are taken as constants."""
        tab = self.table(np.asarray(x, np.float64))
        if points is not None:
            tab[self.n:] = points[self.n:]
        d = tab[self.pe, :3] - x[self.pi]
        r2 = (d * d).sum(1)
        w = np.where(self.mask, tab[self.pe, 3] * law_g(r2, self.rsm), 0.0)
        dv = np.zeros((self.n, 3))
        np.add.at(dv, self.pi, w[:, None] * d)
        return self.c * self.m[:, None] * dv

    def loss(self, x, u, points=None):
        return float((np.asarray(u, np.float64) * self.kick(x, points)).sum())
