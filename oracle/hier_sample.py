"""Timed CPU sample of a refined hierarchy's per-box work (test infrastructure:
the CPU baseline legs of bench.py use it; nothing in the product imports it).

One coarse step of a subcycled hierarchy (ratio 2) advances every box of level
l 2^l times; each advance is an SSP-RK3 step whose stages run the box's
right-hand side - the WENO-Z chain for a regular box, the cut-cell scheme for a
box whose grow(bx, 4) touches the body, nothing for a covered box
(Source/Advance.cpp:201-342) - and the Shu-Osher update.  This module times
that per-box work on the host cores with the oracle restatement (one box per
call of a serial -O3 build, the boxes spread over a thread pool as AMReX's
OpenMP build spreads its tiles, Source/Advance.cpp:197-199) for a sample of a
hierarchy's boxes, and returns the leaf cell-steps the sample stands for (the
cells of each box not covered by the next finer level, times 2^l), so that
leaf cell-steps / seconds is the same metric the GPU reports.  Ghost exchange,
coarse-fine interpolation, reflux and average-down are not timed (the GPU
figure includes them).
"""
from __future__ import annotations

import os
import time
from concurrent.futures import ThreadPoolExecutor

import numpy as np

NG = 4
BOX_REGULAR, BOX_CUT, BOX_COVERED = 0, 1, 2


def leaf_cells(grids):
    """Per level, per box: cells not covered by the next finer level's boxes
    (ratio 2).  grids[l] = [(lo, hi), ...]."""
    out = []
    for l, boxes in enumerate(grids):
        fine = grids[l + 1] if l + 1 < len(grids) else []
        cover = [(tuple(x // 2 for x in lo), tuple(x // 2 for x in hi)) for lo, hi in fine]
        counts = []
        for lo, hi in boxes:
            n = [hi[d] - lo[d] + 1 for d in range(3)]
            mask = np.zeros((n[2], n[1], n[0]), bool)
            for clo, chi in cover:
                a = [max(lo[d], clo[d]) for d in range(3)]
                b = [min(hi[d], chi[d]) for d in range(3)]
                if all(a[d] <= b[d] for d in range(3)):
                    mask[a[2] - lo[2]:b[2] - lo[2] + 1, a[1] - lo[1]:b[1] - lo[1] + 1,
                         a[0] - lo[0]:b[0] - lo[0] + 1] = True
            counts.append(int(mask.size - mask.sum()))
        out.append(counts)
    return out


def classify(eb, grids, dx0, prob_lo):
    """Box class per level and box for a z-aligned cylinder eb = dict(center,
    radius) (covered: every valid cell inside the body; regular: no cut or
    covered cell in grow(bx, 4); else cut, Source/Advance.cpp:213, 231), and the
    cut boxes' geometry (ocfd.geometry, 16 sub-samples).  Boxes whose grown
    rectangle clears the circle are regular without building their geometry."""
    from ocfd import geometry
    cx, cy = eb["center"]
    r = eb["radius"]
    phi = geometry.cylinder_phi(cx, cy, r)
    classes, geoms = [], []
    for l, boxes in enumerate(grids):
        dx = tuple(x / (1 << l) for x in dx0)
        cl, gm = [], []
        for lo, hi in boxes:
            x0 = prob_lo[0] + (lo[0] - NG - 1) * dx[0]
            x1 = prob_lo[0] + (hi[0] + NG + 2) * dx[0]
            y0 = prob_lo[1] + (lo[1] - NG - 1) * dx[1]
            y1 = prob_lo[1] + (hi[1] + NG + 2) * dx[1]
            ddx = max(x0 - cx, 0.0, cx - x1)
            ddy = max(y0 - cy, 0.0, cy - y1)
            if ddx * ddx + ddy * ddy > r * r:
                cl.append(BOX_REGULAR)
                gm.append(None)
                continue
            n = tuple(hi[d] - lo[d] + 1 for d in range(3))
            g = geometry.box_geometry(phi, lo, n, dx, prob_lo, nsub=16)
            typ = g["flag"][0] & 3
            if np.all(typ[NG:-NG, NG:-NG, NG:-NG] == geometry.T_COVERED):
                cl.append(BOX_COVERED)
                gm.append(None)
            elif np.all(typ == geometry.T_REGULAR):
                cl.append(BOX_REGULAR)
                gm.append(None)
            else:
                cl.append(BOX_CUT)
                gm.append(g)
        classes.append(cl)
        geoms.append(gm)
    return classes, geoms


class HierarchySample:
    """grids: box lists per level; fab(l, b) -> grown FAB (5, nz+8, ny+8, nx+8)
    of box b of level l; classes / geoms as classify() returns; dx0 the base
    cell size."""

    def __init__(self, grids, fab, classes, geoms, dx0, redistribute=True, threads=None, cfl=0.5):
        from oracle import Oracle
        self.o = Oracle(fast=True)
        self.grids = grids
        self.fab = fab
        self.classes = classes
        self.geoms = geoms
        self.dx0 = dx0
        self.redist = redistribute
        self.threads = threads or os.cpu_count() or 1
        self.leaf = leaf_cells(grids)
        self.cfl = cfl
        self.tasks = [(l, b) for l in range(len(grids)) for b in range(len(grids[l]))]

    def cells(self, l, b):
        lo, hi = self.grids[l][b]
        return (hi[0] - lo[0] + 1) * (hi[1] - lo[1] + 1) * (hi[2] - lo[2] + 1)

    def select(self, part, nparts):
        """The part-th of nparts interleaved samples of every level's boxes."""
        return [t for i, t in enumerate(self.tasks) if i % nparts == part]

    def _prepare(self, l, b):
        S = np.ascontiguousarray(self.fab(l, b), dtype=np.float64)
        dx = tuple(x / (1 << l) for x in self.dx0)
        est = self.o.estdt(S, dx)
        return S, tuple(1.0 / x for x in dx), self.cfl * est

    def _work(self, job):
        l, b, S, dxinv, dt = job
        cls = self.classes[l][b]
        if cls == BOX_COVERED:
            return
        g = self.geoms[l][b] if cls == BOX_CUT else None
        for _ in range(1 << l):
            self.o.box_rk3_step(S, dxinv, dt, g, self.redist)

    def time(self, sel):
        """Seconds of the per-box work of the boxes `sel` [(level, box)], and the
        leaf and all cell-steps they stand for."""
        jobs = []
        leaf = allc = 0
        for l, b in sorted(sel, key=lambda t: -self.cells(*t) * (1 << t[0])):
            S, dxinv, dt = self._prepare(l, b)
            jobs.append((l, b, S, dxinv, dt))
            leaf += self.leaf[l][b] << l
            allc += self.cells(l, b) << l
        t0 = time.perf_counter()
        with ThreadPoolExecutor(self.threads) as ex:
            list(ex.map(self._work, jobs))
        return time.perf_counter() - t0, leaf, allc
