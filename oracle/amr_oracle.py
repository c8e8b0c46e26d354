"""CPU restatement of the AMR hierarchy step (test infrastructure).

Only tests/ import this module, as the checker of libocfd's ocfd_amr_* path.

It restates, level by level and with whole-level arrays instead of per-box
tables, what one coarse step of the GPU hierarchy does:

* subcycling with ratio 2 (AMReX Amr::timeStep; Source/EBR.cpp:312-360,
  EBR::post_timestep), SSP-RK3 in Shu-Osher form on every level
  (AmrLevel::RK(3, ...), Source/Advance.cpp:141-148), per-box right-hand sides
  from the C oracle (ocfdo_rhs_regular, which restates Source/Advance.cpp:231-342);
* coarse-fine ghost cells: the coarse SSP-RK3 dense output and the Taylor
  expansion of the fine stage states (McCorquodale & Colella, CAMCoS 6 (2011),
  sec. 3), then MC-limited conservative linear interpolation (van Leer) in
  space - the role of FillPatch / FillPatcher::fillRK with cell_cons_interp
  (Source/Setup.cpp:194-196);
* flux registers with the SSP-RK3 stage weights 1/6, 1/6, 2/3 and reflux of
  the uncovered coarse cells (EBFluxRegister CrseAdd / FineAdd / Reflux,
  Source/Advance.cpp:344-360, Source/EBR.cpp:322-330);
* average-down weighted by the fine volume fractions (EB_average_down,
  Source/EBR.cpp:535-559; unit fractions without a body);
* an optional embedded body (a z-aligned cylinder): per box the regular,
  cut-cell (ocfdo_rhs_eb, Source/EB/AdvanceBox.cpp:16-228) or covered scheme of
  the EBR::compute_dSdt box loop (Source/Advance.cpp:201-342), area-fraction
  weighted cut-cell fluxes in the registers and reflux divided by the coarse
  volume fraction (EBFluxRegister with areafrac / volfrac), piecewise-constant
  coarse-fine interpolation next to cut or covered parents;
* dt_0 = cfl * min over levels of est_l * 2^l, limited to 1.1 dt_prev and the
  stop time (EBR::computeNewDt, Source/EBR.cpp:240-305);
* regridding: |d rho| >= refine_dengrad (Source/Tagging.H:11-36) buffered by
  n_error_buf, blocks of blocking_factor cells, proper nesting by 2 coarse
  cells, greedy clustering into boxes of at most max_grid_size;
* with `react`: the CHEM build's EBR::advance on every level and substep
  (Source/Advance.cpp:158-174): 5 + 9 components (conserved state, partial
  densities), chemistry over dt_l / 2 in 4 / 2^l substeps (ocfdo_chem_advance,
  Source/CHEM/ChemAdvance.cpp:27-82), the RK2 multispecies flow step
  (ocfdo_rhs_chem per box, Source/CHEM/FlowAdvance.cpp:9-90) with flow and
  species flux registers (flux_reg / flux_reg_spec), chemistry over dt_l / 2;
  post_timestep: reflux, species renormalisation (Source/EBR.cpp:313-357),
  average-down; the fixed coarse step of the CHEM build (Source/Advance.cpp:54-57).

Parity note: AMReX is not part of the reference tree (empty submodule), so the
coarse-fine operators restate published methods rather than AMReX's code:
parity of this part with the reference is unpinned.  The restatement pins the
GPU implementation (tables, kernels, graph ordering) against an independent
CPU formulation of the same algorithm.
"""
from __future__ import annotations

import math

import numpy as np

from oracle import NG, BCStruct

T_REGULAR, T_CUT, T_COVERED = 0, 1, 3
BOX_REGULAR, BOX_CUT, BOX_COVERED = 0, 1, 2

W_RK3 = (1.0 / 6.0, 1.0 / 6.0, 2.0 / 3.0)
RK_A = (0.0, 0.75, 1.0 / 3.0)
RK_B = (1.0, 0.25, 2.0 / 3.0)
TFRAC = (0.0, 1.0, 0.5)
NEST = 2

# ebr.time_integration (Source/EBR.cpp:36; Source/Advance.cpp:115-149): stages,
# the buffer each stage reads, the times of its ghosts (fractions of dt) and the
# flux-register weights (x dt).  RK3 stages write U^n-weighted Shu-Osher updates;
# RK2 and Euler follow the reference's LinComb / Saxpy order.
SCHEMES = {
    3: dict(nst=3, src=(0, 1, 2), tfrac=TFRAC, w=W_RK3),
    2: dict(nst=2, src=(0, 1), tfrac=(0.0, 1.0), w=(0.5, 0.5)),
    1: dict(nst=1, src=(0,), tfrac=(0.0,), w=(1.0,)),
}


def mix_coefs(kind, theta, r=0.5):
    """Weights of (A, B, C, D) = (u0, U1, U2, U3) of the coarse RK3 step giving a
    fine stage value: kind 0..2 = fine stage 1..3 of the substep starting at
    theta, kind 3 = the coarse dense output at theta + r."""
    def P(th):
        return th - 5.0 / 6.0 * th * th, th * th / 6.0, 2.0 / 3.0 * th * th
    if kind == 3:
        w1, w2, w3 = P(theta + r)
    else:
        w1, w2, w3 = P(theta)
        d1, d2, d3 = 1.0 - 5.0 / 3.0 * theta, theta / 3.0, 4.0 / 3.0 * theta
        e1, e2, e3 = -5.0 / 3.0, 1.0 / 3.0, 4.0 / 3.0
        if kind == 1:
            w1 += r * d1
            w2 += r * d2
            w3 += r * d3
        elif kind == 2:
            w1 += 0.5 * r * d1 + 0.25 * r * r * e1
            w2 += 0.5 * r * d2 + 0.25 * r * r * e2
            w3 += 0.5 * r * d3 + 0.25 * r * r * e3
    return (1.0 - w1 - 3.0 * w2 - 0.5 * w3, w1 - w2, 4.0 * w2 - w3, 1.5 * w3)


def mc_slope(m, c, p):
    dl = c - m
    dr = p - c
    dc = 0.5 * (dl + dr)
    a = np.minimum(np.abs(dc), 2.0 * np.minimum(np.abs(dl), np.abs(dr)))
    s = np.where(dc > 0.0, a, -a)
    return np.where(dl * dr <= 0.0, 0.0, s)


def box_classes(geom, boxes):
    """Class of each box (Source/Advance.cpp:213, 231) from the geometry of its
    level (arrays over the level domain grown by NG): covered when all its cells
    are covered, regular when grow(bx, NG) holds no cut or covered cell."""
    typ = geom["flag"][0] & 3
    out = []
    for lo, hi in boxes:
        valid = typ[NG + lo[2]:NG + hi[2] + 1, NG + lo[1]:NG + hi[1] + 1, NG + lo[0]:NG + hi[0] + 1]
        grown = typ[lo[2]:hi[2] + 2 * NG + 1, lo[1]:hi[1] + 2 * NG + 1, lo[0]:hi[0] + 2 * NG + 1]
        if np.all(valid == T_COVERED):
            out.append(BOX_COVERED)
        elif np.all(grown == T_REGULAR):
            out.append(BOX_REGULAR)
        else:
            out.append(BOX_CUT)
    return out


def _sl(lo, hi, g=0):
    """numpy slices (z, y, x) of the cells lo..hi of an array offset by g."""
    return tuple(slice(lo[d] + g, hi[d] + g + 1) for d in (2, 1, 0))


class AmrOracle:
    def __init__(self, orc, n0, dx0, lo_bc, hi_bc, boxes0, prob_lo=(0.0, 0.0, 0.0), bc_case=0,
                 case_params=(), max_level=1, blocking_factor=(8, 8, 8), max_grid_size=(32, 32, 32),
                 n_error_buf=1, refine_dengrad=0.05, eb=None, time_integration=None, react=None):
        self.orc = orc
        # react: None or dict(dt=..., chem_substeps=4, visc=True)
        self.react = react
        self.nc = 14 if react else 5
        if time_integration is None:
            time_integration = 2 if react else 3
        self.rk = time_integration  # 3: SSP-RK3, 2: RK2 (Heun), 1: Euler
        self.eb = eb          # None or dict(center=(cx, cy), radius=r, nsub=16, redistribute=False)
        self._geoms = {}
        self.n0 = tuple(n0)
        self.dx0 = tuple(dx0)
        self.lo_bc = tuple(lo_bc)
        self.hi_bc = tuple(hi_bc)
        self.prob_lo = tuple(prob_lo)
        self.bc_case = bc_case
        self.case_params = tuple(case_params) + (0.0,) * (16 - len(case_params))
        self.max_level = max_level
        self.bf = tuple(blocking_factor)
        self.mg = tuple(max_grid_size)
        self.nbuf = n_error_buf
        self.thr = refine_dengrad
        self.periodic = tuple(b == 0 for b in lo_bc)
        self.time = 0.0
        self.levels = [self._new_level(0, boxes0)]
        self.dt_prev = -1.0
        self.stop_time = math.inf
        self.est = None

    # ------------------------------------------------------------ structure
    def n(self, l):
        return tuple(x << l for x in self.n0)

    def dx(self, l):
        return tuple(x / (1 << l) for x in self.dx0)

    def geom(self, l):
        """cut-cell geometry of level l over the whole level (None: no body)"""
        if self.eb is None:
            return None
        if l not in self._geoms:
            from ocfd import geometry
            phi = geometry.cylinder_phi(self.eb["center"][0], self.eb["center"][1], self.eb["radius"])
            self._geoms[l] = geometry.box_geometry(phi, (0, 0, 0), self.n(l), self.dx(l), self.prob_lo,
                                                   nsub=self.eb.get("nsub", 16))
        return self._geoms[l]

    def classes(self, l):
        g = self.geom(l)
        boxes = self.levels[l]["boxes"]
        return [BOX_REGULAR] * len(boxes) if g is None else box_classes(g, boxes)

    def _new_level(self, l, boxes):
        n = self.n(l)
        U = np.full((self.nc, n[2] + 2 * NG, n[1] + 2 * NG, n[0] + 2 * NG), np.nan)
        mask = np.zeros((n[2], n[1], n[0]), bool)
        for lo, hi in boxes:
            mask[_sl(lo, hi)] = True
        return dict(boxes=[(tuple(lo), tuple(hi)) for lo, hi in boxes], U=U, mask=mask, time=self.time,
                    dt=0.0, need=None)

    def set_level_fabs(self, l, fab_of_box):
        L = self.levels[l]
        for lo, hi in L["boxes"]:
            fab = fab_of_box(l, lo, hi, self.dx(l))
            L["U"][(slice(None),) + _sl(lo, hi, NG)] = fab[:, NG:-NG, NG:-NG, NG:-NG]

    def valid(self, l):
        L = self.levels[l]
        return L["U"][:, NG:-NG, NG:-NG, NG:-NG], L["mask"]

    def _bc(self, l):
        bc = BCStruct()
        n = self.n(l)
        bc.lo_bc[:] = list(self.lo_bc)
        bc.hi_bc[:] = list(self.hi_bc)
        bc.dirichlet_case = self.bc_case if self.bc_case in (1, 3) else 0
        if self.bc_case == 3:
            bc.jet[:] = list(self.case_params[:8])
        bc.prob_lo[:] = list(self.prob_lo)
        bc.dx[:] = list(self.dx(l))
        bc.dom_lo[:] = [0, 0, 0]
        bc.dom_hi[:] = [x - 1 for x in n]
        bc.dmr_left[:] = list(self.case_params[:5])
        bc.dmr_right[:] = list(self.case_params[5:10])
        return bc

    def _needed(self, l):
        """in-domain cells that are not valid but lie within NG of a box of level
        l (periodic images wrapped): the coarse-fine ghost cells."""
        L = self.levels[l]
        if L["need"] is not None:
            return L["need"]
        n = self.n(l)
        need = np.zeros_like(L["mask"])
        for lo, hi in L["boxes"]:
            idx = []
            for d in range(3):
                r = np.arange(lo[d] - NG, hi[d] + NG + 1)
                if self.periodic[d]:
                    r = np.mod(r, n[d])
                else:
                    r = r[(r >= 0) & (r < n[d])]
                idx.append(r)
            need[np.ix_(idx[2], idx[1], idx[0])] = True
        need &= ~L["mask"]
        L["need"] = need
        return need

    # ------------------------------------------------------------ ghost cells
    def _cf_interp(self, l, U, a, srcs, cells=None):
        kk, jj, ii = np.nonzero(self._needed(l) if cells is None else cells)
        if kk.size == 0:
            return
        M = None
        for q in range(4):
            if a[q] != 0.0:
                M = a[q] * srcs[q] if M is None else M + a[q] * srcs[q]
        pi, pj, pk = ii >> 1, jj >> 1, kk >> 1
        ox = np.where(ii & 1, 0.25, -0.25)
        oy = np.where(jj & 1, 0.25, -0.25)
        oz = np.where(kk & 1, 0.25, -0.25)

        def at(di, dj, dk):
            return M[:, pk + NG + dk, pj + NG + dj, pi + NG + di]
        v0 = at(0, 0, 0)
        sx = mc_slope(at(-1, 0, 0), v0, at(1, 0, 0))
        sy = mc_slope(at(0, -1, 0), v0, at(0, 1, 0))
        sz = mc_slope(at(0, 0, -1), v0, at(0, 0, 1))
        g = self.geom(l - 1)
        if g is not None:
            # piecewise constant where the parent or a face neighbour is cut or covered
            t = g["flag"][0, NG] & 3          # z-invariant: one plane over the grown level
            nonreg = (t[pj + NG, pi + NG] | t[pj + NG, pi + NG - 1] | t[pj + NG, pi + NG + 1] |
                      t[pj + NG - 1, pi + NG] | t[pj + NG + 1, pi + NG]) != 0
            sx = np.where(nonreg, 0.0, sx)
            sy = np.where(nonreg, 0.0, sy)
            sz = np.where(nonreg, 0.0, sz)
        U[:, kk + NG, jj + NG, ii + NG] = v0 + ox * sx + oy * sy + oz * sz

    def fill(self, l, U, a=(1.0, 0.0, 0.0, 0.0), tfrac=0.0, srcs=None):
        L = self.levels[l]
        if l > 0:
            if srcs is None:
                srcs = (self.levels[l - 1]["U"],) * 4
            self._cf_interp(l, U, a, srcs)
        self.orc.fill_ghosts(self._bc(l), U, L["time"] + tfrac * L["dt"])

    def fill_all_sync(self):
        for l in range(len(self.levels)):
            self.fill(l, self.levels[l]["U"])

    # ------------------------------------------------------------ time stepping
    def _estdt(self, l):
        L = self.levels[l]
        m = math.inf
        for lo, hi in L["boxes"]:
            S = np.ascontiguousarray(L["U"][(slice(None),) + _sl((lo[0] - NG, lo[1] - NG, lo[2] - NG),
                                                                 (hi[0] + NG, hi[1] + NG, hi[2] + NG), NG)])
            m = min(m, self.orc.estdt(S, self.dx(l)))
        return m

    def _rhs_level(self, l, S, with_flux):
        """per-box RHS of the stage input S; returns dS over the level (NaN off
        the valid cells) and the level's face fluxes (assembled over boxes)."""
        L = self.levels[l]
        n = self.n(l)
        dxinv = tuple(1.0 / x for x in self.dx(l))
        nc = self.nc
        dS = np.full((nc, n[2], n[1], n[0]), np.nan)
        F = None
        if with_flux:
            F = [np.zeros((nc, n[2] + (d == 2), n[1] + (d == 1), n[0] + (d == 0))) for d in range(3)]
        g = self.geom(l)
        cls = self.classes(l)
        for b, (lo, hi) in enumerate(L["boxes"]):
            if cls[b] == BOX_COVERED:
                dS[(slice(None),) + _sl(lo, hi)] = 0.0
                continue
            Sb = np.ascontiguousarray(S[(slice(None),) + _sl((lo[0] - NG, lo[1] - NG, lo[2] - NG),
                                                             (hi[0] + NG, hi[1] + NG, hi[2] + NG), NG)])
            if self.react:
                d5, ds, f5, fs, _ = self.orc.rhs_chem(np.ascontiguousarray(Sb[:5]), np.ascontiguousarray(Sb[5:]),
                                                      dxinv, do_visc=self.react.get("visc", True))
                d_ = np.concatenate([d5, ds])
                f = [np.concatenate([f5[d], fs[d]]) for d in range(3)]
            elif cls[b] == BOX_REGULAR:
                d_, f = self.orc.rhs_regular(Sb, dxinv)
            else:
                gsl = (slice(None), slice(lo[2], hi[2] + 2 * NG + 1), slice(lo[1], hi[1] + 2 * NG + 1),
                       slice(lo[0], hi[0] + 2 * NG + 1))
                gb = dict(flag=np.ascontiguousarray(g["flag"][gsl]), vfrac=np.ascontiguousarray(g["vfrac"][gsl]))
                ap = []
                for d, key in enumerate(("apx", "apy", "apz")):
                    h = list(hi)
                    h[d] += 1
                    gb[key] = np.ascontiguousarray(g[key][(slice(None),) + _sl(lo, h)])
                    ap.append(gb[key])
                d_, f = self.orc.rhs_eb(Sb, gb, dxinv, do_redistribute=self.eb.get("redistribute", False))
                f = [ap[d] * f[d] for d in range(3)]
            dS[(slice(None),) + _sl(lo, hi)] = d_
            if with_flux:
                for d in range(3):
                    h = list(hi)
                    h[d] += 1
                    F[d][(slice(None),) + _sl(lo, h)] = f[d]
        return dS, F

    def step(self, cfl):
        """One coarse step; returns dt_0."""
        if self.react:
            dt = self.react["dt"]
        else:
            if self.est is None:
                self.est = [self._estdt(l) for l in range(len(self.levels))]
            est = min(e * (1 << l) for l, e in enumerate(self.est))
            dt = cfl * est
            if self.dt_prev > 0 and dt > 1.1 * self.dt_prev:
                dt = 1.1 * self.dt_prev
            if self.time + dt > self.stop_time - 0.001 * dt:
                dt = self.stop_time - self.time
            dt = max(dt, 0.0)
        for l, L in enumerate(self.levels):
            L["dt"] = dt / (1 << l)
            L["time"] = self.time
        self._advance(0, 1)
        self.time += dt
        self.dt_prev = dt
        for L in self.levels:
            L["time"] = self.time
        if not self.react:
            self.est = [self._estdt(l) for l in range(len(self.levels))]
        return dt

    def _boxes_cells(self, l, U, fn):
        """fn(S (5, n), spec (9, n)) on the valid cells of every box of level l, in place"""
        for lo, hi in self.levels[l]["boxes"]:
            gs = (slice(None),) + _sl(lo, hi, NG)
            blk = U[gs]
            a = np.ascontiguousarray(blk[:5].reshape(5, -1))
            b = np.ascontiguousarray(blk[5:].reshape(9, -1))
            fn(a, b)
            U[gs] = np.concatenate([a, b]).reshape(blk.shape)

    def _chem(self, l, U):
        """chemistry over half of level l's step (Source/Advance.cpp:158-173)"""
        it = max(1, self.react.get("chem_substeps", 4) >> l) if l <= 2 else 1
        dt2 = 0.5 * self.levels[l]["dt"] / it

        def go(a, b):
            for _ in range(it):
                self.orc.chem_advance(a, b, dt2)
        self._boxes_cells(l, U, go)

    def _renorm(self, l, U):
        """species clip and rescale, EBR::post_timestep (Source/EBR.cpp:333-357)"""
        self._boxes_cells(l, U, self.orc.spec_renorm)

    def _advance(self, l, it):
        L = self.levels[l]
        has_child = l < len(self.levels) - 1
        theta = 0.5 * (it - 1)
        A = L["U"]
        bufs = [A, A.copy(), A.copy(), A.copy() if has_child else None]
        L["bufs"] = bufs
        parent = self.levels[l - 1]["bufs"] if l > 0 else None
        if has_child:
            L["creg"] = [0.0, 0.0, 0.0]
            self.levels[l + 1]["freg"] = [0.0, 0.0, 0.0]
        sch = SCHEMES[self.rk]
        nst = sch["nst"]
        last = 3 if has_child else 0
        out_of = (1, 2, last) if self.rk == 3 else ((1, last) if self.rk == 2 else (last,))
        if self.react:
            self._chem(l, A)
        for k in range(nst):
            S = bufs[sch["src"][k]]
            self.fill(l, S, self._cf_coefs(k, theta), sch["tfrac"][k], parent)
            dS, F = self._rhs_level(l, S, has_child or l > 0)
            dt = L["dt"]
            O = bufs[out_of[k]]
            # box by box over the valid cells (the boxes of a level are disjoint;
            # the same elementwise arithmetic as over the level's valid mask)
            for lo, hi in L["boxes"]:
                gs = (slice(None),) + _sl(lo, hi, NG)
                vs = (slice(None),) + _sl(lo, hi)
                u0, us = A[gs], S[gs]
                if self.rk == 3:
                    O[gs] = RK_A[k] * u0 + RK_B[k] * (us + dt * dS[vs])
                elif k == 0:
                    O[gs] = 1.0 * us + dt * dS[vs]
                else:
                    O[gs] = (0.5 * us + 0.5 * u0) + (0.5 * dt) * dS[vs]
            w = sch["w"][k] * dt
            if has_child:
                L["creg"] = [L["creg"][d] + w * F[d] for d in range(3)]
            if l > 0:
                L["freg"] = [L["freg"][d] + w * F[d] for d in range(3)]
        if self.react:
            self._chem(l, bufs[last])
            if not has_child:
                self._renorm(l, bufs[last])
        if has_child:
            D = bufs[3]
            self.fill(l, D, self._cf_coefs(3, theta), 1.0, parent)
            for i in (1, 2):
                self._advance(l + 1, i)
            self._reflux(l, D)
            if self.react:
                self._renorm(l, D)
            self._avg_down(l, D)
            L["U"] = D.copy()
        if l > 0:
            L["time"] += L["dt"]

    def _cf_coefs(self, k, theta, r=0.5):
        """Weights of the coarse (A, B, C, D) for fine stage k of the substep at
        theta (k = 3: the coarse end state at theta + r): the RK3 dense output, or
        for RK2 / Euler FillPatch's linear interpolation between the coarse old
        (A) and new (D) states at the stage's time."""
        if self.rk == 3:
            return mix_coefs(k, theta, r)
        th = theta + r if k == 3 else theta + r * SCHEMES[self.rk]["tfrac"][k]
        return (1.0 - th, 0.0, 0.0, th)

    def _covered(self, c):
        m = self.levels[c + 1]["mask"]
        nz, ny, nx = m.shape
        return m.reshape(nz // 2, 2, ny // 2, 2, nx // 2, 2).any(axis=(1, 3, 5))

    def _avg_down(self, c, D):
        F = self.levels[c + 1]["U"][:, NG:-NG, NG:-NG, NG:-NG]
        g = self.geom(c + 1)
        s = 0.0
        if g is None:
            for kk in range(2):
                for jj in range(2):
                    for ii in range(2):
                        s = s + F[:, kk::2, jj::2, ii::2]
            avg = 0.125 * s
        else:
            # volume-fraction weights; all children covered: the first child
            vf = g["vfrac"][:, NG:-NG, NG:-NG, NG:-NG]
            wt = 0.0
            for kk in range(2):
                for jj in range(2):
                    for ii in range(2):
                        w = vf[:, kk::2, jj::2, ii::2]
                        s = s + w * F[:, kk::2, jj::2, ii::2]
                        wt = wt + w
            with np.errstate(all="ignore"):
                avg = np.where(wt > 0.0, s / wt, F[:, 0::2, 0::2, 0::2])
        cov = self._covered(c)
        D[:, NG:-NG, NG:-NG, NG:-NG][:, cov] = avg[:, cov]

    def _reflux(self, c, D):
        C = self.levels[c]
        Fl = self.levels[c + 1]
        cov = self._covered(c)
        dxinv = [1.0 / x for x in self.dx(c)]
        V = D[:, NG:-NG, NG:-NG, NG:-NG]
        for d in range(3):
            ax = 2 - d                       # numpy axis of direction d in (z, y, x)
            n = cov.shape[ax]
            creg = C["creg"][d]
            fe = np.take(Fl["freg"][d], np.arange(0, 2 * n + 1, 2), axis=1 + ax)
            t = [a for a in (0, 1, 2) if a != ax]
            s = 0.0
            for b2 in range(2):
                for b1 in range(2):
                    sl = [slice(None)] * 4
                    sl[1 + t[1]] = slice(b1, None, 2)
                    sl[1 + t[0]] = slice(b2, None, 2)
                    s = s + fe[tuple(sl)]
            favg = 0.25 * s                  # fine side on the coarse faces
            # faces 1..n-1: cell a = face - 1 on the low side, a + 1 on the high side
            cl = np.take(cov, np.arange(0, n - 1), axis=ax)
            cr = np.take(cov, np.arange(1, n), axis=ax)
            for low_uncovered in (True, False):
                m = (~cl & cr) if low_uncovered else (cl & ~cr)
                pos = list(np.nonzero(m))
                face = list(pos)
                face[ax] = pos[ax] + 1
                cell = list(pos)
                if not low_uncovered:
                    cell[ax] = pos[ax] + 1
                fidx = (slice(None),) + tuple(face)
                val = dxinv[d] * (creg[fidx] - favg[fidx])
                self._add_reflux(c, V, tuple(cell), val if low_uncovered else -val)
            if self.periodic[d]:
                c0 = np.take(cov, 0, axis=ax)
                cn = np.take(cov, n - 1, axis=ax)
                for low_uncovered in (True, False):
                    m = (~cn & c0) if low_uncovered else (cn & ~c0)
                    pos = list(np.nonzero(m))
                    if low_uncovered:   # cell n-1, its face n; fine face 0
                        cidx, fc, ff = n - 1, n, 0
                    else:               # cell 0, its face 0; fine face 2n
                        cidx, fc, ff = 0, 0, n
                    def full(v):
                        q = list(pos)
                        q.insert(ax, np.full(len(pos[0]), v, dtype=np.intp))
                        return (slice(None),) + tuple(q)
                    val = dxinv[d] * (creg[full(fc)] - favg[full(ff)])
                    self._add_reflux(c, V, full(cidx)[1:], val if low_uncovered else -val)

    def _add_reflux(self, c, V, cell, val):
        """V[cell] += val, divided by the volume fraction of cut cells, none for
        covered cells"""
        g = self.geom(c)
        if g is None:
            V[(slice(None),) + cell] += val
            return
        vf = g["vfrac"][0, NG:-NG, NG:-NG, NG:-NG][cell]
        cut = self._cut_mask(c)[cell]
        keep = vf > 0.0
        with np.errstate(all="ignore"):
            val = np.where(cut[None], val / vf[None], val)
        sel = tuple(a[keep] for a in cell)
        V[(slice(None),) + sel] += val[:, keep]

    def _cut_mask(self, c):
        """cells of level c in cut boxes"""
        n = self.n(c)
        m = np.zeros((n[2], n[1], n[0]), bool)
        for cl, (lo, hi) in zip(self.classes(c), self.levels[c]["boxes"]):
            if cl == BOX_CUT:
                m[_sl(lo, hi)] = True
        return m

    def average_down_all(self):
        for c in range(len(self.levels) - 2, -1, -1):
            self._avg_down(c, self.levels[c]["U"])

    # ------------------------------------------------------------ regridding
    def _blocks(self, f):
        n = self.n(f)
        bf = [min(self.bf[d], n[d]) for d in range(3)]
        nb = [n[d] // bf[d] for d in range(3)]
        return bf, nb, np.zeros((nb[2], nb[1], nb[0]), bool)

    def _tag_blocks(self, l):
        """blocks of level l+1 holding a tagged cell of level l (+- n_error_buf)"""
        L = self.levels[l]
        U = L["U"]
        r = U[0]
        c = r[NG:-NG, NG:-NG, NG:-NG]
        ax = np.maximum(np.abs(r[NG:-NG, NG:-NG, NG + 1:r.shape[2] - NG + 1] - c),
                        np.abs(c - r[NG:-NG, NG:-NG, NG - 1:r.shape[2] - NG - 1]))
        ay = np.maximum(np.abs(r[NG:-NG, NG + 1:r.shape[1] - NG + 1, NG:-NG] - c),
                        np.abs(c - r[NG:-NG, NG - 1:r.shape[1] - NG - 1, NG:-NG]))
        az = np.maximum(np.abs(r[NG + 1:r.shape[0] - NG + 1, NG:-NG, NG:-NG] - c),
                        np.abs(c - r[NG - 1:r.shape[0] - NG - 1, NG:-NG, NG:-NG]))
        tag = (np.maximum(ax, np.maximum(ay, az)) >= self.thr) & L["mask"]
        bf, nb, blk = self._blocks(l + 1)
        bs = [b // 2 for b in bf]
        n = self.n(l)
        for k, j, i in zip(*np.nonzero(tag)):
            lo = [(max(v - self.nbuf, 0)) // bs[d] for d, v in enumerate((i, j, k))]
            hi = [(min(v + self.nbuf, n[d] - 1)) // bs[d] for d, v in enumerate((i, j, k))]
            blk[lo[2]:hi[2] + 1, lo[1]:hi[1] + 1, lo[0]:hi[0] + 1] = True
        return blk

    def _wrap_pieces(self, l, lo, hi):
        """pieces of the cell region lo..hi of level l inside the domain (periodic
        images wrapped, non-periodic parts dropped)"""
        n = self.n(l)
        pieces = [((), ())]
        for d in range(3):
            new = []
            for plo, phi in pieces:
                if self.periodic[d]:
                    for s in (-n[d], 0, n[d]):
                        a, b = max(lo[d] + s, 0), min(hi[d] + s, n[d] - 1)
                        if a <= b:
                            new.append((plo + (a,), phi + (b,)))
                else:
                    a, b = max(lo[d], 0), min(hi[d], n[d] - 1)
                    if a <= b:
                        new.append((plo + (a,), phi + (b,)))
            pieces = new
        return pieces

    def _cover_mask(self, l, boxes):
        m = np.zeros((self.n(l)[2], self.n(l)[1], self.n(l)[0]), bool)
        for lo, hi in boxes:
            m[_sl(lo, hi)] = True
        return m

    def _cluster(self, f, blk):
        bf, nb, _ = self._blocks(f)
        mg = [max(1, self.mg[d] // bf[d]) for d in range(3)]
        used = np.zeros_like(blk)
        out = []

        def ok(i, j, k):
            return blk[k, j, i] and not used[k, j, i]
        for k in range(nb[2]):
            for j in range(nb[1]):
                for i in range(nb[0]):
                    if not ok(i, j, k):
                        continue
                    ex = ey = ez = 1
                    while i + ex < nb[0] and ex < mg[0] and ok(i + ex, j, k):
                        ex += 1
                    while j + ey < nb[1] and ey < mg[1] and all(ok(i + a, j + ey, k) for a in range(ex)):
                        ey += 1
                    while k + ez < nb[2] and ez < mg[2] and all(ok(i + a, j + b, k + ez)
                                                                for b in range(ey) for a in range(ex)):
                        ez += 1
                    used[k:k + ez, j:j + ey, i:i + ex] = True
                    out.append(((i * bf[0], j * bf[1], k * bf[2]),
                                ((i + ex) * bf[0] - 1, (j + ey) * bf[1] - 1, (k + ez) * bf[2] - 1)))
        return out

    def regrid(self, lbase):
        if lbase >= self.max_level:
            return
        self.fill_all_sync()
        top = min(len(self.levels) - 1, self.max_level - 1)
        T = {}
        for l in range(lbase, top + 1):
            T[l + 1] = self._tag_blocks(l)
        for f in range(top + 1, lbase + 1, -1):
            bf, nb, _ = self._blocks(f)
            cbf, cnb, _ = self._blocks(f - 1)
            for k, j, i in zip(*np.nonzero(T[f])):
                lo = [(v * bf[d]) // 2 - NEST for d, v in enumerate((i, j, k))]
                hi = [((v + 1) * bf[d] - 1) // 2 + NEST for d, v in enumerate((i, j, k))]
                for plo, phi in self._wrap_pieces(f - 1, lo, hi):
                    T[f - 1][plo[2] // cbf[2]:phi[2] // cbf[2] + 1, plo[1] // cbf[1]:phi[1] // cbf[1] + 1,
                             plo[0] // cbf[0]:phi[0] // cbf[0] + 1] = True
        grids = []
        below = self._cover_mask(lbase, self.levels[lbase]["boxes"])
        for f in range(lbase + 1, top + 2):
            bf, nb, _ = self._blocks(f)
            blk = T[f]
            for k, j, i in zip(*np.nonzero(blk)):
                lo = [(v * bf[d]) // 2 - NEST for d, v in enumerate((i, j, k))]
                hi = [((v + 1) * bf[d] - 1) // 2 + NEST for d, v in enumerate((i, j, k))]
                if not all(below[_sl(plo, phi)].all() for plo, phi in self._wrap_pieces(f - 1, lo, hi)):
                    blk[k, j, i] = False
            boxes = self._cluster(f, blk)
            grids.append(boxes)
            if not boxes:
                break
            below = self._cover_mask(f, boxes)
        self.apply_grids(lbase, grids)

    def apply_grids(self, lbase, grids):
        newfinest = lbase
        for q, g in enumerate(grids):
            if not g:
                break
            newfinest = lbase + 1 + q
        for f in range(lbase + 1, newfinest + 1):
            nb = [(tuple(lo), tuple(hi)) for lo, hi in grids[f - lbase - 1]]
            if f < len(self.levels) and self.levels[f]["boxes"] == nb:
                continue
            old = self.levels[f] if f < len(self.levels) else None
            new = self._new_level(f, nb)
            new["time"] = self.time
            if old is None:
                self.levels.append(new)
            else:
                self.levels[f] = new
            self._cf_interp(f, new["U"], (1.0, 0.0, 0.0, 0.0), (self.levels[f - 1]["U"],) * 4, cells=new["mask"])
            if old is not None:
                keep = new["mask"] & old["mask"]
                V = new["U"][:, NG:-NG, NG:-NG, NG:-NG]
                V[:, keep] = old["U"][:, NG:-NG, NG:-NG, NG:-NG][:, keep]
            self.fill(f, new["U"])
        del self.levels[newfinest + 1:]
        # the next step's dt comes from the estimates made at the end of the
        # previous step: a rebuilt level keeps its level's estimate, a new one has none
        if self.est is not None:
            self.est = (self.est + [math.inf] * len(self.levels))[:len(self.levels)]

    def grids(self):
        return [list(L["boxes"]) for L in self.levels]
