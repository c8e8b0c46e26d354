"""Embedded-boundary geometry for a box: cell flags, volume and area fractions.

The reference takes these from AMReX EB2 (Source/Geometry.cpp:9-29), which is not
available; this module builds the same per-box data from an implicit function by
sub-sampling, for a body extruded along z (the cylinder of the multi-level EB
configuration).  Fluid is where phi > 0.

Flag word layout (EBCellFlag as the kernels read it): bits 0-1 cell type
(0 regular, 1 single-valued cut, 3 covered), bits 4..30 connectivity to the 27
neighbours, bit 4 + (i+1) + 3(j+1) + 9(k+1) for offset (i,j,k).

Connectivity rule used here: a non-covered cell is connected to itself, to a
face neighbour when the shared face is open (area fraction > 0) and the
neighbour is not covered, and to an edge/corner neighbour when neither is
covered.  Regular cells carry all 27 bits.
"""
from __future__ import annotations

import numpy as np

NG = 4
T_REGULAR, T_CUT, T_COVERED = 0, 1, 3


def _bit(i, j, k):
    return 4 + (i + 1) + 3 * (j + 1) + 9 * (k + 1)


ALL_NEIGHBOURS = sum(1 << _bit(i, j, k) for i in (-1, 0, 1) for j in (-1, 0, 1) for k in (-1, 0, 1))


def cylinder_phi(cx, cy, r):
    """Implicit function of a z-aligned cylinder: > 0 outside (fluid)."""
    return lambda x, y: (x - cx) ** 2 + (y - cy) ** 2 - r * r


def box_geometry(phi_xy, lo, n, dx, prob_lo=(0.0, 0.0, 0.0), nsub=16, ng=NG):
    """EB data of the box with interior cells lo .. lo+n-1 (absolute indices).

    Returns dict with
      flag  (1, nz+2ng, ny+2ng, nx+2ng) uint32   over the grown box
      vfrac (1, ...) float64                     over the grown box
      apx (1, nz, ny, nx+1), apy (1, nz, ny+1, nx), apz (1, nz+1, ny, nx)
      faces of the interior box.
    """
    nx, ny, nz = n
    gx, gy = nx + 2 * ng, ny + 2 * ng
    # cell-centred sub-sample fractions in the xy plane over the grown box
    s = (np.arange(nsub) + 0.5) / nsub
    i0, j0 = lo[0] - ng, lo[1] - ng
    xs = prob_lo[0] + (i0 + np.arange(gx)[:, None] + s[None, :]) * dx[0]      # (gx, nsub)
    ys = prob_lo[1] + (j0 + np.arange(gy)[:, None] + s[None, :]) * dx[1]      # (gy, nsub)
    inside = phi_xy(xs[None, :, None, :], ys[:, None, :, None]) > 0            # (gy,gx,nsub,nsub)
    vf2 = inside.mean(axis=(2, 3))                                             # (gy, gx)
    # x faces at x = (i)*dx for i in grown range + 1, sub-sampled along y
    xf = prob_lo[0] + (i0 + np.arange(gx + 1)) * dx[0]
    ax2 = (phi_xy(xf[None, :, None], ys[:, None, :]) > 0).mean(axis=2)        # (gy, gx+1)
    yf = prob_lo[1] + (j0 + np.arange(gy + 1)) * dx[1]
    ay2 = (phi_xy(xs[None, :, :], yf[:, None, None]) > 0).mean(axis=2)        # (gy+1, gx)
    gz = nz + 2 * ng
    vfrac = np.broadcast_to(vf2, (gz, gy, gx)).copy()
    apx_g = np.broadcast_to(ax2, (gz, gy, gx + 1))
    apy_g = np.broadcast_to(ay2, (gz, gy + 1, gx))
    # z faces of an extruded body have the open fraction of the column
    apz_g = np.broadcast_to(vf2, (gz + 1, gy, gx))

    covered = vfrac <= 0.0
    full = vfrac >= 1.0
    open_faces = (apx_g[:, :, :-1] >= 1) & (apx_g[:, :, 1:] >= 1) & (apy_g[:, :-1, :] >= 1) & \
                 (apy_g[:, 1:, :] >= 1) & (apz_g[:-1] >= 1) & (apz_g[1:] >= 1)
    regular = full & open_faces
    flag = np.zeros((gz, gy, gx), dtype=np.uint32)
    flag[regular] = np.uint32(T_REGULAR) | np.uint32(ALL_NEIGHBOURS)
    flag[covered] = np.uint32(T_COVERED)
    cut = ~regular & ~covered
    # connectivity of cut cells
    cov_pad = np.pad(covered, 1, constant_values=True)
    conn = np.zeros((gz, gy, gx), dtype=np.uint64)
    for dk in (-1, 0, 1):
        for dj in (-1, 0, 1):
            for di in (-1, 0, 1):
                nb_cov = cov_pad[1 + dk:1 + dk + gz, 1 + dj:1 + dj + gy, 1 + di:1 + di + gx]
                ok = ~nb_cov
                nface = abs(di) + abs(dj) + abs(dk)
                if nface == 1:
                    if di:
                        a = apx_g[:, :, 1:] if di > 0 else apx_g[:, :, :-1]
                    elif dj:
                        a = apy_g[:, 1:, :] if dj > 0 else apy_g[:, :-1, :]
                    else:
                        a = apz_g[1:] if dk > 0 else apz_g[:-1]
                    ok = ok & (a > 0)
                conn |= np.where(ok, np.uint64(1) << np.uint64(_bit(di, dj, dk)), np.uint64(0))
    flag[cut] = (np.uint32(T_CUT) | conn[cut].astype(np.uint32))
    sl = slice(ng, -ng)
    apx = np.ascontiguousarray(apx_g[ng:ng + nz, ng:ng + ny, ng:ng + nx + 1])
    apy = np.ascontiguousarray(apy_g[ng:ng + nz, ng:ng + ny + 1, ng:ng + nx])
    apz = np.ascontiguousarray(apz_g[ng:ng + nz + 1, ng:ng + ny, ng:ng + nx])
    del sl
    return dict(flag=flag[None].copy(), vfrac=vfrac[None].copy(), apx=apx[None].copy(),
                apy=apy[None].copy(), apz=apz[None].copy())


def box_is_regular(phi_xy, lo, n, dx, prob_lo=(0.0, 0.0, 0.0), ng=NG):
    """True when no cell of the box grown by ng is cut or covered
    (the test of Source/Advance.cpp:231)."""
    g = box_geometry(phi_xy, lo, n, dx, prob_lo, nsub=4, ng=ng)
    return bool(np.all((g["flag"] & 3) == T_REGULAR))
