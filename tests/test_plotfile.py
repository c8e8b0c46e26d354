"""Plotfile writer / reader / comparison (host code of libocfd, no GPU):
the files follow the AMReX HyperCLaw-V1.1 layout (checked by an independent
parser written here), and the comparison reproduces fcompare's norms
(Util/Plotfile/fcompare.cpp:150-290) computed with numpy."""
import os

import numpy as np
import pytest

NAMES = ["rho", "xmom", "ymom", "zmom", "Eden"]


def two_levels(rng, n0=(16, 8, 4)):
    dx0 = (1.0 / 16, 1.0 / 16, 1.0 / 16)
    lev0 = dict(boxes=[((0, 0, 0), (7, 7, 3)), ((8, 0, 0), (15, 7, 3))], dx=dx0, step=3)
    lev0["fabs"] = [rng.random((5, 4, 8, 8)) + 1.0 for _ in lev0["boxes"]]
    lev1 = dict(boxes=[((8, 4, 0), (15, 11, 7)), ((16, 4, 0), (19, 11, 7))], dx=tuple(x / 2 for x in dx0), step=6)
    lev1["fabs"] = [rng.random((5, 8, 8, 8)) + 1.0, rng.random((5, 8, 8, 4)) + 1.0]
    return [lev0, lev1], tuple(n - 1 for n in n0)


def parse(path):
    """Independent reader of the layout: header fields and FAB data."""
    with open(os.path.join(path, "Header")) as f:
        lines = f.read().split("\n")
    assert lines[0] == "HyperCLaw-V1.1"
    nc = int(lines[1])
    names = lines[2:2 + nc]
    i = 2 + nc
    dim, time, finest = int(lines[i]), float(lines[i + 1]), int(lines[i + 2])
    i += 3
    plo = [float(x) for x in lines[i].split()]
    phi = [float(x) for x in lines[i + 1].split()]
    ratios = lines[i + 2].split()
    domains = lines[i + 3]
    steps = [int(x) for x in lines[i + 4].split()]
    i += 5
    dxs = [[float(x) for x in lines[i + l].split()] for l in range(finest + 1)]
    i += finest + 1
    assert lines[i] == "0" and lines[i + 1] == "0"
    i += 2
    data = []
    for l in range(finest + 1):
        lev, ngrid, t = lines[i].split()
        assert int(lev) == l
        ngrid = int(ngrid)
        i += 2 + 3 * ngrid
        rel = lines[i]
        i += 1
        cell_h = open(os.path.join(path, rel + "_H")).read().split("\n")
        assert cell_h[0] == "1" and int(cell_h[2]) == nc and cell_h[4].startswith("(%d 0" % ngrid)
        fabs = []
        for b in range(ngrid):
            tag, fname, off = cell_h[7 + ngrid + b].split()
            assert tag == "FabOnDisk:"
            with open(os.path.join(path, "Level_%d" % l, fname), "rb") as f:
                f.seek(int(off))
                hdr = f.readline().decode()
                assert hdr.startswith("FAB ((8, (64 11 52 0 1 12 0 1023)),(8, (1 2 3 4 5 6 7 8)))((")
                box = hdr[hdr.index(")((") + 1:].rsplit(" ", 1)[0]
                lo = [int(x) for x in box[2:box.index(")")].split(",")]
                hi = [int(x) for x in box[box.index(") (") + 3:box.index(") (0")].split(",")]
                n = [hi[d] - lo[d] + 1 for d in range(3)]
                arr = np.frombuffer(f.read(8 * nc * n[0] * n[1] * n[2]), dtype="<f8").reshape(nc, n[2], n[1], n[0])
                fabs.append((tuple(lo), tuple(hi), arr))
        data.append(fabs)
    return dict(names=names, dim=dim, time=time, finest=finest, plo=plo, phi=phi, ratios=ratios, domains=domains,
                steps=steps, dx=dxs, data=data)


def test_layout_round_trip(tmp_path):
    from ocfd import plotfile
    rng = np.random.default_rng(5)
    levels, dhi = two_levels(rng)
    p = str(tmp_path / "plt00003")
    plotfile.write(p, levels, NAMES, dhi, (0.0, 0.0, 0.0), (1.0, 0.5, 0.25), time=0.125)
    d = parse(p)
    assert d["names"] == NAMES and d["dim"] == 3 and d["finest"] == 1 and d["time"] == 0.125
    assert d["ratios"] == ["2"] and d["steps"] == [3, 6]
    assert d["domains"] == "((0,0,0) (15,7,3) (0,0,0)) ((0,0,0) (31,15,7) (0,0,0))"
    assert d["dx"][1] == [1.0 / 32] * 3
    for l, lev in enumerate(levels):
        for (lo, hi, arr), blo_bhi, f in zip(d["data"][l], lev["boxes"], lev["fabs"]):
            assert (lo, hi) == blo_bhi
            assert np.array_equal(arr, f)
    assert plotfile.info(p) == (2, 5)


def test_fcompare_norms(tmp_path):
    from ocfd import plotfile
    rng = np.random.default_rng(6)
    levels, dhi = two_levels(rng)
    a = str(tmp_path / "a")
    b = str(tmp_path / "b")
    plotfile.write(a, levels, NAMES, dhi, (0, 0, 0), (1.0, 0.5, 0.25))
    pert = [dict(l, fabs=[f + 1e-3 * rng.standard_normal(f.shape) for f in l["fabs"]]) for l in levels]
    plotfile.write(b, pert, NAMES, dhi, (0, 0, 0), (1.0, 0.5, 0.25))
    same = plotfile.compare(a, a, norm=1)
    assert (same["abs"] == 0).all() and (same["rel"] == 0).all()
    for norm in (0, 1, 2):
        r = plotfile.compare(a, b, norm=norm)
        for l in range(2):
            A = np.concatenate([f.reshape(5, -1) for f in levels[l]["fabs"]], axis=1)
            B = np.concatenate([f.reshape(5, -1) for f in pert[l]["fabs"]], axis=1)
            dv = np.prod(levels[l]["dx"])
            for n in range(5):
                d = np.abs(B[n] - A[n])
                if norm == 0:
                    ab, rel = d.max(), d.max() / np.abs(A[n]).max()
                elif norm == 1:
                    ab, rel = d.sum() * dv, d.sum() / np.abs(A[n]).sum()
                else:
                    ab, rel = np.sqrt((d * d).sum()) * np.sqrt(dv), np.sqrt((d * d).sum() / (A[n] ** 2).sum())
                assert r["abs"][l, n] == pytest.approx(ab, rel=1e-12)
                assert r["rel"][l, n] == pytest.approx(rel, rel=1e-12)


def test_fcompare_grids_and_nans(tmp_path):
    from ocfd import plotfile
    from ocfd.fcompare import main
    rng = np.random.default_rng(7)
    levels, dhi = two_levels(rng)
    a = str(tmp_path / "a")
    plotfile.write(a, levels, NAMES, dhi, (0, 0, 0), (1, 0.5, 0.25))
    # the same level-0 data split into four boxes
    f0 = np.concatenate(levels[0]["fabs"], axis=3)
    split = dict(levels[0], boxes=[((0, 0, 0), (3, 7, 3)), ((4, 0, 0), (15, 3, 3)), ((4, 4, 0), (15, 7, 3))],
                 fabs=[f0[..., 0:4], f0[:, :, 0:4, 4:16], f0[:, :, 4:8, 4:16]])
    b = str(tmp_path / "b")
    plotfile.write(b, [split, levels[1]], NAMES, dhi, (0, 0, 0), (1, 0.5, 0.25))
    with pytest.raises(Exception):
        plotfile.compare(a, b)
    r = plotfile.compare(a, b, norm=1, allow_diff_grids=True)
    assert (r["abs"] == 0).all()
    assert main([a, b, "-a"]) == 0
    # a NaN is reported and fails the comparison
    bad = [dict(l, fabs=[f.copy() for f in l["fabs"]]) for l in levels]
    bad[1]["fabs"][0][2, 1, 1, 1] = np.nan
    c = str(tmp_path / "c")
    plotfile.write(c, bad, NAMES, dhi, (0, 0, 0), (1, 0.5, 0.25))
    r = plotfile.compare(a, c)
    assert r["nan"][1, 2] == 2 and r["nan"][0].sum() == 0
    assert main([a, c]) == 1
    assert main([a, a]) == 0
