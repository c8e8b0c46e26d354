"""Argument checks of every per-box entry point and of level creation, through the
C ABI: a call that fails its checks returns OCFD_BAD_ARG, launches nothing (its
outputs keep their sentinel values) and leaves the context usable.  The
reference aborts on the host for the same mistakes (amrex::Abort /
amrex::Error, Source/EBR.cpp:178); its device code has no status."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
BAD_ARG = 1


@pytest.fixture(scope="module")
def ctx():
    import ocfd
    return ocfd.Context()


def f64(*shape, fill=np.nan):
    import torch
    return torch.full(shape, fill, dtype=torch.float64, device="cuda")


def bad(fn, *a, **k):
    import ocfd
    with pytest.raises(ocfd.OcfdError) as e:
        fn(*a, **k)
    assert e.value.status == BAD_ARG, str(e.value)


def untouched(t):
    import torch
    torch.cuda.synchronize()
    return bool(torch.isnan(t).all())


def test_regular_box_checks(ctx):
    S = f64(5, 16, 16, 16, fill=1.0)
    dS = f64(5, 8, 8, 8)
    one = [1.0, 1.0, 1.0]
    bad(ctx.rhs_regular_box, S, dS, (0, 0, 0), (-1, 7, 7), one, S_begin=(-4, -4, -4))  # empty
    bad(ctx.rhs_regular_box, S, dS, (0, 0, 0), (8, 7, 7), one, S_begin=(-4, -4, -4))   # dSdt short in x
    bad(ctx.rhs_regular_box, S, dS, (0, 0, 0), (7, 7, 7), one, flags=1 << 20,
        S_begin=(-4, -4, -4))                                                         # unknown flag
    fl = [f64(5, 8 + (d == 2), 8 + (d == 1), 8 + (d == 0) - (d == 0)) for d in range(3)]
    bad(ctx.rhs_regular_box, S, dS, (0, 0, 0), (7, 7, 7), one, flux=fl,
        S_begin=(-4, -4, -4))                                                         # x faces short
    assert untouched(dS) and all(untouched(f) for f in fl)
    ctx.check()


def test_chem_box_checks(ctx):
    S = f64(5, 4, 4, 4, fill=1.0)
    R = f64(9, 4, 4, 4, fill=0.1)
    bad(ctx.chem_advance_box, S, R, (0, 0, 0), (3, 3, 3), -1e-8)              # negative dt
    bad(ctx.chem_advance_box, S, R, (0, 0, 0), (3, 3, -1), 1e-8)              # empty
    bad(ctx.chem_advance_box, S, R[:8], (0, 0, 0), (3, 3, 3), 1e-8)           # 8 species
    bad(ctx.spec_renorm_box, S, R, (0, 0, 0), (4, 3, 3))                      # box past the arrays
    import torch
    torch.cuda.synchronize()
    assert bool((S == 1.0).all()) and bool((R == 0.1).all())
    ctx.check()


def test_chem_rhs_checks(ctx):
    S = f64(5, 14, 14, 14, fill=1.0)      # from lo-4: 2 ghosts on the high side, 3 required
    R = f64(9, 14, 14, 14, fill=0.1)
    dS, dR = f64(5, 8, 8, 8), f64(9, 8, 8, 8)
    bad(ctx.rhs_chem_box, S, R, dS, dR, (0, 0, 0), (7, 7, 7), [1.0, 1.0, 1.0])
    assert untouched(dS) and untouched(dR)
    ctx.check()


def _level(ctx, boxes, domain_hi=(15, 15, 3), lo_bc=(2, 2, 0), hi_bc=(2, 2, 0)):
    from ocfd.level import Level
    return Level(ctx, boxes, domain_hi, lo_bc, hi_bc, (1.0, 1.0, 1.0))


def test_level_checks(ctx):
    good = [((0, 0, 0), (7, 15, 3)), ((8, 0, 0), (15, 15, 3))]
    L = _level(ctx, good)
    assert L.cells() == 16 * 16 * 4
    L.close()
    bad(_level, ctx, [((0, 0, 0), (8, 15, 3)), ((8, 0, 0), (15, 15, 3))])    # overlap in one column
    bad(_level, ctx, [((0, 0, 0), (15, 15, 3)), ((4, 4, 1), (5, 5, 2))])     # nested
    bad(_level, ctx, [((0, 0, 0), (16, 15, 3))])                              # past the domain
    bad(_level, ctx, [((0, 0, 0), (15, 15, 3))], lo_bc=(2, 2, 0), hi_bc=(2, 2, 2))  # half periodic
    bad(_level, ctx, [])                                                      # no boxes
    ctx.check()


def test_level_many_boxes_disjoint(ctx):
    """A level of 8³ boxes tiling 64×64×32 is accepted; moving one box by a cell
    onto its neighbour is not."""
    boxes = [((i, j, k), (i + 7, j + 7, k + 7))
             for k in range(0, 32, 8) for j in range(0, 64, 8) for i in range(0, 64, 8)]
    L = _level(ctx, boxes, domain_hi=(63, 63, 31))
    assert L.cells() == 64 * 64 * 32
    L.close()
    moved = list(boxes)
    (lo, hi) = moved[77]
    moved[77] = ((lo[0] - 1, lo[1], lo[2]), (hi[0] - 1, hi[1], hi[2]))
    bad(_level, ctx, moved, domain_hi=(63, 63, 31))
    ctx.check()
