"""Tile shapes of the stencil pass: the square order-4 tile (32 x 32 nodes) and the default
(64 x 16) give the same bits for every node, level and receiver; the automatic choice follows
the box's node counts; the shapes the square tile does not cover fall back to the default."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _solver(semgb, ex, ey, ez, order, steps, seed, sponge, shape, form=0):
    from semgb import workloads as W
    wl = W.small_random(ex, ey, ez, order, steps, seed=seed, nsrc=2, nrec=40, sponge=sponge)
    m, s = semgb.solver_from_workload(wl, semgb.KERNEL_STENCIL)
    s.set_operator_form(form)
    s.set_tile_shape(shape)
    return m, s


def _close(*pairs):
    for m, s in pairs:
        s.close()
        m.close()


@pytest.mark.parametrize("form", [0, 1], ids=["direct", "difference"])
@pytest.mark.parametrize("dims,sponge", [((7, 6, 9), 2), ((16, 5, 11), 0), ((9, 12, 8), 3)])
def test_square_tile_same_bits(semgb_lib, cuda_device, dims, sponge, form):
    semgb = semgb_lib
    n = 23
    a = _solver(semgb, *dims, 4, n, 41, sponge, semgb.TILE_DEFAULT, form)
    b = _solver(semgb, *dims, 4, n, 41, sponge, semgb.TILE_SQUARE, form)
    a[1].step(n)
    b[1].step(n)
    assert a[1].tile_shape == semgb.TILE_DEFAULT and b[1].tile_shape == semgb.TILE_SQUARE
    assert np.array_equal(a[1].pressure(), b[1].pressure())
    assert np.array_equal(a[1].pressure(semgb.LEVEL_PREVIOUS), b[1].pressure(semgb.LEVEL_PREVIOUS))
    assert np.array_equal(a[1].traces(), b[1].traces())
    _close(a, b)


def test_automatic_shape_and_fallbacks(semgb_lib, cuda_device):
    semgb = semgb_lib
    # 29 nodes per axis: one 32-node tile against a 64 x 16 tile half on the box -> square;
    # 41 nodes: 2 x 2 square tiles against 1 x 3 default tiles -> default
    sq = _solver(semgb, 7, 7, 7, 4, 4, 42, 1, semgb.TILE_AUTO)
    df = _solver(semgb, 10, 10, 10, 4, 4, 43, 1, semgb.TILE_AUTO)
    o3 = _solver(semgb, 7, 7, 7, 3, 4, 44, 1, semgb.TILE_SQUARE)  # order 3: the default
    ref = _solver(semgb, 7, 7, 7, 4, 4, 45, 1, semgb.TILE_SQUARE)
    ref[1].set_rounding(semgb.ROUNDING_REFERENCE)  # the reference rounding: the default
    for _, s in (sq, df, o3, ref):
        assert s.tile_shape == semgb.TILE_AUTO  # nothing built yet
        s.step(4)
    assert sq[1].tile_shape == semgb.TILE_SQUARE
    assert df[1].tile_shape == semgb.TILE_DEFAULT
    assert o3[1].tile_shape == semgb.TILE_DEFAULT
    assert ref[1].tile_shape == semgb.TILE_DEFAULT
    # switching the shape between steps rebuilds the tables and continues the same run
    cont = _solver(semgb, 7, 7, 7, 4, 10, 46, 2, semgb.TILE_SQUARE)
    whole = _solver(semgb, 7, 7, 7, 4, 10, 46, 2, semgb.TILE_DEFAULT)
    cont[1].step(5)
    cont[1].set_tile_shape(semgb.TILE_DEFAULT)
    cont[1].step(5)
    whole[1].step(10)
    assert cont[1].tile_shape == semgb.TILE_DEFAULT
    assert np.array_equal(cont[1].pressure(), whole[1].pressure())
    assert np.array_equal(cont[1].traces(), whole[1].traces())
    _close(sq, df, o3, ref, cont, whole)


def test_group_of_square_members(semgb_lib, cuda_device):
    """Members that step alone on the square tile keep it in a one-launch group, beside a member
    on the default tile."""
    semgb = semgb_lib
    dims = [(7, 7, 7), (7, 5, 6), (16, 5, 11), (9, 6, 8)]
    shapes = [semgb.TILE_SQUARE, semgb.TILE_SQUARE, semgb.TILE_SQUARE, semgb.TILE_DEFAULT]
    solo = [_solver(semgb, *d, 4, 17, 50 + i, 1, sh) for i, (d, sh) in enumerate(zip(dims, shapes))]
    for _, s in solo:
        s.step(17)
    grouped = [_solver(semgb, *d, 4, 17, 50 + i, 1, sh) for i, (d, sh) in enumerate(zip(dims, shapes))]
    for (_, s), sh in zip(grouped, shapes):
        s.step(1)  # the members' own tables
        assert s.tile_shape == sh
    g = semgb.Group([s for _, s in grouped])
    g.step(16)
    g.synchronize()
    assert g.launch == semgb.GROUP_ONE_LAUNCH
    for (_, a), (_, b) in zip(solo, grouped):
        assert np.array_equal(a.pressure(), b.pressure())
        assert np.array_equal(a.traces(), b.traces())
    g.close()
    _close(*solo, *grouped)


@pytest.mark.parametrize("form", [0, 1], ids=["direct", "difference"])
@pytest.mark.parametrize("name", ["c2_shape_q4_12c", "q4_rand"])
def test_square_tile_on_reference_fixtures(semgb_lib, cuda_device, name, form):
    """The square tile on the order-4 fixtures of the compiled reference: the same bits as the
    default tile, so the same errors against the reference and against FP64."""
    import os
    from test_gpu_parity import GOLDEN, rel_l2, solver_for_fixture
    semgb = semgb_lib
    path = [g for g in GOLDEN if os.path.basename(g) == name + ".npz"][0]
    f = np.load(path)
    kernel = "stencil-difference" if form else "stencil"
    runs = []
    for shape in (semgb.TILE_DEFAULT, semgb.TILE_SQUARE):
        m, s = solver_for_fixture(semgb, f, kernel)
        s.set_tile_shape(shape)
        s.step(int(f["nsteps"]))
        assert s.tile_shape == shape
        runs.append((s.traces(), s.pressure(), s.pressure(semgb.LEVEL_PREVIOUS)))
        s.close()
        m.close()
    for a, b in zip(*runs):
        assert np.array_equal(a, b)
    tr, p, _ = runs[1]
    assert rel_l2(tr, f["traces"]) <= 1e-5 + 2 * rel_l2(f["traces"], f["traces64"])
    assert rel_l2(p, f["p_cur"]) <= 1e-5 + 2 * rel_l2(f["p_cur"], f["p_cur64"])
