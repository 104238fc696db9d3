"""Host-side logic of libsemgb (no GPU): GLL tables, Ricker, box indexing, receiver snapping,
sponge profile -- checked against the oracle, indices bit for bit."""
import numpy as np
import pytest

from oracle import oracle as O


@pytest.mark.parametrize("order", [1, 2, 3, 4, 5])
def test_gll_tables(semgb_lib, order):
    xi, w, d = semgb_lib.gll_tables(order)
    oxi, ow, od = O.gll_tables(order)
    assert np.array_equal(xi, oxi) and np.array_equal(w, ow) and np.array_equal(d, od)


@pytest.mark.parametrize("order", [0, 1, 2])
def test_ricker(semgb_lib, order):
    assert np.array_equal(semgb_lib.ricker(700, 3e-4, 9.0, order), O.source_term(700, 3e-4, 9.0, order))


def test_ricker_rejects_bad_order(semgb_lib):
    with pytest.raises(semgb_lib.SemError):
        semgb_lib.ricker(10, 1e-3, 10.0, 3)


@pytest.mark.parametrize("dims", [(3, 4, 5, 1), (4, 3, 2, 2), (3, 3, 4, 3), (2, 3, 2, 4), (2, 2, 2, 5)])
def test_counts_and_connectivity(semgb_lib, dims):
    ex, ey, ez, o = dims
    assert semgb_lib.box_counts(ex, ey, ez, o) == O.box_counts(ex, ey, ez, o)
    assert np.array_equal(semgb_lib.box_connectivity(ex, ey, ez, o), O.connectivity(ex, ey, ez, o))
    part = semgb_lib.box_connectivity(ex, ey, ez, o, e0=3, count=4)
    assert np.array_equal(part, O.connectivity(ex, ey, ez, o)[3:7])


def test_connectivity_range_checked(semgb_lib):
    with pytest.raises(semgb_lib.SemError):
        semgb_lib.box_connectivity(2, 2, 2, 2, e0=7, count=2)


def test_element_from_point_and_nearest_node(semgb_lib):
    rng = np.random.default_rng(1)
    for (ex, ey, ez, o) in [(5, 4, 3, 2), (7, 3, 6, 4), (3, 3, 3, 3)]:
        lx, ly, lz = 10.0 * ex, 12.5 * ey, 7.0 * ez
        pts = rng.uniform(-5, 1.1 * max(lx, ly, lz), (200, 3)).astype(np.float32)
        pts[:10] = np.array([[0, 0, 0], [lx, ly, lz], [10, 12.5, 7], [20, 25, 14]] + [[5, 5, 5]] * 6, np.float32)
        for x, y, z in pts:
            assert semgb_lib.element_from_point(ex, ey, ez, lx, ly, lz, x, y, z) == \
                O.element_from_point(ex, ey, ez, lx, ly, lz, x, y, z)
            assert semgb_lib.nearest_node(ex, ey, ez, lx, ly, lz, o, x, y, z) == \
                O.nearest_node(ex, ey, ez, lx, ly, lz, o, x, y, z)


@pytest.mark.parametrize("thickness,sigma", [(0, 0.06), (2, 0.2), (10, 0.06), (3, 1.5)])
def test_sponge_profile(semgb_lib, thickness, sigma):
    args = (12, 10, 14, 120.0, 100.0, 140.0, 3)
    a = semgb_lib.sponge_profile(*args, thickness, sigma)
    b, _ = O.sponge_profile(*args, thickness, sigma)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    assert all((v > 0).all() and (v <= 1).all() for v in a)


def test_workload_shapes():
    from semgb import workloads as W
    c1 = W.c1_plain_small()
    assert (c1.ex, c1.order, c1.nsteps, len(c1.rec_xyz), c1.sponge_thickness) == (40, 2, 1500, 64, 10)
    assert c1.n_nodes == 81 ** 3
    assert abs(c1.dt - 0.4 * 5.0 / 1500.0) < 1e-9
    c2 = W.c2_plain_scale(8, steps=10)
    assert c2.order == 4 and len(c2.rec_xyz) == 1024
    assert 1500 * 0.95 <= c2.vel.min() and c2.vel.max() <= 4500 * 1.05
    # CFL 0.4 on the smallest GLL spacing
    assert abs(c2.dt - np.float32(0.4 * 10 * (1 - np.sqrt(3 / 7)) / 2 / c2.vel.max())) < 1e-9
