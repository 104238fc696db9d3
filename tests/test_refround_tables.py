"""The reference-rounded stiffness rows and node-class table (SEM_ROUNDING_REFERENCE) against the
oracle's element products, which are pinned bit for bit to the compiled reference.  CPU only: the
tables are built on the host."""
import numpy as np
import pytest

from oracle import oracle as O

# boxes whose float node coordinates are exact in the reference (orders 1-2, integer element
# sizes), with different element sizes per axis
EXACT = [(4, 3, 5, 40.0, 30.0, 50.0, 1), (4, 3, 5, 40.0, 60.0, 75.0, 2), (3, 4, 2, 30.0, 40.0, 20.0, 2)]
INEXACT = [(3, 3, 3, 30.0, 30.0, 30.0, 3), (3, 2, 3, 30.0, 20.0, 30.0, 4), (2, 2, 2, 20.0, 20.0, 20.0, 5)]


def oracle_rows(ex, ey, ez, lx, ly, lz, order, e):
    """R_e(i, j) of the oracle's element product by unit probing: Y = R e_j is exactly column j."""
    npe = (order + 1) ** 3
    P = O.Problem(ex, ey, ez, order, lx, ly, lz, 1e-3, 1, np.full(ex * ey * ez, 1500.0, np.float32),
                  np.zeros(0, np.int64), np.zeros((0, 1), np.float32))
    R = np.zeros((npe, npe), np.float32)
    for j in range(npe):
        pl = np.zeros(npe, np.float32)
        pl[j] = 1.0
        R[:, j] = O.element_apply(P, e, pl)[1]
    return R


def dense_from_rows(rows, order):
    o1 = order + 1
    npe = o1 ** 3
    R = np.zeros((npe, npe), np.float32)
    for i in range(npe):
        i1, i2, i3 = i % o1, (i // o1) % o1, i // (o1 * o1)
        for m in range(o1):
            R[i, m + i2 * o1 + i3 * o1 * o1] += rows[0, i, m]
            if m != i2:
                R[i, i1 + m * o1 + i3 * o1 * o1] += rows[1, i, m]
            if m != i3:
                R[i, i1 + i2 * o1 + m * o1 * o1] += rows[2, i, m]
    return R


def class_from_dense(R, order):
    """Assemble node-class coefficients [a][ly][lz][d+o][lx] from one element's rows (exact sums)."""
    o, o1 = order, order + 1
    W = 2 * o + 1
    C = np.zeros((3, o, o, W, o))

    def members(l):
        return [l] if l else [0, o]
    for ly in range(o):
        for lz in range(o):
            for lx in range(o):
                for ix in members(lx):
                    for iz in members(lz):
                        for iy in members(ly):
                            i = ix + iz * o1 + iy * o1 * o1
                            for m in range(o1):
                                C[0, ly, lz, m - ix + o, lx] += R[i, m + iz * o1 + iy * o1 * o1]
                                if m != iz:
                                    C[1, ly, lz, m - iz + o, lx] += R[i, ix + m * o1 + iy * o1 * o1]
                                if m != iy:
                                    C[2, ly, lz, m - iy + o, lx] += R[i, ix + iz * o1 + m * o1 * o1]
    return C.astype(np.float32)


@pytest.mark.parametrize("box", EXACT, ids=[f"q{b[-1]}-{i}" for i, b in enumerate(EXACT)])
def test_rows_bit_exact_where_reference_coordinates_are_exact(semgb_lib, box):
    ex, ey, ez, lx, ly, lz, order = box
    rows = semgb_lib.refround_rows(*box)
    mine = dense_from_rows(rows, order)
    for e in (0, ex * ey * ez - 1):
        assert np.array_equal(oracle_rows(*box, e), mine)


@pytest.mark.parametrize("box", EXACT, ids=[f"q{b[-1]}-{i}" for i, b in enumerate(EXACT)])
def test_class_table_is_the_assembly_of_the_rows(semgb_lib, box):
    order = box[-1]
    tab = semgb_lib.refround_class_table(*box)
    assert np.array_equal(tab, class_from_dense(oracle_rows(*box, 0), order))


@pytest.mark.parametrize("box", INEXACT, ids=[f"q{b[-1]}" for b in INEXACT])
def test_rows_close_where_reference_coordinates_are_rounded(semgb_lib, box):
    """At orders 3-5 the reference's float node coordinates are rounded per element, so its rows
    differ from the exact-geometry rows by the coordinate rounding (a few 1e-5 at most)."""
    ex, ey, ez, lx, ly, lz, order = box
    mine = dense_from_rows(semgb_lib.refround_rows(*box), order)
    R = oracle_rows(*box, 0)
    mask = mine != 0
    assert np.abs(R[~mask]).max() <= 1e-12 * np.abs(R).max()  # off-line entries: roundoff only
    assert np.max(np.abs(R[mask] - mine[mask]) / np.abs(mine[mask])) < 1e-4
