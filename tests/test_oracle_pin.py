"""The oracle (CPU restatement) pinned against the reference.

* Against the golden fixtures (outputs of the compiled reference, committed): the float oracle
  run with the reference's own GLL tables must reproduce them bit for bit.  Runs anywhere.
* Against the compiled reference itself (oracle/_ref, only where the reference checkout exists):
  tables, mesh indexing, coordinates, Ricker samples, element kernel and whole runs.
"""
import glob
import os

import numpy as np
import pytest

from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")
SMALL = [p for p in sorted(glob.glob(os.path.join(GOLD, "*.npz")))
         if not os.path.basename(p).startswith(("gll_", "c1_full", "c2_shape"))]


def ref_tables_fixture(order):
    t = np.load(os.path.join(GOLD, "gll_ref_tables.npz"))
    return t[f"xi{order}"], t[f"w{order}"], t[f"dphi{order}"]


def problem_from_fixture(f, nsteps=None):
    sp32 = (f["sx"], f["sy"], f["sz"]) if "sx" in f else None
    return O.Problem(int(f["ex"]), int(f["ey"]), int(f["ez"]), int(f["order"]), float(f["lx"]),
                     float(f["ly"]), float(f["lz"]), float(f["dt"]),
                     int(f["nsteps"]) if nsteps is None else nsteps, f["vel"], f["src_elem"],
                     f["wavelet"], f["rec_node"], sp32, None)


def run_with_tables(P, tabs, real=np.float32):
    N = P.n_nodes
    pc, pp = np.zeros(N, real), np.zeros(N, real)
    tr = np.zeros((P.nsteps, max(len(P.rec_node), 1)), real)
    keep = []
    cfg = O._config(P, tabs, keep, 1, real)
    import ctypes as C
    rc = O.lib().or_run_f32(C.byref(cfg), O._ptr(pc, O._F32P), O._ptr(pp, O._F32P), O._ptr(tr, O._F32P))
    assert rc == 0
    return pc, pp, tr[:, :len(P.rec_node)]


@pytest.mark.parametrize("path", SMALL, ids=[os.path.basename(p)[:-4] for p in SMALL])
def test_oracle_bit_exact_vs_reference_fixture(path):
    f = np.load(path)
    P = problem_from_fixture(f)
    pc, pp, tr = run_with_tables(P, ref_tables_fixture(P.order))
    assert np.array_equal(pc, f["p_cur"])
    assert np.array_equal(tr, f["traces"])
    if "p_prev" in f:
        assert np.array_equal(pp, f["p_prev"])


@pytest.mark.parametrize("order", [1, 2, 3, 4, 5])
def test_own_gll_tables_match_reference_literals(order):
    xi, w, d = O.gll_tables(order)
    rxi, rw, rd = ref_tables_fixture(order)
    assert np.abs(xi - rxi).max() < 1e-15
    assert np.array_equal(w, rw)          # weights are 8-decimal literals in the reference
    assert np.abs(d - rd).max() < 1e-13


def test_ricker_known_answers():
    # values printed by the reference's own runs (f0 = 10 Hz, dt = 1 ms, first-derivative form)
    s = O.source_term(201, 1e-3, 10.0, 1)
    assert f"{s[0]:.6g}" == "0.0102097"
    assert f"{s[100]:.6g}" in ("-0", "0")
    assert f"{s[200]:.6g}" == "-0.0102097"


def test_fixture_tables_consistent_with_own_rule():
    """The fixtures' sponge factors, source elements and receiver nodes follow the oracle's
    host rules applied to the stored positions (indices bit-exact)."""
    for path in SMALL:
        f = np.load(path)
        ex, ey, ez, o = int(f["ex"]), int(f["ey"]), int(f["ez"]), int(f["order"])
        lx, ly, lz = float(f["lx"]), float(f["ly"]), float(f["lz"])
        src = [O.element_from_point(ex, ey, ez, lx, ly, lz, *map(float, x)) for x in f["src_xyz"]]
        assert np.array_equal(src, f["src_elem"])
        rec = [O.nearest_node(ex, ey, ez, lx, ly, lz, o, *map(float, x)) for x in f["rec_xyz"]]
        assert np.array_equal(rec, f["rec_node"])
        if "sx" in f:
            sp, _ = O.sponge_profile(ex, ey, ez, lx, ly, lz, o, int(f["sponge_thickness"]),
                                     float(f["sponge_sigma"]))
            for a, b in zip(sp, (f["sx"], f["sy"], f["sz"])):
                assert np.array_equal(a, b)


def test_colour_parallel_matches_sequential_closely():
    """The coloured OpenMP loop (used for CPU timing) only reorders the scatter sums."""
    f = np.load(os.path.join(GOLD, "q3_rand.npz"))
    P = problem_from_fixture(f)
    a = O.run(P, nthreads=1)
    b = O.run(P, nthreads=4)
    assert O.rel_l2(b[0], a[0]) < 1e-6
    assert O.rel_l2(b[2], a[2]) < 1e-6


# ---- against the compiled reference (only where oracle/_ref was built) ----------------------

needs_ref = pytest.mark.skipif(not O.ref_available(2), reason="compiled reference not available")


@needs_ref
@pytest.mark.parametrize("order", [1, 2, 3, 4, 5])
def test_tables_fixture_is_reference(order):
    rxi, rw, rd = O.ref_tables(order)
    fxi, fw, fd = ref_tables_fixture(order)
    assert np.array_equal(rxi, fxi) and np.array_equal(rw, fw) and np.array_equal(rd, fd)


@needs_ref
@pytest.mark.parametrize("order", [2, 3, 4])
def test_mesh_indexing_bit_exact_vs_reference(order):
    import ctypes as C
    ex, ey, ez = 5, 4, 3
    N, NE, NI = O.box_counts(ex, ey, ez, order)
    counts = np.zeros(3, np.int64)
    conn = np.zeros((NE, (order + 1) ** 3), np.int32)
    inter = np.zeros(NI, np.int32)
    X, Y, Z = (np.zeros(conn.shape, np.float32) for _ in range(3))
    O.ref(order).semref_mesh(ex, ey, ez, 50.0, 40.0, 30.0, O._ptr(counts, O._I64P), O._ptr(conn, O._I32P),
                             O._ptr(inter, O._I32P), O._ptr(X, O._F32P), O._ptr(Z, O._F32P), O._ptr(Y, O._F32P))
    assert list(counts) == [N, NE, NI]
    assert np.array_equal(conn, O.connectivity(ex, ey, ez, order))
    assert np.array_equal(inter, O.interior_nodes(ex, ey, ez, order))
    oX, oZ, oY = O.element_coords(ex, ey, ez, 50.0, 40.0, 30.0, order)
    assert np.array_equal(X, oX) and np.array_equal(Y, oY) and np.array_equal(Z, oZ)
    rng = np.random.default_rng(order)
    for _ in range(50):
        x, y, z = rng.uniform(-10, 60, 3).astype(np.float32)
        assert O.ref(order).semref_element_from_point(ex, ey, ez, 50.0, 40.0, 30.0, x, y, z) == \
            O.element_from_point(ex, ey, ez, 50.0, 40.0, 30.0, x, y, z)


@needs_ref
@pytest.mark.parametrize("order", [0, 1, 2])
def test_ricker_bit_exact_vs_reference(order):
    a = O.source_term(500, 7e-4, 12.5, order)
    b = np.zeros(500, np.float32)
    O.ref(2).semref_source_term(500, 7e-4, 12.5, order, O._ptr(b, O._F32P))
    assert np.array_equal(a, b)


@needs_ref
@pytest.mark.parametrize("order", [2, 3, 4])
def test_element_kernel_bit_exact_vs_reference(order):
    from semgb import workloads as W
    wl = W.small_random(3, 3, 2, order, 1, seed=order)
    P = O.problem_from_workload(wl, 1)
    rng = np.random.default_rng(0)
    pl = rng.standard_normal((order + 1) ** 3).astype(np.float32)
    for e in (0, 7, 17):
        M1, Y1 = O.element_apply(P, e, pl, backend="ref")
        M2, Y2 = O.element_apply(P, e, pl, tables="ref")
        assert np.array_equal(M1, M2) and np.array_equal(Y1, Y2)


@needs_ref
@pytest.mark.parametrize("order", [1, 2, 3, 4, 5])
def test_run_bit_exact_vs_reference(order):
    from semgb import workloads as W
    wl = W.small_random(4, 3, 3, order, 25, seed=40 + order, nsrc=2, nrec=6)
    P = O.problem_from_workload(wl)
    r = O.run(P, backend="ref")
    o = O.run(P, tables="ref")
    for a, b in zip(r, o):
        assert np.array_equal(a, b)
