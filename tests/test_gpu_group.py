"""Groups of uneven problems (sem_group_*): every member of a group must give the same bits as
the same solver run alone (same per-node arithmetic, same order of operations), in both launch
forms (one launch per step over all members' tiles, or each member's launches as graph
branches), for even and odd step counts, and solo steps must interleave correctly with group
steps."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# (ex, ey, ez, order, seed, sponge elements): orders 1-4, members with and without a sponge
SHAPES = [(6, 5, 4, 2, 11, 2), (9, 7, 8, 4, 12, 2), (5, 6, 7, 3, 13, 0), (4, 4, 4, 1, 14, 1), (7, 9, 5, 4, 15, 0)]


def _members(semgb, steps, shapes=SHAPES, nrec=7):
    from semgb import workloads as W
    out = []
    for ex, ey, ez, o, seed, sp in shapes:
        wl = W.small_random(ex, ey, ez, o, steps, seed=seed, nsrc=2, nrec=nrec, sponge=sp)
        out.append(semgb.solver_from_workload(wl, semgb.KERNEL_STENCIL))
    return out


def _same(solo, grouped, semgb):
    for (_, a), (_, b) in zip(solo, grouped):
        assert np.array_equal(a.traces(), b.traces())
        assert np.array_equal(a.pressure(), b.pressure())
        assert np.array_equal(a.pressure(semgb.LEVEL_PREVIOUS), b.pressure(semgb.LEVEL_PREVIOUS))


def _close(members, g):
    g.close()
    for m, s in members:
        s.close()
        m.close()


@pytest.mark.parametrize("launch", [0, 1], ids=["one_launch", "branches"])
def test_group_matches_solo_runs(semgb_lib, cuda_device, launch):
    semgb = semgb_lib
    n = 37
    solo = _members(semgb, n)
    for _, s in solo:
        s.step(n)
    grouped = _members(semgb, n)
    g = semgb.Group([s for _, s in grouped], launch=launch)
    g.step(20)
    g.step(17)
    g.synchronize()
    assert g.launch == launch
    _same(solo, grouped, semgb)
    _close(grouped, g)
    for m, s in solo:
        s.close()
        m.close()


@pytest.mark.parametrize("launch", [0, 1], ids=["one_launch", "branches"])
def test_group_and_solo_steps_interleave(semgb_lib, cuda_device, launch):
    semgb = semgb_lib
    solo = _members(semgb, 30)
    for _, s in solo:
        s.step(30)
    grouped = _members(semgb, 30)
    g = semgb.Group([s for _, s in grouped], launch=launch)
    g.step(9)
    for _, s in grouped:
        s.step(3)  # solo steps on the members' own streams between group steps
    g.step(5)
    grouped[1][1].step(1)  # one member one step ahead ...
    for i, (_, s) in enumerate(grouped):
        if i != 1:
            s.step(1)  # ... and the others catch up alone
    g.step(12)
    g.synchronize()
    _same(solo, grouped, semgb)
    _close(grouped, g)


def test_group_falls_back_to_branches(semgb_lib, cuda_device):
    """A member the one-launch form does not cover (order 5; the reference rounding) puts the
    group on branches, with the same bits."""
    semgb = semgb_lib
    shapes = [(5, 4, 6, 2, 21, 1), (3, 3, 4, 5, 22, 1)]
    solo = _members(semgb, 12, shapes)
    for _, s in solo:
        s.step(12)
    grouped = _members(semgb, 12, shapes)
    g = semgb.Group([s for _, s in grouped])
    g.step(12)
    g.synchronize()
    assert g.launch == semgb.GROUP_BRANCHES
    _same(solo, grouped, semgb)
    _close(grouped, g)

    shapes = [(5, 4, 6, 2, 23, 1), (4, 3, 4, 3, 24, 1)]
    solo = _members(semgb, 9, shapes)
    for _, s in solo:
        s.set_rounding(semgb.ROUNDING_REFERENCE)
        s.step(9)
    grouped = _members(semgb, 9, shapes)
    for _, s in grouped:
        s.set_rounding(semgb.ROUNDING_REFERENCE)
    g = semgb.Group([s for _, s in grouped])
    g.step(9)
    g.synchronize()
    assert g.launch == semgb.GROUP_BRANCHES
    _same(solo, grouped, semgb)
    _close(grouped, g)


def test_one_launch_many_tiles_and_chunks(semgb_lib, cuda_device):
    """Members large enough for several x- and z-tiles and y-chunks, receivers spread over many
    CTAs: one launch against solo runs, bit for bit."""
    semgb = semgb_lib
    shapes = [(30, 26, 22, 4, 31, 3), (41, 12, 35, 2, 32, 4), (17, 33, 19, 3, 33, 2), (9, 40, 9, 1, 34, 0)]
    solo = _members(semgb, 14, shapes, nrec=150)
    for _, s in solo:
        s.step(14)
    grouped = _members(semgb, 14, shapes, nrec=150)
    g = semgb.Group([s for _, s in grouped])
    g.step(14)
    g.synchronize()
    assert g.launch == semgb.GROUP_ONE_LAUNCH
    _same(solo, grouped, semgb)
    _close(grouped, g)


@pytest.mark.parametrize("launch", [0, 1], ids=["one_launch", "branches"])
def test_group_across_trace_growth(semgb_lib, cuda_device, launch):
    """More steps than the members' first trace storage (64 steps): the storage grows between
    group steps, the group rebuilds its launch state, and the members still match solo runs."""
    semgb = semgb_lib
    n = 150
    shapes = SHAPES[:3]
    solo = _members(semgb, n, shapes)
    for _, s in solo:
        s.step(n)
    grouped = _members(semgb, n, shapes)
    g = semgb.Group([s for _, s in grouped], launch=launch)
    g.step(50)
    g.step(31)
    g.step(69)
    g.synchronize()
    _same(solo, grouped, semgb)
    _close(grouped, g)
    for m, s in solo:
        s.close()
        m.close()
