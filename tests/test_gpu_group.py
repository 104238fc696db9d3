"""Groups of uneven problems (sem_group_*): every member of a group must give the same bits as
the same solver run alone (same kernels, same order of operations), for even and odd step
counts, and solo steps must interleave correctly with group steps."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPES = [(6, 5, 4, 2, 11), (9, 7, 8, 4, 12), (5, 6, 7, 3, 13), (4, 4, 4, 1, 14)]


def _members(semgb, steps):
    from semgb import workloads as W
    out = []
    for ex, ey, ez, o, seed in SHAPES:
        wl = W.small_random(ex, ey, ez, o, steps, seed=seed, nsrc=2, nrec=7)
        out.append(semgb.solver_from_workload(wl, semgb.KERNEL_STENCIL))
    return out


def test_group_matches_solo_runs(semgb_lib, cuda_device):
    semgb = semgb_lib
    n = 37
    solo = _members(semgb, n)
    for _, s in solo:
        s.step(n)
    grouped = _members(semgb, n)
    g = semgb.Group([s for _, s in grouped])
    g.step(20)
    g.step(17)
    g.synchronize()
    for (_, a), (_, b) in zip(solo, grouped):
        assert np.array_equal(a.traces(), b.traces())
        assert np.array_equal(a.pressure(), b.pressure())
        assert np.array_equal(a.pressure(semgb.LEVEL_PREVIOUS), b.pressure(semgb.LEVEL_PREVIOUS))
    g.close()


def test_group_and_solo_steps_interleave(semgb_lib, cuda_device):
    semgb = semgb_lib
    solo = _members(semgb, 30)
    for _, s in solo:
        s.step(30)
    grouped = _members(semgb, 30)
    g = semgb.Group([s for _, s in grouped])
    g.step(9)
    for _, s in grouped:
        s.step(3)  # solo steps on the members' own streams between group steps
    g.step(18)
    g.synchronize()
    for (_, a), (_, b) in zip(solo, grouped):
        assert np.array_equal(a.traces(), b.traces())
        assert np.array_equal(a.pressure(), b.pressure())
    g.close()
