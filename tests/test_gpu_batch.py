"""Batched form (many shots on one mesh, sem_batch_*): every shot of a batch must give the same
bits as the plain solver run of that shot alone (the plain solver is itself pinned to the
reference): the batch steps the shot-stacked levels with the plain stencil pass's own
arithmetic.  Traces and both pressure levels are compared, for batch sizes that are and are not
multiples of 32, and autotuning must not change the state."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _setup(semgb, order, n_shots, seed):
    from semgb import workloads as W
    wl = W.small_random(8, 6, 7, order, 60, seed=seed, nsrc=n_shots, nrec=9)
    wav = np.stack([semgb.ricker(wl.nsteps, wl.dt, float(f), 1) for f in wl.f0])
    return wl, wav


@pytest.mark.parametrize("order,n_shots", [(1, 7), (2, 40), (3, 33), (4, 64), (5, 12)])
def test_batch_matches_plain_solver_per_shot(semgb_lib, cuda_device, order, n_shots):
    semgb = semgb_lib
    wl, wav = _setup(semgb, order, n_shots, seed=50 + order)
    mesh = semgb.Mesh(wl.ex, wl.ey, wl.ez, wl.lx, wl.ly, wl.lz, order)
    mesh.set_velocity(wl.vel)
    b = semgb.Batch(mesh, wl.dt, n_shots)
    b.set_sponge(wl.sponge_thickness, wl.sponge_sigma)
    b.set_source_points(wl.src_xyz, wav)
    b.set_receivers(wl.rec_xyz)
    b.step(wl.nsteps)
    b.synchronize()
    tr = b.traces()
    assert tr.shape == (wl.nsteps, 9, n_shots)
    for s in (0, n_shots // 2, n_shots - 1):
        p = semgb.Solver(mesh, wl.dt)
        p.set_kernel(semgb.KERNEL_STENCIL)
        p.set_sponge(wl.sponge_thickness, wl.sponge_sigma)
        p.set_source_points(wl.src_xyz[s:s + 1], wav[s:s + 1])
        p.set_receivers(wl.rec_xyz)
        p.step(wl.nsteps)
        assert np.array_equal(tr[:, :, s], p.traces())
        assert np.array_equal(b.pressure(s), p.pressure())
        assert np.array_equal(b.pressure(s, semgb.LEVEL_PREVIOUS), p.pressure(semgb.LEVEL_PREVIOUS))
        p.close()


def test_batch_autotune_keeps_state(semgb_lib, cuda_device):
    semgb = semgb_lib
    wl, wav = _setup(semgb, 4, 64, seed=71)
    res = []
    for tune in (False, True):
        mesh = semgb.Mesh(wl.ex, wl.ey, wl.ez, wl.lx, wl.ly, wl.lz, 4)
        mesh.set_velocity(wl.vel)
        b = semgb.Batch(mesh, wl.dt, 64)
        b.set_sponge(wl.sponge_thickness, wl.sponge_sigma)
        b.set_source_points(wl.src_xyz, wav)
        b.set_receivers(wl.rec_xyz)
        b.step(20)
        if tune:
            pick = b.autotune()
            assert pick["shots_per_cluster"] in (1, 2, 4, 8) and pick["warps_per_cta"] >= 1
        b.step(40)
        res.append((b.traces(), b.pressure(7)))
        b.close()
    assert np.array_equal(res[1][0], res[0][0])
    assert np.array_equal(res[1][1], res[0][1])
