"""Adjoint-state gradient (sem_adjoint_*): the adjoint dot-product test, central finite
differences along seeded random directions, checkpoint invariance, and the forward traces
against the plain solver.  FP64 is used only in the check reductions."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

EX, EY, EZ, ORDER, H = 8, 7, 6, 3, 10.0


def _setup(semgb, nsteps, seed, perturb=0.0):
    from semgb import workloads as W
    rng = np.random.default_rng(seed)
    mesh = semgb.Mesh(EX, EY, EZ, EX * H, EY * H, EZ * H, ORDER)
    c0 = 2000.0
    mesh.set_velocity(np.full(EX * EY * EZ, c0, np.float32))  # source coefficients dt^2 c^2
    nx, ny, nz = EX * ORDER + 1, EY * ORDER + 1, EZ * ORDER + 1
    iy, iz, ix = np.unravel_index(np.arange(nx * ny * nz), (ny, nz, nx))
    # smooth background: slowness^2 of a vertical gradient 2000 -> 2600 m/s
    c = c0 + 600.0 * iz / (nz - 1)
    if perturb:
        r2 = ((ix - nx / 2) ** 2 + (iz - nz / 2) ** 2 + (iy - ny / 2) ** 2) / (0.2 * nx) ** 2
        c = c * (1.0 + perturb * np.exp(-r2))
    m = (1.0 / c ** 2).astype(np.float32)
    mesh.set_slowness2(m)
    dt = W.cfl_dt(H, ORDER, float(c.max()) * 1.05)
    rec = np.stack([rng.uniform(0.15, 0.85, 12) * EX * H, rng.uniform(0.15, 0.85, 12) * EY * H,
                    rng.uniform(0.15, 0.85, 12) * EZ * H], 1).astype(np.float32)
    e_src = 3 + 2 * EX + 3 * EX * EZ  # element (3, 2, 3) in (x, z, y): node 0 at (9, 6, 9), interior
    wav = semgb.ricker(nsteps, dt, 0.15 * c0 / H, 1)[None]
    return mesh, m, dt, rec, e_src, wav


def _adjoint(semgb, mesh, dt, nsteps, every, rec, e_src, wav):
    a = semgb.Adjoint(mesh, dt, nsteps, every)
    a.set_sponge(2, 0.2)
    a.set_sources(np.array([e_src]), wav)
    a.set_receivers(rec)
    return a


def test_forward_traces_match_plain_solver(semgb_lib, cuda_device):
    semgb = semgb_lib
    n = 90
    mesh, m, dt, rec, e_src, wav = _setup(semgb, n, 1)
    a = _adjoint(semgb, mesh, dt, n, 17, rec, e_src, wav)
    d = a.forward()
    s = semgb.Solver(mesh, dt)
    s.set_kernel(semgb.KERNEL_STENCIL)
    s.set_sponge(2, 0.2)
    s.set_sources(np.array([e_src]), wav)
    s.set_receivers(rec)
    s.step(n)
    assert np.array_equal(d, s.traces())
    assert np.abs(d).max() > 0


def test_adjoint_dot_product(semgb_lib, cuda_device):
    """<F w, r> = <w, F^T r>: F maps the source wavelet to the traces; F^T r is read from the
    adjoint run at the source node (row j of the adjoint traces is step n = N-1-j, scaled by
    1/(s a) at that node)."""
    semgb = semgb_lib
    n = 120
    mesh, m, dt, rec, e_src, wav = _setup(semgb, n, 2)
    a = _adjoint(semgb, mesh, dt, n, 25, rec, e_src, wav)
    d = a.forward().astype(np.float64)
    rng = np.random.default_rng(7)
    r = rng.standard_normal(d.shape).astype(np.float32)
    nx, nz = EX * ORDER + 1, EZ * ORDER + 1
    src_node = 9 + 6 * nx + 9 * nx * nz
    a.set_adjoint_receiver_nodes([src_node])
    a.backward(r)
    ta = a.adjoint_traces()[:, 0].astype(np.float64)
    # a = dt^2 / (m W) at the source node, as the mass kernel rounds it; the sponge is 1 there
    _, w, _ = semgb.gll_tables(ORDER)
    detJ = (H / 2) ** 3
    W = w[0] ** 3 * detJ * 8  # local index 0 on all three axes, 2 elements along each
    dt2 = float(np.float32(dt)) ** 2
    a_src = float(np.float32(dt2 / (float(m[src_node]) * W)))
    f32 = np.float32
    coef = float(f32(f32(f32(dt) * f32(dt)) * f32(2000.0)) * f32(2000.0))
    lhs = float(np.sum(d * r))
    rhs = float(np.sum(coef * wav[0].astype(np.float64) * ta[::-1])) / a_src
    print(f"dot test: {lhs:.9e} {rhs:.9e} rel {abs(lhs - rhs) / abs(lhs):.2e}")
    assert abs(lhs - rhs) <= 2e-5 * abs(lhs)


def _loss(d, obs):
    return 0.5 * float(np.sum((d.astype(np.float64) - obs.astype(np.float64)) ** 2))


def test_gradient_central_differences(semgb_lib, cuda_device):
    """dL/dm along 8 seeded random directions against (L(m+eps dm) - L(m-eps dm)) / 2 eps,
    eps = 1e-3 relative."""
    semgb = semgb_lib
    n = 150
    mesh_t, _, dt, rec, e_src, wav = _setup(semgb, n, 3, perturb=0.1)
    obs = _adjoint(semgb, mesh_t, dt, n, 40, rec, e_src, wav).forward()
    mesh, m0, _, _, _, _ = _setup(semgb, n, 3)
    a = _adjoint(semgb, mesh, dt, n, 40, rec, e_src, wav)
    a.forward()
    loss, g = a.gradient(obs)
    assert loss > 0 and np.isfinite(g).all()
    rng = np.random.default_rng(11)
    eps = 1e-3
    for k in range(8):
        dm = (m0 * rng.standard_normal(m0.shape)).astype(np.float64)
        lp = []
        for sgn in (1, -1):
            mesh.set_slowness2((m0 + sgn * eps * dm).astype(np.float32))
            lp.append(_loss(a.forward(), obs))
        mesh.set_slowness2(m0)
        fd = (lp[0] - lp[1]) / (2 * eps)
        an = float(np.dot(g.astype(np.float64), dm))
        print(f"direction {k}: fd {fd:.6e} adjoint {an:.6e} rel {abs(fd - an) / abs(fd):.2e}")
        assert abs(fd - an) <= 1e-2 * abs(fd)


def test_checkpoint_interval_does_not_change_gradient(semgb_lib, cuda_device):
    semgb = semgb_lib
    n = 64
    mesh, m, dt, rec, e_src, wav = _setup(semgb, n, 4)
    rng = np.random.default_rng(5)
    res = rng.standard_normal((n, len(rec))).astype(np.float32)
    grads = []
    for every in (n, 13, 1):
        a = _adjoint(semgb, mesh, dt, n, every, rec, e_src, wav)
        a.forward()
        grads.append(a.backward(res))
        a.close()
    assert np.array_equal(grads[0], grads[1])
    assert np.array_equal(grads[0], grads[2])
    assert np.abs(grads[0]).max() > 0
