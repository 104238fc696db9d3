"""sem_element_step_noalloc: the allocation-free step for callers that cannot allocate device
memory while they step (a host code that hands all device memory to its own pool manager, or one
whose time loop runs where allocation is not allowed).

The test calls the entry point through the C ABI on device buffers the test owns, twice in a row,
and compares each result with the solver's element step (sem_solver_step with
SEM_KERNEL_ELEMENT) from the same state.  Both paths use the same element kernel with float
atomics, so sums may round differently in the last bit; the tolerance is relative L2 <= 2e-6.
This file is collected last so that a failure here leaves every other test already run.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def mass_coefficient(semgb, wl):
    """dt^2 / M_i per node (reference numbering): M_i = w_ix w_iz w_iy |detJ| sum_{e owns i} 1/c_e^2."""
    o = wl.order
    _, w, _ = semgb.gll_tables(o)
    nx, ny, nz = wl.ex * o + 1, wl.ey * o + 1, wl.ez * o + 1
    hx, hy, hz = wl.lx / wl.ex, wl.ly / wl.ey, wl.lz / wl.ez
    detJ = (hx / 2) * (hz / 2) * (hy / 2)
    inv_c2 = 1.0 / wl.vel.astype(np.float64).reshape(wl.ey, wl.ez, wl.ex) ** 2
    S = np.zeros((ny, nz, nx))
    for ky in range(wl.ey):
        for kz in range(wl.ez):
            for kx in range(wl.ex):
                S[ky * o:ky * o + o + 1, kz * o:kz * o + o + 1, kx * o:kx * o + o + 1] += inv_c2[ky, kz, kx]
    wq = np.array([w[i % o] for i in range(max(nx, ny, nz))])
    W = wq[:ny, None, None] * wq[None, :nz, None] * wq[None, None, :nx]
    M = W * detJ * S
    return (np.float64(wl.dt) ** 2 / M).astype(np.float32).reshape(-1)


def test_noalloc_step_matches_solver_element_step(semgb_lib, cuda_device):
    import torch

    from semgb import workloads as W

    semgb = semgb_lib
    lib = semgb.lib()
    wl = W.small_random(7, 5, 6, 3, 2, seed=31, nsrc=0, nrec=0, sponge=2)
    o = wl.order
    nx, ny, nz = wl.ex * o + 1, wl.ey * o + 1, wl.ez * o + 1
    N = nx * ny * nz
    iy, iz, ix = np.unravel_index(np.arange(N), (ny, nz, nx))
    base = np.sin(0.3 * ix + 0.2) * np.cos(0.25 * iz) * np.sin(0.2 * iy + 0.5)
    p0 = base.astype(np.float32)
    q0 = (0.9 * base).astype(np.float32)
    sp = semgb.sponge_profile(wl.ex, wl.ey, wl.ez, wl.lx, wl.ly, wl.lz, o, wl.sponge_thickness, wl.sponge_sigma)

    # the existing entry point: the solver's element step, two steps from (p0, q0)
    mesh = semgb.Mesh(wl.ex, wl.ey, wl.ez, wl.lx, wl.ly, wl.lz, o)
    mesh.set_velocity(wl.vel)
    s = semgb.Solver(mesh, wl.dt)
    s.set_kernel(semgb.KERNEL_ELEMENT)
    s.set_sponge_profile(*sp)
    s.set_pressure(semgb.LEVEL_CURRENT, p0)
    s.set_pressure(semgb.LEVEL_PREVIOUS, q0)
    expect = []
    for _ in range(2):
        s.step(1)
        expect.append((s.pressure(semgb.LEVEL_CURRENT), s.pressure(semgb.LEVEL_PREVIOUS)))

    # the allocation-free entry point on buffers this test owns
    dev = torch.device("cuda", 0)
    conn = torch.from_numpy(mesh.connectivity()).to(dev)
    coef = torch.from_numpy(mass_coefficient(semgb, wl)).to(dev)
    sxyz = [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in sp]
    levels = [torch.from_numpy(p0).to(dev), torch.from_numpy(q0).to(dev)]
    stream = torch.cuda.current_stream(dev)
    cur = 0
    for k in range(2):
        pc, pp = levels[cur], levels[1 - cur]
        rc = lib.sem_element_step_noalloc(wl.ex, wl.ey, wl.ez, wl.lx, wl.ly, wl.lz, o,
                                          C.c_void_p(conn.data_ptr()), C.c_void_p(pc.data_ptr()),
                                          C.c_void_p(pp.data_ptr()), C.c_void_p(coef.data_ptr()),
                                          *[C.c_void_p(a.data_ptr()) for a in sxyz],
                                          C.c_void_p(stream.cuda_stream))
        assert rc == semgb.SEM_OK, lib.sem_last_error_string().decode()
        torch.cuda.synchronize(dev)
        new, damped_old = pp.cpu().numpy(), pc.cpu().numpy()
        cur = 1 - cur
        e_new = rel_l2(new, expect[k][0])
        e_old = rel_l2(damped_old, expect[k][1])
        assert e_new <= 2e-6, (k, e_new)
        assert e_old <= 2e-6, (k, e_old)
        assert np.isfinite(new).all()


def test_noalloc_rejects_meshes_beyond_its_scratch(semgb_lib, cuda_device):
    import torch

    semgb = semgb_lib
    lib = semgb.lib()
    small = torch.zeros(16, device="cuda")  # valid buffers; the size check rejects the call first
    ptr = C.c_void_p(small.data_ptr())
    rc = lib.sem_element_step_noalloc(100, 100, 100, 1000.0, 1000.0, 1000.0, 2, ptr, ptr, ptr, ptr,
                                      None, None, None, None)
    assert rc == semgb.SEM_ERR_ARG
    assert b"at most" in lib.sem_last_error_string()
