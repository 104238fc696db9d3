"""sem_element_step_noalloc: the allocation-free step for callers that cannot allocate device
memory while they step (a host code that hands all device memory to its own pool manager, or one
whose time loop runs where allocation is not allowed).

The test calls the entry point through the C ABI on device buffers the test owns, twice in a row,
and compares each result with the solver's element step (sem_solver_step with
SEM_KERNEL_ELEMENT) from the same state and with the oracle (the reference's arithmetic on the
CPU).  Both GPU paths use the same element kernel with float atomics, so sums may round
differently in the last bit; the tolerance is relative L2 <= 2e-6 against the solver and 5e-6
against the oracle.  After the first call (which loads the library's device code), a call must
leave the device's free memory unchanged.  This file is collected last so that a failure here
leaves every other test already run.
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

    # the oracle: the reference's arithmetic for the same two steps
    from oracle import oracle as O
    P = O.Problem(wl.ex, wl.ey, wl.ez, o, wl.lx, wl.ly, wl.lz, wl.dt, 2, np.ascontiguousarray(wl.vel, np.float32),
                  np.zeros(0, np.int64), np.zeros((0, 2), np.float32), sponge32=sp)
    oracle_out = [O.run(P.__class__(**{**P.__dict__, "nsteps": n}), p0, q0) for n in (1, 2)]

    # the allocation-free entry point on buffers this test owns
    dev = torch.device("cuda", 0)
    conn = torch.from_numpy(mesh.connectivity()).to(dev)
    coef = torch.from_numpy(mass_coefficient(semgb, wl)).to(dev)
    sxyz = [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in sp]
    levels = [torch.from_numpy(p0).to(dev), torch.from_numpy(q0).to(dev)]
    stream = torch.cuda.current_stream(dev)
    torch.cuda.synchronize(dev)
    cur = 0
    for k in range(2):
        pc, pp = levels[cur], levels[1 - cur]
        free_before = torch.cuda.mem_get_info(dev)[0]
        rc = lib.sem_element_step_noalloc(wl.ex, wl.ey, wl.ez, wl.lx, wl.ly, wl.lz, o,
                                          C.c_void_p(conn.data_ptr()), C.c_void_p(pc.data_ptr()),
                                          C.c_void_p(pp.data_ptr()), C.c_void_p(coef.data_ptr()),
                                          *[C.c_void_p(a.data_ptr()) for a in sxyz],
                                          C.c_void_p(stream.cuda_stream))
        assert rc == semgb.SEM_OK, lib.sem_last_error_string().decode()
        torch.cuda.synchronize(dev)
        free_after = torch.cuda.mem_get_info(dev)[0]
        if k > 0:  # the first call in a process may load device code; later calls allocate nothing
            assert free_after == free_before, (free_before, free_after)
        new, damped_old = pp.cpu().numpy(), pc.cpu().numpy()
        cur = 1 - cur
        e_new = rel_l2(new, expect[k][0])
        e_old = rel_l2(damped_old, expect[k][1])
        assert e_new <= 2e-6, (k, e_new)
        assert e_old <= 2e-6, (k, e_old)
        assert np.isfinite(new).all()
        o_new, o_old, _ = oracle_out[k]
        assert rel_l2(new, o_new) <= 5e-6, (k, rel_l2(new, o_new))
        assert rel_l2(damped_old, o_old) <= 5e-6, (k, rel_l2(damped_old, o_old))


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


def test_noalloc_skips_connectivity_outside_the_mesh(semgb_lib, cuda_device):
    """Entries of the caller's map outside [0, n_nodes) are never read or written through: a map
    with one element's row pointing past the mesh changes nothing outside the mesh's nodes (the
    buffers are padded with sentinels that must survive)."""
    import torch

    from semgb import workloads as W

    semgb = semgb_lib
    lib = semgb.lib()
    wl = W.small_random(4, 3, 3, 2, 1, seed=32, nsrc=0, nrec=0, sponge=0)
    o = wl.order
    mesh = semgb.Mesh(wl.ex, wl.ey, wl.ez, wl.lx, wl.ly, wl.lz, o)
    N = mesh.n_nodes
    conn = mesh.connectivity().copy()
    conn[5, :] = N + 7        # past the mesh: inside the padded buffers below
    conn[6, 3] = -1           # negative
    dev = torch.device("cuda", 0)
    pad = 64
    sentinel = 12345.0
    levels = []
    rng = np.random.default_rng(3)
    for _ in range(2):
        a = np.full(N + pad, sentinel, np.float32)
        a[:N] = rng.standard_normal(N).astype(np.float32)
        levels.append(torch.from_numpy(a).to(dev))
    coef = torch.full((N + pad,), 1e-3, device=dev)
    c = torch.from_numpy(conn).to(dev)
    rc = lib.sem_element_step_noalloc(wl.ex, wl.ey, wl.ez, wl.lx, wl.ly, wl.lz, o, C.c_void_p(c.data_ptr()),
                                      C.c_void_p(levels[0].data_ptr()), C.c_void_p(levels[1].data_ptr()),
                                      C.c_void_p(coef.data_ptr()), None, None, None,
                                      C.c_void_p(torch.cuda.current_stream(dev).cuda_stream))
    assert rc == semgb.SEM_OK, lib.sem_last_error_string().decode()
    torch.cuda.synchronize(dev)
    for lv in levels:
        tail = lv.cpu().numpy()[N:]
        assert np.all(tail == sentinel)
        assert np.isfinite(lv.cpu().numpy()[:N]).all()
