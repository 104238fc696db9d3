"""Seeded synthetic workloads for the SEM acoustic step (pure numpy, no GPU).

Each builder returns a :class:`Workload`: a physical description (box mesh, per-element
velocity, source and receiver positions, sponge, dt, steps).  Turning positions into elements
and nodes is left to the consumer (``semgb`` on the GPU side, the oracle on the CPU side), so
that both conversions can be checked against each other.

Axis convention (the reference's, SEMmesh.cpp:142-231): node index = ix + iz*nx + iy*nx*nz; the
coordinate triple is (x, y, z) with z the reference's coordinate column 1, used here as depth.

Synthetic stand-ins: the reference publishes no dataset for this path; every model below is a
seeded synthetic model with the shapes and value ranges of the named configuration.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class Workload:
    name: str
    ex: int
    ey: int
    ez: int
    order: int
    h: float                       # element size (m), same on every axis
    vel: np.ndarray                # float32 [n_elem] (element e = ix + iz*ex + iy*ex*ez)
    dt: float
    nsteps: int
    src_xyz: np.ndarray            # float32 [nsrc, 3]
    f0: np.ndarray                 # float32 [nsrc]
    rec_xyz: np.ndarray            # float32 [nrec, 3]
    sponge_thickness: int = 0      # elements; 0 = no sponge
    sponge_sigma: float = 0.06
    ricker_order: int = 1
    meta: dict = field(default_factory=dict)

    @property
    def lx(self):
        return float(self.ex * self.h)

    @property
    def ly(self):
        return float(self.ey * self.h)

    @property
    def lz(self):
        return float(self.ez * self.h)

    @property
    def n_nodes(self):
        o = self.order
        return (self.ex * o + 1) * (self.ey * o + 1) * (self.ez * o + 1)

    @property
    def n_elem(self):
        return self.ex * self.ey * self.ez


def gll_min_spacing(order: int) -> float:
    """Smallest GLL node spacing on [-1, 1] (between the end point and its neighbour)."""
    from numpy.polynomial import legendre as L
    if order == 1:
        return 2.0
    c = np.zeros(order + 1)
    c[-1] = 1.0
    r = np.sort(np.real(L.legroots(L.legder(c))))
    return float(r[0] + 1.0)


def cfl_dt(h: float, order: int, c_max: float, cfl: float = 0.4) -> float:
    """dt = cfl * dx_min / c_max with dx_min = h * (xi_1 - xi_0) / 2 (the build's CFL rule)."""
    return float(np.float32(cfl * h * gll_min_spacing(order) / 2.0 / c_max))


def _element_centres(ex, ey, ez, h):
    ix = np.arange(ex)
    iy = np.arange(ey)
    iz = np.arange(ez)
    # element e = ix + iz*ex + iy*ex*ez  ->  array index [iy, iz, ix]
    Y, Z, X = np.meshgrid(iy, iz, ix, indexing="ij")
    return (X + 0.5) * h, (Y + 0.5) * h, (Z + 0.5) * h


def _gaussian_filter3(a: np.ndarray, sigma: float) -> np.ndarray:
    """Separable Gaussian filter (reflect padding), numpy only."""
    r = int(np.ceil(3 * sigma))
    k = np.exp(-0.5 * (np.arange(-r, r + 1) / sigma) ** 2)
    k /= k.sum()
    out = a.astype(np.float64)
    for ax in range(3):
        pad = [(0, 0)] * 3
        pad[ax] = (r, r)
        b = np.pad(out, pad, mode="reflect")
        acc = np.zeros_like(out)
        for i, kv in enumerate(k):
            sl = [slice(None)] * 3
            sl[ax] = slice(i, i + out.shape[ax])
            acc += kv * b[tuple(sl)]
        out = acc
    return out


def layered_velocity(ex, ey, ez, h, n_layers, vmin, vmax, rng, perturb=0.0, sigma_elems=5.0):
    """Horizontal layers in depth (z) with seeded uniform speeds, optionally times
    (1 + perturb * n) where n is seeded white noise Gaussian-filtered at sigma_elems and scaled
    to max |n| = 1.  Evaluated per element (at its centre).  Returns float32 [n_elem]."""
    speeds = rng.uniform(vmin, vmax, n_layers)
    _, _, Zc = _element_centres(ex, ey, ez, h)
    layer = np.minimum((Zc / (ez * h) * n_layers).astype(int), n_layers - 1)
    v = speeds[layer]
    if perturb:
        noise = rng.standard_normal((ey, ez, ex))
        f = _gaussian_filter3(noise, sigma_elems)
        f /= np.abs(f).max()
        v = v * (1.0 + perturb * f)
    return np.ascontiguousarray(v.reshape(-1), np.float32)


def c1_plain_small(steps: int = 1500) -> Workload:
    """Plain SEM, CPU-runnable: 40^3 elements of 10 m, GLL order 2, c = 1500 m/s, Ricker 5 Hz at
    the domain centre (200,200,200), 10-element sponge on all faces, dt at CFL 0.4, 1500 steps,
    64 receivers on a seeded random line at z = 50 m."""
    ex = ey = ez = 40
    h, order = 10.0, 2
    vel = np.full(ex * ey * ez, 1500.0, np.float32)
    dt = cfl_dt(h, order, 1500.0)
    rng = np.random.default_rng(20240512)
    a, b = rng.uniform(0.0, ex * h, 2), rng.uniform(0.0, ey * h, 2)
    t = np.linspace(0.0, 1.0, 64)
    rec = np.stack([a[0] + (a[1] - a[0]) * t, b[0] + (b[1] - b[0]) * t, np.full(64, 50.0)], 1)
    return Workload("c1_plain_40c_q2", ex, ey, ez, order, h, vel, dt, steps,
                    np.array([[200.0, 200.0, 200.0]], np.float32), np.array([5.0], np.float32),
                    rec.astype(np.float32), sponge_thickness=10)


def c2_plain_scale(n: int = 200, steps: int = 1000, seed: int = 2) -> Workload:
    """Plain SEM at scale: n^3 (200^3) hex elements of 10 m, GLL order 4; velocity = 5 horizontal
    layers with seeded uniform speeds in [1500, 4500] m/s times a smooth Gaussian-filtered
    (sigma 5 elements) seeded perturbation of +-5 %; 20-element sponge; Ricker 10 Hz at depth
    100 m (centred in x and y); CFL 0.4; 1000 steps; 1024 receivers on a 32 x 32 grid two elements
    below the top face."""
    ex = ey = ez = n
    h, order = 10.0, 4
    rng = np.random.default_rng(seed)
    if n <= 256:
        vel = layered_velocity(ex, ey, ez, h, 5, 1500.0, 4500.0, rng, perturb=0.05, sigma_elems=5.0)
    else:  # too large to filter in numpy quickly: layers only
        vel = layered_velocity(ex, ey, ez, h, 5, 1500.0, 4500.0, rng)
    dt = cfl_dt(h, order, float(vel.max()))
    L = n * h
    g = (np.arange(32) + 0.5) / 32 * L
    X, Y = np.meshgrid(g, g, indexing="ij")
    # the top face is a Dirichlet (pressure-free) surface, so receivers sit two elements below it
    rec = np.stack([X.ravel(), Y.ravel(), np.full(X.size, 2 * h)], 1)
    return Workload(f"c2_plain_{n}c_q4", ex, ey, ez, order, h, vel, dt, steps,
                    np.array([[L / 2, L / 2, 100.0]], np.float32), np.array([10.0], np.float32),
                    rec.astype(np.float32), sponge_thickness=min(20, n // 4))


def small_random(ex, ey, ez, order, steps, seed, h=10.0, nsrc=1, nrec=16, sponge=2,
                 vmin=1500.0, vmax=3000.0) -> Workload:
    """A small seeded problem for parity tests: layered + perturbed velocity, random sources
    and receivers inside the box."""
    rng = np.random.default_rng(seed)
    vel = layered_velocity(ex, ey, ez, h, 3, vmin, vmax, rng, perturb=0.05, sigma_elems=1.5)
    dt = cfl_dt(h, order, float(vel.max()))
    Ls = np.array([ex * h, ey * h, ez * h])
    src = rng.uniform(0.2, 0.8, (nsrc, 3)) * Ls
    f0 = rng.uniform(0.1, 0.2, nsrc) * float(vel.min()) / h
    rec = rng.uniform(0.0, 1.0, (nrec, 3)) * Ls
    return Workload(f"rand_{ex}x{ey}x{ez}_q{order}_s{seed}", ex, ey, ez, order, h, vel, dt, steps,
                    src.astype(np.float32), f0.astype(np.float32), rec.astype(np.float32),
                    sponge_thickness=sponge, sponge_sigma=0.2)


def c3_batched_shots(n: int = 100, n_shots: int = 64, steps: int = 800, seed: int = 3) -> Workload:
    """Batched shots on one mesh: n^3 (100^3) hex elements of 10 m, GLL order 4, the velocity
    recipe of :func:`c2_plain_scale` with another seed; n_shots (64) Ricker 8 Hz sources on a
    seeded jittered 8 x 8 grid spanning the undamped part of the surface, at the depth of the
    plain workload's source (100 m); the 32 x 32 receiver grid of :func:`c2_plain_scale`;
    800 steps.  ``src_xyz`` / ``f0`` hold one row per shot."""
    w = c2_plain_scale(n, steps, seed)
    rng = np.random.default_rng(seed + 1000)
    L = n * w.h
    k = int(round(np.sqrt(n_shots)))
    a = w.sponge_thickness * w.h
    g = a + (np.arange(k) + 0.5) / k * (L - 2 * a)
    X, Y = np.meshgrid(g, g, indexing="ij")
    jit = rng.uniform(-0.25, 0.25, (k * k, 2)) * ((L - 2 * a) / k)
    src = np.stack([X.ravel() + jit[:, 0], Y.ravel() + jit[:, 1], np.full(k * k, 100.0)], 1)[:n_shots]
    return Workload(f"c3_batched_{n}c_q4_{n_shots}shots", w.ex, w.ey, w.ez, w.order, w.h, w.vel, w.dt,
                    steps, src.astype(np.float32), np.full(len(src), 8.0, np.float32), w.rec_xyz,
                    sponge_thickness=w.sponge_thickness)


def c3_uneven_batch(n_problems: int = 32, steps: int = 800, seed: int = 31, lo: int = 40, hi: int = 120):
    """Uneven batch: n_problems (32) independent problems with element counts drawn per axis from
    [lo, hi] ([40, 120]) and GLL order from {2, 3, 4}, elements of 10 m, each with the velocity
    recipe of :func:`c2_plain_scale` (its own seed), a Ricker 8 Hz source at 100 m depth centred in
    x and y, the 32 x 32 receiver grid two elements below the top face and a 20-element sponge
    (capped at a quarter of the smallest axis); dt at CFL 0.4 per problem."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n_problems):
        ex, ey, ez = (int(v) for v in rng.integers(lo, hi + 1, 3))
        order = int(rng.choice([2, 3, 4]))
        h = 10.0
        r = np.random.default_rng(seed * 1000 + i)
        vel = layered_velocity(ex, ey, ez, h, 5, 1500.0, 4500.0, r)
        dt = cfl_dt(h, order, float(vel.max()))
        gx = (np.arange(32) + 0.5) / 32 * ex * h
        gy = (np.arange(32) + 0.5) / 32 * ey * h
        X, Y = np.meshgrid(gx, gy, indexing="ij")
        rec = np.stack([X.ravel(), Y.ravel(), np.full(X.size, 2 * h)], 1)
        out.append(Workload(f"uneven_{i}_{ex}x{ey}x{ez}_q{order}", ex, ey, ez, order, h, vel, dt, steps,
                            np.array([[ex * h / 2, ey * h / 2, 100.0]], np.float32), np.array([8.0], np.float32),
                            rec.astype(np.float32), sponge_thickness=min(20, min(ex, ey, ez) // 4)))
    return out


def node_coordinates(ex, ey, ez, order, h):
    """Node coordinates (x, y, z) in the reference node numbering (node = ix + iz*nx + iy*nx*nz),
    with GLL points inside each element."""
    xi = np.array(_gll_points(order))
    def axis(ne):
        e = np.arange(ne * order + 1) // order
        l = np.arange(ne * order + 1) - e * order
        e = np.minimum(e, ne - 1)
        l = np.where(np.arange(ne * order + 1) == ne * order, order, l)
        return e * h + (1.0 + xi[l]) * 0.5 * h
    x, y, z = axis(ex), axis(ey), axis(ez)
    Y, Z, X = np.meshgrid(y, z, x, indexing="ij")
    return X.reshape(-1), Y.reshape(-1), Z.reshape(-1)


def _gll_points(order):
    # Gauss-Lobatto-Legendre points: -1, 1 and the roots of P'_order
    if order == 1:
        return [-1.0, 1.0]
    c = np.zeros(order + 1)
    c[-1] = 1.0
    inner = np.sort(np.real(np.polynomial.legendre.legroots(np.polynomial.legendre.legder(c))))
    return [-1.0, *inner.tolist(), 1.0]


def c4_adjoint(n: int = 96, order: int = 3, steps: int = 2000, n_shots: int = 16, n_rec: int = 256,
               seed: int = 4, h: float = 10.0):
    """Adjoint gradient: n^3 (96^3) elements of 10 m, GLL order 3; true model = two layers
    (2000 / 3000 m/s, interface at mid-depth) times (1 + 0.1 g) with g a Gaussian bump of radius 8
    elements at a seeded position in the lower half of the interior; current model = the layered
    background smoothed over 4 elements in depth; both per node as squared slowness.  n_shots (16)
    Ricker 8 Hz sources on a seeded jittered 4 x 4 grid at 60 m depth, n_rec (256) receivers on a
    16 x 16 grid at 20 m depth, steps (2000), dt at CFL 0.4 of 3300 m/s.  Returns a dict."""
    rng = np.random.default_rng(seed)
    L = n * h
    X, Y, Z = node_coordinates(n, n, n, order, h)
    zi = L / 2
    width = 4 * h  # smoothing length of the background's interface
    c_bg = 2000.0 + 1000.0 * 0.5 * (1.0 + np.tanh((Z - zi) / width))
    c_layers = np.where(Z < zi, 2000.0, 3000.0)
    centre = np.array([rng.uniform(0.35, 0.65) * L, rng.uniform(0.35, 0.65) * L, rng.uniform(0.55, 0.7) * L])
    r2 = ((X - centre[0]) ** 2 + (Y - centre[1]) ** 2 + (Z - centre[2]) ** 2) / (8 * h) ** 2
    c_true = c_layers * (1.0 + 0.1 * np.exp(-r2))
    k = int(round(np.sqrt(n_shots)))
    g = (np.arange(k) + 0.5) / k * L
    SX, SY = np.meshgrid(g, g, indexing="ij")
    jit = rng.uniform(-0.2, 0.2, (k * k, 2)) * (L / k)
    src = np.stack([SX.ravel() + jit[:, 0], SY.ravel() + jit[:, 1], np.full(k * k, 60.0)], 1)[:n_shots]
    m = int(round(np.sqrt(n_rec)))
    gr = (np.arange(m) + 0.5) / m * L
    RX, RY = np.meshgrid(gr, gr, indexing="ij")
    rec = np.stack([RX.ravel(), RY.ravel(), np.full(m * m, 20.0)], 1)[:n_rec]
    dt = cfl_dt(h, order, 3300.0)
    return {"name": f"c4_adjoint_{n}c_q{order}", "ex": n, "ey": n, "ez": n, "order": order, "h": h,
            "m_true": (1.0 / c_true ** 2).astype(np.float32), "m0": (1.0 / c_bg ** 2).astype(np.float32),
            "vel_elem": np.full(n * n * n, 2000.0, np.float32), "dt": dt, "steps": steps,
            "src_xyz": src.astype(np.float32), "f0": 8.0, "rec_xyz": rec.astype(np.float32),
            "checkpoint_every": 50, "sponge_thickness": 10, "sponge_sigma": 0.06}
