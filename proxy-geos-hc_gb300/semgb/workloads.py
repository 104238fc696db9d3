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
