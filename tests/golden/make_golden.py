"""Generates the golden fixtures in this directory by running the reference's own SEM code.

The reference's sources are compiled by oracle/build_ref.sh (they exist only where the reference
checkout does), so this script runs only there; its outputs are committed and read by the tests
on any machine.  Each fixture holds the problem's inputs (velocity, source elements and wavelets,
receiver nodes, sponge factors, dt) and the reference's outputs after ``nsteps`` steps (newest
and previous pressure levels and receiver traces), plus the same scheme run in FP64 by the
oracle, so that tests can state each code's error against FP64.

Usage:  python tests/golden/make_golden.py [--only NAME] [--c1]
"""
from __future__ import annotations

import argparse
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "proxy-geos-hc_gb300"))

from oracle import oracle as O  # noqa: E402
from semgb import workloads as W  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))

SMALL = {
    # name: (workload builder, nsteps); step counts keep the pulse inside the box at the end
    "q1_rand": (lambda: W.small_random(9, 8, 7, 1, 80, seed=11, nsrc=2, nrec=10), 80),
    "q2_rand": (lambda: W.small_random(8, 7, 6, 2, 90, seed=12, nsrc=2, nrec=12), 90),
    "q3_rand": (lambda: W.small_random(6, 5, 5, 3, 100, seed=13, nsrc=1, nrec=12), 100),
    "q4_rand": (lambda: W.small_random(5, 5, 4, 4, 110, seed=14, nsrc=2, nrec=12), 110),
    "q5_rand": (lambda: W.small_random(4, 4, 4, 5, 100, seed=15, nsrc=1, nrec=8), 100),
    "q2_nosponge_edge": (lambda: _edge_case(), 80),
    "c2_shape_q4_12c": (lambda: W.c2_plain_scale(n=12, steps=150, seed=7), 150),
    "c1_shape_q2_16c": (lambda: _c1_small(16, 300), 300),
}


def _edge_case() -> W.Workload:
    """No sponge; one source on a boundary corner element (node 0 is a Dirichlet node) and one
    outside the box (the reference maps it to element 0 per axis); receivers on boundary nodes."""
    wl = W.small_random(5, 4, 6, 2, 80, seed=21, nsrc=1, nrec=6, sponge=0)
    wl.src_xyz = np.array([[0.0, 0.0, 0.0], [-5.0, 1e4, 25.0], [31.0, 22.0, 47.0]], np.float32)
    wl.f0 = np.array([30.0, 25.0, 20.0], np.float32)
    wl.rec_xyz = np.concatenate([wl.rec_xyz, [[0.0, 0.0, 0.0], [50.0, 40.0, 60.0], [1e4, -1, 3]]]).astype(np.float32)
    return wl


def _c1_small(n: int, steps: int) -> W.Workload:
    wl = W.c1_plain_small(steps)
    scale = n / wl.ex
    wl.name = f"c1_shape_q2_{n}c"
    wl.ex = wl.ey = wl.ez = n
    wl.vel = np.full(n ** 3, 1500.0, np.float32)
    wl.src_xyz = (wl.src_xyz * scale).astype(np.float32)
    wl.rec_xyz = (wl.rec_xyz * np.array([scale, scale, 1.0])).astype(np.float32)
    wl.sponge_thickness = 4
    return wl


def save(name: str, wl: W.Workload, nsteps: int, full_fields=True):
    P = O.problem_from_workload(wl, nsteps)
    t = time.time()
    pc, pp, tr = O.run(P, backend="ref")
    t_ref = time.time() - t
    t = time.time()
    pc64, pp64, tr64 = O.run(P, real=np.float64, nthreads=os.cpu_count() or 1)
    t64 = time.time() - t
    out = dict(
        ex=wl.ex, ey=wl.ey, ez=wl.ez, order=wl.order, h=wl.h, lx=wl.lx, ly=wl.ly, lz=wl.lz,
        dt=np.float32(wl.dt), nsteps=nsteps, vel=P.vel, src_elem=P.src_elem, wavelet=P.wavelet,
        src_xyz=wl.src_xyz, f0=wl.f0, ricker_order=wl.ricker_order, rec_xyz=wl.rec_xyz,
        rec_node=P.rec_node, sponge_thickness=wl.sponge_thickness, sponge_sigma=wl.sponge_sigma,
        traces=tr, traces64=tr64.astype(np.float32),
        p_cur=pc, p_cur64=pc64.astype(np.float32),
        p_prev_norm=np.float64(np.linalg.norm(pp.astype(np.float64))),
        p_prev64_norm=np.float64(np.linalg.norm(pp64)),
    )
    if full_fields:
        out["p_prev"] = pp
        out["p_prev64"] = pp64.astype(np.float32)
    if P.sponge32 is not None:
        out.update(sx=P.sponge32[0], sy=P.sponge32[1], sz=P.sponge32[2])
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
    e_tr = O.rel_l2(tr, tr64)
    e_p = O.rel_l2(pc, pc64)
    print(f"{name}: N={P.n_nodes} steps={nsteps} ref {t_ref:.1f}s fp64 {t64:.1f}s "
          f"|p|max={np.abs(pc).max():.3g} ref-vs-fp64 traces {e_tr:.2e} p {e_p:.2e}", flush=True)


def save_tables():
    """The reference's own GLL tables (its 15-digit closed forms), for runs of the oracle that
    must match the reference bit for bit on machines without the reference checkout."""
    out = {}
    for q in range(1, 6):
        xi, w, d = O.ref_tables(q)
        out[f"xi{q}"], out[f"w{q}"], out[f"dphi{q}"] = xi, w, d
    np.savez(os.path.join(HERE, "gll_ref_tables.npz"), **out)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", default=None)
    ap.add_argument("--c1", action="store_true", help="also the full 40^3 Q2 1500-step case (minutes)")
    a = ap.parse_args()
    save_tables()
    for name, (mk, n) in SMALL.items():
        if a.only and a.only != name:
            continue
        save(name, mk(), n)
    if a.c1 or a.only == "c1_full":
        save("c1_full", W.c1_plain_small(1500), 1500, full_fields=False)


if __name__ == "__main__":
    main()
