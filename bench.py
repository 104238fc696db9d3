"""Benchmark of the SEM acoustic step (plain form) on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload c2|c1] [--kernel auto|element|stencil]

Metric: Gnode-steps/s (global nodes x time steps / second), FP32 fields.  Default workload: the
at-scale plain configuration, 200^3 hexahedra of 10 m, GLL order 4 (513,922,401 nodes), layered
+ perturbed velocity, 20-element sponge, one Ricker source, 1024 receivers (synthetic inputs,
seeded).  A "step" is one leapfrog step of the whole mesh.  Fields are 2 GB each, far larger than
L2, so no L2 flush is needed between steps.

Rank 0 prints one JSON line.  Under torchrun (N > 1) every rank runs an independent replica of
the workload (the plain step does not shard in this build) and `value` is the sum over ranks of
node-steps divided by the slowest rank's time.

--impl reference times the reference's CPU implementation of the same step on this machine's
host cores: the oracle's C restatement (oracle/sem_oracle.c, bit-exact with the compiled
reference where the reference is available), OpenMP over all cores with race-free element
colouring, on a bounded sub-box of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "proxy-geos-hc_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "SEM Gnode-steps/s on 1 GB300 (Q4, fp32)"
PEAKS_FILE = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0


def hbm_peak():
    try:
        with open(PEAKS_FILE) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def reduce_max(x: float, ws: int) -> float:
    """Max of a per-rank value over all ranks (the value itself on one rank)."""
    if ws <= 1:
        return float(x)
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank: float, ws: int, t_local_s: float) -> float:
    """Whole-job throughput of replicas: the units all ranks processed over the slowest rank's
    time (every rank runs the same workload; no data moves between ranks)."""
    return units_per_rank * ws / reduce_max(t_local_s, ws)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.rows = []
        self.proc = None
        self.thread = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 8:
                self.rows.append(parts)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(r[1]) for r in self.rows if num(r[1]) is not None]
        mx = [num(r[2]) for r in self.rows if num(r[2]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[4 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def make_workload(name: str, elems: int = 200):
    from semgb import workloads as W
    if name == "c2":
        return W.c2_plain_scale(elems, steps=1000)
    if name == "c1":
        return W.c1_plain_small(1500)
    raise SystemExit(f"unknown workload {name}")


# ---------------------------------------------------------------------------------------------
# CPU side (oracle restatement of the reference's step)
# ---------------------------------------------------------------------------------------------

def cpu_sample(wl, n_elems_axis: int):
    """A bounded sub-box of the workload for the CPU timing: same order, element size and
    velocity recipe (the box's first elements along each axis), same source/sponge rules."""
    from semgb import workloads as W
    import copy
    s = copy.deepcopy(wl)
    n = n_elems_axis
    v = wl.vel.reshape(wl.ey, wl.ez, wl.ex)[:n, :n, :n]
    s.ex = s.ey = s.ez = n
    s.vel = np.ascontiguousarray(v.reshape(-1))
    s.src_xyz = np.array([[n * wl.h / 2, n * wl.h / 2, min(100.0, n * wl.h / 2)]], np.float32)
    s.rec_xyz = wl.rec_xyz[:16] * (n / wl.ex)
    s.sponge_thickness = min(wl.sponge_thickness, max(1, n // 4))
    s.name = f"{wl.name}_cpu_sample_{n}c"
    return s


def time_cpu(wl, steps: int, threads: int):
    from oracle import oracle as O
    P = O.problem_from_workload(wl, steps)
    t0 = time.perf_counter()
    O.run(P, nthreads=threads)
    dt = time.perf_counter() - t0
    return P.n_nodes * steps / dt, dt, P.n_nodes


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    wl = make_workload(args.workload, args.elems)
    n = args.cpu_elems
    sw = cpu_sample(wl, n)
    from oracle import oracle as O
    O.lib()
    if args.warmup:
        time_cpu(sw, 1, threads)
    rate, secs, nodes = time_cpu(sw, args.steps, threads)
    g = rate / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": g, "unit": "Gnode-steps/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": secs / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": f"{wl.name} (CPU sample: {n}^3 elements of the same recipe)",
                   "order": wl.order, "nodes": nodes, "parallelism": f"openmp x{threads}"},
        "cpu_baseline": {"value": g, "unit": "Gnode-steps/s", "cores": threads, "kind": "port",
                         "sample": f"{n}^3-element sub-box of {wl.name}, {args.steps} steps"},
        "e2e": {"value": g, "unit": "Gnode-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------------------------
# GPU side
# ---------------------------------------------------------------------------------------------

def traffic_per_node(kernel_name: str):
    """DRAM bytes per node per launch from the committed ncu summary (profiles/), if any."""
    p = os.path.join(ROOT, "profiles", "dram_bytes_per_node.json")
    try:
        with open(p) as f:
            return float(json.load(f)[kernel_name])
    except Exception:
        return None


# Algorithmic (compulsory) DRAM bytes per node and launch.
#  stencil (fused pass): read p^n, p^{n-1}, dt^2/M; write p^{n+1}                    = 16 B
#  element kernel: connectivity (o+1)^3*4/o^3, gather of p^n, y read-modify-write    = see below
#  update kernel: read p^n, p^{n-1}, y, dt^2/M; write p^{n+1}, y                    = 24 B
def element_bytes_per_node(order: int) -> float:
    return 4.0 * (order + 1) ** 3 / order ** 3 + 4.0 + 8.0


def run_ours(args):
    import torch
    import torch.distributed as dist

    import semgb

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    wl = make_workload(args.workload, args.elems)
    kernel = {"auto": semgb.KERNEL_AUTO, "element": semgb.KERNEL_ELEMENT,
              "stencil": semgb.KERNEL_STENCIL}[args.kernel]
    mesh, s = semgb.solver_from_workload(wl, kernel)
    s.set_tile_shape({"auto": semgb.TILE_AUTO, "default": semgb.TILE_DEFAULT, "square": semgb.TILE_SQUARE}[args.tile])
    stream = torch.cuda.Stream()
    s.set_stream(stream.cuda_stream)
    N = mesh.n_nodes
    W = max(args.warmup, 3)

    def barrier():
        if ws > 1:
            dist.barrier()

    # warm-up (also builds the graphs and the mass coefficients)
    s.step(W)
    torch.cuda.synchronize()
    barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        ev0.record(stream)
        s.step(args.steps)
        ev1.record(stream)
        torch.cuda.synchronize()
    barrier()
    t_ms = ev0.elapsed_time(ev1)
    s.synchronize()
    t_max = reduce_max(t_ms, ws)
    value = job_rate(N * args.steps, ws, t_ms / 1e3) / 1e9

    # per-kernel device time (CUDA events on the solver's stream, un-captured launches)
    kms = [float(x) for x in s.time_kernels(max(5, min(20, args.steps)))]
    resolved = "stencil" if kernel in (semgb.KERNEL_AUTO, semgb.KERNEL_STENCIL) else "element"
    peak, peak_kind = hbm_peak()
    if resolved == "stencil":
        bpn, kname, kt = 16.0, "sem_stencil", kms[1]
        launches_per_step = 2
    else:
        bpn, kname, kt = element_bytes_per_node(wl.order), "sem_element", kms[1]
        launches_per_step = 3
    achieved = bpn * N / (kt / 1e3) / 1e9
    tpn = traffic_per_node(kname)
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "traffic": (tpn * N if tpn else None),
            "kernel": kname, "bytes_per_node": bpn, "kernel_ms": kt, "peak_kind": peak_kind}
    extra = {}
    if resolved == "element":
        upd_b = 24.0 * N
        extra["roofline_update"] = {"bound": "hbm", "achieved": upd_b / (kms[2] / 1e3) / 1e9,
                                    "peak": peak, "unit": "GB/s",
                                    "frac": upd_b / (kms[2] / 1e3) / 1e9 / peak, "kernel_ms": kms[2]}
    # whole-step bytes under the two-phase byte model (32.3 B/node at Q4) for comparison
    o = wl.order
    model_b = 20.0 + 4.0 * (o + 1) ** 3 / o ** 3 + 32.0 / o ** 3
    step_ms = t_max / args.steps
    extra["two_phase_model"] = {"bytes_per_node": model_b,
                                "equivalent_GBps": model_b * N / (step_ms / 1e3) / 1e9,
                                "frac": model_b * N / (step_ms / 1e3) / 1e9 / peak}

    # end to end through the public streaming call with host buffers: per step, this step's
    # wavelet sample goes host->device and the step's receiver samples come back
    nsrc, nrec = s.nsrc, s.nrec
    wav_h = torch.empty((1, nsrc), dtype=torch.float32, pin_memory=True)
    tr_h = torch.empty((1, nrec), dtype=torch.float32, pin_memory=True)
    wav_np, tr_np = wav_h.numpy(), tr_h.numpy()
    src_w = semgb.ricker(wl.nsteps, wl.dt, float(wl.f0[0]), wl.ricker_order)
    s.reset()
    e2e_steps = min(args.steps, wl.nsteps - 2)
    for i in range(2):  # warm-up of the streaming path
        wav_np[0, :] = src_w[i]
        s.step_host(1, wav_np, tr_np)
    barrier()
    t0 = time.perf_counter()
    for i in range(e2e_steps):
        wav_np[0, :] = src_w[(i + 2) % len(src_w)]
        s.step_host(1, wav_np, tr_np)
    t_e2e = time.perf_counter() - t0
    e2e_val = job_rate(N * e2e_steps, ws, t_e2e) / 1e9

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        sw = cpu_sample(wl, args.cpu_elems)
        rate, secs, nodes = time_cpu(sw, args.cpu_steps, threads)
        cpu = {"value": rate / 1e9, "unit": "Gnode-steps/s", "cores": threads, "kind": "port",
               "sample": f"{args.cpu_elems}^3-element sub-box of {wl.name} ({nodes} nodes), "
                         f"{args.cpu_steps} steps, {secs:.1f} s"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "Gnode-steps/s", "n_gpus": ws,
            "steps": args.steps, "warmup": W, "ms_per_step": t_max / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded layered+perturbed velocity model)",
            "config": {"workload": wl.name, "elements": [wl.ex, wl.ey, wl.ez], "order": wl.order,
                       "nodes": N, "kernel": resolved, "tile": ({0: "default", 1: "square"}.get(s.tile_shape, "n/a")
                                                                if resolved == "stencil" else "n/a"),
                       "parallelism": "replicas" if ws > 1 else "single",
                       "l2": "inputs larger than L2 (2 GB per field), no flush"},
            "roofline": roof,
            **extra,
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_val, "unit": "Gnode-steps/s", "h2d_bytes_per_step": 4 * nsrc,
                    "d2h_bytes_per_step": 4 * nrec, "steps": e2e_steps},
            "gpu_launches": launches_per_step * args.steps,
            "clocks": clk.summary(),
            "kernel_ms": {"source": float(kms[0]), "stiffness": float(kms[1]), "update": float(kms[2])},
        }
        if not args.no_rows and ws == 1:
            s.close()
            mesh.close()
            torch.cuda.synchronize()
            line["rows"] = {"operator_forms": measure_forms(args.elems), "orders": measure_orders(), "element_path": measure_element(args.elems, args.steps),
                            "rounding": measure_rounding(args.elems),
                            "batched": measure_batched(), "uneven": measure_uneven(),
                            "uneven_small": measure_uneven(200, 8, 24, "c3_uneven_32_small"), "adjoint": measure_adjoint(),
                            "learned_boundary": measure_learned()}
        print(json.dumps(line), flush=True)
    s.close()
    mesh.close()
    if ws > 1:
        dist.destroy_process_group()


# ---------------------------------------------------------------------------------------------
# the other rows of the path: batched shots, uneven groups, adjoint gradient (rank 0, after the
# headline measurement; each frees its device memory before the next)
# ---------------------------------------------------------------------------------------------

def _ev_time(stream, fn):
    import torch
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    fn()
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1)


def measure_forms(n: int = 200, steps: int = 20):
    """Both operator forms of the stencil pass on the headline workload: node-steps/s of the
    direct form (default) and of the difference form (sem_solver_set_operator_form)."""
    import torch
    import semgb
    wl = make_workload("c2", n)
    out = {}
    for name, form in (("direct", semgb.FORM_DIRECT), ("difference", semgb.FORM_DIFFERENCE)):
        mesh, s = semgb.solver_from_workload(wl, semgb.KERNEL_STENCIL)
        s.set_operator_form(form)
        stream = torch.cuda.Stream()
        s.set_stream(stream.cuda_stream)
        s.step(4)
        ms = _ev_time(stream, lambda: s.step(steps)) / steps
        out[name] = {"ms_per_step": ms, "Gnode_steps_per_s": mesh.n_nodes / (ms / 1e3) / 1e9}
        s.close()
        mesh.close()
    return out


def measure_rounding(n: int = 200, steps: int = 20):
    """The stencil pass on the headline workload in both roundings of the operator: the build's
    own (default) and the reference's float-rounded element rows (sem_solver_set_rounding), which
    keeps FP32 results within 1e-5 of the reference on long runs; node-steps/s and the fraction
    of the measured HBM bandwidth at 16 B per node."""
    import torch
    import semgb
    wl = make_workload("c2", n)
    peak, _ = hbm_peak()
    out = {}
    for name, rnd in (("default", semgb.ROUNDING_DEFAULT), ("reference", semgb.ROUNDING_REFERENCE)):
        mesh, s = semgb.solver_from_workload(wl, semgb.KERNEL_STENCIL)
        s.set_rounding(rnd)
        stream = torch.cuda.Stream()
        s.set_stream(stream.cuda_stream)
        s.step(4)
        ms = _ev_time(stream, lambda: s.step(steps)) / steps
        N = mesh.n_nodes
        out[name] = {"ms_per_step": ms, "Gnode_steps_per_s": N / (ms / 1e3) / 1e9,
                     "frac": 16.0 * N / (ms / 1e3) / 1e9 / peak}
        s.close()
        mesh.close()
    return out


def measure_orders(steps: int = 20, nodes_axis: int = 801):
    """The stencil pass at every GLL order on boxes of about nodes_axis^3 nodes (constant 2000
    m/s, 20-element sponge, one source): node-steps/s and the fraction of the measured HBM
    bandwidth at 16 B per node (the headline recipe is order 4)."""
    import torch
    import semgb
    from semgb import workloads as W
    peak, _ = hbm_peak()
    out = {}
    for o in (1, 2, 3, 4, 5):
        e = (nodes_axis - 1) // o
        h = 10.0
        mesh = semgb.Mesh(e, e, e, e * h, e * h, e * h, o)
        mesh.set_velocity(np.full(e ** 3, 2000.0, np.float32))
        dt = W.cfl_dt(h, o, 2000.0)
        s = semgb.Solver(mesh, dt)
        s.set_kernel(semgb.KERNEL_STENCIL)
        stream = torch.cuda.Stream()
        s.set_stream(stream.cuda_stream)
        s.set_sponge(min(20, e // 4), 0.06)
        s.set_source_points(np.array([[e * h / 2] * 3], np.float32), semgb.ricker(steps + 8, dt, 10.0, 1)[None])
        s.step(4)
        ms = _ev_time(stream, lambda: s.step(steps)) / steps
        N = mesh.n_nodes
        out[f"q{o}"] = {"elements": e, "nodes": N, "ms_per_step": ms, "Gnode_steps_per_s": N / (ms / 1e3) / 1e9,
                        "frac": 16.0 * N / (ms / 1e3) / 1e9 / peak}
        s.close()
        mesh.close()
    return out


def measure_element(n: int = 200, steps: int = 20):
    """The reference-shaped element path (SEM_KERNEL_ELEMENT: gather through the connectivity,
    sum-factorised K_e.p, atomic scatter, then the update pass) on the headline workload:
    node-steps/s and each kernel's fraction of the measured HBM bandwidth under its own byte
    model (element pass: connectivity + gather + scatter read-modify-write; update: 24 B)."""
    import torch
    import semgb
    wl = make_workload("c2", n)
    mesh, s = semgb.solver_from_workload(wl, semgb.KERNEL_ELEMENT)
    stream = torch.cuda.Stream()
    s.set_stream(stream.cuda_stream)
    N = mesh.n_nodes
    steps = max(5, min(steps, 20))
    s.step(3)
    step_ms = _ev_time(stream, lambda: s.step(steps)) / steps
    kms = [float(x) for x in s.time_kernels(steps)]
    s.close()
    mesh.close()
    peak, peak_kind = hbm_peak()
    eb = element_bytes_per_node(wl.order)
    return {"workload": wl.name, "nodes": N, "steps": steps, "ms_per_step": step_ms,
            "Gnode_steps_per_s": N / (step_ms / 1e3) / 1e9,
            "element_kernel": {"ms": kms[1], "bytes_per_node": eb,
                               "frac": eb * N / (kms[1] / 1e3) / 1e9 / peak},
            "update_kernel": {"ms": kms[2], "bytes_per_node": 24.0,
                              "frac": 24.0 * N / (kms[2] / 1e3) / 1e9 / peak},
            "peak_kind": peak_kind}


def measure_batched(steps: int = 40, n: int = 100, shots: int = 64):
    """64 shots on one 100^3 Q4 mesh (sem_batch_*, autotuned launch shape) against the plain step
    of one shot on the same mesh: shot-node-steps/s of both, inputs larger than L2."""
    import torch
    import semgb
    from semgb import workloads as W
    wl = W.c3_batched_shots(n, shots, 800)
    mesh = semgb.Mesh(wl.ex, wl.ey, wl.ez, wl.lx, wl.ly, wl.lz, wl.order)
    mesh.set_velocity(wl.vel)
    wav = np.stack([semgb.ricker(wl.nsteps, wl.dt, float(f), 1) for f in wl.f0])
    N = mesh.n_nodes
    stream = torch.cuda.Stream()
    s = semgb.Solver(mesh, wl.dt)
    s.set_kernel(semgb.KERNEL_STENCIL)
    s.set_stream(stream.cuda_stream)
    s.set_sponge(wl.sponge_thickness, wl.sponge_sigma)
    s.set_source_points(wl.src_xyz[:1], wav[:1])
    s.set_receivers(wl.rec_xyz)
    s.step(4)
    plain_ms = _ev_time(stream, lambda: s.step(steps)) / steps
    s.close()
    b = semgb.Batch(mesh, wl.dt, shots)
    b.set_stream(stream.cuda_stream)
    b.set_sponge(wl.sponge_thickness, wl.sponge_sigma)
    b.set_source_points(wl.src_xyz, wav)
    b.set_receivers(wl.rec_xyz)
    b.step(4)
    pick = b.autotune()
    b.step(2)
    batch_ms = _ev_time(stream, lambda: b.step(steps)) / steps
    b.synchronize()
    b.close()
    mesh.close()
    plain = N / (plain_ms / 1e3) / 1e9
    batch = N * shots / (batch_ms / 1e3) / 1e9
    return {"workload": wl.name, "nodes": N, "shots": shots, "steps": steps,
            "plain_Gshot_node_steps_per_s": plain, "plain_ms_per_shot_step": plain_ms,
            "batched_Gshot_node_steps_per_s": batch, "batched_ms_per_step": batch_ms,
            "speedup_vs_plain": batch / plain, "tuning": pick,
            "bytes_per_shot_node": 12.0 + 4.0 / shots,
            "batched_GBps": batch * (12.0 + 4.0 / shots)}


def measure_uneven(steps: int = 20, lo: int = 40, hi: int = 120, name: str = "c3_uneven_32"):
    """32 independent problems (per-axis elements in [lo, hi], orders {2, 3, 4}) advanced as one
    group -- one launch per step over every member's tiles (the default), and each member's own
    launches as branches of one graph -- against the same solvers stepped one after another:
    node-steps/s over the whole batch."""
    import torch
    import semgb
    from semgb import workloads as W
    wls = W.c3_uneven_batch(32, 800, lo=lo, hi=hi)
    stream = torch.cuda.Stream()
    members = [semgb.solver_from_workload(w, semgb.KERNEL_STENCIL) for w in wls]
    nodes = sum(m.n_nodes for m, _ in members)
    for _, s in members:
        s.set_stream(stream.cuda_stream)
        s.step(2)
    seq_ms = _ev_time(stream, lambda: [s.step(steps) for _, s in members])
    res = {}
    for form in (semgb.GROUP_ONE_LAUNCH, semgb.GROUP_BRANCHES):
        g = semgb.Group([s for _, s in members], launch=form)
        g.step(2)
        g.synchronize()
        ms = g.time_step(steps) * steps
        g.synchronize()
        res[form] = (ms, g.launch)
        g.close()
    for m, s in members:
        s.close()
        m.close()
    one_ms, one_form = res[semgb.GROUP_ONE_LAUNCH]
    br_ms, _ = res[semgb.GROUP_BRANCHES]
    return {"workload": name, "problems": len(wls), "elements_per_axis": [lo, hi], "nodes": nodes, "steps": steps,
            "orders": sorted({w.order for w in wls}),
            "one_launch": one_form == semgb.GROUP_ONE_LAUNCH,
            "launches_per_step": 2 if one_form == semgb.GROUP_ONE_LAUNCH else 2 * len(wls),
            "group_Gnode_steps_per_s": nodes * steps / (one_ms / 1e3) / 1e9,
            "branches_Gnode_steps_per_s": nodes * steps / (br_ms / 1e3) / 1e9,
            "sequential_Gnode_steps_per_s": nodes * steps / (seq_ms / 1e3) / 1e9,
            "speedup_vs_sequential": seq_ms / one_ms,
            "branches_speedup_vs_sequential": seq_ms / br_ms}


def measure_adjoint(shots: int = 16, fd_dirs: int = 8, n: int = 96, steps: int = 2000):
    """Adjoint gradient on the 96^3 Q3 two-layer model (16 shots, 256 receivers, 2000 steps,
    checkpoint every 50 steps): wall time per shot gradient through the public API (forward with
    checkpoints, then the gradient call: recompute, adjoint with the imaging term, gradient
    copied to the host), against three plain steps per step (the floor of a checkpointed
    gradient), and a central-difference check of the 16-shot gradient along 8 seeded random
    directions (FP64 reductions)."""
    import torch
    import semgb
    from semgb import workloads as W
    c = W.c4_adjoint(n=n, steps=steps)
    mesh = semgb.Mesh(c["ex"], c["ey"], c["ez"], c["ex"] * c["h"], c["ey"] * c["h"], c["ez"] * c["h"], c["order"])
    mesh.set_velocity(c["vel_elem"])
    a = semgb.Adjoint(mesh, c["dt"], steps, c["checkpoint_every"])
    a.set_sponge(c["sponge_thickness"], c["sponge_sigma"])
    a.set_receivers(c["rec_xyz"])
    wav = semgb.ricker(steps, c["dt"], c["f0"], 1)[None]
    N = mesh.n_nodes
    obs = []
    mesh.set_slowness2(c["m_true"])
    for k in range(shots):
        a.set_source_points(c["src_xyz"][k:k + 1], wav)
        obs.append(a.forward())
    mesh.set_slowness2(c["m0"])
    loss = 0.0
    shot_grads = []
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(shots):
        a.set_source_points(c["src_xyz"][k:k + 1], wav)
        a.forward()
        l, g = a.gradient(obs[k])
        loss += l
        shot_grads.append(g)
    t_grad = (time.perf_counter() - t0) / shots
    # the sum over shots (an application step, in float64 on the host) is outside the timed region
    grad = np.zeros(N, np.float64)
    for g in shot_grads:
        grad += g
    rng = np.random.default_rng(8)
    checks = []
    eps = 1e-3
    for _ in range(fd_dirs):
        dm = c["m0"].astype(np.float64) * rng.standard_normal(N)
        lp = []
        for sgn in (1, -1):
            mesh.set_slowness2((c["m0"] + sgn * eps * dm).astype(np.float32))
            tot = 0.0
            for k in range(shots):
                a.set_source_points(c["src_xyz"][k:k + 1], wav)
                d = a.forward().astype(np.float64)
                tot += 0.5 * float(np.sum((d - obs[k]) ** 2))
            lp.append(tot)
        fd = (lp[0] - lp[1]) / (2 * eps)
        an = float(np.dot(grad, dm))
        checks.append({"fd": fd, "adjoint": an, "rel_err": abs(fd - an) / abs(fd)})
    mesh.set_slowness2(c["m0"])
    a.close()
    # the plain step on the same mesh and model
    s = semgb.Solver(mesh, c["dt"])
    s.set_kernel(semgb.KERNEL_STENCIL)
    stream = torch.cuda.Stream()
    s.set_stream(stream.cuda_stream)
    s.set_sponge(c["sponge_thickness"], c["sponge_sigma"])
    s.set_source_points(c["src_xyz"][:1], wav)
    s.set_receivers(c["rec_xyz"])
    s.step(4)
    plain_ms = _ev_time(stream, lambda: s.step(100)) / 100
    s.close()
    mesh.close()
    return {"workload": c["name"], "nodes": N, "steps": steps, "shots": shots, "receivers": int(len(c["rec_xyz"])),
            "checkpoint_every": c["checkpoint_every"], "loss": loss,
            "seconds_per_shot_gradient": t_grad,
            "plain_ms_per_step": plain_ms,
            "gradient_vs_three_plain_steps": t_grad / (3 * steps * plain_ms / 1e3),
            "Gnode_steps_per_s": 3 * N * steps / t_grad / 1e9,
            "note": "3 passes per gradient: forward with checkpoints, recompute with K.p recorded, adjoint",
            "fd_checks": checks, "fd_max_rel_err": max(ch["rel_err"] for ch in checks)}


def measure_learned(steps_time: int = 40):
    """Learned absorbing boundary.  Quality on a small region of interest (6^3 Q4 elements): the
    network (trained here, on the boundary nodes of a 3-element sponge: rounds of samples, the
    best round kept, then steepest descent on the reflected energy of whole runs with the
    gradient from the adjoint of the time loop) against the same sponge alone and a 20-element
    sponge, reflected energy against a padded run, for the training source and for a source
    position not used in training, after the sample rounds and after the adjoint training; and
    the trained network on a region twice as large (12^3 elements, twice the run length).
    Speed at the 120^3 size: 120^3 Q4 with a 20-element sponge (region of interest 80^3)
    against 86^3 Q4 with a 3-element sponge and the network, ms per step of each time loop
    (CUDA events)."""
    import torch
    import semgb
    from semgb import learned_boundary as LB
    from semgb import workloads as W
    c, h, o = 2000.0, 10.0, 4
    dt = W.cfl_dt(h, o, c)
    common = dict(interior=6, order=o, h=h, c=c, sponge_p=6, f0=40.0, dt=dt, steps=260, src_frac=(0.25, 0.5, 0.5))
    # the thin sponge under the network damps gently (sigma 0.015: a steep 3-element sponge
    # reflects from its own damping gradient); the 20-element sponge it replaces keeps 0.06
    thin_sigma = 0.015
    thin = LB.Setup(sponge_t=3, pad=12, layer=0, sigma=thin_sigma, **common)
    thick = LB.Setup(sponge_t=20, pad=12, layer=0, **common)
    thick_gentle = LB.Setup(sponge_t=20, pad=12, layer=0, sigma=thin_sigma, **common)
    held = dict(common, src_frac=(0.6, 0.35, 0.55))  # source position not used in training
    thin_h = LB.Setup(sponge_t=3, pad=12, layer=0, sigma=thin_sigma, **held)
    net = semgb.Mlp(3)
    t0 = time.perf_counter()
    log = LB.train_network(thin, net, rounds=3, epochs=10, per_step=3000, seed=0)
    t_train = time.perf_counter() - t0
    e_sup, _ = LB.reflected_energy(thin, net)
    e_sup_h, _ = LB.reflected_energy(thin_h, net)
    t0 = time.perf_counter()
    adj_hist = LB.train_through_adjoint(thin, net, iters=30)
    t_adj = time.perf_counter() - t0
    e_net, _ = LB.reflected_energy(thin, net)
    e_thin, _ = LB.reflected_energy(thin, None)
    e_thick, _ = LB.reflected_energy(thick, None)
    e_thick_g, _ = LB.reflected_energy(thick_gentle, None)
    e_net_h, _ = LB.reflected_energy(thin_h, net)
    e_thin_h, _ = LB.reflected_energy(thin_h, None)
    # the same network on a region twice as large (12^3 elements; run length and padding scaled
    # with it, the padded run's own boundary still too far to reflect back in time): how the
    # trained boundary carries over to a larger model than it was trained on
    big = dict(common, interior=12, steps=520)
    thin_b = LB.Setup(sponge_t=3, pad=24, layer=0, sigma=thin_sigma, **big)
    thick_b = LB.Setup(sponge_t=20, pad=24, layer=0, **big)
    t0 = time.perf_counter()
    e_net_b, _ = LB.reflected_energy(thin_b, net)
    e_thin_b, _ = LB.reflected_energy(thin_b, None)
    e_thick_b, _ = LB.reflected_energy(thick_b, None)
    t_big = time.perf_counter() - t0
    # speed at size
    stream = torch.cuda.Stream()
    out = {}
    for name, ne, sponge, use_net in (("sponge20_120c", 120, 20, False), ("net_sponge3_86c", 86, 3, True)):
        mesh = semgb.Mesh(ne, ne, ne, ne * h, ne * h, ne * h, o)
        mesh.set_velocity(np.full(ne ** 3, c, np.float32))
        sol = semgb.Solver(mesh, dt)
        sol.set_kernel(semgb.KERNEL_STENCIL)
        sol.set_stream(stream.cuda_stream)
        sol.set_sponge(sponge, thin_sigma if use_net else 0.06)
        sol.set_source_points(np.array([[ne * h / 2] * 3], np.float32), semgb.ricker(200, dt, 10.0, 1)[None])
        abc = semgb.Abc(sol, net, 0) if use_net else None
        run = (lambda k: abc.step(k)) if use_net else (lambda k: sol.step(k))
        run(4)
        ms = _ev_time(stream, lambda: run(steps_time)) / steps_time
        sol.synchronize()
        out[name] = {"elements": ne, "nodes": mesh.n_nodes, "ms_per_step": ms,
                     "boundary_nodes": abc.n_nodes if abc else 0}
        if abc:
            abc.close()
        sol.close()
        mesh.close()
    net.close()
    return {"quality": {"region": "6^3 Q4 elements", "thin_sponge_sigma": thin_sigma, "sponge20_sigma": thick.sigma,
                        "reflected_energy_network_sponge3": e_net,
                        "reflected_energy_sponge3": e_thin, "reflected_energy_sponge20": e_thick,
                        "reflected_energy_sponge20_sigma_thin": e_thick_g,
                        "held_out_source": {"reflected_energy_network_sponge3": e_net_h,
                                            "reflected_energy_sponge3": e_thin_h,
                                            "reflected_energy_network_samples_only": e_sup_h},
                        "reflected_energy_network_samples_only": e_sup,
                        "region_12c": {"steps": big["steps"], "reflected_energy_network_sponge3": e_net_b,
                                       "reflected_energy_sponge3": e_thin_b, "reflected_energy_sponge20": e_thick_b,
                                       "seconds": t_big},
                        "training": log, "training_seconds": t_train,
                        "adjoint_training": {"loss_per_iteration": adj_hist, "seconds": t_adj,
                                             "method": "steepest descent, line searches along the adjoint gradient and along its sign scaled by each parameter"}},
            "speed": out,
            "speedup_per_step": out["sponge20_120c"]["ms_per_step"] / out["net_sponge3_86c"]["ms_per_step"]}


def run_case(name: str):
    """Small fixed cases for kernel profiles (no JSON line): `batch40` steps a 64-shot batch on a
    40^3 Q4 mesh 6 times; `abc86` runs 6 steps of an 86^3 Q4 mesh with the boundary network;
    `q5_80` runs 6 stencil steps of an 80^3 order-5 box (401^3 nodes, constant 2000 m/s,
    20-element sponge, one source); `uneven_small` steps the 32 small uneven problems (8-24
    elements per axis, orders 2-4) as one group 6 times."""
    import semgb
    from semgb import workloads as W
    if name == "batch40":
        wl = W.c3_batched_shots(40, 64, 50)
        mesh = semgb.Mesh(wl.ex, wl.ey, wl.ez, wl.lx, wl.ly, wl.lz, wl.order)
        mesh.set_velocity(wl.vel)
        wav = np.stack([semgb.ricker(wl.nsteps, wl.dt, float(f), 1) for f in wl.f0])
        b = semgb.Batch(mesh, wl.dt, 64)
        b.set_sponge(wl.sponge_thickness, wl.sponge_sigma)
        b.set_source_points(wl.src_xyz, wav)
        b.set_receivers(wl.rec_xyz)
        b.step(6)
        b.synchronize()
        print("batch40 ok", mesh.n_nodes)
    elif name == "abc86":
        ne, o, h, c = 86, 4, 10.0, 2000.0
        dt = W.cfl_dt(h, o, c)
        mesh = semgb.Mesh(ne, ne, ne, ne * h, ne * h, ne * h, o)
        mesh.set_velocity(np.full(ne ** 3, c, np.float32))
        sol = semgb.Solver(mesh, dt)
        sol.set_kernel(semgb.KERNEL_STENCIL)
        sol.set_sponge(3, 0.06)
        sol.set_source_points(np.array([[ne * h / 2] * 3], np.float32), semgb.ricker(200, dt, 10.0, 1)[None])
        net = semgb.Mlp(3)
        abc = semgb.Abc(sol, net, 0)
        abc.step(6)
        sol.synchronize()
        print("abc86 ok", abc.n_nodes)
    elif name == "q5_80":
        ne, o, h, c = 80, 5, 10.0, 2000.0
        dt = W.cfl_dt(h, o, c)
        mesh = semgb.Mesh(ne, ne, ne, ne * h, ne * h, ne * h, o)
        mesh.set_velocity(np.full(ne ** 3, c, np.float32))
        sol = semgb.Solver(mesh, dt)
        sol.set_kernel(semgb.KERNEL_STENCIL)
        sol.set_sponge(20, 0.06)
        sol.set_source_points(np.array([[ne * h / 2] * 3], np.float32), semgb.ricker(200, dt, 10.0, 1)[None])
        sol.step(6)
        sol.synchronize()
        print("q5_80 ok", mesh.n_nodes)
    elif name == "uneven_small":
        wls = W.c3_uneven_batch(32, 800, lo=8, hi=24)
        members = [semgb.solver_from_workload(w, semgb.KERNEL_STENCIL) for w in wls]
        g = semgb.Group([s for _, s in members])
        g.step(6)
        g.synchronize()
        print("uneven_small ok", sum(m.n_nodes for m, _ in members), "one launch:", g.launch == semgb.GROUP_ONE_LAUNCH)
        g.close()
        for m, s in members:
            s.close()
            m.close()
    else:
        raise SystemExit(f"unknown case {name}")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["c2", "c1"], default="c2")
    ap.add_argument("--kernel", choices=["auto", "element", "stencil"], default="auto")
    ap.add_argument("--elems", type=int, default=200, help="elements per axis of the c2 recipe")
    ap.add_argument("--cpu-elems", type=int, default=100,
                    help="CPU sub-box of the workload (elements per axis), timed by both the cpu_baseline leg "
                         "and --impl reference")
    ap.add_argument("--cpu-steps", type=int, default=6, help="cpu_baseline steps")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--tile", choices=["auto", "default", "square"], default="auto",
                    help="tile shape of the stencil pass (auto: chosen per box; square: order 4 only)")
    ap.add_argument("--no-rows", action="store_true", help="skip the element-path / batched / uneven / adjoint / learned-boundary rows")
    ap.add_argument("--case", choices=["batch40", "abc86", "q5_80", "uneven_small"], default=None,
                    help="run a small fixed case for a kernel profile instead of the benchmark")
    args = ap.parse_args()
    if args.case:
        run_case(args.case)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
