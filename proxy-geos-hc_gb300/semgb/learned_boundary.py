"""Learned absorbing boundary: training data from padded-domain runs, training, evaluation.

A truncated problem (mesh T: the region of interest plus a thin sponge) and a padded problem
(mesh P: the same region with `pad` extra elements on every side, its own sponge far away) share
the element size, order, velocity and source.  The padded run gives the reflection-free field
on T's nodes.

Training data (teacher forcing): at every step n, T's levels are set to the padded run's
(p^n, p^{n-1}) on T's nodes, T takes one plain step, and each strip node contributes the
network inputs of that step (sem_abc_features) with the target p_P^{n+1} / scale on boundary
nodes (the face value of the padded run) or (p_P^{n+1} - p_T^{n+1}) / scale on interior strip
nodes (the correction that would have reproduced the padded run).

Evaluation: T runs from rest with and without the network; the reflected energy is the sum over
steps and the nodes of the region of interest of (p_T - p_P)^2, divided by the same sum of p_P^2.
Set-ups with different sponges around the same region of interest compare directly.

Training through the adjoint (train_through_adjoint): the reflected energy of a whole run of T
is itself the loss, its gradient with respect to the network's parameters comes from the adjoint
of the time loop (sem_abc_bptt), and Adam steps follow it.
"""
from __future__ import annotations

import time
from dataclasses import dataclass

import numpy as np

from . import LEVEL_CURRENT, LEVEL_PREVIOUS, KERNEL_STENCIL, Abc, Mesh, Mlp, Solver, ricker


@dataclass
class Setup:
    interior: int            # elements per axis of the region of interest
    sponge_t: int            # sponge of T around it (elements): T has interior + 2 sponge_t elements
    order: int
    h: float
    c: float                 # velocity (m/s)
    pad: int                 # extra elements per side of the padded mesh P around T
    sponge_p: int            # sponge of P (elements)
    layer: int               # strip of the network (elements; 0: the boundary nodes)
    f0: float
    dt: float
    steps: int
    src_frac: tuple = (0.5, 0.5, 0.5)  # source position as a fraction of the region of interest
    sigma: float = 0.06

    @property
    def ex(self):
        return self.interior + 2 * self.sponge_t

    @property
    def nx_t(self):
        return self.ex * self.order + 1

    @property
    def off(self):
        return self.pad * self.order


def _solver(s: Setup, ne: int, sponge: int, shift: float):
    """Box of ne elements whose region of interest starts at `shift` metres."""
    L = ne * s.h
    mesh = Mesh(ne, ne, ne, L, L, L, s.order)
    mesh.set_velocity(np.full(ne ** 3, s.c, np.float32))
    sol = Solver(mesh, s.dt)
    sol.set_kernel(KERNEL_STENCIL)
    if sponge > 0:
        sol.set_sponge(sponge, s.sigma)
    Li = s.interior * s.h
    xyz = np.array([[shift + f * Li for f in s.src_frac]], np.float32)
    sol.set_source_points(xyz, ricker(s.steps + 2, s.dt, s.f0, 1)[None])
    return mesh, sol


def make_solvers(s: Setup):
    """(mesh_T, solver_T), (mesh_P, solver_P) with the source at the same physical point."""
    return (_solver(s, s.ex, s.sponge_t, s.sponge_t * s.h),
            _solver(s, s.ex + 2 * s.pad, s.sponge_p, (s.pad + s.sponge_t) * s.h))


def restrict(s: Setup, field_p):
    """Field of mesh P (reference numbering) restricted to T's nodes."""
    n_p = (s.ex + 2 * s.pad) * s.order + 1
    f = np.asarray(field_p).reshape(n_p, n_p, n_p)  # [y][z][x]
    o, n = s.off, s.nx_t
    return np.ascontiguousarray(f[o:o + n, o:o + n, o:o + n]).reshape(-1)


def _target(s: Setup, ref, plain):
    """Network target before the division by the scale: the padded run's value on boundary nodes
    (layer 0), the correction from T's plain update to it on interior strip nodes."""
    return ref if s.layer == 0 else ref - plain


def teacher_forced_samples(s: Setup, per_step: int = 4000, seed: int = 0, min_rel_scale: float = 1e-4):
    """(x [N][81], t [N]) from the padded run, `per_step` strip nodes sampled per step among
    those whose field is not negligible."""
    rng = np.random.default_rng(seed)
    (mt, st), (mp, sp) = make_solvers(s)
    net0 = Mlp(seed)  # not used for the plain step; Abc needs one to gather features
    abc = Abc(st, net0, s.layer)
    strip = abc.nodes()
    xs, ts = [], []
    smax = 0.0
    for n in range(s.steps):
        pc = restrict(s, sp.pressure(LEVEL_CURRENT))
        pq = restrict(s, sp.pressure(LEVEL_PREVIOUS))
        st.set_pressure(LEVEL_CURRENT, pc)
        st.set_pressure(LEVEL_PREVIOUS, pq)
        abc.set_history(pq)
        st.step(1)
        sp.step(1)
        x, sc = abc.features()
        target = _target(s, restrict(s, sp.pressure(LEVEL_CURRENT))[strip], st.pressure(LEVEL_CURRENT)[strip])
        smax = max(smax, float(sc.max()))
        keep = np.nonzero(sc > min_rel_scale * max(smax, 1e-30))[0]
        if len(keep) == 0:
            continue
        pick = rng.choice(keep, min(per_step, len(keep)), replace=False)
        xs.append(x[pick])
        ts.append((target[pick] / sc[pick]).astype(np.float32))
    for o in (abc, net0, st, sp, mt, mp):
        o.close()
    if not xs:
        return np.zeros((0, Mlp.N_IN), np.float32), np.zeros(0, np.float32)
    return np.concatenate(xs), np.concatenate(ts)


def rollout_samples(s: Setup, net: Mlp, per_step: int = 4000, seed: int = 0, min_rel_scale: float = 1e-4,
                    blowup: float = 1e3):
    """(x, t) from a run of T with the network (the states the method itself produces): at every
    step the target is the correction that would bring T's new level on the strip to the padded
    run's, from T's own plain update.  Stops early if T's field exceeds `blowup` times the padded
    run's largest value."""
    rng = np.random.default_rng(seed)
    (mt, st), (mp, sp) = make_solvers(s)
    abc = Abc(st, net, s.layer)
    strip = abc.nodes()
    xs, ts = [], []
    smax = 0.0
    pmax = 1e-30
    for n in range(s.steps):
        st.step(1)
        sp.step(1)
        x, sc = abc.features()
        ref = restrict(s, sp.pressure(LEVEL_CURRENT))
        pmax = max(pmax, float(np.abs(ref).max()))
        target = _target(s, ref[strip], st.pressure(LEVEL_CURRENT)[strip])
        smax = max(smax, float(sc.max()))
        if smax > blowup * pmax:
            break
        keep = np.nonzero(sc > min_rel_scale * max(smax, 1e-30))[0]
        if len(keep):
            pick = rng.choice(keep, min(per_step, len(keep)), replace=False)
            xs.append(x[pick])
            ts.append(np.clip(target[pick] / sc[pick], -1.0, 1.0).astype(np.float32))
        abc.correct()
    for o in (abc, st, sp, mt, mp):
        o.close()
    if not xs:
        return np.zeros((0, Mlp.N_IN), np.float32), np.zeros(0, np.float32)
    return np.concatenate(xs), np.concatenate(ts)


def train_network(s: Setup, net: Mlp, rounds: int = 3, epochs: int = 12, per_step: int = 3000, batch: int = 2048,
                  lr: float = 1e-3, seed: int = 0, select: bool = True):
    """Teacher-forced samples first, then `rounds` rounds of samples from runs with the current
    network, each followed by training on everything gathered so far.  With `select`, every
    round's network is scored by its reflected energy on `s` and the best one is kept (the
    rounds do not improve monotonically: the teacher-forced network alone reflects more than
    the sponge, the first rollout round far less, later ones drift).  Returns the per-round
    sample counts, final losses and scores."""
    xs, ts = [], []
    x, t = teacher_forced_samples(s, per_step, seed)
    xs.append(x)
    ts.append(np.clip(t, -1.0, 1.0))
    log = []
    best = None  # (energy, params, round)
    for r in range(rounds + 1):
        X, Tt = np.concatenate(xs), np.concatenate(ts)
        losses = net.train(X, Tt, epochs=epochs, batch=batch, lr=lr, seed=seed + r)
        entry = {"round": r, "samples": int(len(X)), "loss": float(losses[-1]) if len(losses) else None}
        if select:
            e, _ = reflected_energy(s, net)
            entry["reflected_energy"] = e
            if best is None or e < best[0]:
                best = (e, net.params.copy(), r)
        log.append(entry)
        if r < rounds:
            x, t = rollout_samples(s, net, per_step, seed + 100 + r)
            xs.append(x)
            ts.append(t)
    if select and best is not None:
        net.params = best[1]
        log.append({"selected_round": best[2], "reflected_energy": best[0]})
    return log


def descent_step(theta, g, e: float, step: float, step0: float, loss_at, method: str = "line+relative"):
    """One iteration of train_through_adjoint's searches from parameters theta (FP32) with loss e
    and gradient g: returns (theta, step, ok), ok False when the gradient is zero or not finite.
    loss_at(p) evaluates the loss at parameters p.  The gradient search tries step * 2^k along the
    normalised negative gradient (k = -2..2); "line+relative" also tries -sign(g) * max(|theta|,
    1e-3) * 2^-j (j = 9, 7, 5, 3).  The lowest loss below e is taken (the relative search on a
    tie); `step` follows an accepted gradient step, is quartered when neither search lowers the
    loss, and is reset to step0 once it has shrunk a thousandfold."""
    d = -g
    nrm = float(np.linalg.norm(d))
    if not np.isfinite(nrm) or nrm == 0.0:
        return theta, step, False
    d = (d / nrm).astype(np.float32)
    tried = [(loss_at(theta + step * (2.0 ** k) * d), k) for k in (-2, -1, 0, 1, 2)]
    lk, k = min(tried)
    lr_best, cand = np.inf, None
    if method == "line+relative":
        rel = (-np.sign(g) * np.maximum(np.abs(theta.astype(np.float64)), 1e-3)).astype(np.float32)
        for j in (9, 7, 5, 3):
            th = theta + np.float32(2.0 ** -j) * rel
            lj = loss_at(th)
            if lj < lr_best:
                lr_best, cand = lj, th
    if lr_best < min(lk, e):
        return cand, step, True
    if lk < e:
        return theta + step * (2.0 ** k) * d, step * 2.0 ** k, True
    step *= 0.25
    if step < step0 * 1e-3:
        step = step0  # no progress at any step length: search again from the start
    return theta, step, True


def train_through_adjoint(s, net: Mlp, iters: int = 20, step: float = 0.01, lr: float = 1e-3,
                          method: str = "line+relative", keep_best: bool = True):
    """Trains the network on the reflected energy itself, through the adjoint of the whole time
    loop.  `s` is one Setup or a list of Setups (e.g. several source positions around the same
    region of interest: the loss is then the mean of theirs).  Every evaluation runs T with the
    network from rest (s.steps steps); a set-up's loss is sum over steps and region-of-interest
    nodes of (p_T - p_P)^2 / sum p_P^2 (the padded run P restricted to T), and its gradient with
    respect to the network's parameters comes from the adjoint pass (sem_abc_bptt: the
    network's backward kernels at the boundary nodes and the adjoint leapfrog of the stencil
    pass).  Layer 0 only.

    method "line": steepest descent with a search along the normalised negative gradient (steps
    step * 2^k, k = -2..2, the best kept; `step` follows the accepted one, quartered when none
    lowers the loss and reset when it has shrunk a thousandfold): a 260-step rollout makes the
    loss rough, and a search along the exact gradient never accepts a step that raises it.
    method "line+relative": the same search, and beside it one along -sign(g) scaled by each
    parameter's magnitude (relative steps 2^-9 .. 2^-3): the BF16 weight matrices keep 8
    significant bits, so steps along the normalised gradient small enough to lower a rough loss
    often change no weight at all, while a relative step moves every weight whose gradient is
    not zero; the lower of the two searches is taken.
    method "adam": one Adam step of rate `lr` per gradient.  With keep_best the parameters of
    the lowest loss seen are kept.  Returns the loss after every iteration (entry 0: before
    training)."""
    setups = list(s) if isinstance(s, (list, tuple)) else [s]
    if any(x.layer != 0 for x in setups):
        raise ValueError("training through the adjoint needs the network on the boundary nodes (layer 0)")
    runs = []  # (roi, ref, den, abc, objects to close)
    for x in setups:
        (mt, st), (mp, sp) = make_solvers(x)
        mask = interior_mask(x)
        roi = np.nonzero(mask)[0]
        ref = np.empty((x.steps, len(roi)), np.float32)
        for n in range(x.steps):
            sp.step(1)
            ref[n] = restrict(x, sp.pressure(LEVEL_CURRENT))[mask]
        den = max(float(np.sum(ref.astype(np.float64) ** 2)), 1e-300)
        abc = Abc(st, net, 0)
        runs.append((roi, ref, den, abc, (abc, st, sp, mt, mp)))

    def evaluate(grad: bool):
        loss, g = 0.0, None
        for roi, ref, den, abc, _ in runs:
            l, gg = abc.bptt(roi, ref, grad=grad)
            loss += l / den / len(runs)
            if grad:
                g = gg.astype(np.float64) / den / len(runs) if g is None else g + gg.astype(np.float64) / den / len(runs)
        return loss, g

    def loss_at(p):
        net.params = p
        return evaluate(False)[0]

    theta = net.params.copy()
    step0 = step
    history = []
    best = (np.inf, theta.copy())
    for it in range(iters + 1):
        net.params = theta
        e, g = evaluate(it < iters)
        history.append(e)
        if e < best[0]:
            best = (e, theta.copy())
        if it == iters:
            break
        if method == "adam":
            net.adam_step(g.astype(np.float32), lr)
            theta = net.params.copy()
            continue
        theta, step, ok = descent_step(theta, g, e, step, step0, loss_at, method)
        if not ok:
            break
    net.params = best[1] if keep_best else theta
    for *_, objs in runs:
        for o in objs:
            o.close()
    return history


def interior_mask(s: Setup):
    """T's nodes in the region of interest (reference numbering)."""
    n = s.nx_t
    lo, hi = s.sponge_t * s.order, (s.sponge_t + s.interior) * s.order
    i = np.arange(n)
    a = (i >= lo) & (i <= hi)
    return (a[:, None, None] & a[None, :, None] & a[None, None, :]).reshape(-1)


def reflected_energy(s: Setup, net: Mlp | None, sample_every: int = 4):
    """Reflected energy of T (with the network when given) against the padded run, over the
    interior of T; also the wall time per step of T's time loop."""
    (mt, st), (mp, sp) = make_solvers(s)
    abc = Abc(st, net, s.layer) if net is not None else None
    mask = interior_mask(s)
    num = den = 0.0
    t_loop = 0.0
    for n0 in range(0, s.steps, sample_every):
        k = min(sample_every, s.steps - n0)
        t0 = time.perf_counter()
        if abc is not None:
            abc.step(k)
        else:
            st.step(k)
        st.synchronize()
        t_loop += time.perf_counter() - t0
        sp.step(k)
        ref = restrict(s, sp.pressure(LEVEL_CURRENT))[mask].astype(np.float64)
        got = st.pressure(LEVEL_CURRENT)[mask].astype(np.float64)
        num += float(np.sum((got - ref) ** 2))
        den += float(np.sum(ref ** 2))
    for o in (abc, st, sp, mt, mp):
        if o is not None:
            o.close()
    return num / max(den, 1e-300), t_loop / s.steps
