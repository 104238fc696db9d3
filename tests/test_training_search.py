"""The line searches of the learned boundary's adjoint training (learned_boundary.descent_step),
on the host with a synthetic loss that, like the network's, reads most parameters through BF16
rounding: the searches never raise the loss, and where the gradient steps are too short to
change any BF16 value (as they must be on the rough loss of a whole rollout), the relative
search still moves the BF16 parameters."""
import numpy as np

from semgb import learned_boundary as LB


def bf16(x):
    """Round FP32 to BF16 (nearest, ties to even), returned as FP32."""
    u = np.asarray(x, np.float32).view(np.uint32)
    r = (u + np.uint32(0x7FFF) + ((u >> np.uint32(16)) & np.uint32(1))) & np.uint32(0xFFFF0000)
    return r.astype(np.uint32).view(np.float32)


def make_problem(seed=0, n_w=8000, n_f=200):
    """Targets t (BF16-exact for the first n_w parameters, read through BF16 rounding), start
    on the BF16 value nearest 2^-5 relative above them (a grid point: the nearest rounding
    boundary is half a BF16 step away), and FP32 parameters 0.05 off theirs."""
    rng = np.random.default_rng(seed)
    t = rng.uniform(0.2, 1.0, n_w + n_f).astype(np.float32)
    t[:n_w] = bf16(t[:n_w])
    theta = t.copy()
    theta[:n_w] = bf16(theta[:n_w] * np.float32(1 + 2.0 ** -5))
    theta[n_w:] += np.float32(0.05)

    def seen(p):
        q = np.asarray(p, np.float32).copy()
        q[:n_w] = bf16(q[:n_w])
        return q.astype(np.float64)

    def loss(p):
        return float(np.sum((seen(p) - t) ** 2))

    def grad(p):
        return 2.0 * (seen(p) - t)  # the gradient at the parameters the loss reads

    return theta, loss, grad


def test_searches_never_raise_the_loss():
    for method in ("line", "line+relative"):
        theta, loss, grad = make_problem()
        step = step0 = 0.01
        hist = [loss(theta)]
        for _ in range(25):
            theta, step, ok = LB.descent_step(theta, grad(theta), hist[-1], step, step0, loss, method)
            if not ok:  # fitted exactly: no gradient left
                break
            hist.append(loss(theta))
        assert all(b <= a for a, b in zip(hist, hist[1:])), method
        assert hist[-1] < 1e-3 * hist[0], method


def test_relative_search_moves_bf16_parameters():
    theta, loss, grad = make_problem(n_f=0)
    e, g = loss(theta), grad(theta)
    # gradient steps of at most 4e-5 along a unit direction, against half a BF16 step of at least
    # 2^-9 * 0.2: no BF16 value changes
    th_line, _, ok = LB.descent_step(theta, g, e, 1e-5, 0.01, loss, "line")
    assert ok and loss(th_line) == e
    assert np.array_equal(bf16(th_line), bf16(theta))
    th_rel, _, ok = LB.descent_step(theta, g, e, 1e-5, 0.01, loss, "line+relative")
    assert ok and loss(th_rel) < 0.5 * e
    assert np.count_nonzero(bf16(th_rel) != bf16(theta)) > 0.9 * theta.size


def test_step_length_follows_the_searches():
    theta, loss, grad = make_problem(n_f=0)
    e, g = loss(theta), grad(theta)
    # nothing lowers the loss: the step is quartered, and reset once it has shrunk a thousandfold
    _, step, _ = LB.descent_step(theta, g, e, 1e-3, 1e-3, loss, "line")
    assert step == 0.25e-3
    _, step, _ = LB.descent_step(theta, g, e, 1e-6, 1e-3, loss, "line")
    assert step == 1e-3


def test_zero_gradient_stops():
    theta, loss, _ = make_problem()
    out, step, ok = LB.descent_step(theta, np.zeros(theta.size), loss(theta), 0.01, 0.01, loss)
    assert not ok and out is theta and step == 0.01
