"""Learned absorbing boundary: the network's GPU kernels (BF16 tensor-core forward, training pass)
against the CPU oracle, the strip correction against the oracle on the solver's own features, a
zero network reproducing the plain solver, and the trained network reducing the reflected energy
of the same thin sponge."""
import numpy as np
import pytest

from oracle import mlp_oracle as M

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _params(seed, scale=0.3):
    rng = np.random.default_rng(seed)
    p = rng.standard_normal(M.N_PARAMS) * scale
    return p.astype(np.float32)


def test_forward_matches_oracle(semgb_lib, cuda_device):
    semgb = semgb_lib
    net = semgb.Mlp(1)
    p = _params(2)
    net.params = p
    x = np.random.default_rng(3).uniform(-1, 1, (1000, 81)).astype(np.float32)
    y = net.forward(x)
    yo, _ = M.forward(p, x)
    assert rel_l2(y, yo) < 2e-3


def test_loss_and_gradient_match_oracle(semgb_lib, cuda_device):
    semgb = semgb_lib
    net = semgb.Mlp(1)
    p = _params(4, 0.2)
    net.params = p
    rng = np.random.default_rng(5)
    x = rng.uniform(-1, 1, (777, 81)).astype(np.float32)  # not a multiple of the 128-row tile
    t = rng.standard_normal(777).astype(np.float32)
    loss, g = net.loss_grad(x, t)
    lo, go = M.loss_grad(p, x, t)
    assert abs(loss - lo) <= 2e-3 * lo
    assert rel_l2(g, go) < 5e-3
    for name, (a, b) in {"W1": (0, 64 * 81), "W2": (64 * 81 + 64, 64 * 81 + 64 + 4096)}.items():
        assert rel_l2(g[a:b], go[a:b]) < 5e-3, name


def test_training_reduces_loss(semgb_lib, cuda_device):
    semgb = semgb_lib
    net = semgb.Mlp(7)
    rng = np.random.default_rng(8)
    x = rng.uniform(-1, 1, (20000, 81)).astype(np.float32)
    t = (np.tanh(x[:, :27].sum(1) * 0.3) - 0.2 * x[:, 40]).astype(np.float32)
    l0, _ = net.loss_grad(x, t)
    losses = net.train(x, t, epochs=15, batch=1024, lr=2e-3, seed=1)
    l1, _ = net.loss_grad(x, t)
    assert l1 < 0.05 * l0, (l0, l1, losses)


def test_training_is_reproducible(semgb_lib, cuda_device):
    """Per-CTA partial gradients are added in CTA order (no atomics): the same seed and data give
    the same parameters and losses bit for bit, so the boundary's training is repeatable."""
    semgb = semgb_lib
    rng = np.random.default_rng(18)
    x = rng.uniform(-1, 1, (9000, 81)).astype(np.float32)
    t = (np.tanh(x[:, :27].sum(1) * 0.3) - 0.2 * x[:, 40]).astype(np.float32)
    runs = []
    for _ in range(2):
        net = semgb.Mlp(17)
        losses = net.train(x, t, epochs=3, batch=1000, lr=2e-3, seed=5)
        g = net.loss_grad(x, t)
        runs.append((net.params, losses, g[0], g[1]))
        net.close()
    assert np.array_equal(runs[0][0], runs[1][0])
    assert np.array_equal(runs[0][1], runs[1][1])
    assert runs[0][2] == runs[1][2] and np.array_equal(runs[0][3], runs[1][3])


def _solver(semgb, wl):
    mesh, s = semgb.solver_from_workload(wl, semgb.KERNEL_STENCIL)
    return mesh, s


def test_zero_network_is_the_plain_step(semgb_lib, cuda_device):
    semgb = semgb_lib
    from semgb import workloads as W
    wl = W.small_random(8, 7, 6, 3, 40, seed=31, nsrc=1, nrec=6)
    m1, plain = _solver(semgb, wl)
    plain.step(40)
    m2, s = _solver(semgb, wl)
    net = semgb.Mlp(0)
    net.params = np.zeros(net.n_params, np.float32)
    abc = semgb.Abc(s, net, 1)
    abc.step(40)
    assert np.array_equal(s.pressure(), plain.pressure())
    assert np.array_equal(s.traces(), plain.traces())


def test_strip_correction_matches_oracle(semgb_lib, cuda_device):
    semgb = semgb_lib
    from semgb import workloads as W
    wl = W.small_random(8, 8, 8, 2, 30, seed=32, nsrc=1, nrec=4)
    mesh, s = _solver(semgb, wl)
    net = semgb.Mlp(0)
    p = _params(9, 0.05)
    net.params = p
    abc = semgb.Abc(s, net, 2)
    abc.step(29)  # fields reach the strip; history filled by the corrections
    s.step(1)     # one plain step; the correction for it is applied below
    x, sc = abc.features()
    nodes = abc.nodes()
    before = s.pressure()
    abc.correct()
    got = s.pressure()[nodes] - before[nodes]
    yo, _ = M.forward(p, x)
    want = sc * yo
    big = np.abs(want) > 1e-3 * np.abs(want).max()
    assert big.sum() > 100
    assert rel_l2(got[big], want[big]) < 5e-3
    # only the strip changes
    other = np.ones(mesh.n_nodes, bool)
    other[nodes] = False
    assert np.array_equal(s.pressure()[other], before[other])


def test_trained_network_reduces_reflections(semgb_lib, cuda_device):
    """Thin sponge (3 elements) with and without the trained network on the boundary nodes,
    against a padded run: the network (best of its training rounds) lowers the reflected energy
    in the interior, for the training source and for a source position not used in training.
    Training is bit-reproducible (per-CTA gradient sums added in order), so the ratios are fixed:
    measured 0.590 for the training source (bound 0.6) and 0.394 for the held-out source (bound
    0.75)."""
    semgb = semgb_lib
    from semgb import learned_boundary as LB
    from semgb import workloads as W
    c, h, o = 2000.0, 10.0, 4
    dt = W.cfl_dt(h, o, c)
    common = dict(interior=6, sponge_t=3, order=o, h=h, c=c, pad=12, sponge_p=6, layer=0, f0=40.0, dt=dt,
                  steps=260)
    s = LB.Setup(src_frac=(0.25, 0.5, 0.5), **common)
    held = LB.Setup(src_frac=(0.6, 0.35, 0.55), **common)
    net = semgb.Mlp(3)
    log = LB.train_network(s, net, rounds=3, epochs=10, per_step=3000, seed=0)
    print(log)
    assert log[0]["samples"] > 50000
    for setup, bound in ((s, 0.6), (held, 0.75)):
        e_plain, _ = LB.reflected_energy(setup, None)
        e_net, _ = LB.reflected_energy(setup, net)
        print(f"reflected energy: sponge only {e_plain:.3e}, sponge + network {e_net:.3e}")
        assert e_net < bound * e_plain


@pytest.mark.parametrize("sponge", [0, 2])
def test_face_tiled_correction_matches_oracle(semgb_lib, cuda_device, sponge):
    """Boundary nodes (layer 0) are corrected by the face-tiled kernel: each tile stages its three
    levels on the face and the plane inside it once and builds every node's features from there,
    and writes p^n of the two-node shell for the next step.  After 29 corrected steps and one
    plain one, the correction equals the oracle network on the features the host gathers from the
    same levels, every face (edges and corners included) is corrected, and nothing else changes."""
    semgb = semgb_lib
    from semgb import workloads as W
    wl = W.small_random(9, 7, 8, 2, 30, seed=33, nsrc=1, nrec=4, sponge=sponge)
    mesh, s = _solver(semgb, wl)
    net = semgb.Mlp(0)
    p = _params(10, 0.05)
    net.params = p
    abc = semgb.Abc(s, net, 0)
    abc.step(29)
    s.step(1)
    x, sc = abc.features()
    nodes = abc.nodes()
    nx, ny, nz = wl.ex * 2 + 1, wl.ey * 2 + 1, wl.ez * 2 + 1
    assert len(nodes) == nx * ny * nz - (nx - 2) * (ny - 2) * (nz - 2)
    before = s.pressure()
    abc.correct()
    after = s.pressure()
    yo, _ = M.forward(p, x)
    want = sc * np.clip(yo, -1.0, 1.0)
    got = after[nodes]
    big = np.abs(want) > 1e-3 * np.abs(want).max()
    assert big.sum() > 100
    assert rel_l2(got[big], want[big]) < 5e-3
    other = np.ones(mesh.n_nodes, bool)
    other[nodes] = False
    assert np.array_equal(after[other], before[other])
