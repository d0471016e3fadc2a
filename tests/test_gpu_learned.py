"""Learned warm start on the GPU: network kernels against the FP64 oracle
(with BF16 rounding emulated at the kernels' rounding points), training, and
what the trained network gains over plain Gauss-Newton."""
import numpy as np
import pytest

from conftest import make_setup

pytestmark = pytest.mark.gpu


def _rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _random_net(mp, torch, dims, seed):
    net = mp.MLP(*dims, seed=seed)
    rng = np.random.default_rng(seed)
    flat = np.zeros(net.param_count, np.float32)
    o = net.offsets
    i, h1, h2, out = dims
    for k, (rows, cols) in enumerate(((h1, i), (h2, h1), (out, h2))):
        flat[o[2 * k]:o[2 * k] + rows * cols] = (rng.standard_normal(rows * cols) / np.sqrt(cols)).astype(np.float32)
        flat[o[2 * k + 1]:o[2 * k + 1] + rows] = 0.1 * rng.standard_normal(rows).astype(np.float32)
    net.set_parameters(torch.tensor(flat, device="cuda"))
    return net


@pytest.mark.parametrize("batch", [128, 100])
def test_mlp_forward_and_gradients_match_oracle(batch):
    from oracle import mlp_oracle as mo
    import mpflow_gb300 as mp
    import torch
    dims = (128, 256, 128, 384)
    net = _random_net(mp, torch, dims, seed=3)
    rng = np.random.default_rng(7)
    x = rng.standard_normal((batch, dims[0])).astype(np.float32)
    valid = 300
    t = rng.standard_normal((batch, valid)).astype(np.float32)
    xt, tt = torch.tensor(x, device="cuda"), torch.tensor(t, device="cuda")
    params = net.unpack(net.parameters())
    # inference
    y = net.forward(xt).cpu().numpy()
    yo = mo.forward(params, x)["Y"]
    assert _rel(y, yo) < 2e-3, _rel(y, yo)
    # loss and gradients
    loss = net.backward(xt, tt, valid=valid)
    lo, go = mo.loss_and_gradients(params, x, t, valid)
    assert abs(loss - lo) <= 1e-3 * lo
    grads = net.unpack(net.gradients())
    for name, g, r in zip(("dW1", "db1", "dW2", "db2", "dW3", "db3"), grads, go):
        assert _rel(g, r) < 1e-2, (name, _rel(g, r))


def test_mlp_training_reduces_loss():
    import mpflow_gb300 as mp
    import torch
    dims = (128, 256, 256, 256)
    net = mp.MLP(*dims, seed=1)
    rng = np.random.default_rng(2)
    A = rng.standard_normal((dims[0], dims[3])).astype(np.float32) / np.sqrt(dims[0])
    x = rng.standard_normal((512, dims[0])).astype(np.float32)
    t = np.tanh(x @ A).astype(np.float32)
    xt, tt = torch.tensor(x, device="cuda"), torch.tensor(t, device="cuda")
    first = net.backward(xt[:256], tt[:256])
    for step in range(200):
        b = (step % 2) * 256
        net.backward(xt[b:b + 256], tt[b:b + 256], want_loss=False)
        net.adam(2e-3)
    last = net.backward(xt[:256], tt[:256])
    assert last < 0.2 * first, (first, last)


def test_learned_warm_start_saves_gauss_newton_updates():
    """Trained on forward-model pairs, the network's start needs fewer
    Gauss-Newton updates than the homogeneous start on held-out frames, and
    every frame still reaches the target."""
    import mpflow_gb300 as mp
    from mpflow_gb300.learned import generate_pairs, inclusion_frames, round_up, train_warm_start
    import torch
    mesh, src, _ = make_setup(rings=20, ports=16, logarithmic=True)
    E = mesh.elements.shape[0]
    model = mp.EIT(mesh, src, 1.0, logarithmic=True)
    cent = mesh.nodes[mesh.elements].mean(axis=1)
    rng = np.random.default_rng(11)
    opts = mp.SolveOptions(tol=1e-6, max_iter=4000)
    Vtr, gtr = generate_pairs(model, inclusion_frames(cent, 2048, rng), batch=128, options=opts)
    L = Vtr.shape[1] * Vtr.shape[2]
    net = mp.MLP(L, 512, 512, round_up(E, 128), seed=5)
    losses, _ = train_warm_start(model, net, Vtr, gtr, epochs=40, batch=256, lr=1e-3, snr_db=60.0)
    assert losses[-1] < 0.8 * losses[0], losses
    # held-out frames, noise-free measurements from the refined forward model
    gte = inclusion_frames(cent, 32, np.random.default_rng(99))
    Vte = model.solve(torch.tensor(gte, device="cuda"), mp.SolveOptions(tol=1e-6, refine_tol=1e-10)).contiguous()
    _, J0 = model.solve(torch.zeros((1, E), device="cuda"), mp.SolveOptions(tol=1e-6), jacobian=True)
    lam = 2e-2 * float(J0.norm() / np.sqrt(J0.shape[1]))
    target = 1e-3
    g0 = torch.zeros((32, E), device="cuda")
    it_plain, res_plain, st_plain = model.gn_solve(g0, Vte, lam, target=target, max_iters=15, options=opts)
    g1, it_learn, res_learn, acc, st_learn = model.gn_solve_learned(net, Vte, lam, target=target, max_iters=15,
                                                                   options=opts)
    print(f"plain GN updates {it_plain.mean():.3f}, learned {it_learn.mean():.3f}, accepted {acc.sum()}/32, "
          f"loss {losses[0]:.3f} -> {losses[-1]:.3f}")
    assert st_plain.frames_converged == 32 and st_learn.frames_converged == 32
    assert acc.sum() >= 16
    assert it_learn.mean() < it_plain.mean(), (it_learn.mean(), it_plain.mean())
