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


def test_mlp_adam_and_train_step():
    """Adam (k_adam_flat / k_adam_wt) against an FP32 numpy Adam from the
    kernels' own gradients; gradients after the step against the oracle at
    the updated parameters (the backward products read the transposed BF16
    copies that the Adam kernel writes); and mpf_mlp_train_step on rows
    gathered by index equal to backward + adam on gathered copies, bit for
    bit."""
    from oracle import mlp_oracle as mo
    import mpflow_gb300 as mp
    import torch
    dims = (128, 256, 128, 384)
    rng = np.random.default_rng(11)
    X = rng.standard_normal((300, dims[0])).astype(np.float32)
    valid = 300
    T = rng.standard_normal((300, 320)).astype(np.float32)
    rows = rng.permutation(300)[:200].astype(np.int32)
    Xt, Tt = torch.tensor(X, device="cuda"), torch.tensor(T, device="cuda")
    rt = torch.tensor(rows, device="cuda")
    lr, wd, b1, b2, eps = 1e-3, 1e-2, 0.9, 0.999, 1e-8
    a = _random_net(mp, torch, dims, seed=5)
    b = _random_net(mp, torch, dims, seed=5)
    p0 = a.parameters().cpu().numpy().astype(np.float64)
    b.backward(Xt[rt.long()], Tt[rt.long()], valid=valid, want_loss=False)
    g = b.gradients().cpu().numpy().astype(np.float64)
    b.adam(lr, weight_decay=wd)
    a.train_step(Xt, Tt, rows=rt, valid=valid, lr=lr, weight_decay=wd)
    pa, pb = a.parameters().cpu().numpy(), b.parameters().cpu().numpy()
    assert np.array_equal(pa, pb)
    # FP64 Adam from the same gradients; weights decay, biases do not
    o = a.offsets
    decay = np.zeros(a.param_count, bool)
    for k, (r, c) in enumerate(((dims[1], dims[0]), (dims[2], dims[1]), (dims[3], dims[2]))):
        decay[o[2 * k]:o[2 * k] + r * c] = True
    m, v = (1 - b1) * g, (1 - b2) * g * g
    w = p0 - np.where(decay, lr * wd * p0, 0.0)
    w = w - lr * (m / (1 - b1)) / (np.sqrt(v / (1 - b2)) + eps)
    assert np.abs(pa - w).max() <= 1e-6 * max(np.abs(w).max(), 1.0), np.abs(pa - w).max()
    # second step: gradients at the updated parameters against the oracle
    a.backward(Xt[rt.long()], Tt[rt.long()], valid=valid, want_loss=False)
    grads = a.unpack(a.gradients())
    _, go = mo.loss_and_gradients(a.unpack(a.parameters()), X[rows], T[rows][:, :valid], valid)
    for name, gg, r in zip(("dW1", "db1", "dW2", "db2", "dW3", "db3"), grads, go):
        assert _rel(gg, r) < 1e-2, (name, _rel(gg, r))
    # more train steps stay identical to backward + adam
    for step in range(3):
        a.train_step(Xt, Tt, rows=rt, valid=valid, lr=lr, weight_decay=wd)
        b.backward(Xt[rt.long()], Tt[rt.long()], valid=valid, want_loss=False)
        b.adam(lr, weight_decay=wd)
    assert np.array_equal(a.parameters().cpu().numpy(), b.parameters().cpu().numpy())


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


def _prior_setup(frames=8):
    import mpflow_gb300 as mp
    from mpflow_gb300.learned import inclusion_frames
    import torch
    mesh, src, _ = make_setup(rings=20, ports=16, logarithmic=True)
    E = mesh.elements.shape[0]
    model = mp.EIT(mesh, src, 1.0, logarithmic=True)
    cent = mesh.nodes[mesh.elements].mean(axis=1)
    gte = inclusion_frames(cent, frames, np.random.default_rng(17))
    Vte = model.solve(torch.tensor(gte, device="cuda"), mp.SolveOptions(tol=1e-6, refine_tol=1e-10)).contiguous()
    _, J0 = model.solve(torch.zeros((1, E), device="cuda"), mp.SolveOptions(tol=1e-6), jacobian=True)
    lam = 2e-2 * float(J0.norm() / np.sqrt(J0.shape[1]))
    return mp, torch, model, mesh, cent, E, Vte, lam


def test_learned_prior_is_the_first_gauss_newton_update():
    """prior(x) equals one Gauss-Newton step from the homogeneous start
    (mpf_gn_step: split-BF16 Gram there, FP64 Gram in the prior), and the
    accumulate modes add and subtract it."""
    mp, torch, model, mesh, cent, E, Vte, lam = _prior_setup()
    F = Vte.shape[0]
    model.learned_prior(lam)
    x = model.learned_input(Vte)
    gp = model.learned_prior_apply(x)
    g1 = torch.zeros((F, E), device="cuda")
    model.gn_step(g1, Vte, lam, mp.SolveOptions(tol=1e-7, refine_tol=1e-10))
    for f in range(F):
        assert _rel(gp[f].cpu().numpy(), g1[f].cpu().numpy()) < 2e-3, f
    acc = torch.ones((F, E), device="cuda")
    model.learned_prior_apply(x, acc, mode=1)
    assert _rel((acc - 1.0).cpu().numpy(), gp.cpu().numpy()) < 1e-6
    model.learned_prior_apply(x, acc, mode=-1)
    assert _rel(acc.cpu().numpy(), np.ones((F, E))) < 1e-6
    model.learned_prior(0.0)
    with pytest.raises(mp.MpfError):
        model.learned_prior_apply(x)


def test_looser_acceptance_solve_keeps_the_decisions():
    """accept_tol: the solve at the start's prediction runs at a looser CG
    tolerance, frames below target (1 - margin) are decided on it and skipped
    afterwards, the others continue to the full tolerance.  On 64 held-out
    frames from the linear prior (zero network) the accepted flags and the
    updates per frame equal those of the full-tolerance run and the final
    residuals stay below the target."""
    from mpflow_gb300.learned import round_up, zero_network
    mp, torch, model, mesh, cent, E, Vte, lam = _prior_setup(frames=64)
    model.learned_prior(lam)
    F = Vte.shape[0]
    L = Vte.shape[1] * Vte.shape[2]
    net0 = zero_network(L, round_up(E, 128))
    target = 1e-3
    full = mp.SolveOptions(tol=1e-6, max_iter=4000, warm_start="homogeneous")
    loose = mp.SolveOptions(tol=1e-6, max_iter=4000, warm_start="homogeneous", accept_tol=1e-4, accept_margin=0.1)
    _, it_f, res_f, acc_f, st_f = model.gn_solve_learned(net0, Vte, lam, target=target, max_iters=15, options=full)
    g_l, it_l, res_l, acc_l, st_l = model.gn_solve_learned(net0, Vte, lam, target=target, max_iters=15,
                                                           options=loose)
    print(f"accepted {acc_f.sum()}/{F}, decided on the loose solve {st_l.accepted_loose}, "
          f"CG iterations {st_l.cg_iterations} against {st_f.cg_iterations}")
    assert np.array_equal(acc_l, acc_f) and np.array_equal(it_l, it_f)
    assert st_l.frames_converged == st_f.frames_converged == F
    assert (res_l <= target).all()
    assert st_l.accepted_loose > 0 and st_f.accepted_loose == 0


def test_learned_prior_and_network_save_gauss_newton_updates():
    """With the linear prior, the learned start (prior + a correction trained
    on where Gauss-Newton from the prior converges) needs fewer updates than
    the homogeneous start and than the prior alone (zero network) on 64
    held-out frames.  The training set size decides it: at 20 rings the
    network trained on 2048 pairs needed more updates than the prior alone
    (1.03 against 0.89), on 8192 pairs fewer (0.72)."""
    from mpflow_gb300.learned import (generate_pairs, gn_labels, inclusion_frames, round_up, train_warm_start,
                                      zero_network)
    mp, torch, model, mesh, cent, E, Vte, lam = _prior_setup(frames=64)
    opts = mp.SolveOptions(tol=1e-6, max_iter=4000)
    model.learned_prior(lam)
    Vtr, gtr = generate_pairs(model, inclusion_frames(cent, 16384, np.random.default_rng(11)), batch=128,
                              options=opts)
    L = Vtr.shape[1] * Vtr.shape[2]
    labels, conv = gn_labels(model, Vtr, lam, target=1e-3, options=opts)
    assert conv > 0.9, conv
    net = mp.MLP(L, 512, 512, round_up(E, 128), seed=5)
    losses, _ = train_warm_start(model, net, Vtr, labels, epochs=40, batch=256, lr=1e-3, snr_db=60.0, prior=True)
    assert losses[-1] < losses[0], losses
    target = 1e-3
    F = Vte.shape[0]
    g0 = torch.zeros((F, E), device="cuda")
    it_plain, _, st_plain = model.gn_solve(g0, Vte, lam, target=target, max_iters=15, options=opts)
    _, it_prior, _, acc_p, st_prior = model.gn_solve_learned(zero_network(L, round_up(E, 128)), Vte, lam,
                                                             target=target, max_iters=15, options=opts)
    _, it_learn, _, acc, st_learn = model.gn_solve_learned(net, Vte, lam, target=target, max_iters=15,
                                                           options=opts)
    print(f"GN updates: plain {it_plain.mean():.3f}, prior only {it_prior.mean():.3f} "
          f"(direct {np.mean(it_prior == 0):.2f}), prior + network {it_learn.mean():.3f} "
          f"(direct {np.mean(it_learn == 0):.2f}, accepted {acc.sum()}/{F}); loss {losses[0]:.3g} -> {losses[-1]:.3g}")
    assert st_plain.frames_converged == F and st_prior.frames_converged == F and st_learn.frames_converged == F
    assert acc_p.sum() >= 0.75 * F and acc.sum() >= 0.75 * F
    assert it_prior.mean() < it_plain.mean()
    # what the trained network gains over the method without it
    assert it_learn.mean() < it_prior.mean(), (it_learn.mean(), it_prior.mean())


def test_network_checkpoint_round_trip(tmp_path):
    """MLP.save / MLP.load keep the parameters bit for bit, so a trained
    warm start can be reused without training again."""
    import mpflow_gb300 as mp
    import torch
    net = mp.MLP(256, 128, 128, 384, seed=3)
    x = torch.randn((128, 256), device="cuda")
    y0 = net.forward(x)
    path = str(tmp_path / "net.mpf")
    net.save(path)
    back = mp.MLP.load(path)
    assert (back.inputs, back.hidden1, back.hidden2, back.outputs) == (256, 128, 128, 384)
    assert torch.equal(back.parameters(), net.parameters())
    assert torch.equal(back.forward(x), y0)
