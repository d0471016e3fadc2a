"""Host logic of the learned warm start on the CPU (a fake model stands in
for the GPU one): which training label each frame gets, and the guards of
the training entry points."""
import numpy as np
import pytest
import torch

from mpflow_gb300.learned import gn_labels, inclusion_frames, train_warm_start


class _Mesh:
    def __init__(self, E):
        self.elements = np.zeros((E, 3), np.int32)


class FakeModel:
    """GN 'converges' for even-numbered frames (label = 10 + frame index);
    odd frames stay above the target; the prior of a frame is -(frame
    index), read back from its input."""

    def __init__(self, E=5, prior=True):
        self.mesh = _Mesh(E)
        self.device = 0
        self.prior_lambda = 0.1 if prior else None
        self.calls = []

    def gn_solve_learned(self, net, V, lam, target, max_iters, options=None):
        F = V.shape[0]
        ids = V[:, 0, 0].round().long()
        g = (10.0 + ids.float())[:, None].repeat(1, self.mesh.elements.shape[0])
        res = np.where(ids.numpy() % 2 == 0, 0.5 * target, 10.0 * target)
        self.calls.append((net, F, lam, target, max_iters))
        return g, np.ones(F, np.int32), res, np.ones(F, np.int32), None

    def learned_input(self, V):
        return V.reshape(V.shape[0], -1).clone()

    def learned_prior_apply(self, x, out=None, mode=0):
        p = (-x[:, 0])[:, None].repeat(1, self.mesh.elements.shape[0])
        if out is None:
            return p
        out += mode * p
        return out


def test_gn_labels_keep_the_prior_where_gn_does_not_converge():
    model = FakeModel()
    V = torch.arange(7, dtype=torch.float32)[:, None, None].repeat(1, 2, 2)
    net0 = object()
    labels, conv = gn_labels(model, V, 0.1, target=1e-3, max_iters=3, batch=3, net0=net0)
    assert conv == pytest.approx(4 / 7)
    for f in range(7):
        want = 10.0 + f if f % 2 == 0 else -float(f)
        assert torch.all(labels[f] == want), (f, labels[f])
    # batches of 3: 3 + 3 + 1 frames, each with the given network and limits
    assert [c[1] for c in model.calls] == [3, 3, 1]
    assert all(c[0] is net0 and c[3] == 1e-3 and c[4] == 3 for c in model.calls)


def test_gn_labels_and_training_need_the_prior():
    model = FakeModel(prior=False)
    V = torch.zeros((2, 2, 2))
    with pytest.raises(ValueError, match="linear prior"):
        gn_labels(model, V, 0.1, net0=object())
    with pytest.raises(ValueError, match="linear prior"):
        train_warm_start(model, object(), V, torch.zeros((2, 5)), epochs=1, batch=128, prior=True)


def test_training_batch_must_be_a_multiple_of_128():
    with pytest.raises(ValueError, match="multiple of 128"):
        train_warm_start(FakeModel(), object(), torch.zeros((2, 2, 2)), torch.zeros((2, 5)), batch=100)


def test_inclusion_frames_family():
    import mpflow_gb300 as mp
    mesh = mp.IrregularMesh.ring(30)
    cent = mesh.nodes[mesh.elements].mean(axis=1)
    g = inclusion_frames(cent, 50, np.random.default_rng(1))
    assert g.shape == (50, mesh.elements.shape[0]) and g.dtype == np.float32
    # background 0 dB, inclusions within +-10 dB (contrast 0.1 .. 10), every frame has one
    assert np.all(np.abs(g) <= 10.0 + 1e-5)
    assert np.all((g != 0).sum(axis=1) > 0)


def test_checkpoint_reader_rejects_foreign_and_truncated_files(tmp_path):
    """The network checkpoint reader checks the magic and the length before
    any parameter reaches a device."""
    import numpy as np
    import pytest
    from mpflow_gb300.learned import MLP
    bad = tmp_path / "bad.bin"
    bad.write_bytes(b"not a checkpoint at all, just bytes........")
    with pytest.raises(ValueError):
        MLP.read_checkpoint(str(bad))
    head = np.array([4, 128, 128, 8, 10], dtype="<i8").tobytes()
    good = tmp_path / "good.bin"
    good.write_bytes(MLP.MAGIC + head + np.arange(10, dtype="<f4").tobytes())
    dims, flat = MLP.read_checkpoint(str(good))
    assert dims == (4, 128, 128, 8) and np.array_equal(flat, np.arange(10, dtype=np.float32))
    short = tmp_path / "short.bin"
    short.write_bytes(MLP.MAGIC + head + np.arange(9, dtype="<f4").tobytes())
    with pytest.raises(ValueError):
        MLP.read_checkpoint(str(short))
