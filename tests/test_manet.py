"""The Monge-Ampere warm-start network: the FP64 oracle against torch autograd (CPU), and the
GPU BF16 tensor-core kernels (forward, backward-data, weight gradients, Adam) against the oracle."""
import numpy as np
import pytest

import oracle
import mitos_gb300.lib as ml


def _layers_from_params(p):
    """per-layer (w, b) with the real channel counts, from a padded parameter vector"""
    out = []
    for l, (w, b) in enumerate(ml.manet_layers(p)):
        cin, cout = oracle.MANET_CIN[l], oracle.MANET_COUT[l]
        out.append((w[:, :cin, :cout].astype(np.float64), b[:cout].astype(np.float64)))
    return out


def _random_layers(rng):
    layers = []
    for cin, cout in zip(oracle.MANET_CIN, oracle.MANET_COUT):
        layers.append((rng.standard_normal((27, cin, cout)) * np.sqrt(2.0 / (27 * cin)),
                       rng.standard_normal(cout) * 0.1))
    return layers


def test_bf16_rounding_matches_torch():
    torch = pytest.importorskip("torch")
    x = np.random.default_rng(1).standard_normal(4096) * np.logspace(-8, 8, 4096)
    ref = torch.tensor(x, dtype=torch.float32).to(torch.bfloat16).to(torch.float64).numpy()
    assert np.array_equal(oracle.bf16(x), ref)


def test_oracle_network_matches_torch_autograd():
    torch = pytest.importorskip("torch")
    F = torch.nn.functional
    rng = np.random.default_rng(7)
    N = 8
    x = rng.standard_normal((N, N, N, 3))
    t = rng.standard_normal((N, N, N))
    layers = _random_layers(rng)
    loss, pred, grads = oracle.manet_loss_grad(x, t, layers, round_bf16=False)

    # torch: channels-first, circular padding; weight[co][ci][dx][dy][dz] = w[t][ci][co]
    h = torch.tensor(x, dtype=torch.float64).permute(3, 0, 1, 2)[None]
    params = []
    for l, (w, b) in enumerate(layers):
        cin, cout = w.shape[1], w.shape[2]
        wt = torch.tensor(w.reshape(3, 3, 3, cin, cout).transpose(4, 3, 0, 1, 2).copy(), requires_grad=True)
        bt = torch.tensor(b, requires_grad=True)
        params.append((wt, bt))
        h = F.conv3d(F.pad(h, (1, 1, 1, 1, 1, 1), mode="circular"), wt, bt)
        if l < 3:
            h = torch.relu(h)
    tl = ((h[0, 0] - torch.tensor(t)) ** 2).mean()
    tl.backward()
    assert abs(tl.item() - loss) <= 1e-12 * abs(loss)
    assert np.allclose(h[0, 0].detach().numpy(), pred, rtol=1e-12, atol=1e-12)
    for (wt, bt), (dw, db) in zip(params, grads):
        tw = wt.grad.numpy().transpose(2, 3, 4, 1, 0).reshape(dw.shape)
        assert np.allclose(tw, dw, rtol=1e-9, atol=1e-14 * np.abs(dw).max())
        assert np.allclose(bt.grad.numpy(), db, rtol=1e-9, atol=1e-14 * max(np.abs(db).max(), 1e-300))


def _fp32_grid(N, arr):
    g = ml.alloc_local_grid(N, 1.0, ml.FP32)
    ml.set_box(g, arr)
    return g


@pytest.mark.gpu
def test_network_forward_and_gradients_match_oracle():
    """GPU BF16 / FP32-accumulate kernels against the oracle with the same BF16 roundings;
    tolerances cover FP32-vs-FP64 accumulation and rare BF16 rounding-boundary flips."""
    N = 32
    rng = np.random.default_rng(3)
    x = rng.uniform(-1, 1, (N, N, N, 3))
    t = rng.standard_normal((N, N, N)) * 0.3
    grids = [_fp32_grid(N, x[..., c]) for c in range(3)] + [_fp32_grid(N, t)]
    net = ml.manet_init(11)
    try:
        p = ml.manet_params(net)
        loss = ml.manet_loss_grad(net, N, N + 2, *grids)
        g = ml.manet_grads(net)
        out = _fp32_grid(N, np.zeros((N, N, N)))
        ml.manet_infer(net, N, N + 2, grids[0], grids[1], grids[2], out)
        pred_gpu = ml.get_box(out)[..., :N]
        # the GPU stores the inputs in BF16 after an FP32 product: round them the same way
        xq = oracle.bf16(x.astype(np.float32))
        oloss, opred, ograds = oracle.manet_loss_grad(xq, t.astype(np.float32), _layers_from_params(p))
        assert abs(loss - oloss) <= 2e-3 * oloss
        assert np.sqrt(np.mean((pred_gpu - opred) ** 2)) <= 2e-3 * np.sqrt(np.mean(opred ** 2))
        for l, ((gw, gb), (ow, ob)) in enumerate(zip(ml.manet_layers(g), ograds)):
            cin, cout = oracle.MANET_CIN[l], oracle.MANET_COUT[l]
            gw = gw[:, :cin, :cout]
            err = np.sqrt(np.mean((gw - ow) ** 2)) / np.sqrt(np.mean(ow ** 2))
            assert err < 2e-2, (l, err)
            assert np.allclose(gb[:cout], ob, rtol=5e-2, atol=2e-2 * np.abs(ob).max()), l
            # padded channels carry no gradient
            assert not np.any(ml.manet_layers(g)[l][0][:, cin:, :]) and not np.any(ml.manet_layers(g)[l][0][:, :, cout:])
        ml.free_local_grid(out)
    finally:
        ml.manet_free(net)
        for gr in grids:
            ml.free_local_grid(gr)


@pytest.mark.gpu
def test_network_training_fits_a_teacher():
    """Adam on the GPU drives the student towards the output of a fixed teacher network."""
    N = 32
    rng = np.random.default_rng(9)
    x = rng.uniform(-1, 1, (N, N, N, 3))
    grids = [_fp32_grid(N, x[..., c]) for c in range(3)]
    target = _fp32_grid(N, np.zeros((N, N, N)))
    teacher, student = ml.manet_init(101), ml.manet_init(202)
    try:
        ml.manet_infer(teacher, N, N + 2, *grids, target)
        losses = [ml.manet_train_step(student, N, N + 2, *grids, target, 3e-3) for _ in range(300)]
        assert np.all(np.isfinite(losses))
        assert np.mean(losses[-10:]) < 0.25 * np.mean(losses[:3])
    finally:
        ml.manet_free(teacher)
        ml.manet_free(student)
        for gr in grids + [target]:
            ml.free_local_grid(gr)
