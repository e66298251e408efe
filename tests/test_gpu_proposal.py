"""Learned flip proposals: the hand-written network kernels against PyTorch on
the CPU (forward, loss and every parameter gradient), and what the trained
network gains: on a held-out design, the flips it ranks first are better
than average, which an untrained network's are not."""
import numpy as np
import pytest

from conftest import case_G

pytestmark = pytest.mark.gpu


def torch_net(params, C, x, target, mask):
    """The same network in PyTorch (CPU, float32), weights rounded to BF16 as
    the GPU kernels use them."""
    import torch
    import torch.nn.functional as F
    cin = [3, C, C, C]
    cout = [C, C, C, 1]
    off = 0
    ws, bs = [], []
    for l in range(4):
        n = cout[l] * cin[l] * 9
        w = torch.tensor(params[off:off + n].reshape(cout[l], cin[l], 3, 3)).to(torch.bfloat16).float()
        off += n
        b = torch.tensor(params[off:off + cout[l]])
        off += cout[l]
        ws.append(w.requires_grad_(True))
        bs.append(b.requires_grad_(True))
    h = torch.tensor(x)
    for l in range(4):
        h = F.conv2d(h, ws[l], bs[l], padding=1)
        if l < 3:
            h = torch.relu(h)
    out = h[:, 0]
    t = torch.tensor(target)
    m = torch.tensor(mask)
    loss = (((out - t) * m) ** 2).sum() / m.sum()
    loss.backward()
    grads = []
    for l in range(4):
        grads += [ws[l].grad.numpy().ravel(), bs[l].grad.numpy().ravel()]
    return out.detach().numpy(), float(loss), np.concatenate(grads)


# (tiles_x, tiles_y, channels, batch): square maps in one band of the tiled
# kernels, a wide map cut into several bands (25 wide: 5-row bands), and a
# channel count the tiled kernels do not take (the general kernels).
@pytest.mark.parametrize("tx,ty,C,B", [(7, 7, 32, 3), (25, 13, 16, 5), (9, 7, 12, 2)])
def test_network_matches_torch_cpu(tx, ty, C, B, cases, built_lib):
    from pngf_gb300 import lib
    h = lib.Handle(tx, ty, [30e9], max_flips=1)
    p = lib.Proposal(h, channels=C, seed=3)
    rng = np.random.default_rng(0)
    params = (rng.standard_normal(p.num_params()) * 0.2).astype(np.float32)
    p.set_params(params)
    x = rng.standard_normal((B, 3, ty, tx)).astype(np.float32)
    target = rng.standard_normal((B, ty, tx)).astype(np.float32)
    mask = (rng.random((B, ty, tx)) < 0.6).astype(np.float32)
    out, grad, loss = p.forward_backward(x, target, mask)
    out_t, loss_t, grad_t = torch_net(params, C, x, target, mask)
    np.testing.assert_allclose(out, out_t, rtol=1e-4, atol=1e-4 * np.abs(out_t).max())
    assert abs(loss - loss_t) <= 1e-4 * abs(loss_t)
    np.testing.assert_allclose(grad, grad_t, rtol=1e-3, atol=1e-4 * np.abs(grad_t).max())


def gains_at(h, tiles):
    """Exact objective change of each single-tile flip at the handle's design."""
    F0 = h.objective()
    _, F = h.eval_candidates([[t] for t in tiles])
    return F - F0


def test_trained_network_ranks_held_out_flips(cases, built_lib):
    from pngf_gb300 import lib
    c = cases["single_11x11_f3_seed2"]
    Gs, gobj = case_G(c, built_lib)
    Gs, gobj, freqs = Gs[:2], gobj[:2], c["freqs"][:2]
    a = 11

    def handle():
        h = lib.Handle(a, a, freqs, max_flips=1)
        for f, G in enumerate(Gs):
            h.load_G(f, G, gobj[f])
        return h

    # Training pairs from plain DBS runs (every exact evaluation is recorded).
    h = handle()
    prop = lib.Proposal(h, channels=32, seed=1)
    for seed in (2, 3):
        d = lib.Dbs(h, mode=lib.DBS_SINGLE, init=lib.INIT_RANDOM, seed=seed, max_evals=400)
        lib.dbs_set_proposal(d, prop, topk=0)
        d.run()
        d.close()
    assert prop.num_samples() > 20
    untrained = prop.params()
    loss = prop.train(400, batch=32, lr=2e-3)
    assert np.isfinite(loss)
    # A held-out design: a run from another seed, stopped midway.
    d = lib.Dbs(h, mode=lib.DBS_SINGLE, init=lib.INIT_RANDOM, seed=11, max_evals=60)
    d.run()
    mid = (a - 1) // 2
    elig = [t for t in range(a * a) if not (t // a == mid and abs(t % a - mid) <= 1)]
    true = gains_at(h, elig)
    k = 16

    def topk_mean(pred):
        order = np.argsort([pred[t] for t in elig])[:k]
        return true[order].mean()

    trained_mean = topk_mean(prop.predict())
    prop.set_params(untrained)
    untrained_mean = topk_mean(prop.predict())
    overall = true.mean()
    assert trained_mean < overall
    assert trained_mean < untrained_mean
