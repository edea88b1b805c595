"""The warm-start network trained by the library's kernels against the CPU reference
(oracle/nn_reference.py): forward outputs, every layer's weight / bias gradients, the training
loss and one Adam step. BF16 tolerances (stated per check): relative error of a layer's whole
gradient tensor (Frobenius norm of the difference over the reference's) <= 5e-2, outputs <= 2e-2."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup(ps, H=128, W=128, B=2, seed=3):
    import torch

    from ps_gb300 import nn

    net = nn.Net(H, W, max_batch=B, seed=seed)
    g = torch.Generator(device="cuda").manual_seed(seed)
    x = torch.randn(B, H, W, 2, device="cuda", generator=g)
    return net, x


def _relerr(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def test_network_forward_matches_reference(ps):
    import torch

    from oracle.nn_reference import Reference

    net, x = _setup(ps)
    y = net.forward(x).cpu().numpy()
    ref = Reference(net.get_params())
    with torch.no_grad():
        yr = ref.forward(x.cpu()).numpy()
    e = _relerr(y, yr)
    assert e <= 2e-2, e
    assert np.abs(y).max() > 0


def _layer_errors(gg, gr):
    from oracle.nn_reference import layer_spec

    out, o = [], 0
    for cin, cout, k in layer_spec():
        nw = cout * k * k * cin
        out.append((_relerr(gg[o:o + nw], gr[o:o + nw]), _relerr(gg[o + nw:o + nw + cout], gr[o + nw:o + nw + cout])))
        o += nw + cout
    return out


def test_network_gradients_per_layer(ps):
    """Per layer, relative error of the weight and bias gradients:
    - against the reference that sees the GPU run's hidden activations (values and ReLU masks)
      and rounds gradients where the GPU does (bf16 at each convolution's input gradient):
      <= 5e-3, FP32 summation order only;
    - against the reference's own forward and plain FP32 backward: <= 0.15. Its activations differ
      from the GPU's by ~0.4 % (FP32 summation order flips bf16 roundings), which flips the ReLU
      mask where a pre-activation is near zero; a fraction f of flipped entries moves a layer's
      gradient by ~sqrt(f), 5-10 % here."""
    import torch

    from oracle.nn_reference import Reference

    net, x = _setup(ps, seed=4)
    p0 = net.get_params()
    y = net.forward(x)
    g = torch.Generator(device="cuda").manual_seed(9)
    dy = torch.randn(y.shape, device="cuda", generator=g)
    net.zero_grad()
    net.backward(dy)
    gg = net.get_grads()
    acts = [net.activation(i, x.shape[0]) for i in range(14)]
    errs = {}
    for forced in (True, False):
        ref = Reference(p0, round_grads=forced)
        yr = ref.forward(x.cpu(), forced=acts if forced else None)
        (yr * dy.cpu()).sum().backward()
        errs[forced] = _layer_errors(gg, ref.grads())
    assert max(max(e) for e in errs[True]) <= 5e-3, errs[True]
    assert max(max(e) for e in errs[False]) <= 0.15, errs[False]
    # backward accumulates until zero_grad
    net.backward(dy)
    # (split-K weight gradients add partial sums with FP32 atomics in any order: compare norm-wise)
    assert _relerr(net.get_grads(), 2 * gg) <= 1e-5


def test_train_step_loss_and_adam(ps):
    import torch

    from oracle.nn_reference import Reference

    net, x = _setup(ps, seed=5)
    p0 = net.get_params()
    g = torch.Generator(device="cuda").manual_seed(11)
    t = torch.randn(x.shape[0], x.shape[1], x.shape[2], 3, device="cuda", generator=g)
    lr = 1e-3
    loss = net.train_step(x, t, lr)
    ref = Reference(p0)
    yr = ref.forward(x.cpu())
    lr_ref = ((yr - t.cpu()) ** 2).mean().detach()
    assert abs(loss - float(lr_ref)) <= 2e-2 * float(lr_ref), (loss, float(lr_ref))
    # first Adam step: p1 = p0 - lr * g / (|g| + eps) elementwise (bias-corrected moments)
    gr = net.get_grads()
    p1 = net.get_params()
    expect = p0 - lr * gr / (np.abs(gr) + 1e-8)
    assert np.allclose(p1, expect, rtol=1e-4, atol=1e-6)


def test_training_reduces_loss(ps):
    """A few hundred Adam steps on a fixed batch drive the loss down (the kernels learn)."""
    import torch

    net, x = _setup(ps, seed=6)
    t = torch.tanh(x[..., :1].repeat(1, 1, 1, 3) * torch.tensor([1.0, -0.5, 0.25], device="cuda"))
    first = net.train_step(x, t, 2e-3)
    for _ in range(200):
        last = net.train_step(x, t, 2e-3)
    assert last < 0.1 * first, (first, last)


def test_save_load_roundtrip(ps, tmp_path):
    net, x = _setup(ps, seed=7)
    net.scales = [0.5, 2.0, 0.0, 1.0, 3.0, 4.0, 5.0, 0.0]
    y0 = net.forward(x).cpu().numpy()
    path = tmp_path / "w.bin"
    net.save(path)
    net2, _ = _setup(ps, seed=8)
    net2.load(path)
    assert net2.scales[:7] == [0.5, 2.0, 0.0, 1.0, 3.0, 4.0, 5.0]
    y1 = net2.forward(x).cpu().numpy()
    # saved weights are bf16 (what the forward pass uses), so the outputs agree exactly
    assert np.array_equal(y0, y1)
