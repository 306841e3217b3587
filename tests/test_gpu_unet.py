"""The learned-guess U-Net's own CUDA kernels vs the PyTorch CPU oracle
(marked gpu).

Forward and gradient are compared with the oracle run on the same BF16
weights, with every activation rounded to BF16 where the library stores
it; the library additionally rounds pre-activation gradients to BF16 for
the tensor-core products, so gradients agree to a few parts in a hundred
(relative L2 per layer, stated below), not bit for bit.  Adam is FP32
arithmetic and agrees to 1e-5 relative.
"""
import numpy as np
import pytest

import unet_oracle as UO

pytestmark = pytest.mark.gpu

FWD_TOL = 2e-2     # relative L2 of the network output
GRAD_TOL = 5e-2    # relative L2 of each layer's weight and bias gradient


def _net(seed=3):
    import vfs_poisson as V
    net = V.UNet(seed)
    p = net.get_params()
    rng = np.random.default_rng(seed)
    p[-17:] = rng.normal(size=17).astype(np.float32) * 0.3   # non-zero head
    off = 0
    for ci, co in UO.LAYERS:                                  # non-zero biases
        off += 27 * ci * co
        p[off:off + co] = rng.normal(size=co).astype(np.float32) * 0.05
        off += co
    net.set_params(p)
    return net, p


def _data(dims, seed=0):
    import torch
    nx, ny, nz = dims
    rng = np.random.default_rng(seed)
    f = rng.normal(size=(4, nz, ny, nx)).astype(np.float32)
    f[3] = (rng.uniform(size=(nz, ny, nx)) > 0.1)
    t = rng.normal(size=(nz, ny, nx)).astype(np.float32)
    w = f[3].copy()
    dev = [torch.from_numpy(a).cuda() for a in (f, t, w)]
    return (f, t, w), dev


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


@pytest.mark.parametrize("dims", [(16, 16, 8), (20, 12, 8), (32, 8, 12)])
def test_forward_matches_oracle(cuda_lib, dims):
    import torch
    import vfs_poisson as V
    net, p = _net()
    (f, t, w), (fd, td, wd) = _data(dims)
    out = torch.zeros(dims[::-1], device="cuda")
    net.forward(V.UNet.batch(fd), out)
    torch.cuda.synchronize()
    ref, _ = UO.forward(p, f)
    assert _rel(out.cpu().numpy(), ref.detach().numpy()) < FWD_TOL
    net.close()


def test_forward_on_sub_box(cuda_lib):
    import torch
    import vfs_poisson as V
    net, p = _net()
    (f, t, w), (fd, td, wd) = _data((24, 20, 16))
    out = torch.zeros((8, 12, 16), device="cuda")
    net.forward(V.UNet.batch(fd, origin=(4, 8, 4), size=(16, 12, 8)), out)
    sub = torch.zeros((8, 12, 16), device="cuda")
    fs = fd[:, 4:12, 8:20, 4:20].contiguous()
    net.forward(V.UNet.batch(fs), sub)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(out.cpu().numpy(), sub.cpu().numpy())
    net.close()


@pytest.mark.parametrize("dims", [(16, 16, 8), (20, 12, 8)])
def test_gradient_matches_oracle(cuda_lib, dims):
    import vfs_poisson as V
    net, p = _net()
    (f, t, w), (fd, td, wd) = _data(dims, seed=1)
    g = np.zeros(net.num_params, np.float32)
    loss = net.gradient(V.UNet.batch(fd, td, wd), g)
    lref, gref = UO.loss_and_grad(p, f, t, w)
    assert abs(loss - lref) <= 1e-2 * abs(lref)
    off = 0
    for li, (ci, co) in enumerate(UO.LAYERS):
        nw = 27 * ci * co
        gw, rw = g[off:off + nw], gref[off:off + nw]
        if li == 0:   # only the 4 fed input channels carry gradient
            gw = gw.reshape(27, ci, co)[:, :4].ravel()
            rw = rw.reshape(27, ci, co)[:, :4].ravel()
            assert np.all(g[off:off + nw].reshape(27, ci, co)[:, 4:] == 0)
        assert _rel(gw, rw) < GRAD_TOL, f"layer {li} weights"
        off += nw
        assert _rel(g[off:off + co], gref[off:off + co]) < GRAD_TOL, f"layer {li} bias"
        off += co
    assert _rel(g[off:], gref[off:]) < GRAD_TOL, "head"
    net.close()


def test_adam_matches_oracle(cuda_lib):
    net, p = _net()
    rng = np.random.default_rng(5)
    m = np.zeros_like(p, dtype=np.float64)
    v = np.zeros_like(p, dtype=np.float64)
    ref = p.astype(np.float64)
    for t in range(1, 4):
        g = rng.normal(size=p.shape).astype(np.float32)
        net.set_grads(g)
        net.adam(1e-3)
        ref, m, v = UO.adam(ref, g, m, v, t, 1e-3)
    got = net.get_params()
    assert np.max(np.abs(got - ref)) <= 1e-5 * max(1.0, np.max(np.abs(ref)))
    net.close()


def test_training_reduces_loss(cuda_lib):
    import vfs_poisson as V
    net, p = _net()
    (f, t, w), (fd, td, wd) = _data((16, 16, 16), seed=2)
    # a learnable target: a smooth function of the features
    import torch
    td.copy_(0.5 * fd[0] - 0.25 * fd[1] + 0.1)
    b = V.UNet.batch(fd, td, wd)
    first = net.gradient(b)
    for _ in range(60):
        last = net.train_step(b, 2e-3)
    assert last < 0.5 * first
    net.close()


def test_residual_loss_gradient_matches_oracle(cuda_lib):
    """The operator-residual loss (the quantity the solver judges a guess
    by) and its gradient, with a random 19-point operator."""
    import torch
    import vfs_poisson as V
    net, p = _net()
    dims = (16, 12, 8)
    (f, t, w), (fd, td, wd) = _data(dims, seed=4)
    rng = np.random.default_rng(9)
    op = rng.normal(size=(19,) + dims[::-1]).astype(np.float32) * 0.3
    opd = torch.from_numpy(op).cuda()
    g = np.zeros(net.num_params, np.float32)
    b = V.UNet.batch(fd, td, wd, op=opd, op_scale=0.7, mse_weight=0.25, res_weight=1.0)
    loss = net.gradient(b, g)
    lref, gref = UO.loss_and_grad(p, f, t, w, op=op, op_scale=0.7, mse_weight=0.25, res_weight=1.0)
    assert abs(loss - lref) <= 2e-2 * abs(lref)
    assert _rel(g, gref) < GRAD_TOL
    net.close()
