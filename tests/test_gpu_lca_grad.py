"""dL/dW of unrolled LCA through the C ABI (pvgpu_lca_grad_*: the unrolled forward, the segment
recomputation and the adjoint in one CUDA graph), for L = 0.5 ||x - W^T a_T||^2 + lambda ||a_T||_1
(lambda = VThresh = 0.1, tau = 100, checkpoint every 10):
  * against the autograd harness over the delivery kernels and their adjoints
    (tests/lca_autograd.py), whose gradient is checked against FP64 central differences: loss
    within 1e-5 relative, dW within 1e-4 of max|dW| (30 steps) and 1e-3 (100 steps, full size);
  * against FP64 central differences (h = 1e-3) of the oracle's LCA directly, at 2e-3;
  * the full-size configuration (32 images 64x64x1, V1 16x16x256 stride 4, 16x16x1 patches,
    100 steps): two runs of the graph give the same bits."""
import numpy as np
import pytest

from tests.test_gpu_dictionary_learning import LAM, dictionary, fp64_loss, one_over_f

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from openpv_gb300 import build
    build.build()
    return torch


def c_abi_gradient(torch, w, x, v1, P, steps, k=10):
    from openpv_gb300 import capi
    nb, n = x.shape[0], x.shape[1]
    g = capi.LcaGrad(nb, (n, n, 1), v1, P, LAM, LAM, steps, checkpoint_every=k)
    wd = torch.from_numpy(w).cuda()
    xd = torch.from_numpy(x).cuda()
    dw = torch.empty_like(wd)
    loss = torch.zeros(1, dtype=torch.float64, device="cuda")
    g.run(wd, xd, dw, loss)
    torch.cuda.synchronize()
    return g, wd, xd, dw, loss


def harness_gradient(torch, w, x, v1, P, steps):
    from tests import lca_autograd as LA
    nb, n = x.shape[0], x.shape[1]
    geo = LA.Geometry(nb, (n, n, 1), v1, P)
    wd = torch.from_numpy(w).cuda().requires_grad_(True)
    loss = LA.unrolled_lca_loss(wd, torch.from_numpy(x).cuda(), geo, steps, LAM, LAM, checkpoint_every=10)
    loss.backward()
    return wd.grad.cpu().numpy(), float(loss.item())


def test_c_abi_gradient_matches_harness_and_fp64_differences(torch, oracle):
    rng = np.random.default_rng(6)
    nb, n, v1, P, steps = 2, 32, (8, 8, 16), 16, 30
    w = dictionary(rng, v1[2], P)
    x = one_over_f(rng, nb, n)
    g, _, _, dw, loss = c_abi_gradient(torch, w, x, v1, P, steps)
    gh, lh = harness_gradient(torch, w, x, v1, P, steps)
    got = dw.cpu().numpy()
    assert abs(loss.item() - lh) <= 1e-5 * abs(lh), (loss.item(), lh)
    assert np.abs(got - gh).max() <= 1e-4 * np.abs(gh).max()
    l64 = fp64_loss(oracle, w, x, steps, nb, n, v1)
    assert abs(loss.item() - l64) <= 1e-4 * abs(l64)
    h = 1e-3
    for trial in range(3):
        D = rng.normal(size=w.shape)
        D /= np.linalg.norm(D)
        fd = (fp64_loss(oracle, w + h * D, x, steps, nb, n, v1) - fp64_loss(oracle, w - h * D, x, steps, nb, n, v1)) / (
            2 * h)
        assert abs((got * D).sum() - fd) <= 2e-3 * abs(fd) + 1e-5, (trial, (got * D).sum(), fd)
    print("GEMMs as FP32 emulated on the BF16 tensor cores:", g.emulated_fp32())


def test_c_abi_gradient_full_size(torch):
    rng = np.random.default_rng(1234 + 4)
    nb, n, v1, P, steps = 32, 64, (16, 16, 256), 16, 100
    w = dictionary(rng, v1[2], P)
    x = one_over_f(rng, nb, n)
    g, wd, xd, dw, loss = c_abi_gradient(torch, w, x, v1, P, steps)
    first = dw.cpu().numpy().copy()
    l1 = loss.item()
    g.run(wd, xd, dw, loss)  # the graph again
    torch.cuda.synchronize()
    assert np.array_equal(dw.cpu().numpy().view(np.uint32), first.view(np.uint32)) and loss.item() == l1
    gh, lh = harness_gradient(torch, w, x, v1, P, steps)
    assert abs(l1 - lh) <= 1e-5 * abs(lh), (l1, lh)
    assert np.abs(first - gh).max() <= 1e-3 * np.abs(gh).max()
