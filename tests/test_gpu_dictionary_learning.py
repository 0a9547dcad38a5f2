"""Differentiable dictionary learning through the C-ABI adjoint delivery kernels.

Loss: L(W) = 0.5 ||x - W^T a_T||^2 + lambda ||a_T||_1 after T unrolled LCA timesteps from V = 0
(lambda = VThresh = 0.1, soft threshold, tau = 100), checkpointed every 10 steps.  Checks:
  * the explicit gradient (a fixed) equals minus the reference's Hebbian update (dWMax = 1,
    normalize_dW off) of the same a and residual, and matches FP64 central differences;
  * the unrolled gradient matches FP64 central differences (h = 1e-3) of the oracle's LCA;
  * the full-size configuration (32 images 64x64, V1 16x16x256 stride 4, 16x16 patches,
    100 steps, checkpoint every 10) runs, and a gradient step lowers the loss."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from openpv_gb300 import build
    build.build()
    return torch


def one_over_f(rng, nb, n):
    f = np.sqrt(np.fft.fftfreq(n)[:, None] ** 2 + np.fft.fftfreq(n)[None, :] ** 2)
    f[0, 0] = 1.0
    amp = 1.0 / f
    amp[0, 0] = 0.0
    out = np.real(np.fft.ifft2(amp[None] * np.exp(1j * rng.uniform(0, 2 * np.pi, (nb, n, n)))))
    out = (out - out.mean(axis=(1, 2), keepdims=True)) / out.std(axis=(1, 2), keepdims=True)
    return np.ascontiguousarray(out[..., None].astype(np.float32))


def dictionary(rng, nf, p):
    w = rng.normal(size=(nf, p, p, 1))
    return (w / np.sqrt((w ** 2).sum(axis=(1, 2, 3), keepdims=True))).astype(np.float32)


LAM = 0.1
SMALL = dict(nb=2, n=32, v1=(8, 8, 16), P=16)


def fp64_loss(oracle, w, x, steps, nb, n, v1):
    """Oracle (FP64) LCA for `steps` timesteps, then L = 0.5||x - W^T a||^2 + lam ||a||_1."""
    vy, vx, vf = v1
    P = w.shape[1]
    p = oracle.lca_params(nbatch=nb, inNx=n, inNy=n, inNf=1, v1Nx=vx, v1Ny=vy, v1Nf=vf, nxp=P, nyp=P,
                          VThresh=LAM, AShift=LAM, AMin=0.0, tau=100.0)
    _, a, _, _ = oracle.lca_run(p, w.astype(np.float64), x[None].astype(np.float64), steps,
                                np.zeros((nb, vy, vx, vf)), f64=True, want_recon=False)
    return explicit_loss_f64(oracle, w, x, a, nb, n, v1)


def explicit_loss_f64(oracle, w, x, a, nb, n, v1):
    vy, vx, vf = v1
    P = w.shape[1]
    m = (P // (n // vx)) // 2
    pre = oracle.Loc.make(nb, vx, vy, vf, m)
    post = oracle.Loc.make(nb, n, n, 1, 0)
    ae = np.zeros(pre.ext_shape())
    ae[:, m:m + vy, m:m + vx, :] = a
    rec = oracle.deliver_pre_f64(pre, post, P, P, w.astype(np.float64), ae)
    r = x.astype(np.float64) - rec
    return 0.5 * (r * r).sum() + LAM * np.abs(a).sum()


def test_explicit_gradient_is_minus_hebbian_and_matches_fd(torch, oracle):
    from tests import lca_autograd as LA
    rng = np.random.default_rng(4)
    nb, n, v1, P = SMALL["nb"], SMALL["n"], SMALL["v1"], SMALL["P"]
    geo = LA.Geometry(nb, (n, n, 1), v1, P)
    w = dictionary(rng, v1[2], P)
    x = one_over_f(rng, nb, n)
    a = (np.maximum(rng.normal(0, 0.3, (nb,) + v1) - 0.2, 0)).astype(np.float32)
    wd = torch.from_numpy(w).cuda().requires_grad_(True)
    ad = torch.from_numpy(a).cuda()
    xd = torch.from_numpy(x).cuda()
    r = xd - LA.Recon.apply(ad, wd, geo)
    loss = 0.5 * (r * r).sum() + LAM * ad.abs().sum()
    loss.backward()
    g = wd.grad.cpu().numpy()
    # minus the reference's Hebbian update on the same a and residual (dWMax = 1)
    m_v1, m_err = geo.v1.halo.lt, geo.err.halo.lt
    ae = np.pad(a, ((0, 0), (m_v1, m_v1), (m_v1, m_v1), (0, 0)))
    re = np.pad(r.detach().cpu().numpy(), ((0, 0), (m_err, m_err), (m_err, m_err), (0, 0)))
    opre = oracle.Loc.make(nb, v1[1], v1[0], v1[2], m_v1)
    opost = oracle.Loc.make(nb, n, n, 1, m_err)
    dw = oracle.hebbian_dw(opre, opost, P, P, ae, re, 1.0)
    np.testing.assert_allclose(-g, dw, rtol=1e-5, atol=1e-5 * np.abs(dw).max())
    # central differences in FP64
    h = 1e-3
    for trial in range(3):
        D = rng.normal(size=w.shape)
        D /= np.linalg.norm(D)
        fd = (explicit_loss_f64(oracle, w + h * D, x, a, nb, n, v1)
              - explicit_loss_f64(oracle, w - h * D, x, a, nb, n, v1)) / (2 * h)
        assert abs((g * D).sum() - fd) <= 1e-4 * abs(fd) + 1e-6, (trial, (g * D).sum(), fd)


def test_unrolled_gradient_matches_fp64_finite_differences(torch, oracle):
    from tests import lca_autograd as LA
    rng = np.random.default_rng(6)
    nb, n, v1, P = SMALL["nb"], SMALL["n"], SMALL["v1"], SMALL["P"]
    steps = 30
    geo = LA.Geometry(nb, (n, n, 1), v1, P)
    w = dictionary(rng, v1[2], P)
    x = one_over_f(rng, nb, n)
    wd = torch.from_numpy(w).cuda().requires_grad_(True)
    xd = torch.from_numpy(x).cuda()
    loss = LA.unrolled_lca_loss(wd, xd, geo, steps, LAM, LAM, checkpoint_every=10)
    loss.backward()
    g = wd.grad.cpu().numpy()
    l64 = fp64_loss(oracle, w, x, steps, nb, n, v1)
    assert abs(loss.item() - l64) <= 1e-4 * abs(l64)
    h = 1e-3
    for trial in range(3):
        D = rng.normal(size=w.shape)
        D /= np.linalg.norm(D)
        fd = (fp64_loss(oracle, w + h * D, x, steps, nb, n, v1) - fp64_loss(oracle, w - h * D, x, steps, nb, n, v1)) / (
            2 * h)
        assert abs((g * D).sum() - fd) <= 2e-3 * abs(fd) + 1e-5, (trial, (g * D).sum(), fd)


def test_full_size_dictionary_learning_step(torch):
    """32 images 64x64x1, V1 16x16x256 stride 4, 16x16x1 dictionary, 100 unrolled steps with a
    checkpoint every 10: the gradient exists, is finite, and a normalised step lowers the loss."""
    from tests import lca_autograd as LA
    rng = np.random.default_rng(1234 + 4)
    nb, n, v1, P = 32, 64, (16, 16, 256), 16
    geo = LA.Geometry(nb, (n, n, 1), v1, P)
    w = torch.from_numpy(dictionary(rng, v1[2], P)).cuda().requires_grad_(True)
    x = torch.from_numpy(one_over_f(rng, nb, n)).cuda()
    loss = LA.unrolled_lca_loss(w, x, geo, 100, LAM, LAM, checkpoint_every=10)
    loss.backward()
    g = w.grad
    assert torch.isfinite(g).all() and g.abs().max() > 0
    with torch.no_grad():
        w2 = w - 1e-3 * g / g.norm() * w.norm()
        w2 = w2 / w2.flatten(1).norm(dim=1).view(-1, 1, 1, 1)
        loss2 = LA.unrolled_lca_loss(w2.contiguous(), x, geo, 100, LAM, LAM)
    assert loss2.item() < loss.item()
