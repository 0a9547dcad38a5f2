"""The expiry path of a bounded device wait, on the GPU, without a fault or a hang: a CTA waits
on an mbarrier that nothing arrives at, with a short time limit; the wait gives up, the other
role sees the abort flag, tensor memory is freed, and the host gets PVGPU_ERR_TIMEOUT.  The
context stays usable: a tensor-memory kernel (the LCA solver) runs correctly right after."""
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


def test_bounded_wait_expires_with_timeout_status(torch, oracle):
    from openpv_gb300 import capi
    for limit_ns in (2_000_000, 20_000_000):
        st, expired, waited = capi.selftest_wait_expiry(limit_ns)
        assert st == capi.PVGPU_ERR_TIMEOUT and expired == 1, (st, expired)
        assert limit_ns <= waited < limit_ns + 50_000_000, (limit_ns, waited)
    assert capi.selftest_wait_expiry(0)[0] == capi.PVGPU_ERR_BAD_ARG  # a zero limit is refused
    # the context and tensor memory are intact: a short BF16 solve meets its bar
    rng = np.random.default_rng(7)
    w = rng.normal(size=(64, 8, 8, 1))
    w = (w / np.sqrt((w ** 2).sum(axis=(1, 2, 3), keepdims=True))).astype(np.float32)
    x = rng.normal(size=(2, 32, 32, 1)).astype(np.float32)
    p = oracle.lca_params(nbatch=2)
    _, _, _, e64 = oracle.lca_run(p, w.astype(np.float64), x[None].astype(np.float64), 5, np.zeros((2, 16, 16, 64)),
                                  f64=True, want_recon=False)
    s = capi.LcaSolver(2, (32, 32, 1), (16, 16, 64), 8, 0.1)
    s.set_weights(torch.from_numpy(w).cuda())
    s.reset()
    xd = torch.from_numpy(x).cuda()
    s.run(xd, 5, precision=capi.LCA_BF16)
    e = torch.zeros(2, dtype=torch.float64, device="cuda")
    s.energy(xd, e)
    torch.cuda.synchronize()
    assert s.error_flag() == 0
    assert (np.abs(e.cpu().numpy() - e64[-1]) / np.abs(e64[-1])).max() < 1e-3
