"""The compaction entry point that allocates nothing (pvgpu_compact_active_noalloc), through the
C ABI, against the ordinary one (pvgpu_compact_active, caller scratch).

It serves callers that cannot allocate device memory where they call (loops that must not pay
cudaMalloc's implicit synchronisation, hosts that own all device memory through their own pool);
its scratch is a fixed array in the library's device image.  Two calls in a row check that the
shared array carries nothing over between calls.  This file is collected last on purpose."""
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


def _entries(torch, nb, n):
    return torch.zeros((nb, n, 2), dtype=torch.int32, device="cuda")


@pytest.mark.parametrize("nb,n,p_seq", [(3, 25600, (0.05, 0.3)), (2, 204800, (0.5, 0.01)), (1, 4097, (1.0, 0.0))])
def test_noalloc_compaction_equals_scratch_version(torch, nb, n, p_seq):
    from openpv_gb300 import capi
    rng = np.random.default_rng(n)
    for p in p_seq:  # two calls in a row, different inputs
        a = ((rng.random((nb, n)) < p) * rng.normal(size=(nb, n))).astype(np.float32)
        ad = torch.from_numpy(a).cuda()
        e_ref, n_ref = _entries(torch, nb, n), torch.full((nb,), -1, dtype=torch.int64, device="cuda")
        e_new, n_new = _entries(torch, nb, n), torch.full((nb,), -2, dtype=torch.int64, device="cuda")
        capi.compact_active(ad, nb, n, e_ref, n_ref)
        capi.compact_active_noalloc(ad, nb, n, e_new, n_new)
        torch.cuda.synchronize()
        assert torch.equal(n_ref, n_new)
        for b in range(nb):
            k = int(n_ref[b].item())
            assert torch.equal(e_ref[b, :k], e_new[b, :k])


def test_noalloc_rejects_sizes_beyond_its_fixed_scratch(torch):
    from openpv_gb300 import capi
    nb, n = 129, 4096 * 4096  # 129 * 1024 chunks of 16384 values > 131071
    a = torch.zeros(1, device="cuda")
    e = torch.zeros(1, device="cuda")
    num = torch.zeros(nb, dtype=torch.int64, device="cuda")
    with pytest.raises(capi.PvgpuError) as exc:
        capi.compact_active_noalloc(a, nb, n, e, num)
    assert exc.value.status == 1
    assert "131071" in capi.last_error()
