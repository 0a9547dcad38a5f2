"""Tensor-core deliveries (pvgpu_deliver_post_tc / pvgpu_deliver_pre_tc: one-to-one
connections as an implicit GEMM on tcgen05 with split-TF32 operands) against the oracle's FP32
post- and pre-perspective deliveries, through the C ABI.  Tolerance: the FAST mode's 1e-5
relative (the split leaves about 2^-21 relative error per product, and the chains of tensor-core
accumulation are summed with round-to-nearest)."""
import numpy as np
import pytest

from tests.test_gpu_kernels import OL, H, T, sparse_activity

pytestmark = pytest.mark.gpu

RTOL = 1e-5


@pytest.fixture(scope="module")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from openpv_gb300 import build
    build.build()
    from openpv_gb300 import capi
    capi.lib()
    return torch


# (nb, nx, ny, pre nf, pre halo), (post nf, post halo), patch, dt_factor
TC_CASES = [
    ((2, 40, 12, 32, 3), (64, 0), 7, 1.0),      # one column tile shorter than 128 positions
    ((1, 130, 9, 64, 3), (32, 1), 7, 1.0),      # two column tiles, the second 2 wide; odd rows
    ((1, 128, 8, 256, 3), (64, 0), 7, 1.0),     # the 128x128x256 -> 64 microbenchmark's shape, 8 rows
    ((2, 33, 10, 32, 4), (96, 0), 9, 1.0),      # widest patch, 96 post features
    ((1, 64, 6, 32, 1), (256, 0), 3, 1.0),      # 256 post features (one row per unit)
    ((2, 50, 7, 64, 0), (32, 2), 1, 0.5),       # 1x1 patch, dt_factor
    ((1, 70, 11, 32, 4), (64, 0), 5, 1.0),      # halo above the margin
    ((1, 40, 5, 32, 2), (160, 0), 5, 1.0),      # five 32-feature tiles
    ((1, 24, 4, 64, 1), (384, 1), 3, 1.0),      # three 128-feature tiles
]


def _case(oracle, capi, case, seed):
    (nb, nx, ny, nf, h), (qf, qh), p, dtf = case
    pre = capi.Loc.make(nb, nx, ny, nf, h)
    post = capi.Loc.make(nb, nx, ny, qf, qh)
    rng = np.random.default_rng(seed)
    a = sparse_activity(rng, pre, 0.3, zero_halo=False)
    w = rng.normal(0, 0.05, (nf, p, p, qf)).astype(np.float32)
    g0 = rng.normal(size=post.res_shape()).astype(np.float32)
    conn = capi.conn_desc(pre, post, p, p, dtf)
    return pre, post, a, w, g0, conn


@pytest.mark.parametrize("case", TC_CASES)
def test_deliver_post_tc_matches_oracle(cuda, oracle, case):
    torch = cuda
    from openpv_gb300 import capi
    pre, post, a, w, g0, conn = _case(oracle, capi, case, seed=case[0][1] + case[1][0])
    p, dtf = case[2], case[3]
    w_post = oracle.transpose_shared(OL(oracle, pre), OL(oracle, post), p, p, w)
    ref = oracle.deliver_post(OL(oracle, pre), OL(oracle, post), p, p, w_post, a, dt_factor=dtf, gsyn=g0.copy())
    ws = torch.empty(capi.deliver_tc_workspace_bytes(conn), dtype=torch.uint8, device="cuda")
    g = T(torch, g0)
    capi.deliver_post_tc(conn, T(torch, a), T(torch, w_post), g, ws)
    out = H(g)
    assert capi.deliver_tc_check_error() == 0
    np.testing.assert_allclose(out, ref, rtol=RTOL, atol=RTOL * np.abs(ref).max())


@pytest.mark.parametrize("case", TC_CASES[:4])
def test_deliver_pre_tc_matches_oracle(cuda, oracle, case):
    """The presynaptic entry (transpose on the device, then the same GEMM) against the oracle's
    presynaptic scatter of the same activity."""
    torch = cuda
    from openpv_gb300 import capi
    pre, post, a, w, g0, conn = _case(oracle, capi, case, seed=case[0][2] * 3 + case[1][0])
    p, dtf = case[2], case[3]
    ent, num = oracle.compact(a.reshape(pre.nbatch, -1))
    ref = oracle.deliver_pre(OL(oracle, pre), OL(oracle, post), p, p, w, entries=ent, num_active=num,
                             dt_factor=dtf, gsyn=g0.copy())
    ws = torch.empty(capi.deliver_tc_workspace_bytes(conn), dtype=torch.uint8, device="cuda")
    g = T(torch, g0)
    capi.deliver_pre_tc(conn, T(torch, a), T(torch, w), g, ws)
    out = H(g)
    assert capi.deliver_tc_check_error() == 0
    np.testing.assert_allclose(out, ref, rtol=RTOL, atol=RTOL * np.abs(ref).max())


def test_deliver_tc_repeated_calls_accumulate(cuda, oracle):
    """Two calls add twice (GSyn is accumulated into, as the reference's deliveries do), and a
    call on a zero activity leaves GSyn unchanged."""
    torch = cuda
    from openpv_gb300 import capi
    pre, post, a, w, g0, conn = _case(oracle, capi, TC_CASES[0], seed=11)
    w_post = oracle.transpose_shared(OL(oracle, pre), OL(oracle, post), 7, 7, w)
    ws = torch.empty(capi.deliver_tc_workspace_bytes(conn), dtype=torch.uint8, device="cuda")
    g1 = torch.zeros(post.res_shape(), device="cuda")
    capi.deliver_post_tc(conn, T(torch, a), T(torch, w_post), g1, ws)
    g2 = torch.zeros(post.res_shape(), device="cuda")
    capi.deliver_post_tc(conn, T(torch, a), T(torch, w_post), g2, ws)
    capi.deliver_post_tc(conn, T(torch, a), T(torch, w_post), g2, ws)
    np.testing.assert_allclose(H(g2), 2 * H(g1), rtol=1e-6, atol=1e-6 * np.abs(H(g1)).max())
    g = T(torch, g0)
    capi.deliver_post_tc(conn, torch.zeros(pre.ext_shape(), device="cuda"), T(torch, w_post), g, ws)
    assert np.array_equal(H(g), g0)


def test_deliver_tc_refuses_other_shapes(cuda):
    torch = cuda
    from openpv_gb300 import capi
    ws = torch.empty(1 << 20, dtype=torch.uint8, device="cuda")
    a = torch.zeros(1 << 16, device="cuda")
    g = torch.zeros(1 << 16, device="cuda")
    w = torch.zeros(1 << 16, device="cuda")
    bad = [
        capi.conn_desc(capi.Loc.make(1, 16, 16, 24, 3), capi.Loc.make(1, 16, 16, 32, 0), 7, 7),  # pre nf % 32
        capi.conn_desc(capi.Loc.make(1, 16, 16, 32, 3), capi.Loc.make(1, 16, 16, 48, 0), 7, 7),  # post nf % 32
        capi.conn_desc(capi.Loc.make(1, 32, 32, 32, 3), capi.Loc.make(1, 16, 16, 32, 0), 4, 4),  # many-to-one
        capi.conn_desc(capi.Loc.make(1, 16, 16, 32, 5), capi.Loc.make(1, 16, 16, 32, 0), 11, 11),  # patch > 9
    ]
    for conn in bad:
        assert capi.deliver_tc_workspace_bytes(conn) == 0  # the size query tells the shape apart too
        with pytest.raises(capi.PvgpuError) as e:
            capi.deliver_post_tc(conn, a, w, g, ws)
        assert e.value.status == capi.PVGPU_ERR_UNSUPPORTED_SHAPE
