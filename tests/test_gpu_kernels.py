"""GPU parity of the delivery / update kernels against the CPU oracle, called through
the C ABI (libpvgpu.so).  Integer work (compaction, geometry) and the update kernels are
compared bit for bit; FP32 delivery sums within 1e-5 relative in FAST mode and bit for
bit in REFERENCE_ORDER mode (the reference's single-thread order)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL_FP32 = 1e-5  # FP32 sums in a different order than the reference


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


def T(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def H(t):
    return t.cpu().numpy()


def OL(O, loc):
    return O.Loc.make(loc.nbatch, loc.nx, loc.ny, loc.nf, loc.halo.lt, loc.halo.dn)


def sparse_activity(rng, loc, p, zero_halo=True):
    a = np.zeros(loc.ext_shape(), np.float32)
    h = loc.halo
    core = (rng.random(loc.res_shape()) < p) * rng.uniform(1e-3, 1.0, loc.res_shape())
    a[:, h.up:h.up + loc.ny, h.lt:h.lt + loc.nx, :] = core
    if not zero_halo:
        a += (rng.random(loc.ext_shape()) < p) * rng.uniform(1e-3, 1.0, loc.ext_shape())
    return a.astype(np.float32)


# ---- a1: compaction --------------------------------------------------------------------

# Sizes: float4 units (n % 4 == 0) and scalar units, one chunk of 16384 and long look-back
# chains (the delivery microbenchmark's 16 x 134x134x256 extended activity: 281 chunks per
# image), empty and full activity.  `offset` starts the activity one float past an aligned
# address, which forces scalar units on an aligned size.
@pytest.mark.parametrize("nb,n,p,offset", [(3, 25600, 0.05, 0), (2, 4097, 0.5, 0), (1, 4096, 1.0, 0),
                                           (4, 777, 0.0, 0), (2, 204800, 0.02, 0), (1, 1, 1.0, 0),
                                           (16, 134 * 134 * 256, 0.01, 0), (5, 1000003, 0.3, 0),
                                           (3, 25600, 0.05, 1), (2, 8192 * 3, 1.0, 1), (2, 16384 * 3, 1.0, 0),
                                           (2, 16384 * 3 + 5, 0.4, 1)])
def test_compaction_bitexact(cuda, oracle, nb, n, p, offset):
    torch = cuda
    from openpv_gb300 import capi
    rng = np.random.default_rng(n)
    a = ((rng.random((nb, n)) < p) * rng.normal(size=(nb, n))).astype(np.float32)
    ent_ref, num_ref = oracle.compact(a)
    ent = torch.zeros((nb, n, 2), dtype=torch.int32, device="cuda")
    num = torch.full((nb,), -7, dtype=torch.int64, device="cuda")
    buf = torch.zeros(nb * n + offset, device="cuda")
    buf[offset:] = T(torch, a.reshape(-1))
    capi.compact_active(buf[offset:], nb, n, ent, num)
    num_h = H(num)
    ent_h = H(ent).view(np.uint8).reshape(nb, n, 8).view(capi.ENTRY_DTYPE).reshape(nb, n)
    assert np.array_equal(num_h, num_ref)
    for b in range(nb):
        k = num_ref[b]
        assert np.array_equal(ent_h[b, :k]["index"], ent_ref[b, :k]["index"])
        assert np.array_equal(ent_h[b, :k]["value"].view(np.uint32), ent_ref[b, :k]["value"].view(np.uint32))


# ---- a4: presynaptic delivery ------------------------------------------------------------

# (pre nb,nx,ny,nf,halo), (post nx,ny,nf,halo), nxp, nyp
PRE_CASES = [
    ((2, 16, 16, 64, 2), (32, 32, 1, 3), 8, 8),     # LCA reconstruction V1 -> error
    ((2, 16, 16, 24, 2), (32, 32, 3, 3), 8, 8),     # colour reconstruction
    ((2, 24, 20, 16, 3), (24, 20, 8, 0), 7, 7),     # one-to-one, shrunken at borders
    ((1, 32, 32, 4, 6), (8, 8, 5, 0), 4, 4),        # many-to-one x4
    ((3, 12, 8, 3, 1), (24, 16, 2, 2), 6, 4),       # one-to-many, unequal axes
    ((1, 20, 20, 40, 0), (20, 20, 600, 0), 3, 3),   # post features above one tile
    # one-to-one with 32 / 64 / 128 post features: the row-sliding kernel in FAST mode
    ((2, 40, 70, 16, 3), (40, 70, 64, 0), 7, 7),    # several row segments, the last partial
    ((1, 13, 37, 8, 2), (13, 37, 32, 0), 5, 5),     # columns not a multiple of 8
    ((2, 24, 33, 4, 1), (24, 33, 128, 0), 3, 3),
    ((1, 20, 40, 8, 4), (20, 40, 64, 1), 5, 5),     # pre halo above the margin, post halo
    ((1, 16, 40, 8, 1), (16, 40, 32, 0), 7, 7),     # pre halo below the margin
    ((2, 20, 36, 6, 4), (20, 36, 64, 0), 5, 9),     # unequal patch axes
    ((1, 30, 40, 1, 5), (30, 40, 32, 0), 11, 11),   # 11x11 (Gauss2D-style LIF input), 32 features
    ((2, 20, 36, 4, 6), (20, 36, 64, 0), 13, 13),   # tallest patch of the row-sliding kernel
    # the reference's GPU system tests (tests/GPUSystemTest/input), their layer sizes:
    ((1, 32, 32, 3, 1), (64, 64, 3, 0), 6, 6),      # preTest.params: TransposeConn of a 3x3 many-to-one, one-to-many x2
    ((4, 32, 32, 3, 8), (16, 16, 64, 0), 9, 9),     # preRecvBatch.params: batch 4, many-to-one x2, 9x9
]


@pytest.mark.parametrize("case", PRE_CASES)
@pytest.mark.parametrize("sparse", [True, False])
def test_deliver_pre_matches_oracle(cuda, oracle, case, sparse):
    torch = cuda
    from openpv_gb300 import capi
    (nb, nx, ny, nf, h), (qx, qy, qf, qh), nxp, nyp = case
    pre = capi.Loc.make(nb, nx, ny, nf, h)
    post = capi.Loc.make(nb, qx, qy, qf, qh)
    rng = np.random.default_rng(nx * 7 + qf)
    a = sparse_activity(rng, pre, 0.1, zero_halo=False)
    nk = (nx // qx if nx > qx else 1) * (ny // qy if ny > qy else 1) * nf
    w = rng.normal(0, 0.05, (nk, nyp, nxp, qf)).astype(np.float32)
    g0 = rng.normal(size=post.res_shape()).astype(np.float32)
    ent, num = oracle.compact(a.reshape(nb, -1))
    ref = oracle.deliver_pre(OL(oracle, pre), OL(oracle, post), nxp, nyp, w, entries=ent, num_active=num,
                             gsyn=g0.copy())
    conn = capi.conn_desc(pre, post, nxp, nyp)
    for mode in (capi.DELIVER_FAST, capi.DELIVER_REFERENCE_ORDER):
        g = T(torch, g0)
        if sparse:
            ent_d = T(torch, ent.view(np.uint8))
            capi.deliver_pre(conn, T(torch, w), g, entries=ent_d, num_active=T(torch, num), mode=mode)
        else:
            capi.deliver_pre(conn, T(torch, w), g, a_ext=T(torch, a), mode=mode)
        out = H(g)
        if mode == capi.DELIVER_REFERENCE_ORDER:
            assert np.array_equal(out.view(np.uint32), ref.view(np.uint32))
        else:
            np.testing.assert_allclose(out, ref, rtol=RTOL_FP32, atol=1e-5 * np.abs(ref).max())


@pytest.mark.parametrize("p,nb", [(0.01, 2), (0.05, 2), (0.2, 1)])
def test_deliver_pre_full_size_microbenchmark_connection(cuda, oracle, p, nb):
    """The delivery microbenchmark's connection at full size -- pre 128x128x256 (halo 3, zero),
    Bernoulli(p) x uniform(0,1] activity, post 128x128x64 one-to-one, 7x7 shared weights
    N(0, 0.05^2) -- on nb images: the SparseList delivery in REFERENCE_ORDER mode bit for bit
    against the oracle (the reference CPU loop's order), FAST mode and the tensor-core entry
    (dense activity, split-TF32) within 1e-5 of max|GSyn|."""
    torch = cuda
    from openpv_gb300 import capi
    pre = capi.Loc.make(nb, 128, 128, 256, 3)
    post = capi.Loc.make(nb, 128, 128, 64, 0)
    rng = np.random.default_rng(1234 + 2)
    a = np.zeros(pre.ext_shape(), np.float32)
    core = (rng.random(pre.res_shape()) < p) * (1.0 - rng.random(pre.res_shape()))
    a[:, 3:131, 3:131, :] = core
    w = rng.normal(0, 0.05, (256, 7, 7, 64)).astype(np.float32)
    ent, num = oracle.compact(a.reshape(nb, -1))
    ref = oracle.deliver_pre(OL(oracle, pre), OL(oracle, post), 7, 7, w, entries=ent, num_active=num)
    scale = np.abs(ref).max()
    conn = capi.conn_desc(pre, post, 7, 7)
    ad, wd = T(torch, a), T(torch, w)
    ent_d = torch.zeros((nb, pre.num_ext, 2), dtype=torch.int32, device="cuda")
    num_d = torch.zeros(nb, dtype=torch.int64, device="cuda")
    capi.compact_active(ad, nb, pre.num_ext, ent_d, num_d)
    assert np.array_equal(H(num_d), num)
    for mode in (capi.DELIVER_REFERENCE_ORDER, capi.DELIVER_FAST):
        g = torch.zeros(post.res_shape(), device="cuda")
        capi.deliver_pre(conn, wd, g, entries=ent_d, num_active=num_d, mode=mode)
        out = H(g)
        if mode == capi.DELIVER_REFERENCE_ORDER:
            assert np.array_equal(out.view(np.uint32), ref.view(np.uint32))
        else:
            assert np.abs(out - ref).max() <= 1e-5 * scale
    ws = torch.empty(capi.deliver_tc_workspace_bytes(conn), dtype=torch.uint8, device="cuda")
    g = torch.zeros(post.res_shape(), device="cuda")
    capi.deliver_pre_tc(conn, ad, wd, g, ws)
    assert capi.deliver_tc_check_error() == 0
    assert np.abs(H(g) - ref).max() <= 1e-5 * scale


def test_deliver_pre_empty_activity(cuda, oracle):
    torch = cuda
    from openpv_gb300 import capi
    pre = capi.Loc.make(2, 16, 16, 8, 2)
    post = capi.Loc.make(2, 32, 32, 1, 3)
    g0 = np.arange(2 * 32 * 32, dtype=np.float32).reshape(post.res_shape())
    g = T(torch, g0)
    ent = torch.zeros((2, pre.num_ext, 2), dtype=torch.int32, device="cuda")
    num = torch.zeros(2, dtype=torch.int64, device="cuda")
    capi.deliver_pre(capi.conn_desc(pre, post, 8, 8), torch.ones(8 * 64, device="cuda"), g, entries=ent,
                     num_active=num)
    assert np.array_equal(H(g), g0)


# ---- a5: postsynaptic delivery ------------------------------------------------------------

# conn pre -> post with the pre layer's halo at least the post-perspective margin
POST_CASES = [
    ((2, 32, 32, 1, 3), (16, 16, 64, 2), 4, 4),     # error -> V1 (LCA), many-to-one x2, 8x8 receptive field
    ((2, 32, 32, 3, 3), (16, 16, 48, 2), 4, 4),     # colour LCA
    ((1, 24, 24, 16, 3), (24, 24, 8, 0), 7, 7),     # one-to-one
    ((2, 8, 8, 6, 2), (16, 16, 4, 1), 4, 4),        # one-to-many x2 (kernel phases)
    ((1, 64, 64, 1, 6), (16, 16, 32, 2), 4, 4),     # stride-4 dictionary, 16x16 receptive field
    # the reference's GPU system tests (tests/GPUSystemTest/input), their layer sizes:
    ((1, 64, 64, 3, 8), (32, 32, 64, 0), 9, 9),     # postTest.params: TransposeConn of an 18x18 dictionary
    ((16, 64, 64, 3, 8), (32, 32, 64, 0), 9, 9),    # postRecvBatch.params: batch 16
    ((1, 32, 32, 64, 8), (64, 64, 3, 0), 18, 18),   # postTestOneToMany.params: one-to-many x2
    ((1, 32, 32, 3, 5), (16, 16, 192, 0), 6, 6),    # oneToTwo.params / twoToOneAccumulation.params, 192 features
    ((1, 32, 32, 3, 3), (16, 16, 192, 0), 4, 4),
]


@pytest.mark.parametrize("case", POST_CASES)
def test_deliver_post_matches_oracle(cuda, oracle, case):
    torch = cuda
    from openpv_gb300 import capi
    (nb, nx, ny, nf, h), (qx, qy, qf, qh), nxp, nyp = case
    pre = capi.Loc.make(nb, nx, ny, nf, h)
    post = capi.Loc.make(nb, qx, qy, qf, qh)
    rng = np.random.default_rng(qf + nx)
    a = rng.normal(size=pre.ext_shape()).astype(np.float32)
    nk = (nx // qx if nx > qx else 1) * (ny // qy if ny > qy else 1) * nf
    w = rng.normal(0, 0.05, (nk, nyp, nxp, qf)).astype(np.float32)
    w_post = oracle.transpose_shared(OL(oracle, pre), OL(oracle, post), nxp, nyp, w)
    # the GPU transpose agrees with the oracle bit for bit
    conn = capi.conn_desc(pre, post, nxp, nyp)
    w_post_d = torch.zeros(w_post.size, dtype=torch.float32, device="cuda")
    capi.transpose_weights(conn, T(torch, w), w_post_d)
    assert np.array_equal(H(w_post_d).reshape(w_post.shape), w_post)
    g0 = rng.normal(size=post.res_shape()).astype(np.float32)
    nxpP = oracle.post_patch_size(nxp, nx, qx)
    nypP = oracle.post_patch_size(nyp, ny, qy)
    ref = oracle.deliver_post(OL(oracle, pre), OL(oracle, post), nxpP, nypP, w_post, a, gsyn=g0.copy())
    for mode in (capi.DELIVER_FAST, capi.DELIVER_REFERENCE_ORDER):
        g = T(torch, g0)
        capi.deliver_post(conn, T(torch, a), w_post_d, g, mode=mode)
        out = H(g)
        if mode == capi.DELIVER_REFERENCE_ORDER:
            assert np.array_equal(out.view(np.uint32), ref.view(np.uint32))
        else:
            np.testing.assert_allclose(out, ref, rtol=RTOL_FP32, atol=1e-5 * np.abs(ref).max())


# (pre nbatch, nx, ny, nf), (post nx, ny, nf), patch of the pre -> post connection
PRE_POST_CASES = [
    ((2, 32, 32, 8), (16, 16, 16), 4),
    # tests/ReceiveFromPostTest/input of the reference, their layer sizes:
    ((1, 32, 32, 3), (16, 16, 10), 2),     # manyToOnePatchSizeTest.params
    ((1, 4, 4, 3), (8, 8, 10), 4),         # oneToManyPatchSizeTest.params
    ((1, 16, 16, 96), (8, 8, 384), 3),     # postTest.params: TransposeConn of a 6x6x96 one-to-many
    ((1, 32, 32, 3), (16, 16, 3), 3),      # postTest_ManyToOne.params
    ((1, 16, 16, 3), (32, 32, 3), 10),     # postTest_OneToMany.params
]


@pytest.mark.parametrize("case", PRE_POST_CASES)
def test_pre_and_post_perspective_agree(cuda, oracle, case):
    """ReceiveFromPostTest's property: pre- and post-perspective delivery of the same
    connection give the same GSyn, to the rounding of the terms summed per element
    (n * 2^-24 of the largest value; postTest.params:176 allows 3e-3)."""
    torch = cuda
    from openpv_gb300 import capi
    (nb, nx, ny, nf), (qx, qy, qf), p = case
    pp = oracle.post_patch_size(p, nx, qx)
    h = max(oracle.required_margin(nx, qx, p), oracle.required_margin(qx, nx, pp))
    pre = capi.Loc.make(nb, nx, ny, nf, h)
    post = capi.Loc.make(nb, qx, qy, qf, 0)
    rng = np.random.default_rng(5)
    a = sparse_activity(rng, pre, 0.3)
    nk = (nx // qx if nx > qx else 1) * (ny // qy if ny > qy else 1) * nf
    w = rng.normal(0, 0.1, (nk, p, p, qf)).astype(np.float32)
    conn = capi.conn_desc(pre, post, p, p)
    g_pre = torch.zeros(post.res_shape(), device="cuda")
    capi.deliver_pre(conn, T(torch, w), g_pre, a_ext=T(torch, a))
    w_post = torch.zeros(w.size, device="cuda")
    capi.transpose_weights(conn, T(torch, w), w_post)
    g_post = torch.zeros(post.res_shape(), device="cuda")
    capi.deliver_post(conn, T(torch, a), w_post, g_post)
    n_inputs = pp * pp * nf
    np.testing.assert_allclose(H(g_pre), H(g_post), atol=n_inputs * 2.0 ** -24 * np.abs(H(g_pre)).max())


# ---- a6..a9: layer update ------------------------------------------------------------------

def test_update_kernels_bitexact(cuda, oracle):
    torch = cuda
    from openpv_gb300 import capi
    rng = np.random.default_rng(9)
    loc = capi.Loc.make(5, 16, 16, 64, 2)
    ol = OL(oracle, loc)
    v = rng.normal(0, 0.3, loc.res_shape()).astype(np.float32)
    gs = rng.normal(0, 0.3, (2,) + loc.res_shape()).astype(np.float32)
    a = oracle.ann_activity(ol, rng.normal(0, 0.3, loc.res_shape()).astype(np.float32), 0.1, 0.0, np.inf, 0.1, 0.0)
    dt = np.array([1.0, 0.5, 0.25, 2.0, 1.0], np.float64)
    coeffs = np.array([1.0, -1.0], np.float32)
    # accumulate
    g_ref = oracle.gsyn_accumulate(gs, coeffs)
    g = torch.zeros(loc.res_shape(), device="cuda")
    capi.gsyn_accumulate(loc.num_res * 5, [1.0, -1.0], T(torch, gs), g)
    assert np.array_equal(H(g).view(np.uint32), g_ref.view(np.uint32))
    # LCA membrane update
    v_ref = oracle.lca_update(ol, g_ref, a, v, dt, 100.0)
    vd = T(torch, v)
    capi.lca_update(loc, True, T(torch, dt), 100.0, g, T(torch, a), vd)
    assert np.array_equal(H(vd).view(np.uint32), v_ref.view(np.uint32))
    # thresholds: soft, firm, clipped, identity
    for th in [(0.1, 0.0, np.inf, 0.1, 0.0), (0.025, 0.0, np.inf, 0.0, 0.025), (0.1, 0.0, 0.2, 0.1, 0.0),
               (-np.inf, -np.inf, np.inf, 0.0, 0.0)]:
        a_ref = oracle.ann_activity(ol, v_ref, *th, a_ext=a)
        ad = T(torch, a)
        capi.ann_activity(loc, vd, *th, ad)
        assert np.array_equal(H(ad).view(np.uint32), a_ref.view(np.uint32)), th
    # fused
    import ctypes
    desc = capi.LcaLayerDesc(loc, 2, (ctypes.c_float * 4)(1.0, -1.0, 0.0, 0.0), 1, 100.0, 0.1, 0.0, np.inf, 0.1, 0.0)
    a2_ref = oracle.ann_activity(ol, v_ref, 0.1, 0.0, np.inf, 0.1, 0.0, a_ext=a)
    vd2 = T(torch, v)
    ad2 = T(torch, a)
    capi.lca_layer_update(desc, T(torch, gs), T(torch, dt), vd2, ad2)
    assert np.array_equal(H(vd2).view(np.uint32), v_ref.view(np.uint32))
    assert np.array_equal(H(ad2).view(np.uint32), a2_ref.view(np.uint32))


def test_momentum_and_ista_updates_bitexact(cuda, oracle):
    """MomentumLCAInternalStateBuffer.kpp and ISTAInternalStateBuffer.kpp on the GPU equal the
    oracle (itself pinned to the reference .kpp code) bit for bit, over several steps."""
    torch = cuda
    from openpv_gb300 import capi
    rng = np.random.default_rng(23)
    loc = capi.Loc.make(4, 12, 10, 32, 2)
    ol = OL(oracle, loc)
    dt = np.array([1.0, 0.5, 0.25, 2.0], np.float64)
    v = rng.normal(0, 0.3, loc.res_shape()).astype(np.float32)
    pd = np.zeros_like(v)
    vd, pdd = T(torch, v), T(torch, pd)
    vi, vid = v.copy(), T(torch, v)
    for step in range(4):
        g = rng.normal(0, 0.3, loc.res_shape()).astype(np.float32)
        a = oracle.ann_activity(ol, rng.normal(0, 0.3, loc.res_shape()).astype(np.float32), 0.1, 0.0, np.inf, 0.1, 0.0)
        v, pd = oracle.momentum_lca_update(ol, g, a, pd, v, dt, 50.0, 0.6, step % 2 == 0)
        capi.momentum_lca_update(loc, step % 2 == 0, 0.6, T(torch, dt), 50.0, T(torch, g), T(torch, a), pdd, vd)
        assert np.array_equal(H(vd).view(np.uint32), v.view(np.uint32))
        assert np.array_equal(H(pdd).view(np.uint32), pd.view(np.uint32))
        vi = oracle.ista_update(ol, g, a, vi, dt, 20.0, 0.1)
        capi.ista_update(loc, 0.1, T(torch, dt), 20.0, T(torch, g), T(torch, a), vid)
        assert np.array_equal(H(vid).view(np.uint32), vi.view(np.uint32))


# ---- a11: energy ---------------------------------------------------------------------------

@pytest.mark.parametrize("kind,p0,p1", [(0, 0.0, 0.0), (1, 0.0, 0.0), (2, 0.025, 0.025)])
def test_cost_sum_fp64(cuda, oracle, kind, p0, p1):
    torch = cuda
    from openpv_gb300 import capi
    rng = np.random.default_rng(kind)
    loc = capi.Loc.make(4, 16, 16, 64, 2)
    buf = rng.normal(0, 0.1, loc.ext_shape()).astype(np.float32)
    ref = oracle.cost_sum(OL(oracle, loc), buf, kind, p0, p1)
    out = torch.zeros(4, dtype=torch.float64, device="cuda")
    capi.cost_sum(loc, T(torch, buf), kind, p0, p1, out)
    np.testing.assert_allclose(H(out), ref, rtol=1e-12)


# ---- a12: Hebbian ----------------------------------------------------------------------------

@pytest.mark.parametrize("case", [((3, 16, 16, 8, 2), (32, 32, 1, 3), 8, 8),
                                  ((2, 10, 10, 4, 1), (10, 10, 3, 1), 3, 3),
                                  ((2, 16, 16, 4, 3), (8, 8, 2, 0), 2, 2)])
def test_hebbian_bitexact(cuda, oracle, case):
    torch = cuda
    from openpv_gb300 import capi
    (nb, nx, ny, nf, h), (qx, qy, qf, qh), nxp, nyp = case
    pre = capi.Loc.make(nb, nx, ny, nf, h)
    post = capi.Loc.make(nb, qx, qy, qf, qh)
    rng = np.random.default_rng(2)
    a = sparse_activity(rng, pre, 0.3)
    r = rng.normal(size=post.ext_shape()).astype(np.float32)
    ref = oracle.hebbian_dw(OL(oracle, pre), OL(oracle, post), nxp, nyp, a, r, 1.0)
    dw = torch.zeros(ref.size, device="cuda")
    capi.hebbian_dw(capi.conn_desc(pre, post, nxp, nyp), 1.0, T(torch, a), T(torch, r), dw)
    assert np.array_equal(H(dw).reshape(ref.shape).view(np.uint32), ref.view(np.uint32))


# ---- tcgen05 building block ------------------------------------------------------------------

@pytest.mark.parametrize("M,N,K", [(128, 64, 64), (256, 192, 512), (384, 256, 192), (128, 16, 128)])
def test_tc_gemm_bf16(cuda, M, N, K):
    """TMA -> SW128 smem -> tcgen05.mma -> TMEM -> tcgen05.ld against an FP32 host GEMM of
    the same BF16 values (FP32 accumulation: only summation order differs)."""
    torch = cuda
    from openpv_gb300 import capi
    g = torch.Generator().manual_seed(M + N + K)
    A = torch.randn(M, K, generator=g).to(torch.bfloat16)
    B = torch.randn(N, K, generator=g).to(torch.bfloat16)
    ref = A.float() @ B.float().T
    C = torch.zeros(M, N, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    capi.tc_gemm_bf16(A.cuda(), B.cuda(), C, M, N, K, err)
    torch.cuda.synchronize()
    assert int(err.item()) == 0, "a bounded device wait timed out"
    np.testing.assert_allclose(C.cpu().numpy(), ref.numpy(), rtol=1e-4, atol=1e-3)


@pytest.mark.parametrize("M,N,K", [(128, 64, 64), (256, 192, 512), (128, 256, 128)])
def test_tc_gemm_bf16_mn_major_b(cuda, M, N, K):
    """The MN-major B operand (B stored [K][N], 128-byte rows along K, 64-column groups 8 KB apart:
    a K-major weight tile read transposed) against the same host GEMM."""
    torch = cuda
    from openpv_gb300 import capi
    g = torch.Generator().manual_seed(7 * M + N + K)
    A = torch.randn(M, K, generator=g).to(torch.bfloat16)
    B = torch.randn(K, N, generator=g).to(torch.bfloat16)
    ref = A.float() @ B.float()
    C = torch.zeros(M, N, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    capi.tc_gemm_bf16_kn(A.cuda(), B.cuda(), C, M, N, K, err)
    torch.cuda.synchronize()
    assert int(err.item()) == 0, "a bounded device wait timed out"
    np.testing.assert_allclose(C.cpu().numpy(), ref.numpy(), rtol=1e-4, atol=1e-3)


@pytest.mark.parametrize("M,N,K", [(128, 64, 64), (256, 192, 192), (128, 256, 256)])
def test_tc_gemm_bf16_a_from_tmem(cuda, M, N, K):
    """A read by tcgen05.mma from tensor memory (row m in lane m, two K elements per 32-bit
    column, stored with tcgen05.st) against the same host GEMM."""
    torch = cuda
    from openpv_gb300 import capi
    g = torch.Generator().manual_seed(3 * M + N + K)
    A = torch.randn(M, K, generator=g).to(torch.bfloat16)
    B = torch.randn(N, K, generator=g).to(torch.bfloat16)
    ref = A.float() @ B.float().T
    C = torch.zeros(M, N, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    capi.tc_gemm_bf16_atmem(A.cuda(), B.cuda(), C, M, N, K, err)
    torch.cuda.synchronize()
    assert int(err.item()) == 0, "a bounded device wait timed out"
    np.testing.assert_allclose(C.cpu().numpy(), ref.numpy(), rtol=1e-4, atol=1e-3)


def test_deliver_ident_matches_reference_rule(cuda, oracle):
    """IdentDelivery (delivery/IdentDelivery.cpp:99-180): GSyn += the restricted activity, from the
    dense extended buffer or from the SparseList (entries in the halo skipped); one contribution
    per element, so bit-exact."""
    torch = cuda
    from openpv_gb300 import capi
    pre = capi.Loc.make(3, 20, 12, 5, 2)
    post = capi.Loc.make(3, 20, 12, 5, 0)
    rng = np.random.default_rng(21)
    a = sparse_activity(rng, pre, 0.3, zero_halo=False)  # halo entries present: must be skipped
    g0 = rng.normal(size=post.res_shape()).astype(np.float32)
    ref = g0 + a[:, 2:14, 2:22, :]
    ent, num = oracle.compact(a.reshape(3, -1))
    L = capi.lib()
    for sparse in (False, True):
        g = T(torch, g0)
        if sparse:
            ent_d = T(torch, ent.view(np.uint8))
            st = L.pvgpu_deliver_ident(C.byref(pre), C.byref(post), capi._ptr(ent_d), capi._ptr(T(torch, num)), None,
                                       capi._ptr(g), capi._stream())
        else:
            st = L.pvgpu_deliver_ident(C.byref(pre), C.byref(post), None, None, capi._ptr(T(torch, a)), capi._ptr(g),
                                       capi._stream())
        assert st == 0
        assert np.array_equal(H(g).view(np.uint32), ref.view(np.uint32)), sparse
    # errScale: V *= s, elementwise in FP32
    v = rng.normal(size=1000).astype(np.float32)
    vd = T(torch, v)
    assert L.pvgpu_err_scale(v.size, C.c_float(0.3), capi._ptr(vd), capi._stream()) == 0
    assert np.array_equal(H(vd), v * np.float32(0.3))


@pytest.mark.parametrize("method", ["v", "s", "a"])
def test_momentum_weight_update_bitexact(cuda, oracle, method):
    """MomentumUpdater::updateWeights on the device (pvgpu_momentum_update_weights) equals the
    oracle's restatement over several updates, with the Hebbian dW of each update from
    pvgpu_hebbian_dw (itself bit-exact vs the oracle)."""
    torch = cuda
    from openpv_gb300 import capi
    rng = np.random.default_rng(ord(method))
    n = 64 * 8 * 8 * 3 + 5
    f_d = capi.momentum_factors(method, 0.8 if method != "v" else 20.0, 0.01, 0.5)
    f_o = oracle.momentum_factors(method, 0.8 if method != "v" else 20.0, 0.01, 0.5)
    assert f_d == f_o
    w = rng.normal(size=n).astype(np.float32)
    prev = np.zeros(n, np.float32)
    wd, pd = T(torch, w), T(torch, prev)
    for _ in range(4):
        dw = rng.normal(0, 0.1, n).astype(np.float32)
        dd = T(torch, dw)
        dw, prev, w = oracle.momentum_update_weights(dw, prev, w, *f_o)
        capi.momentum_update_weights(dd, pd, wd, *f_d)
        for a, b in ((dd, dw), (pd, prev), (wd, w)):
            assert np.array_equal(H(a).view(np.uint32), b.view(np.uint32))


@pytest.mark.parametrize("vertices", ["soft", "firm", "list"])
def test_ann_vertices_bitexact(cuda, oracle, vertices):
    """pvgpu_ann_vertices (the reference GPU path's vertex form, device vertex arrays) against the
    oracle's vertex form, itself pinned to the reference's kernel: bit for bit, potentials on the
    vertices included."""
    torch = cuda
    from openpv_gb300 import capi
    rng = np.random.default_rng(21)
    loc = capi.Loc.make(3, 20, 12, 7, 2)
    v = (rng.normal(size=loc.res_shape()) * 0.5).astype(np.float32)
    if vertices == "list":
        vV = np.array([-0.5, 0.0, 0.0, 0.25, 1.0], np.float32)
        vA = np.array([-0.5, 0.0, 0.1, 0.3, 0.7], np.float32)
        sl = np.array([1.0, 1.0, 0.0, 0.8, 0.533, 2.0], np.float32)
        v.reshape(-1)[:5] = vV
    else:
        th = (0.1, 0.0, np.inf, 0.1, 0.0) if vertices == "soft" else (0.1, 0.0, np.inf, 0.0, 0.05)
        vV, vA, sl = oracle.ann_vertices(*[np.float32(x) for x in th])
    ref = oracle.apply_vertices(OL(oracle, loc), v, vV, vA, sl)
    a = torch.full(loc.ext_shape(), 7.0, device="cuda")
    a_ref = ref.copy()
    h = loc.halo
    mask = np.ones(loc.ext_shape(), bool)
    mask[:, h.up:h.up + loc.ny, h.lt:h.lt + loc.nx, :] = False
    a_ref[mask] = 7.0  # the halo is left as it was
    capi.ann_vertices(loc, T(torch, vV), T(torch, vA), T(torch, sl), T(torch, v), a)
    assert np.array_equal(H(a).view(np.uint32), a_ref.view(np.uint32))
