"""The C++ host side (libpvhost.so) runs the LCA module from an OpenPV params file on the GPU:
IdentConn input -> residual, HyPerConn V1 -> residual (presynaptic perspective), TransposeConn
residual -> V1 (postsynaptic perspective), ANNErrorLayer and HyPerLCALayer updates in phase order.

With receiveGpu = false every delivery is the reference's "...ConvolveDelivery" keyword, run by
the REFERENCE_ORDER kernels: V and A of V1 equal the FP32 oracle's LCA (the reference CPU loops
restated and pinned bit for bit) exactly, whether V1 publishes a SparseList or dense activity.
With receiveGpu = true the "...GPUDelivery" keywords run the FAST kernels: within 1e-5 relative
(V) of the same oracle after the same steps."""
import numpy as np
import pytest

from tests.lca_params import lca_params

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def capi():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from openpv_gb300 import build
    build.build()
    from openpv_gb300 import capi
    return capi


def inputs(nb, n, c, nf, nxp, seed=11):
    rng = np.random.default_rng(seed)
    x = rng.normal(size=(nb, n, n, c)).astype(np.float32)
    x = (x - x.mean(axis=(1, 2, 3), keepdims=True)) / x.std(axis=(1, 2, 3), keepdims=True)
    w = rng.normal(size=(nf, nxp, nxp, c))
    w = (w / np.sqrt((w ** 2).sum(axis=(1, 2, 3), keepdims=True))).astype(np.float32)
    return x, w


def oracle_lca(oracle, x, w, steps, nb, n, c, nf, nxp, vthresh=0.1, tau=100.0, err_scale=1.0):
    p = oracle.lca_params(nbatch=nb, inNx=n, inNy=n, inNf=c, v1Nx=n // 2, v1Ny=n // 2, v1Nf=nf, nxp=nxp, nyp=nxp,
                          VThresh=vthresh, AShift=vthresh, AMin=0.0, VWidth=0.0, tau=tau, errScale=err_scale,
                          dtFixed=1.0)
    v0 = np.zeros((nb, n // 2, n // 2, nf), np.float32)
    v, a, _, _ = oracle.lca_run(p, w, x[None], steps, v0, want_recon=False)
    return v, a


def run_column(capi, text, x, w, steps):
    col = capi.Column(text)
    col.set_weights("V1ToResidual", w)
    col.set_input("Input", x[None])
    col.advance(steps)
    return col, col.read("V1", "V"), col.read("V1", "A")


@pytest.mark.parametrize("sparse", [True, False])
def test_convolve_deliveries_equal_the_reference_cpu_path(capi, oracle, sparse):
    nb, n, c, nf, nxp, steps = 2, 32, 1, 16, 8, 12
    x, w = inputs(nb, n, c, nf, nxp)
    col, v, a = run_column(capi, lca_params(nb=nb, n=n, c=c, nf=nf, nxp=nxp, receive_gpu=False, sparse=sparse), x, w,
                           steps)
    assert col.delivery("V1ToResidual") == "PresynapticPerspectiveConvolveDelivery"
    assert col.delivery("ResidualToV1") == "PostsynapticPerspectiveConvolveDelivery"
    assert col.delivery("InputToResidual") == "IdentDelivery"
    assert col.delivery_engine("ResidualToV1") == "reference-order"
    # halos from the connections' margins (requiredConvolveMargin), as the reference sizes them
    assert col.layer_info("V1")["halo"] == 2 and col.layer_info("Residual")["halo"] == 3
    v_ref, a_ref = oracle_lca(oracle, x, w, steps, nb, n, c, nf, nxp)
    assert (a_ref > 0).any() and (a_ref == 0).any()  # a sparse, nontrivial code
    assert np.array_equal(v.view(np.uint32), v_ref.view(np.uint32))
    assert np.array_equal(a.view(np.uint32), a_ref.view(np.uint32))


def test_colour_and_err_scale(capi, oracle):
    nb, n, c, nf, nxp, steps = 1, 32, 3, 32, 8, 8
    x, w = inputs(nb, n, c, nf, nxp, seed=5)
    text = lca_params(nb=nb, n=n, c=c, nf=nf, nxp=nxp, receive_gpu=False, err_scale=0.75)
    _, v, a = run_column(capi, text, x, w, steps)
    v_ref, a_ref = oracle_lca(oracle, x, w, steps, nb, n, c, nf, nxp, err_scale=0.75)
    assert np.array_equal(v.view(np.uint32), v_ref.view(np.uint32))
    assert np.array_equal(a.view(np.uint32), a_ref.view(np.uint32))


def test_gpu_deliveries_within_fp32_tolerance(capi, oracle):
    nb, n, c, nf, nxp, steps = 2, 32, 1, 16, 8, 12
    x, w = inputs(nb, n, c, nf, nxp)
    col, v, a = run_column(capi, lca_params(nb=nb, n=n, c=c, nf=nf, nxp=nxp, receive_gpu=True), x, w, steps)
    assert col.delivery("V1ToResidual") == "PresynapticPerspectiveGPUDelivery"
    assert col.delivery("ResidualToV1") == "PostsynapticPerspectiveGPUDelivery"
    v_ref, a_ref = oracle_lca(oracle, x, w, steps, nb, n, c, nf, nxp)
    vs = np.abs(v_ref).max()
    np.testing.assert_allclose(v, v_ref, rtol=1e-5, atol=1e-5 * vs)
    np.testing.assert_allclose(a, a_ref, rtol=1e-5, atol=1e-5 * vs)


def test_presynaptic_transpose_and_errors(capi, oracle):
    """The transpose delivered from the presynaptic perspective (its weights transposed on the
    device) gives the same V1 within FP32 summation-order tolerance; unsupported switches are
    refused with the reference's wording."""
    nb, n, c, nf, nxp, steps = 1, 32, 1, 16, 8, 6
    x, w = inputs(nb, n, c, nf, nxp)
    col, v, _ = run_column(capi, lca_params(nb=nb, n=n, c=c, nf=nf, nxp=nxp, post_perspective=False), x, w, steps)
    assert col.delivery("ResidualToV1") == "PresynapticPerspectiveConvolveDelivery"
    v_ref, _ = oracle_lca(oracle, x, w, steps, nb, n, c, nf, nxp)
    np.testing.assert_allclose(v, v_ref, rtol=1e-5, atol=1e-5 * np.abs(v_ref).max())
    bad = lca_params().replace('pvpatchAccumulateType = "convolve";\n};\n\nTransposeConn',
                               'pvpatchAccumulateType = "stochastic";\n};\n\nTransposeConn')
    assert "stochastic" in bad
    with pytest.raises(RuntimeError, match="PresynapticPerspectiveStochasticDelivery"):
        capi.Column(bad)
    with pytest.raises(RuntimeError, match="pvpatchAccumulateType"):
        capi.Column(lca_params().replace('"convolve"', '"maxpooling"', 1))


def module_oracle(oracle, x, w, steps, nb, n, c, nf, nxp, kind, vthresh=0.1, tau=100.0, rate=0.0):
    """The LCA module composed from the oracle's pinned pieces in the reference's phase order,
    with the V1 membrane update of HyPerLCALayer, MomentumLCALayer or ISTALayer."""
    v1n = n // 2
    v1 = oracle.Loc.make(nb, v1n, v1n, nf, 2)
    er = oracle.Loc.make(nb, n, n, c, 3)
    fmax = np.float32(3.4028234663852886e38)
    v = np.zeros(v1.res_shape(), np.float32)
    prev = np.zeros_like(v)
    a1 = oracle.ann_activity(v1, v, vthresh, 0.0, fmax, vthresh, 0.0)
    dt = np.ones(nb, np.float64)
    for _ in range(steps):
        ch1 = oracle.deliver_pre(v1, er, nxp, nxp, w, a_ext=a1)
        g = oracle.gsyn_accumulate(np.stack([x + np.float32(0), ch1]), np.array([1.0, -1.0], np.float32))
        ae = oracle.ann_activity(er, g, -fmax, -fmax, fmax, 0.0, 0.0)
        g1 = oracle.gsyn_accumulate(oracle.deliver_post(er, v1, nxp, nxp, w, ae)[None], np.array([1.0, -1.0], np.float32))
        if kind == "HyPerLCALayer":
            v = oracle.lca_update(v1, g1, a1, v, dt, tau)
        elif kind == "MomentumLCALayer":
            v, prev = oracle.momentum_lca_update(v1, g1, a1, prev, v, dt, tau, rate)
        else:
            v = oracle.ista_update(v1, g1, a1, v, dt, tau, vthresh)
        a1 = oracle.ann_activity(v1, v, vthresh, 0.0, fmax, vthresh, 0.0)
    return v, a1[:, 2:-2, 2:-2, :]


@pytest.mark.parametrize("kind, rate", [("HyPerLCALayer", 0.0), ("MomentumLCALayer", 0.5), ("ISTALayer", 0.0)])
def test_lca_variants_equal_the_reference_composition(capi, oracle, kind, rate):
    """MomentumLCALayer (MomentumLCAInternalStateBuffer.kpp) and ISTALayer
    (ISTAInternalStateBuffer.kpp) in the params-built column, Convolve deliveries: V and A equal
    the oracle pieces composed in phase order, bit for bit (HyPerLCALayer as the control)."""
    nb, n, c, nf, nxp, steps = 2, 32, 1, 16, 8, 10
    x, w = inputs(nb, n, c, nf, nxp, seed=3)
    tau = 100.0 if kind != "ISTALayer" else 20.0
    text = lca_params(nb=nb, n=n, c=c, nf=nf, nxp=nxp, tau=tau, v1_keyword=kind, momentum=rate)
    _, v, a = run_column(capi, text, x, w, steps)
    v_ref, a_ref = module_oracle(oracle, x, w, steps, nb, n, c, nf, nxp, kind, tau=tau, rate=rate)
    assert np.array_equal(v.view(np.uint32), v_ref.view(np.uint32)), kind
    assert np.array_equal(a.view(np.uint32), a_ref.view(np.uint32)), kind
    if kind == "HyPerLCALayer":  # the composition is the oracle's LCA module itself
        v2, _ = oracle_lca(oracle, x, w, steps, nb, n, c, nf, nxp)
        assert np.array_equal(v_ref.view(np.uint32), v2.view(np.uint32))


def one_to_one_params(nb, nx, ny, cin, cout, p, perspective_post):
    return f"""
HyPerCol "column" = {{ nx = {nx}; ny = {ny}; nbatch = {nb}; dt = 1.0; stopTime = 10; }};
ImageLayer "Input" = {{ nxScale = 1; nyScale = 1; nf = {cin}; phase = 0; displayPeriod = 0; inputPath = "in.txt"; }};
HyPerLayer "Out" = {{ nxScale = 1; nyScale = 1; nf = {cout}; phase = 1; InitVType = "ZeroV"; sparseLayer = false; }};
HyPerConn "InToOut" = {{
   preLayerName = "Input"; postLayerName = "Out"; channelCode = 0;
   nxp = {p}; nyp = {p}; nfp = {cout}; sharedWeights = true; weightInitType = "FileWeight";
   initWeightsFile = "w.pvp"; plasticityFlag = false; receiveGpu = true;
   updateGSynFromPostPerspective = {"true" if perspective_post else "false"}; pvpatchAccumulateType = "convolve";
}};
"""


@pytest.mark.parametrize("post", [True, False])
def test_one_to_one_gpu_delivery_in_the_column(capi, oracle, post):
    """A one-to-one HyPerConn with 32 / 64 features: the postsynaptic GPU keyword runs the
    tensor-core delivery, the presynaptic one the sparse kernel; both within 1e-5 of the oracle's
    FP32 delivery of the input frame (HyPerLayer: V = GSyn)."""
    nb, nx, ny, cin, cout, p = 2, 40, 12, 32, 64, 5
    rng = np.random.default_rng(17)
    x = ((rng.random((nb, ny, nx, cin)) < 0.3) * rng.uniform(0, 1, (nb, ny, nx, cin))).astype(np.float32)
    w = rng.normal(0, 0.05, (cin, p, p, cout)).astype(np.float32)
    col = capi.Column(one_to_one_params(nb, nx, ny, cin, cout, p, post))
    assert col.delivery("InToOut") == ("PostsynapticPerspectiveGPUDelivery" if post else
                                       "PresynapticPerspectiveGPUDelivery")
    col.set_weights("InToOut", w)
    col.set_input("Input", x[None])
    col.advance(1)
    assert col.delivery_engine("InToOut") == ("tensor-core" if post else "simt")
    v = col.read("Out", "V")
    h = col.layer_info("Input")["halo"]
    pre = oracle.Loc.make(nb, nx, ny, cin, h, h)
    postl = oracle.Loc.make(nb, nx, ny, cout, 0, 0)
    a = np.zeros(pre.ext_shape(), np.float32)
    a[:, h:h + ny, h:h + nx, :] = x
    ref = oracle.deliver_pre(pre, postl, p, p, w, a_ext=a)
    np.testing.assert_allclose(v, ref, rtol=1e-5, atol=1e-5 * np.abs(ref).max())


def lif_network_params(nb, n, p, outdir, inpath, method):
    return f"""
HyPerCol "column" = {{ nx = {n}; ny = {n}; nbatch = {nb}; dt = 1.0; stopTime = 10; randomSeed = 5;
   outputPath = "{outdir}"; }};
PvpLayer "Spikes" = {{ nxScale = 1; nyScale = 1; nf = 1; phase = 0; displayPeriod = 1; inputPath = "{inpath}";
   sparseLayer = true; writeStep = 1; }};
LIFLayer "Exc" = {{ nxScale = 1; nyScale = 1; nf = 4; phase = 1; InitVType = "ConstantV"; valueV = -70;
   method = "{method}"; sparseLayer = true; writeStep = 1; }};
HyPerConn "SpikesToExc" = {{ preLayerName = "Spikes"; postLayerName = "Exc"; channelCode = 0;
   nxp = {p}; nyp = {p}; nfp = 4; sharedWeights = true; weightInitType = "FileWeight"; initWeightsFile = "w.pvp";
   plasticityFlag = false; receiveGpu = false; updateGSynFromPostPerspective = false;
   pvpatchAccumulateType = "convolve"; }};
"""


def test_lif_network_from_params_with_pvp_input_and_output(capi, oracle, tmp_path):
    """A spiking network from an OpenPV params file: a PvpLayer replays Poisson spike frames from
    a .pvp file (byFile batching), a HyPerConn delivers them (Convolve keyword: reference order)
    into the EXC channel of a LIFLayer (Heun method), and both layers write their activity to
    <outputPath>/<layer>.pvp every step from t = 0.  The written frames equal the oracle's network
    composed from the pinned pieces, bit for bit."""
    nb, n, p, steps, F = 2, 24, 5, 5, 6
    rng = np.random.default_rng(41)
    frames = (rng.random((F, n, n, 1)) < 0.08).astype(np.float32)
    inpath = tmp_path / "spikes.pvp"
    with capi.PvpWriter(inpath, n, n, 1, True) as w:
        for f in range(F):
            idx = np.nonzero(frames[f].reshape(-1))[0]
            w.write_sparse(idx, np.ones(len(idx), np.float32), float(f))
    w = (0.8 * rng.uniform(0.5, 1.5, (1, p, p, 4))).astype(np.float32)
    col = capi.Column(lif_network_params(nb, n, p, tmp_path, inpath, "beginning"))
    col.set_weights("SpikesToExc", w)
    col.advance(steps)
    del col  # closes the files
    # oracle
    h = 2
    pre = oracle.Loc.make(nb, n, n, 1, h, h)
    post = oracle.Loc.make(nb, n, n, 4, 0, 0)
    nres = nb * n * n * 4
    st = {"rnd": oracle.taus_init(nres, 5), "V": np.full(nres, -70.0, np.float32),
          "Vth": np.full(nres, -55.0, np.float32), "GE": np.zeros(nres, np.float32),
          "GI": np.zeros(nres, np.float32), "GIB": np.zeros(nres, np.float32)}
    a = np.zeros(post.ext_shape(), np.float32)
    prm = oracle.lif_params_array()
    want_exc, want_in = [a[:, :, :, :].copy()], []
    for t in range(1, steps + 1):
        x = np.zeros(pre.ext_shape(), np.float32)
        for b in range(nb):
            x[b, h:h + n, h:h + n, :] = frames[(b + (t - 1) * nb) % F]
        want_in.append(x[:, h:h + n, h:h + n, :].copy())
        e, c = oracle.compact(x.reshape(nb, -1))
        g = oracle.deliver_pre(pre, post, p, p, w, entries=e, num_active=c)
        gs = np.stack([g.reshape(-1), np.zeros(nres, np.float32), np.zeros(nres, np.float32)])
        st, a = oracle.lif_update("b", post, prm, 1.0, st, gs, a)
        want_exc.append(a.copy())
    assert sum(float(x.sum()) for x in want_exc) > 0
    with capi.PvpReader(tmp_path / "Exc.pvp") as r:
        assert r.header["fileType"] == 6 and r.num_frames == (steps + 1) * nb
        for t in range(steps + 1):
            for b in range(nb):
                v, ts = r.read_dense(t * nb + b)
                assert ts == float(t)
                assert np.array_equal(v, want_exc[t][b]), (t, b)
    with capi.PvpReader(tmp_path / "Spikes.pvp") as r:
        assert r.num_frames == (steps + 1) * nb
        for t in range(1, steps + 1):
            for b in range(nb):
                assert np.array_equal(r.read_dense(t * nb + b)[0], want_in[t - 1][b])
