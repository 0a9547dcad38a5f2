"""LIF on the device (pvgpu_lif_update, pvgpu_taus_init) against the oracle's restatement of
LIFActivityComponent.cpp, itself pinned bit for bit to the reference's own update loops
(tests/test_oracle_vs_ref.py).  Method 'b' and the generator are compared bit for bit; 'a' and
'o' bit for bit in everything but V, which carries the device's expf / powf / logf in the filter
coefficients (within 2e-6 relative).  A spiking network step -- Poisson spikes as a SparseList,
presynaptic delivery into the EXC channel, the LIF update, compaction of the spikes -- is checked
against the oracle composed the same way."""
import numpy as np
import pytest

from tests.test_gpu_kernels import OL, H, T

pytestmark = pytest.mark.gpu


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


def state(oracle, n, rng, seed):
    return {"rnd": oracle.taus_init(n, seed),
            "V": rng.uniform(-75.0, -50.0, n).astype(np.float32),
            "Vth": rng.uniform(-57.0, -48.0, n).astype(np.float32),
            "GE": rng.uniform(0.0, 2.0, n).astype(np.float32),
            "GI": rng.uniform(0.0, 1.0, n).astype(np.float32),
            "GIB": rng.uniform(0.0, 0.5, n).astype(np.float32)}


def to_dev(torch, st):
    return {k: T(torch, v.view(np.uint32).reshape(-1, 4).view(np.int32) if k == "rnd" else v) for k, v in st.items()}


def from_dev(d, dtype):
    return {k: (H(v).view(np.uint32).reshape(-1).view(dtype) if k == "rnd" else H(v)) for k, v in d.items()}


def test_taus_init_bitexact(cuda, oracle):
    torch = cuda
    from openpv_gb300 import capi
    for n, seed in [(1, 0), (1000, 17), (70000, 123456)]:
        d = torch.zeros((n, 4), dtype=torch.int32, device="cuda")
        capi.taus_init(d, n, seed)
        ref = oracle.taus_init(n, seed)
        assert np.array_equal(H(d).view(np.uint32).reshape(-1), ref.view(np.uint32))


@pytest.mark.parametrize("method", ["b", "a", "o"])
@pytest.mark.parametrize("noise", [False, True])
def test_lif_update_matches_oracle(cuda, oracle, method, noise):
    torch = cuda
    from openpv_gb300 import capi
    loc = capi.Loc.make(3, 40, 17, 8, 2)
    ol = OL(oracle, loc)
    n = loc.nbatch * loc.nx * loc.ny * loc.nf
    rng = np.random.default_rng(ord(method) * 3 + noise)
    kw = dict(noiseAmpE=0.5, noiseAmpI=0.3, noiseAmpIB=0.2, noiseFreqE=300.0) if noise else {}
    p_o, p_d = oracle.lif_params_array(**kw), capi.LifParams.make(**kw)
    st = state(oracle, n, rng, seed=5)
    dev = to_dev(torch, st)
    a_o = np.zeros(loc.ext_shape(), np.float32)
    a_d = T(torch, a_o)
    fired = 0
    for step in range(5):
        gs = np.stack([rng.uniform(0, 1.5, n), rng.uniform(0, 0.8, n), rng.uniform(0, 0.3, n)]).astype(np.float32)
        st, a_o = oracle.lif_update(method, ol, p_o, 1.0, st, gs, a_o)
        capi.lif_update(loc, method, p_d, 1.0, dev["rnd"], dev["V"], dev["Vth"], dev["GE"], dev["GI"], dev["GIB"],
                        T(torch, gs), a_d)
        got = from_dev(dev, oracle.TAUS_DTYPE)
        assert np.array_equal(H(a_d), a_o), step
        fired += int(a_o.sum())
        for k in ("rnd", "Vth", "GE", "GI", "GIB") + (("V",) if method == "b" else ()):
            assert np.array_equal(got[k].view(np.uint32), st[k].view(np.uint32)), (k, step)
        if method != "b":
            np.testing.assert_allclose(got["V"], st["V"], rtol=2e-6, atol=0)
            st["V"] = got["V"].copy()  # continue both from the same state
    assert fired > 0


def test_lif_rejects_unknown_method(cuda):
    torch = cuda
    from openpv_gb300 import capi
    loc = capi.Loc.make(1, 4, 4, 1, 0)
    z = torch.zeros(64, device="cuda")
    with pytest.raises(capi.PvgpuError):
        capi.lif_update(loc, "x", capi.LifParams.make(), 1.0, z, z, z, z, z, z, z, z)


@pytest.mark.parametrize("method, mode", [("b", "reference"), ("a", "fast")])
def test_spiking_network_steps(cuda, oracle, method, mode):
    """Poisson input spikes (pre-generated, 64x64x1, rate 30 Hz at dt = 1 ms) -> 11x11 Gauss2D-like
    weights -> excitatory LIF layer 64x64x8 over 8 steps: the input SparseList is delivered into
    the EXC channel, the layer updates and its spikes are compacted each step.  Reference-order
    delivery with method 'b' is bit for bit; FAST delivery with 'a' within tolerance and the same
    spikes."""
    torch = cuda
    from openpv_gb300 import capi
    nb, n, nfo, p, steps = 2, 64, 8, 11, 8
    pre = capi.Loc.make(nb, n, n, 1, 5)
    post = capi.Loc.make(nb, n, n, nfo, 0)
    rng = np.random.default_rng(29)
    yy, xx = np.mgrid[-5:6, -5:6]
    gauss = np.exp(-(xx ** 2 + yy ** 2) / (2 * 2.5 ** 2))
    w = (0.4 * gauss[None, :, :, None] * rng.uniform(0.5, 1.5, (1, p, p, nfo))).astype(np.float32)
    nres = nb * n * n * nfo
    st = state(oracle, nres, rng, seed=9)
    st["V"][:] = -70.0
    st["Vth"][:] = -55.0
    st["GE"][:] = 0
    st["GI"][:] = 0
    st["GIB"][:] = 0
    dev = to_dev(torch, st)
    a_o = np.zeros(post.ext_shape(), np.float32)
    a_d = T(torch, a_o)
    conn = capi.conn_desc(pre, post, p, p)
    dmode = capi.DELIVER_REFERENCE_ORDER if mode == "reference" else capi.DELIVER_FAST
    gs_d = torch.zeros((3, nres), device="cuda")
    ent = torch.zeros((nb, pre.num_ext, 2), dtype=torch.int32, device="cuda")
    num = torch.zeros(nb, dtype=torch.int64, device="cuda")
    total_spikes = 0
    p_o, p_d = oracle.lif_params_array(), capi.LifParams.make()
    for step in range(steps):
        x = np.zeros(pre.ext_shape(), np.float32)
        x[:, 5:5 + n, 5:5 + n, :] = (rng.random((nb, n, n, 1)) < 0.03).astype(np.float32)
        # oracle: SparseList of the input, delivery, update
        e_o, c_o = oracle.compact(x.reshape(nb, -1))
        g_exc = oracle.deliver_pre(OL(oracle, pre), OL(oracle, post), p, p, w, entries=e_o, num_active=c_o)
        gs = np.stack([g_exc.reshape(-1), np.zeros(nres, np.float32), np.zeros(nres, np.float32)])
        st, a_o = oracle.lif_update(method, OL(oracle, post), p_o, 1.0, st, gs, a_o)
        # device: compaction, delivery into the EXC channel, update
        capi.compact_active(T(torch, x), nb, pre.num_ext, ent, num)
        gs_d.zero_()
        capi.deliver_pre(conn, T(torch, w), gs_d[0], entries=ent, num_active=num, mode=dmode)
        capi.lif_update(post, method, p_d, 1.0, dev["rnd"], dev["V"], dev["Vth"], dev["GE"], dev["GI"], dev["GIB"],
                        gs_d, a_d)
        got = from_dev(dev, oracle.TAUS_DTYPE)
        assert np.array_equal(H(a_d), a_o), step
        total_spikes += int(a_o.sum())
        if method == "b":
            for k in st:
                assert np.array_equal(got[k].view(np.uint32), st[k].view(np.uint32)), (k, step)
        else:
            for k in ("V", "GE"):
                np.testing.assert_allclose(got[k], st[k], rtol=1e-5, atol=1e-5)
            st = {k: (v.copy() if k == "rnd" else got[k].copy()) for k, v in st.items()}
    assert total_spikes > 0


def gauss_w(nfpre, p, nfpost, sigma, peak):
    r = np.arange(p) - (p - 1) / 2.0
    g = np.exp(-(r[:, None] ** 2 + r[None, :] ** 2) / (2 * sigma ** 2))
    return np.ascontiguousarray(np.broadcast_to(peak * g[None, :, :, None], (nfpre, p, p, nfpost))).astype(np.float32)


def network_spike_counts(torch, oracle, method, mode, nb, n, ne, ni, steps, seed=77):
    """input -> exc (11x11 Gaussian sigma 3 peak 0.5, EXC), exc -> inh (stride 2, 3x3 weights 0.05,
    EXC), inh -> exc (8x8 Gaussian sigma 2 peak 1, INH), Poisson input at U[5, 50] Hz, default LIF
    parameters, noise off; run on the device through the C ABI and by the oracle composed the
    same way.  Returns the spike counts per neuron (device exc, oracle exc, device inh, oracle inh)."""
    from openpv_gb300 import capi
    inp, exc, inh = capi.Loc.make(nb, n, n, 1, 5), capi.Loc.make(nb, n, n, ne, 2), capi.Loc.make(nb, n // 2, n // 2, ni, 2)
    exc_r, inh_r = capi.Loc.make(nb, n, n, ne, 0), capi.Loc.make(nb, n // 2, n // 2, ni, 0)
    conns = [(capi.conn_desc(inp, exc_r, 11, 11), gauss_w(1, 11, ne, 3.0, 0.5)),
             (capi.conn_desc(exc, inh_r, 3, 3), np.full((ne * 4, 3, 3, ni), 0.05, np.float32)),
             (capi.conn_desc(inh, exc_r, 8, 8), gauss_w(ni, 8, ne, 2.0, 1.0))]
    dmode = capi.DELIVER_REFERENCE_ORDER if mode == "reference" else capi.DELIVER_FAST
    rng = np.random.default_rng(seed)
    rates = rng.uniform(5, 50, (nb, n, n, 1))
    ne_res, ni_res = nb * n * n * ne, nb * (n // 2) ** 2 * ni
    p_o, p_d = oracle.lif_params_array(), capi.LifParams.make()

    def init(m, seed):
        return {"rnd": oracle.taus_init(m, seed), "V": np.full(m, -70.0, np.float32), "Vth": np.full(m, -55.0, np.float32),
                "GE": np.zeros(m, np.float32), "GI": np.zeros(m, np.float32), "GIB": np.zeros(m, np.float32)}

    so_e, so_h = init(ne_res, 17), init(ni_res, 18)
    sd_e, sd_h = to_dev(torch, so_e), to_dev(torch, so_h)
    ao_e, ao_h = np.zeros(exc.ext_shape(), np.float32), np.zeros(inh.ext_shape(), np.float32)
    ad_e, ad_h = T(torch, ao_e), T(torch, ao_h)
    gd_e, gd_h = torch.zeros((3, ne_res), device="cuda"), torch.zeros((3, ni_res), device="cuda")
    wd = [T(torch, w) for _, w in conns]
    cnt_o_e, cnt_d_e = np.zeros(ne_res), np.zeros(ne_res)
    cnt_o_h, cnt_d_h = np.zeros(ni_res), np.zeros(ni_res)

    def sparse(torch_a, loc):
        ent = torch.zeros((nb, loc.num_ext, 2), dtype=torch.int32, device="cuda")
        num = torch.zeros(nb, dtype=torch.int64, device="cuda")
        capi.compact_active(torch_a, nb, loc.num_ext, ent, num)
        return ent, num

    res = lambda a, h: a[:, h:a.shape[1] - h, h:a.shape[2] - h, :].reshape(-1)
    for t in range(steps):
        x = np.zeros(inp.ext_shape(), np.float32)
        x[:, 5:5 + n, 5:5 + n, :] = (rng.random((nb, n, n, 1)) < rates * 1e-3).astype(np.float32)
        # oracle
        e0, c0 = oracle.compact(x.reshape(nb, -1))
        eh, ch = oracle.compact(ao_h.reshape(nb, -1))
        g0 = oracle.deliver_pre(OL(oracle, inp), OL(oracle, exc_r), 11, 11, conns[0][1], entries=e0, num_active=c0)
        g1 = oracle.deliver_pre(OL(oracle, inh), OL(oracle, exc_r), 8, 8, conns[2][1], entries=eh, num_active=ch)
        so_e, ao_e = oracle.lif_update(method, OL(oracle, exc), p_o, 1.0, so_e,
                                       np.stack([g0.reshape(-1), g1.reshape(-1), 0 * g0.reshape(-1)]), ao_e)
        ee, ce = oracle.compact(ao_e.reshape(nb, -1))
        gi = oracle.deliver_pre(OL(oracle, exc), OL(oracle, inh_r), 3, 3, conns[1][1], entries=ee, num_active=ce).reshape(-1)
        so_h, ao_h = oracle.lif_update(method, OL(oracle, inh), p_o, 1.0, so_h, np.stack([gi, 0 * gi, 0 * gi]), ao_h)
        # device
        gd_e.zero_()
        gd_h.zero_()
        ent, num = sparse(T(torch, x), inp)
        capi.deliver_pre(conns[0][0], wd[0], gd_e[0], entries=ent, num_active=num, mode=dmode)
        ent, num = sparse(ad_h, inh)
        capi.deliver_pre(conns[2][0], wd[2], gd_e[1], entries=ent, num_active=num, mode=dmode)
        capi.lif_update(exc, method, p_d, 1.0, sd_e["rnd"], sd_e["V"], sd_e["Vth"], sd_e["GE"], sd_e["GI"], sd_e["GIB"],
                        gd_e, ad_e)
        ent, num = sparse(ad_e, exc)
        capi.deliver_pre(conns[1][0], wd[1], gd_h[0], entries=ent, num_active=num, mode=dmode)
        capi.lif_update(inh, method, p_d, 1.0, sd_h["rnd"], sd_h["V"], sd_h["Vth"], sd_h["GE"], sd_h["GI"], sd_h["GIB"],
                        gd_h, ad_h)
        cnt_o_e += res(ao_e, 2)
        cnt_o_h += res(ao_h, 2)
        cnt_d_e += res(H(ad_e), 2)
        cnt_d_h += res(H(ad_h), 2)
    return cnt_d_e, cnt_o_e, cnt_d_h, cnt_o_h


@pytest.mark.parametrize("method, mode", [("b", "reference"), ("a", "fast")])
def test_exc_inh_network_spike_counts(cuda, oracle, method, mode):
    """The spiking configuration at reduced size (2 images, input 48x48, exc 48x48x8, inh 24x24x4,
    40 steps), arma or Heun.  Spike counts per neuron against the oracle: identical for Heun with
    reference-order delivery; for arma with FAST delivery the total within 1 % and at least 99 % of
    neurons with identical counts."""
    cnt_d_e, cnt_o_e, cnt_d_h, cnt_o_h = network_spike_counts(cuda, oracle, method, mode, 2, 48, 8, 4, 40)
    assert cnt_o_e.sum() > 0 and cnt_o_h.sum() > 0
    if method == "b":
        assert np.array_equal(cnt_d_e, cnt_o_e) and np.array_equal(cnt_d_h, cnt_o_h)
    else:
        for d, o in ((cnt_d_e, cnt_o_e), (cnt_d_h, cnt_o_h)):
            assert abs(d.sum() - o.sum()) <= 0.01 * o.sum()
            assert np.mean(d == o) >= 0.99


def test_lif_network_full_size_spike_counts(cuda, oracle):
    """The spiking configuration at its full layer sizes (input 256x256x1, exc 256x256x32, inh
    128x128x8) for one image over 120 timesteps (the oracle takes about 0.15-0.25 s per step on one
    host core), arma with FAST delivery as in the network benchmark: the total spike count of each
    layer within 1 % of the oracle's and at least 99 % of the neurons with identical counts."""
    cnt_d_e, cnt_o_e, cnt_d_h, cnt_o_h = network_spike_counts(cuda, oracle, "a", "fast", 1, 256, 32, 8, 120, seed=1234 + 5)
    assert cnt_o_e.sum() > 0 and cnt_o_h.sum() > 0
    same = []
    for d, o in ((cnt_d_e, cnt_o_e), (cnt_d_h, cnt_o_h)):
        assert abs(d.sum() - o.sum()) <= 0.01 * o.sum(), (d.sum(), o.sum())
        same.append(float(np.mean(d == o)))
        assert same[-1] >= 0.99, same
    print(f"LIF network full size, 120 steps: exc spikes {int(cnt_d_e.sum())} (oracle {int(cnt_o_e.sum())}), "
          f"inh {int(cnt_d_h.sum())} (oracle {int(cnt_o_h.sum())}); identical per-neuron counts exc {same[0]:.4f}, "
          f"inh {same[1]:.4f}")
