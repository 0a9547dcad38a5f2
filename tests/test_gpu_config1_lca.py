"""The plain LCA configuration exactly, step by step: input 32x32x1 uniform[0,1] minus its mean,
V1 16x16x64 at stride 2, 64 features of 8x8x1 drawn N(0,1) and L2-normalised, VThresh = AShift =
0.1, AMin = 0, tau = 100, dt = 1, 200 timesteps, batch 1, topology of the LCA tutorial
(Input -> Error by IdentConn on channel 0, V1 -> Error by a presynaptic sparse HyPerConn on
channel 1, Error -> V1 by a postsynaptic TransposeConn).

Per timestep the V1 GSyn, V and A, the error layer's GSyn and activity, the reconstruction and
the total energy are compared with the oracle (the reference CPU path's loops, pinned to the
reference's own compiled code):
  * the C ABI entry points composed in the reference's phase order with
    PVGPU_DELIVER_REFERENCE_ORDER: bit for bit on every buffer, the FP64 energy probes within
    1e-12 relative (only the reduction order differs);
  * the LCA solver's FP32 form: V and A within 1e-5 relative to the largest |V| of the step, the
    energy within 1e-5 relative, on every step.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STEPS = 200
VT = 0.1


@pytest.fixture(scope="module")
def torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from openpv_gb300 import build
    build.build()
    return torch


def config1_inputs():
    rng = np.random.default_rng(1234 + 1)
    x = rng.uniform(0.0, 1.0, (1, 32, 32, 1))
    x = (x - x.mean()).astype(np.float32)
    w = rng.normal(size=(64, 8, 8, 1))
    w = (w / np.sqrt((w ** 2).sum(axis=(1, 2, 3), keepdims=True))).astype(np.float32)
    return x, w


def oracle_steps(O, x, w):
    """The module stepped with the oracle's primitives (float, the reference's order)."""
    v1 = O.Loc.make(1, 16, 16, 64, 2)
    er = O.Loc.make(1, 32, 32, 1, 3)
    inf = np.float32(np.inf)
    v = np.zeros(v1.res_shape(), np.float32)
    a1 = O.ann_activity(v1, v, VT, 0.0, inf, VT, 0.0)
    rec = np.zeros(er.res_shape(), np.float32)
    dt = np.ones(1)
    out = []
    for _ in range(STEPS):
        ge = O.gsyn_accumulate(np.stack([x, rec]), [1.0, -1.0])
        ae = O.ann_activity(er, ge, -inf, -inf, inf, 0.0, 0.0)
        g1 = O.deliver_post(er, v1, 8, 8, w, ae)
        v = O.lca_update(v1, g1, a1, v, dt, 100.0)
        a1 = O.ann_activity(v1, v, VT, 0.0, inf, VT, 0.0)
        ent, num = O.compact(a1.reshape(1, -1))
        rec = O.deliver_pre(v1, er, 8, 8, w, entries=ent, num_active=num)
        energy = 0.5 * O.cost_sum(er, ae, O.COST_L2)[0] + float(np.float32(VT)) * O.cost_sum(v1, a1, O.COST_L1)[0]
        out.append(dict(ge=ge, ae=ae, g1=g1, v=v.copy(), a1=a1.copy(), rec=rec, energy=energy))
    return out


@pytest.fixture(scope="module")
def reference(oracle):
    x, w = config1_inputs()
    steps = oracle_steps(oracle, x, w)
    # the step-by-step composition is the oracle's own module loop, bit for bit
    p = oracle.lca_params()
    v_run, _, recon, e_run = oracle.lca_run(p, w, x[None], STEPS, np.zeros((1, 16, 16, 64), np.float32))
    assert np.array_equal(v_run.view(np.uint32), steps[-1]["v"].view(np.uint32))
    for t in (0, STEPS // 2, STEPS - 1):
        assert np.array_equal(recon[t].view(np.uint32), steps[t]["rec"].view(np.uint32))
        assert abs(e_run[t, 0] - steps[t]["energy"]) <= 1e-12 * abs(e_run[t, 0])
    return x, w, steps


def test_config1_reference_order_every_step_bitexact(torch, oracle, reference):
    from openpv_gb300 import capi
    x, w, ref = reference
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    v1 = capi.Loc.make(1, 16, 16, 64, 2)
    er = capi.Loc.make(1, 32, 32, 1, 3)
    inf = float("inf")
    wd = dev(w)
    pre_conn = capi.conn_desc(v1, er, 8, 8)    # V1 -> Error, presynaptic, sparse
    post_conn = capi.conn_desc(er, v1, 4, 4)   # Error -> V1 (TransposeConn), postsynaptic
    v = torch.zeros(v1.res_shape(), device="cuda")
    a1 = torch.zeros(v1.ext_shape(), device="cuda")
    capi.ann_activity(v1, v, VT, 0.0, inf, VT, 0.0, a1)
    gsyn_e = torch.zeros((2,) + er.res_shape(), device="cuda")  # ch0 input, ch1 reconstruction
    gsyn_e[0] = dev(x)
    ge = torch.zeros(er.res_shape(), device="cuda")
    ae = torch.zeros(er.ext_shape(), device="cuda")
    g1 = torch.zeros(v1.res_shape(), device="cuda")
    ent = torch.zeros((1, v1.num_ext, 2), dtype=torch.int32, device="cuda")
    num = torch.zeros(1, dtype=torch.int64, device="cuda")
    dt = torch.ones(1, dtype=torch.float64, device="cuda")
    l2 = torch.zeros(1, dtype=torch.float64, device="cuda")
    l1 = torch.zeros(1, dtype=torch.float64, device="cuda")
    u32 = lambda t: t.cpu().numpy().view(np.uint32)
    for t in range(STEPS):
        r = ref[t]
        # phase 1: error layer
        capi.gsyn_accumulate(er.num_res, [1.0, -1.0], gsyn_e, ge)
        capi.ann_activity(er, ge, -inf, -inf, inf, 0.0, 0.0, ae)
        # phase 2: V1
        g1.zero_()
        capi.deliver_post(post_conn, ae, wd, g1, mode=capi.DELIVER_REFERENCE_ORDER)
        capi.lca_update(v1, True, dt, 100.0, g1, a1, v)
        capi.ann_activity(v1, v, VT, 0.0, inf, VT, 0.0, a1)
        # phase 3: reconstruction from V1's SparseList into the error layer's channel 1
        capi.compact_active(a1, 1, v1.num_ext, ent, num)
        gsyn_e[1].zero_()
        capi.deliver_pre(pre_conn, wd, gsyn_e[1], entries=ent, num_active=num, mode=capi.DELIVER_REFERENCE_ORDER)
        capi.cost_sum(er, ae, capi.COST_L2, 0.0, 0.0, l2)
        capi.cost_sum(v1, a1, capi.COST_L1, 0.0, 0.0, l1)
        torch.cuda.synchronize()
        assert np.array_equal(u32(ge), r["ge"].view(np.uint32)), t
        assert np.array_equal(u32(ae), r["ae"].view(np.uint32)), t
        assert np.array_equal(u32(g1), r["g1"].view(np.uint32)), t
        assert np.array_equal(u32(v), r["v"].view(np.uint32)), t
        assert np.array_equal(u32(a1), r["a1"].view(np.uint32)), t
        assert np.array_equal(u32(gsyn_e[1]), r["rec"].view(np.uint32)), t
        e = 0.5 * float(l2.item()) + float(np.float32(VT)) * float(l1.item())
        assert abs(e - r["energy"]) <= 1e-12 * abs(r["energy"]), (t, e, r["energy"])
    assert int(num.item()) > 0  # the code is sparse but not empty


def test_config1_fp32_solver_every_step_within_1e5(torch, oracle, reference):
    from openpv_gb300 import capi
    x, w, ref = reference
    s = capi.LcaSolver(1, (32, 32, 1), (16, 16, 64), 8, VT)
    s.set_weights(torch.from_numpy(w).cuda())
    s.reset()
    xd = torch.from_numpy(x).cuda()
    v = torch.zeros((1, 16, 16, 64), device="cuda")
    a = torch.zeros((1, 16, 16, 64), device="cuda")
    e = torch.zeros(1, dtype=torch.float64, device="cuda")
    worst_v = worst_e = 0.0
    for t in range(STEPS):
        s.run(xd, 1, precision=capi.LCA_FP32)
        s.state(v, a)
        s.energy(xd, e)
        torch.cuda.synchronize()
        r = ref[t]
        vmax = np.abs(r["v"]).max()
        a_ref = r["a1"][:, 2:18, 2:18, :]
        dv = np.abs(v.cpu().numpy() - r["v"]).max() / vmax
        da = np.abs(a.cpu().numpy() - a_ref).max() / vmax
        de = abs(float(e.item()) - r["energy"]) / abs(r["energy"])
        assert dv <= 1e-5 and da <= 1e-5, (t, dv, da)
        assert de <= 1e-5, (t, de)
        worst_v, worst_e = max(worst_v, dv, da), max(worst_e, de)
    assert s.error_flag() == 0
    print(f"config 1, FP32 solver, 200 steps: max |dV|,|dA| / max|V| = {worst_v:.2e}, energy {worst_e:.2e}")
