"""The reference's LCA system test (tests/LCATest, described in tests/lcatest_case.py) run on
the GPU through the C ABI, composed in the column's phase order the way the drop-in's
translation units are called: residual (GSyn accumulate, identity activity), V1 (postsynaptic
TransposeConn delivery, HyPerLCA update with the adaptive time step, firm threshold),
reconstruction (SparseList compaction, presynaptic CloneConn delivery into the residual's
channel 1), energy probes (FP64 L2 and firm-threshold cost sums).  The adaptive time step is
the column's host-side probe (stand-in: lcatest_case.timescale_update) fed by the GPU's
energies.

Per timestep, against the oracle's composition (pinned to the reference's correct.pvp by
tests/test_oracle_lcatest.py): the time step and energy within 1e-12 relative, V, A, the residual
and the reconstruction bit for bit while the time steps agree bit for bit (they do unless an
FP64 energy sum rounds differently), else within the reference's 1e-6.  At the fixture's
timesteps the reconstruction equals the reference's known answer to 1e-6."""
import numpy as np
import pytest

from tests import lcatest_case as L

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from openpv_gb300 import build
    build.build()
    return torch


def test_lcatest_through_the_c_abi(torch, oracle):
    from openpv_gb300 import capi
    frames, steps, correct = L.fixture()
    v0, w = L.initial_state(oracle)
    ref = L.oracle_steps(oracle, frames, v0, w)

    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    v1, er = L.locs(capi)
    inf = float("inf")
    wd = dev(w)
    pre_conn = capi.conn_desc(v1, er, L.NXP, L.NXP)            # CloneConn V1 -> Reconstruction
    post_conn = capi.conn_desc(er, v1, L.NXP // 2, L.NXP // 2)  # TransposeConn Residual -> V1
    v = dev(v0)
    a1 = torch.zeros(v1.ext_shape(), device="cuda")
    capi.ann_activity(v1, v, L.VTHRESH, 0.0, inf, 0.0, L.VWIDTH, a1)
    gsyn_e = torch.zeros((2,) + er.res_shape(), device="cuda")   # ch0 input, ch1 reconstruction
    ge = torch.zeros(er.res_shape(), device="cuda")
    ae = torch.zeros(er.ext_shape(), device="cuda")
    g1 = torch.zeros(v1.res_shape(), device="cuda")
    ent = torch.zeros((1, v1.num_ext, 2), dtype=torch.int32, device="cuda")
    num = torch.zeros(1, dtype=torch.int64, device="cuda")
    dt = torch.zeros(1, dtype=torch.float64, device="cuda")
    l2 = torch.zeros(1, dtype=torch.float64, device="cuda")
    cost = torch.zeros(1, dtype=torch.float64, device="cuda")
    xs = [dev(f.reshape(er.res_shape())) for f in frames]
    state, energy = [L.BASE_MIN, L.BASE_MAX, -1.0], 0.0
    exact_dt = True
    worst = 0.0
    for t in range(1, L.STEPS + 1):
        r = ref[t - 1]
        state = L.timescale_update(state, -1.0 if (t - 1) % L.DISPLAY == 0 else energy)
        dt.fill_(state[0])
        gsyn_e[0].copy_(xs[(t - 1) // L.DISPLAY])
        # phase 1: residual
        capi.gsyn_accumulate(er.num_res, [1.0, -1.0], gsyn_e, ge)
        capi.ann_activity(er, ge, -inf, -inf, inf, 0.0, 0.0, ae)
        # phase 2: V1
        g1.zero_()
        capi.deliver_post(post_conn, ae, wd, g1, mode=capi.DELIVER_REFERENCE_ORDER)
        capi.lca_update(v1, True, dt, L.TAU, g1, a1, v)
        capi.ann_activity(v1, v, L.VTHRESH, 0.0, inf, 0.0, L.VWIDTH, a1)
        # phase 3: reconstruction from V1's SparseList
        capi.compact_active(a1, 1, v1.num_ext, ent, num)
        gsyn_e[1].zero_()
        capi.deliver_pre(pre_conn, wd, gsyn_e[1], entries=ent, num_active=num, mode=capi.DELIVER_REFERENCE_ORDER)
        # probes
        capi.cost_sum(er, ae, capi.COST_L2, 0.0, 0.0, l2)
        capi.cost_sum(v1, a1, capi.COST_FIRM, L.VTHRESH, L.VWIDTH, cost)
        torch.cuda.synchronize()
        energy = 0.5 * float(l2.item()) + float(np.float32(L.VTHRESH)) * float(cost.item())
        assert abs(state[0] - r["dt"]) <= 1e-12 * r["dt"], (t, state[0], r["dt"])
        assert abs(energy - r["energy"]) <= 1e-12 * abs(r["energy"]), (t, energy, r["energy"])
        exact_dt = exact_dt and state[0] == r["dt"]
        rec = gsyn_e[1].cpu().numpy()
        if exact_dt:
            for name, got in (("ae", ae), ("v", v), ("a1", a1)):
                assert np.array_equal(got.cpu().numpy().view(np.uint32), r[name].view(np.uint32)), (t, name)
            assert np.array_equal(rec.view(np.uint32), r["rec"].view(np.uint32)), t
        else:
            assert np.abs(rec - r["rec"]).max() <= L.BAR, t
        if t in steps:
            d = np.abs(rec.reshape(L.IN_NY, L.IN_NX) - correct[list(steps).index(t), :, :, 0]).max()
            assert d <= L.BAR, (t, d)
            worst = max(worst, d)
    assert int(num.item()) > 0
    print(f"LCATest through the C ABI: time steps {'bit-exact' if exact_dt else 'within 1e-12'}, "
          f"max |recon - correct.pvp| = {worst:.2e} at steps {steps.tolist()}")
