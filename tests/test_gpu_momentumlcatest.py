"""The reference's momentum-LCA system test (tests/MomentumLCATest, described in
tests/momentumlcatest_case.py) run on the GPU through the C ABI in the column's phase order:
residual (GSyn accumulate of the input and of V1's delivery on channel 1, identity activity), V1
(postsynaptic TransposeConn delivery, momentum LCA update with the adaptive time step, firm
threshold), V1 -> residual (SparseList compaction, presynaptic delivery), energy probes.  The
time step is the column's host-side probe (lcatest_case.timescale_update) fed by the GPU's
energies.

Per timestep, against the oracle's composition (which reproduces the test's correct.pvp bit for
bit, tests/test_oracle_lcatest.py): the time step and energy within 1e-12 relative; V, the
momentum state, A, the residual and the reconstruction bit for bit while the time steps agree
bit for bit, else within the test's 1e-4; the reconstruction against the known answer likewise."""
import numpy as np
import pytest

from tests import momentumlcatest_case as M

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from openpv_gb300 import build
    build.build()
    return torch


def test_momentumlcatest_through_the_c_abi(torch, oracle):
    from openpv_gb300 import capi
    x, correct = M.fixture()
    v0, w = M.initial_state(oracle)
    ref = M.oracle_steps(oracle, x, v0, w)

    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    v1, er = M.locs(capi)
    inf = float("inf")
    wd = dev(w)
    pre_conn = capi.conn_desc(v1, er, M.NXP, M.NXP)            # V1 -> Residual
    post_conn = capi.conn_desc(er, v1, M.NXP // 2, M.NXP // 2)  # TransposeConn Residual -> V1
    v = dev(v0)
    prev = torch.zeros(v1.res_shape(), device="cuda")
    a1 = torch.zeros(v1.ext_shape(), device="cuda")
    capi.ann_activity(v1, v, M.VTHRESH, 0.0, inf, 0.0, M.VWIDTH, a1)
    gsyn_e = torch.zeros((2,) + er.res_shape(), device="cuda")   # ch0 input, ch1 V1's delivery
    gsyn_e[0] = dev(x.reshape(er.res_shape()))
    ge = torch.zeros(er.res_shape(), device="cuda")
    ae = torch.zeros(er.ext_shape(), device="cuda")
    g1 = torch.zeros(v1.res_shape(), device="cuda")
    ent = torch.zeros((1, v1.num_ext, 2), dtype=torch.int32, device="cuda")
    num = torch.zeros(1, dtype=torch.int64, device="cuda")
    dt = torch.zeros(1, dtype=torch.float64, device="cuda")
    l2 = torch.zeros(1, dtype=torch.float64, device="cuda")
    cost = torch.zeros(1, dtype=torch.float64, device="cuda")

    def deliver_v1():
        capi.compact_active(a1, 1, v1.num_ext, ent, num)
        gsyn_e[1].zero_()
        capi.deliver_pre(pre_conn, wd, gsyn_e[1], entries=ent, num_active=num, mode=capi.DELIVER_REFERENCE_ORDER)

    deliver_v1()  # V1's initial activity reaches the residual at timestep 1
    state, energy = [M.BASE_MIN, M.BASE_MAX, -1.0], 0.0
    exact_dt = True
    for t in range(1, M.STEPS + 1):
        r = ref[t - 1]
        state = M.step_timescale(state, -1.0 if (t - 1) % M.DISPLAY == 0 else energy)
        dt.fill_(state[0])
        # phase 1: residual
        capi.gsyn_accumulate(er.num_res, [1.0, -1.0], gsyn_e, ge)
        capi.ann_activity(er, ge, -inf, -inf, inf, 0.0, 0.0, ae)
        # phase 2: V1
        g1.zero_()
        capi.deliver_post(post_conn, ae, wd, g1, mode=capi.DELIVER_REFERENCE_ORDER)
        capi.momentum_lca_update(v1, True, M.RATE, dt, M.TAU, g1, a1, prev, v)
        capi.ann_activity(v1, v, M.VTHRESH, 0.0, inf, 0.0, M.VWIDTH, a1)
        # V1 -> residual (and the identical CloneConn reconstruction)
        deliver_v1()
        # probes
        capi.cost_sum(er, ae, capi.COST_L2, 0.0, 0.0, l2)
        capi.cost_sum(v1, a1, capi.COST_FIRM, M.VTHRESH, M.VWIDTH, cost)
        torch.cuda.synchronize()
        energy = 0.5 * float(l2.item()) + float(np.float32(M.VTHRESH)) * float(cost.item())
        assert abs(state[0] - r["dt"]) <= 1e-12 * r["dt"], (t, state[0], r["dt"])
        assert abs(energy - r["energy"]) <= 1e-12 * abs(r["energy"]), (t, energy, r["energy"])
        exact_dt = exact_dt and state[0] == r["dt"]
        rec = gsyn_e[1].cpu().numpy()
        want = correct[t - 1].reshape(rec.shape)
        if exact_dt:
            for name, got in (("ae", ae), ("v", v), ("prev", prev), ("a1", a1)):
                assert np.array_equal(got.cpu().numpy().view(np.uint32), r[name].view(np.uint32)), (t, name)
            assert np.array_equal(rec.view(np.uint32), r["rec"].view(np.uint32)), t
            assert np.array_equal(rec.view(np.uint32), want.view(np.uint32)), t
        else:
            assert np.abs(rec - r["rec"]).max() <= M.BAR, t
            assert np.abs(rec - want).max() <= M.BAR, t
    assert int(num.item()) > 0
    print(f"MomentumLCATest through the C ABI: time steps {'bit-exact' if exact_dt else 'within 1e-12'}, "
          f"reconstruction {'bit for bit' if exact_dt else 'within 1e-4'} of correct.pvp on all {M.STEPS} steps")
