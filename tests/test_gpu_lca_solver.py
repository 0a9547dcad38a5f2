"""The fused LCA solver (both precisions) against the CPU oracle's LCA module
(pvo_lca_run: input -> error <-> V1 in the reference's phase order), through the C ABI.

FP32 form: same math as the reference path, only GEMM summation order differs -> V and A
agree with the FP32 oracle within 1e-5 relative to max|V| (normwise: single elements near the
threshold or near zero have no meaningful elementwise relative error) and the probe energy
within 1e-5 relative.  BF16 form: the final energy must be within 1e-3 relative of the FP64
oracle (the stated BF16 bar)."""
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


def dictionary(rng, nf, p, c):
    w = rng.normal(size=(nf, p, p, c))
    w /= np.sqrt((w ** 2).sum(axis=(1, 2, 3), keepdims=True))
    return w.astype(np.float32)


def one_over_f(rng, nb, ny, nx, c):
    fy = np.fft.fftfreq(ny)[:, None]
    fx = np.fft.fftfreq(nx)[None, :]
    f = np.sqrt(fy ** 2 + fx ** 2)
    f[0, 0] = 1.0
    amp = 1.0 / f
    amp[0, 0] = 0.0
    out = np.zeros((nb, ny, nx, c))
    for b in range(nb):
        for ch in range(c):
            ph = rng.uniform(0, 2 * np.pi, (ny, nx))
            img = np.real(np.fft.ifft2(amp * np.exp(1j * ph)))
            out[b, :, :, ch] = img
        out[b] = (out[b] - out[b].mean()) / out[b].std()
    return out.astype(np.float32)


CASES = {
    # name: nb, (in y,x,c), (v1 y,x,f), nxp, VThresh, steps
    "plain_lca": (2, (32, 32, 1), (16, 16, 64), 8, 0.1, 30),
    "colour": (2, (32, 32, 3), (16, 16, 128), 8, 0.15, 30),
    "stride4": (1, (64, 64, 1), (16, 16, 64), 16, 0.1, 20),
    # four 128-position blocks per image: interior blocks sum bands from both neighbours
    "tall": (2, (64, 32, 3), (32, 16, 128), 8, 0.15, 20),
}
# BF16x3 is offered where its operands fit in shared memory: 8x8 patches and input images of at
# most ~4 K floats (kernel R holds x twice and the reconstruction of one image beside two
# double-width stages)
X3_CASES = ("plain_lca", "colour")


def setup(oracle, name, seed=3):
    nb, ins, v1s, nxp, vth, steps = CASES[name]
    rng = np.random.default_rng(seed)
    w = dictionary(rng, v1s[2], nxp, ins[2])
    x = one_over_f(rng, nb, *ins)
    p = oracle.lca_params(nbatch=nb, inNx=ins[1], inNy=ins[0], inNf=ins[2], v1Nx=v1s[1], v1Ny=v1s[0],
                          v1Nf=v1s[2], nxp=nxp, nyp=nxp, VThresh=vth, AShift=vth, AMin=0.0, VWidth=0.0, tau=100.0,
                          dtFixed=1.0)
    return nb, ins, v1s, nxp, vth, steps, w, x, p


@pytest.mark.parametrize("name", list(CASES))
def test_lca_fp32_form_matches_oracle(torch, oracle, name):
    from openpv_gb300 import capi
    nb, ins, v1s, nxp, vth, steps, w, x, p = setup(oracle, name)
    v0 = np.zeros((nb,) + v1s, np.float32)
    v_ref, a_ref, _, e_ref = oracle.lca_run(p, w, x[None], steps, v0, want_recon=False)
    s = capi.LcaSolver(nb, ins, v1s, nxp, vth)
    s.set_weights(torch.from_numpy(w).cuda())
    s.reset()
    xd = torch.from_numpy(x).cuda()
    s.run(xd, steps, precision=capi.LCA_FP32)
    v = torch.zeros((nb,) + v1s, device="cuda")
    a = torch.zeros((nb,) + v1s, device="cuda")
    s.state(v, a)
    e = torch.zeros(nb, dtype=torch.float64, device="cuda")
    s.energy(xd, e)
    torch.cuda.synchronize()
    assert s.error_flag() == 0
    vs = np.abs(v_ref).max()
    dv = np.abs(v.cpu().numpy() - v_ref).max() / vs
    da = np.abs(a.cpu().numpy() - a_ref).max() / vs
    assert dv <= 1e-5 and da <= 1e-5, (dv, da)
    np.testing.assert_allclose(e.cpu().numpy(), e_ref[-1], rtol=1e-5)


@pytest.mark.parametrize("name", list(CASES))
def test_lca_bf16_form_energy_within_1e3_of_fp64(torch, oracle, name):
    from openpv_gb300 import capi
    nb, ins, v1s, nxp, vth, steps, w, x, p = setup(oracle, name)
    v0 = np.zeros((nb,) + v1s)
    _, _, _, e64 = oracle.lca_run(p, w.astype(np.float64), x[None].astype(np.float64), steps, v0, f64=True,
                                  want_recon=False)
    s = capi.LcaSolver(nb, ins, v1s, nxp, vth)
    s.set_weights(torch.from_numpy(w).cuda())
    xd = torch.from_numpy(x).cuda()
    e = torch.zeros(nb, dtype=torch.float64, device="cuda")
    for x3 in ((0, 5) if name in X3_CASES else (0,)):
        s.reset()
        s.run(xd, steps, x3_steps=x3, precision=capi.LCA_BF16)
        s.energy(xd, e)
        torch.cuda.synchronize()
        assert s.error_flag() == 0
        rel = np.abs(e.cpu().numpy() - e64[-1]) / np.abs(e64[-1])
        assert rel.max() < 1e-3, (x3, rel)


def test_lca_bf16_x3_closer_than_bf16(torch, oracle):
    """BF16x3 split products bring the state closer to the FP32 oracle than plain BF16."""
    from openpv_gb300 import capi
    nb, ins, v1s, nxp, vth, steps, w, x, p = setup(oracle, "colour")
    v0 = np.zeros((nb,) + v1s, np.float32)
    v_ref, _, _, _ = oracle.lca_run(p, w, x[None], steps, v0, want_recon=False)
    s = capi.LcaSolver(nb, ins, v1s, nxp, vth)
    s.set_weights(torch.from_numpy(w).cuda())
    xd = torch.from_numpy(x).cuda()
    errs = []
    for x3 in (0, steps):
        s.reset()
        s.run(xd, steps, x3_steps=x3, precision=capi.LCA_BF16)
        v = torch.zeros((nb,) + v1s, device="cuda")
        s.state(v)
        torch.cuda.synchronize()
        errs.append(np.abs(v.cpu().numpy() - v_ref).max())
    assert errs[1] < 0.25 * errs[0], errs


def test_lca_bf16_graph_replay_equals_kernel_by_kernel(torch, oracle):
    """A BF16 run is replayed as one CUDA graph with programmatic dependent launches between its
    kernels; the state it leaves is bit-identical to the kernel-by-kernel run (per-kernel timing
    mode), also after the graph is rebuilt for another input buffer and step count, and when run
    on a side stream."""
    from openpv_gb300 import capi
    nb, ins, v1s, nxp, vth, steps, w, x, p = setup(oracle, "colour")
    wd = torch.from_numpy(w).cuda()

    def solve(xd, n, x3, direct, stream=None):
        s = capi.LcaSolver(nb, ins, v1s, nxp, vth)
        s.set_weights(wd)
        s.reset()
        if direct:
            s.profile_begin(n)
        s.run(xd, n, x3_steps=x3, precision=capi.LCA_BF16, stream=stream)
        if direct:
            s.profile_end()
        v = torch.zeros((nb,) + v1s, device="cuda")
        s.state(v, stream=stream)
        torch.cuda.synchronize()
        assert s.error_flag() == 0
        return v.cpu().numpy()

    xd = torch.from_numpy(x).cuda()
    x2 = (xd * 0.5).contiguous()
    for xi, n, x3 in ((xd, steps, 0), (x2, steps + 3, 4)):
        ref = solve(xi, n, x3, direct=True)
        assert np.array_equal(solve(xi, n, x3, direct=False).view(np.uint32), ref.view(np.uint32))
    side = torch.cuda.Stream()
    with torch.cuda.stream(side):
        got = solve(x2, steps + 3, 4, direct=False, stream=side)
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))

    # one solver, graph reused across runs and rebuilt when the input changes
    s = capi.LcaSolver(nb, ins, v1s, nxp, vth)
    s.set_weights(wd)
    outs = []
    for xi in (xd, xd, x2):
        s.reset()
        s.run(xi, steps, precision=capi.LCA_BF16)
        v = torch.zeros((nb,) + v1s, device="cuda")
        s.state(v)
        torch.cuda.synchronize()
        outs.append(v.cpu().numpy())
    assert np.array_equal(outs[0], outs[1])
    assert np.array_equal(outs[0], solve(xd, steps, 0, direct=True))
    assert np.array_equal(outs[2], solve(x2, steps, 0, direct=True))


def test_lca_autotune_picks_valid_shapes_and_keeps_parity(torch, oracle):
    """The autotuner times every kernel shape that fits, keeps the fastest (reported by
    plan_info), hands it to later solvers of the same geometry, and the tuned solver still meets
    the 1e-3 energy bar against the FP64 oracle."""
    from openpv_gb300 import capi
    nb, ins, v1s, nxp, vth, steps, w, x, p = setup(oracle, "colour")
    v0 = np.zeros((nb,) + v1s)
    _, _, _, e64 = oracle.lca_run(p, w.astype(np.float64), x[None].astype(np.float64), steps, v0, f64=True,
                                  want_recon=False)
    s = capi.LcaSolver(nb, ins, v1s, nxp, vth)
    s.set_weights(torch.from_numpy(w).cuda())
    xd = torch.from_numpy(x).cuda()
    s.autotune(xd, trial_steps=2)
    info = s.plan_info()
    for form in ("bf16", "bf16x3"):
        q = info[form]
        assert q["feature_tile"] in (64, 128) and v1s[2] % q["feature_tile"] == 0, info
        assert 1 <= q["v_slots"] <= 3 and 1 <= q["w_slots"] <= 2 and 2 <= q["recon_stages"] <= 4, info
    assert info["bf16x3"]["a_staged"] == 0
    sched = s.schedule()
    assert sched["chains"] in (1, 2) and sched["recon_ctas"] == 0, sched
    assert sched["post_ctas"] == 0 or sched["chains"] == 2, sched  # capped grids only with two chains
    s2 = capi.LcaSolver(nb, ins, v1s, nxp, vth)
    assert s2.plan_info() == info and s2.schedule() == sched
    e = torch.zeros(nb, dtype=torch.float64, device="cuda")
    for x3 in (0, 5):
        s.reset()
        s.run(xd, steps, x3_steps=x3, precision=capi.LCA_BF16)
        s.energy(xd, e)
        torch.cuda.synchronize()
        assert s.error_flag() == 0
        rel = np.abs(e.cpu().numpy() - e64[-1]) / np.abs(e64[-1])
        assert rel.max() < 1e-3, (x3, rel, info)


@pytest.mark.parametrize("nb", [3, 6])
def test_lca_bf16_schedules_leave_identical_state(torch, oracle, nb):
    """The graph's schedule -- one chain or two half-batch chains on parallel branches (halves of
    4 + 2 and 2 + 1 images), capped
    persistent grids, with and without programmatic edges -- moves work between CTAs and SMs
    only: the state is bit-identical to the kernel-by-kernel run, BF16x3 steps included."""
    from openpv_gb300 import capi
    _, ins, v1s, nxp, vth, steps, w, _, _ = setup(oracle, "colour")
    x = one_over_f(np.random.default_rng(11), nb, *ins)
    wd = torch.from_numpy(w).cuda()
    xd = torch.from_numpy(x).cuda()
    s = capi.LcaSolver(nb, ins, v1s, nxp, vth)
    s.set_weights(wd)
    assert s.schedule() == {"chains": 1, "recon_ctas": 0, "post_ctas": 0, "programmatic": True, "fused": True}

    def state(direct):
        s.reset()
        if direct:
            s.profile_begin(steps)
        s.run(xd, steps, x3_steps=4, precision=capi.LCA_BF16)
        if direct:
            s.profile_end()
        v = torch.zeros((nb,) + v1s, device="cuda")
        s.state(v)
        torch.cuda.synchronize()
        assert s.error_flag() == 0
        return v.cpu().numpy().view(np.uint32)

    ref = state(direct=True)
    for sc in ((2, 0, 0, True), (2, 0, 0, False), (2, 2, 5, True), (1, 2, 3, False), (2, 4, 16, True)):
        s.set_schedule(*sc)
        assert s.schedule()["chains"] == sc[0]
        assert np.array_equal(state(direct=False), ref), sc
    with pytest.raises(capi.PvgpuError):
        s.set_schedule(chains=3)
    one = capi.LcaSolver(1, ins, v1s, nxp, vth)
    with pytest.raises(capi.PvgpuError):
        one.set_schedule(chains=2)  # one image has no second half


@pytest.mark.parametrize("name", list(CASES))
def test_lca_fused_steps_match_unfused_and_oracle(torch, oracle, name):
    """Fused timesteps (kernel F: post delivery, update and the reconstruction of the new
    activity in one launch, residual windows summed from the previous step's bands) against the
    two-kernel form: the same final energy to 1e-4 relative, V within 1e-3 of max|V|, both within
    the 1e-3 bar of the FP64 oracle; the profiled run reports the expected number of fused
    steps; graph replay (one and two chains) equals the kernel-by-kernel run bit for bit."""
    from openpv_gb300 import capi
    nb, ins, v1s, nxp, vth, steps, w, x, p = setup(oracle, name)
    v0 = np.zeros((nb,) + v1s)
    _, _, _, e64 = oracle.lca_run(p, w.astype(np.float64), x[None].astype(np.float64), steps, v0, f64=True,
                                  want_recon=False)
    wd = torch.from_numpy(w).cuda()
    xd = torch.from_numpy(x).cuda()
    s = capi.LcaSolver(nb, ins, v1s, nxp, vth)
    s.set_weights(wd)
    info = s.fused_plan_info()
    assert info["feature_tile"] > 0, info
    e = torch.zeros(nb, dtype=torch.float64, device="cuda")

    def run(fused, x3, n=steps, direct=False, chains=1):
        s.set_schedule(chains=chains, fused=fused)
        s.reset()
        if direct:
            s.profile_begin(n)
        s.run(xd, n, x3_steps=x3, precision=capi.LCA_BF16)
        prof = s.profile_end_fused() if direct else None
        s.energy(xd, e)
        v = torch.zeros((nb,) + v1s, device="cuda")
        s.state(v)
        torch.cuda.synchronize()
        assert s.error_flag() == 0
        return v.cpu().numpy(), e.cpu().numpy().copy(), prof

    for x3 in ((0, 4) if name in X3_CASES else (0,)):
        vf, ef, prof = run(True, x3, direct=True)
        assert prof[3] == steps and prof[4] == steps - x3 - (1 if x3 == 0 else 0), prof
        vu, eu, prof_u = run(False, x3, direct=True)
        assert prof_u[4] == 0
        assert np.abs(ef - eu).max() / np.abs(eu).max() < 1e-4, (ef, eu)
        assert np.abs(vf - vu).max() <= 1e-3 * np.abs(vu).max()
        rel = np.abs(ef - e64[-1]) / np.abs(e64[-1])
        assert rel.max() < 1e-3, rel
        for chains in ((1, 2) if nb >= 2 else (1,)):
            vg, _, _ = run(True, x3, chains=chains)
            assert np.array_equal(vg.view(np.uint32), vf.view(np.uint32)), chains
    # the shortest fused run: R + F (residual window), F (bands, writes A), R + P
    vf3, _, _ = run(True, 0, n=3, direct=True)
    vu3, _, _ = run(False, 0, n=3, direct=True)
    assert np.abs(vf3 - vu3).max() <= 1e-3 * max(np.abs(vu3).max(), 1e-6)


def test_lca_fused_plan_shapes(torch, oracle):
    """Every fused-kernel shape that fits: the ring depths change nothing (bit-identical state for
    one feature tile); other feature tiles split the reconstruction into other bands and stay
    within 1e-3 of max|V| of the two-kernel form."""
    from openpv_gb300 import capi
    nb, ins, v1s, nxp, vth, steps, w, x, p = setup(oracle, "colour")
    wd = torch.from_numpy(w).cuda()
    xd = torch.from_numpy(x).cuda()
    s = capi.LcaSolver(nb, ins, v1s, nxp, vth)
    s.set_weights(wd)

    def state():
        s.reset()
        s.run(xd, steps, x3_steps=0, precision=capi.LCA_BF16)
        v = torch.zeros((nb,) + v1s, device="cuda")
        s.state(v)
        torch.cuda.synchronize()
        assert s.error_flag() == 0
        return v.cpu().numpy()

    s.set_schedule(fused=False)
    ref = state()
    s.set_schedule(fused=True)
    per_tile = {}
    for ft in (64, 128):
        for nv in (2, 4):
            for nw in (2, 3, 4):
                try:
                    s.set_fused_plan(ft, nv, nw)
                except capi.PvgpuError:
                    continue
                assert s.fused_plan_info() == {"feature_tile": ft, "v_slots": nv, "w_slots": nw}
                v = state()
                if ft in per_tile:
                    assert np.array_equal(v.view(np.uint32), per_tile[ft].view(np.uint32)), (ft, nv, nw)
                else:
                    per_tile[ft] = v
                assert np.abs(v - ref).max() <= 1e-3 * np.abs(ref).max(), (ft, nv, nw)
    assert set(per_tile) == {64, 128}
    with pytest.raises(capi.PvgpuError):
        s.set_fused_plan(96, 2, 2)  # not a multiple of 64
    for nv, nw in ((1, 2), (3, 2), (2, 5)):  # odd V rings (the two epilogue groups own every other slot)
        with pytest.raises(capi.PvgpuError):
            s.set_fused_plan(64, nv, nw)


def test_lca_config3_geometry_every_fused_shape(torch, oracle):
    """The batched configuration's geometry -- 32x32x3 inputs (1/f spectrum, unit std) -> V1
    16x16x512 at stride 2, 512 features of 8x8x3, VThresh = AShift = 0.15 -- on 4 images for 100
    timesteps with the last 12 in BF16x3.  Every fused-kernel shape the solver accepts (feature
    tiles 64..512, V rings of 2 and 4 slots, weight rings of 2 to 4, among them the 512-feature
    tile with 4 V and 3 weight slots) against the two-kernel form: V within 1e-3 of max|V|; the final
    energy within 1e-3 relative of the FP64 oracle for each, and for the autotuner's own pick;
    no bounded device wait gives up."""
    from openpv_gb300 import capi
    nb, ins, v1s, nxp, vth, steps, x3 = 4, (32, 32, 3), (16, 16, 512), 8, 0.15, 100, 12
    rng = np.random.default_rng(1234 + 3)
    w = dictionary(rng, v1s[2], nxp, ins[2])
    x = one_over_f(rng, nb, *ins)
    p = oracle.lca_params(nbatch=nb, inNx=32, inNy=32, inNf=3, v1Nx=16, v1Ny=16, v1Nf=512, nxp=8, nyp=8,
                          VThresh=vth, AShift=vth, AMin=0.0, VWidth=0.0, tau=100.0, dtFixed=1.0)
    _, _, _, e64 = oracle.lca_run(p, w.astype(np.float64), x[None].astype(np.float64), steps,
                                  np.zeros((nb,) + v1s), f64=True, threads=nb, want_recon=False)
    s = capi.LcaSolver(nb, ins, v1s, nxp, vth)
    s.set_weights(torch.from_numpy(w).cuda())
    xd = torch.from_numpy(x).cuda()
    e = torch.zeros(nb, dtype=torch.float64, device="cuda")

    def solve():
        s.reset()
        s.run(xd, steps, x3_steps=x3, precision=capi.LCA_BF16)
        s.energy(xd, e)
        v = torch.zeros((nb,) + v1s, device="cuda")
        s.state(v)
        torch.cuda.synchronize()
        assert s.error_flag() == 0
        rel = np.abs(e.cpu().numpy() - e64[-1]) / np.abs(e64[-1])
        return v.cpu().numpy(), rel.max()

    s.set_schedule(fused=False)
    ref, rel_u = solve()
    assert rel_u < 1e-3, rel_u
    s.set_schedule(fused=True)
    accepted = []
    for ft in (64, 128, 256, 512):
        for nv in (2, 4):
            for nw in (2, 3, 4):
                try:
                    s.set_fused_plan(ft, nv, nw)
                except capi.PvgpuError:
                    continue
                v, rel = solve()
                accepted.append((ft, nv, nw))
                assert np.abs(v - ref).max() <= 1e-3 * np.abs(ref).max(), (ft, nv, nw)
                assert rel < 1e-3, (ft, nv, nw, rel)
    assert (512, 4, 3) in accepted and (512, 2, 4) in accepted, accepted
    s.autotune(xd, trial_steps=2)
    _, rel = solve()
    assert rel < 1e-3, (rel, s.fused_plan_info(), s.schedule())
