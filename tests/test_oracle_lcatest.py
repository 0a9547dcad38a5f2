"""The oracle's LCA module against the reference's own known answer for it: the reconstruction
of the LCA system test (tests/LCATest/input/correct.pvp, LCATest.params), which the reference
compares with its Reconstruction layer at every timestep to 1e-6.  The case is described in
tests/lcatest_case.py: random initial V and weights from the column's seed, normalizeL2, a
firm threshold, sparse V1, and the adaptive time step driven by the total energy.

Both forms of the module are checked: the oracle's module loop (pvo_lca_run, reconstruction by
the dense presynaptic loop) and the step-by-step composition from the oracle's primitives with
the reconstruction delivered from V1's SparseList (the composition the GPU test mirrors through
the C ABI).  Neither is bit-exact with the file (about a third of the pixels match bit for bit,
the rest within 1.2e-7: the file's summation order, e.g. per-thread accumulation, is not
recorded), both are well inside the test's 1e-6."""
import os

import numpy as np
import pytest

from tests import lcatest_case as L
from tests.refbuild import REF_ROOT


def _module_run(oracle, frames, v0, w):
    p = L.oracle_params(oracle)
    _, _, recon, energy = oracle.lca_run(p, w, frames.reshape(2, 1, L.IN_NY, L.IN_NX, 1), L.STEPS, v0)
    return recon[:, 0, :, :, 0], energy[:, 0]


def test_lca_module_reproduces_lcatest_known_answer(oracle):
    frames, steps, correct = L.fixture()
    v0, w = L.initial_state(oracle)
    assert (w != 0).mean() < 0.15  # sparseFraction 0.9
    assert np.allclose((w.astype(np.float64) ** 2).sum(axis=(1, 2, 3)), 1.0, rtol=1e-5)
    recon, energy = _module_run(oracle, frames, v0, w)
    seq = L.oracle_steps(oracle, frames, v0, w)
    worst = 0.0
    for i, t in enumerate(steps):
        want = correct[i, :, :, 0]
        d_run = np.abs(recon[t - 1] - want).max()
        d_seq = np.abs(seq[t - 1]["rec"].reshape(L.IN_NY, L.IN_NX) - want).max()
        assert d_run <= L.BAR and d_seq <= L.BAR, (t, d_run, d_seq)
        worst = max(worst, d_run, d_seq)
    # the two forms agree on the energy that drives the time step
    for t in range(L.STEPS):
        assert abs(seq[t]["energy"] - energy[t]) <= 1e-9 * abs(energy[t]), t
    # the time step follows the probe: base at both frame onsets, growing in between
    assert seq[0]["dt"] == L.BASE_MIN and seq[L.DISPLAY]["dt"] == L.BASE_MIN
    assert seq[L.DISPLAY - 1]["dt"] > seq[1]["dt"] >= L.BASE_MIN
    print(f"LCATest known answer at steps {steps.tolist()}: max |recon - correct| = {worst:.2e} (bar {L.BAR})")


def _reference_correct():
    path = os.path.join(REF_ROOT, "tests", "LCATest", "input", "correct.pvp")
    if not os.path.exists(path):
        pytest.skip("reference tree not present")
    from tests.golden.make_lcatest_fixture import read_dense_pvp
    return read_dense_pvp(path)


def test_lca_module_reproduces_every_frame_of_correct_pvp(oracle):
    """All 40 frames of the reference's file (read where the reference tree is present), and
    the fixture's frames are the file's."""
    c, t = _reference_correct()
    frames, steps, correct = L.fixture()
    assert np.array_equal(c[steps - 1], correct)
    v0, w = L.initial_state(oracle)
    recon, _ = _module_run(oracle, frames, v0, w)
    err = np.abs(recon - c[:, :, :, 0]).reshape(L.STEPS, -1).max(axis=1)
    assert np.all(err <= L.BAR), err
    # the seed order matters: the weights drawn first (seeds 1234567890 ..) miss by far
    w_first = oracle.normalize_l2(
        oracle.uniform_random_weights(L.V1_NF, L.NXP * L.NXP, -1.0, 1.0, 0.9, L.SEED)).reshape(w.shape)
    v_second = oracle.uniform_random_v(L.V1_NX, L.V1_NY, L.V1_NF, -1.0, 0.1, L.SEED + L.V1_NF)[None]
    recon_bad, _ = _module_run(oracle, frames, v_second, w_first)
    assert np.abs(recon_bad[0] - c[0, :, :, 0]).max() > 1e-2


def test_random_initial_state_matches_the_gpu_lca_test_files(oracle):
    """tests/GPULCATest/input holds V1's initial V (initialV1.pvp) and the weights
    (weights.pvp) that the same seeded initialisation produced: the oracle's UniformRandomV
    equals the V file bit for bit, its UniformRandomWeight + normalizeL2 the weight file to
    within one rounding of the normalisation (6e-8)."""
    d = os.path.join(REF_ROOT, "tests", "GPULCATest", "input")
    if not os.path.isdir(d):
        pytest.skip("reference tree not present")
    from tests.golden.make_lcatest_fixture import read_dense_pvp
    v_file, _ = read_dense_pvp(os.path.join(d, "initialV1.pvp"))
    v0, w = L.initial_state(oracle)
    assert np.array_equal(v_file[0].view(np.uint32), v0[0].view(np.uint32))
    # a shared-weight file (PVP_KERNEL_FILE_TYPE): 104-byte header, then per kernel an 8-byte
    # patch header and nxp*nyp*nfp floats
    raw = open(os.path.join(d, "weights.pvp"), "rb").read()
    hdr = np.frombuffer(raw, np.int32, 26)
    assert hdr[0] == 104 and hdr[2] == 5 and tuple(hdr[20:23]) == (L.NXP, L.NXP, 1) and hdr[25] == L.V1_NF
    n = L.NXP * L.NXP
    w_file = np.stack([np.frombuffer(raw, np.float32, n, 104 + k * (8 + 4 * n) + 8) for k in range(L.V1_NF)])
    assert np.abs(w_file.reshape(w.shape) - w).max() <= 1e-7


def test_host_timescale_stand_in_matches_the_oracle(oracle):
    """The host-side time-scale update the GPU test uses in place of the column's probe equals
    the oracle's AdaptiveTimeScaleController restatement step for step: resets (-1), repeated
    energies, growth up to the cap, an energy increase."""
    energies = [-1.0, 3171.0, 3190.1, 3176.5, 3100.0, 3050.0, 3049.9, 3049.9, 3000.0, 3500.0, 3400.0, -1.0, 2900.0,
                2800.0, 2700.0, 2650.0, 2640.0, 2639.0]
    py = [L.BASE_MIN, L.BASE_MAX, -1.0]
    c = np.array([[L.BASE_MIN, L.BASE_MAX, -1.0]])
    for e in energies:
        py = L.timescale_update(py, e)
        c = oracle.adaptive_timescale(c, [e], L.BASE_MAX, L.BASE_MIN, L.TAU_FACTOR, L.GROWTH)
        assert py == list(c[0]), (e, py, c[0])


def test_momentum_lca_module_reproduces_momentumlcatest_bit_for_bit(oracle):
    """The reference's momentum-LCA system test (tests/MomentumLCATest, described in
    tests/momentumlcatest_case.py): V1 feeding the residual directly (its initial activity at
    timestep 1), MomentumLCALayer, the time step triggered by the input every 5 steps.  The
    oracle's composition from its pinned primitives reproduces all 10 known-answer frames bit for
    bit (the test itself allows 1e-4)."""
    from tests import momentumlcatest_case as M
    x, correct = M.fixture()
    v0, w = M.initial_state(oracle)
    steps = M.oracle_steps(oracle, x, v0, w)
    for t in range(M.STEPS):
        got = steps[t]["rec"].reshape(M.IN_N, M.IN_N)
        assert np.array_equal(got.view(np.uint32), correct[t, :, :, 0].view(np.uint32)), t
    assert steps[0]["dt"] == M.BASE_MIN and steps[M.DISPLAY]["dt"] == M.BASE_MIN
    c, _ = _reference_file("MomentumLCATest", "correct.pvp")
    if c is not None:
        assert np.array_equal(c, correct)


def _reference_file(test, name):
    path = os.path.join(REF_ROOT, "tests", test, "input", name)
    if not os.path.exists(path):
        return None, None
    from tests.golden.make_lcatest_fixture import read_dense_pvp
    return read_dense_pvp(path)
