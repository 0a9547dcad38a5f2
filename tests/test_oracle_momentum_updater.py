"""The oracle's MomentumUpdater restatement against the reference's own known-answer model of it
(tests/MomentumConnSimpleCheckpointerTest/src/CorrectState.cpp, restated below): one input and
one output neuron joined by one weight (IdentWeight 1), input ceil(t / 4), output = input * w,
a weight update every fourth step with the Hebbian dW = input * output (dWMax 1), and
momentumMethod "simple" with timeConstantTau 0.75 and no decay (the test's params file)."""
import math

import numpy as np

F = np.float32


def correct_state(steps, tau):
    """CorrectState::update, float arithmetic; the (weight, dw) after every step."""
    w, dw, out = F(1.0), F(0.0), []
    for t in range(1, steps + 1):
        x = F(math.ceil(F(t) / F(4.0)))
        y = x * w
        if abs(math.fmod(t + 1, 4.0) - 1) < 0.5:  # doesWeightUpdate
            base = x * y
            dw = (F(1) - tau) * base + tau * dw
            w = w + dw
        out.append((w, dw))
    return out


def test_simple_momentum_matches_reference_known_answers(oracle):
    tau = F(0.75)
    dwf, wf = oracle.momentum_factors("s", tau, 0.0, 1.0)
    assert (dwf, wf) == (tau, 0.0)
    want = correct_state(40, tau)
    w = np.array([1.0], np.float32)
    prev = np.array([0.0], np.float32)
    dw = np.array([0.0], np.float32)
    for t in range(1, 41):
        x = F(math.ceil(F(t) / F(4.0)))
        if abs(math.fmod(t + 1, 4.0) - 1) < 0.5:
            y = x * w[0]
            dw = np.array([x * y], np.float32)  # HebbianUpdater dW of this update
            dw, prev, w = oracle.momentum_update_weights(dw, prev, w, dwf, wf)
        assert w[0] == want[t - 1][0] and prev[0] == want[t - 1][1], t


def test_momentum_factors(oracle):
    tau = 12.5
    # expf of the float quotient, correctly rounded (the C library's expf is, for this argument)
    arg = float(np.float32(-1.0) / np.float32(tau))
    assert oracle.momentum_factors("v", tau, 0.01, 2.0) == (float(np.float32(math.exp(arg))), np.float32(0.01))
    assert oracle.momentum_factors("v", 0.0, 0.0, 1.0)[0] == 0.0
    a = oracle.momentum_factors("a", 0.5, 0.1, 3.0)
    assert a[0] == np.float32(0.5) and a[1] == np.float32(np.float32(0.1) * np.float32(3.0))
