"""The reference's momentum-LCA system test (tests/MomentumLCATest/input/MomentumLCATest.params)
as a test case.

Topology: Input (PvpLayer, 60x60x1, one image shown for 5 timesteps at a time) -> Residual
(ANNErrorLayer) by IdentConn on channel 0; V1 (MomentumLCALayer, 30x30x32, VThresh = VWidth =
0.025, AMin = AShift = 0, tau 100, LCAMomentumRate 0.4, selfInteract, sparse) feeds the residual's
channel 1 directly through V1ToResidual (HyPerConn, 18x18x1 shared weights, presynaptic
perspective: at timestep 1 the residual already receives V1's initial activity) and receives the
residual through its TransposeConn (postsynaptic perspective); Reconstruction (ANNLayer,
identity) receives V1 through a CloneConn.  V1's time step comes from an AdaptiveTimeScaleProbe
(baseMax 5, baseMin 0.125, tauFactor 0.05, growthFactor 0, triggered by the input) on the total
energy (0.5 * the residual's squared L2 norm + VThresh * the firm-threshold cost of V1).  The test
compares the reconstruction with correct.pvp (10 frames) at every timestep to 1e-4.

Initial state from the column's random seed 1234567890 in the order the column initialises its
objects: V1's UniformRandomV (minV -1, maxV 0.1) takes seeds 1234567890 .. + 899, the weights
(UniformRandomWeight, wMin -1, wMax 1, sparseFraction 0.9) the next 32, then normalizeL2.

TEST INFRASTRUCTURE: the oracle builds the initial state and the expected trajectory.
"""
import os

import numpy as np

from tests.lcatest_case import timescale_update

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURE = os.path.join(HERE, "golden", "momentumlcatest_correct.npz")

SEED = 1234567890
IN_N, V1_N, V1_NF, NXP = 60, 30, 32, 18
VTHRESH = VWIDTH = 0.025
TAU = 100.0
RATE = 0.4
DISPLAY = 5
STEPS = 10
BASE_MAX, BASE_MIN, TAU_FACTOR, GROWTH = 5.0, 0.125, 0.05, 0.0
BAR = 1e-4  # RequireAllZeroActivityProbe "ComparisonTest" nnzThreshold (MomentumLCATest.params)


def fixture():
    z = np.load(FIXTURE)
    return z["input_frame"], z["correct"]


def initial_state(O):
    """(V0 [1][30][30][32], W [32][18][18][1]) from the column's seed."""
    v0 = O.uniform_random_v(V1_N, V1_N, V1_NF, -1.0, 0.1, SEED)[None]
    w = O.uniform_random_weights(V1_NF, NXP * NXP, -1.0, 1.0, 0.9, SEED + V1_N * V1_N)
    return v0, O.normalize_l2(w).reshape(V1_NF, NXP, NXP, 1)


def locs(O_or_capi):
    """V1 and residual layer geometries with the margins the connections need."""
    L = O_or_capi.Loc
    return L.make(1, V1_N, V1_N, V1_NF, 4), L.make(1, IN_N, IN_N, 1, 8)


def step_timescale(state, energy):
    return timescale_update(state, energy, BASE_MAX, BASE_MIN, TAU_FACTOR, GROWTH)


def oracle_steps(O, x, v0, w):
    """The module stepped with the oracle's primitives in the column's phase order (residual from
    the input and V1's current activity, V1's momentum update, the reconstruction from V1's
    SparseList, probes); per timestep the time step, the residual, V1's V and A, the
    reconstruction and the total energy."""
    v1, er = locs(O)
    inf = np.float32(np.inf)
    v = v0.copy()
    a1 = O.ann_activity(v1, v, VTHRESH, 0.0, inf, 0.0, VWIDTH)
    prev = np.zeros(v1.res_shape(), np.float32)
    ent, num = O.compact(a1.reshape(1, -1))
    rec = O.deliver_pre(v1, er, NXP, NXP, w, entries=ent, num_active=num)
    xin = x.reshape(er.res_shape())
    state, energy = [BASE_MIN, BASE_MAX, -1.0], 0.0
    out = []
    for t in range(1, STEPS + 1):
        state = step_timescale(state, -1.0 if (t - 1) % DISPLAY == 0 else energy)
        dt = np.array([state[0]])
        ge = O.gsyn_accumulate(np.stack([xin, rec]), [1.0, -1.0])
        ae = O.ann_activity(er, ge, -inf, -inf, inf, 0.0, 0.0)
        g1 = O.deliver_post(er, v1, NXP, NXP, w, ae)
        v, prev = O.momentum_lca_update(v1, g1, a1, prev, v, dt, TAU, RATE)
        a1 = O.ann_activity(v1, v, VTHRESH, 0.0, inf, 0.0, VWIDTH)
        ent, num = O.compact(a1.reshape(1, -1))
        rec = O.deliver_pre(v1, er, NXP, NXP, w, entries=ent, num_active=num)
        energy = (0.5 * O.cost_sum(er, ae, O.COST_L2)[0]
                  + float(np.float32(VTHRESH)) * O.cost_sum(v1, a1, O.COST_FIRM, VTHRESH, VWIDTH)[0])
        out.append(dict(dt=float(dt[0]), ae=ae, v=v.copy(), a1=a1.copy(), prev=prev.copy(), rec=rec,
                        energy=energy))
    return out
