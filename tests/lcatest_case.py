"""The reference's LCA system test (tests/LCATest/input/LCATest.params) as a test case.

Topology: Input (PvpLayer, 128x64x1, two frames shown for 20 timesteps each) -> Residual
(ANNErrorLayer, errScale 1) by IdentConn on channel 0; V1 (HyPerLCALayer, 64x32x24, VThresh =
VWidth = 0.025, AMin = AShift = 0, tau 100, selfInteract, sparse) receives the residual through
the TransposeConn of V1ToResidual (18x18x1 shared weights, postsynaptic perspective);
Reconstruction (ANNLayer, identity) receives V1 through a CloneConn of V1ToResidual (presynaptic
perspective) and feeds the residual's channel 1 by IdentConn.  V1's time step comes from an
AdaptiveTimeScaleProbe (baseMax 0.55, baseMin 0.5, tauFactor 0.1, growthFactor 0.01, triggered by
the input) on the total energy: 0.5 * the residual's squared L2 norm (L2NormProbe) plus the
firm-threshold cost of V1 (FirmThresholdCostFnLCAProbe, coefficient VThresh).  The test compares
the reconstruction with correct.pvp at every timestep to 1e-6 (RequireAllZeroActivityProbe).

Initial state from the column's random seed 1234567890, seeds handed out in the order the
column initialises its objects (V1 before V1ToResidual): V1's UniformRandomV (minV -1, maxV 0.1)
takes seeds 1234567890 .. + 2047 (one per restricted position), the weights
(UniformRandomWeight, wMin -1, wMax 1, sparseFraction 0.9, one generator per feature) the next
24, followed by normalizeL2 (strength 1).

TEST INFRASTRUCTURE: the oracle builds the initial state and the expected trajectory.
"""
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURE = os.path.join(HERE, "golden", "lcatest_correct.npz")

SEED = 1234567890
IN_NX, IN_NY = 128, 64
V1_NX, V1_NY, V1_NF = 64, 32, 24
NXP = 18
VTHRESH = VWIDTH = 0.025
TAU = 100.0
DISPLAY = 20
STEPS = 40
BASE_MAX, BASE_MIN, TAU_FACTOR, GROWTH = 0.55, 0.5, 0.1, 0.01
BAR = 1e-6  # RequireAllZeroActivityProbe "ComparisonTest" nnzThreshold (LCATest.params)


def fixture():
    z = np.load(FIXTURE)
    return z["input_frames"], z["steps"], z["correct"]


def initial_state(O):
    """(V0 [1][32][64][24], W [24][18][18][1]) from the column's seed."""
    v0 = O.uniform_random_v(V1_NX, V1_NY, V1_NF, -1.0, 0.1, SEED)[None]
    w = O.uniform_random_weights(V1_NF, NXP * NXP, -1.0, 1.0, 0.9, SEED + V1_NX * V1_NY)
    return v0, O.normalize_l2(w).reshape(V1_NF, NXP, NXP, 1)


def locs(O_or_capi):
    """V1 and residual layer geometries with the margins the connections need."""
    L = O_or_capi.Loc
    return L.make(1, V1_NX, V1_NY, V1_NF, 4), L.make(1, IN_NX, IN_NY, 1, 8)


def timescale_update(state, energy, base_max=BASE_MAX, base_min=BASE_MIN, tau_factor=TAU_FACTOR, growth=GROWTH):
    """AdaptiveTimeScaleController::calcTimesteps (components/AdaptiveTimeScaleController.cpp:57-86)
    for one batch element; state = [timeScale, timeScaleMax, timeScaleTrue], energy = the total
    energy of the previous timestep, or -1 where the trigger layer updates this timestep."""
    ts, tsmax, e0 = state
    if energy == e0:
        return state
    dE = (e0 - energy) / ts
    if dE < 0.0 or e0 <= 0.0 or energy <= 0.0:
        return [base_min, base_max, energy]
    ts = tau_factor * (e0 / dE)
    if ts >= tsmax:
        ts = tsmax
        tsmax = tsmax * (1 + growth)
    return [ts, tsmax, energy]


def oracle_steps(O, frames, v0, w):
    """The module stepped with the oracle's primitives in the column's phase order (residual,
    V1, reconstruction from V1's SparseList, probes); per timestep the time step, the residual,
    V1's V and A, the reconstruction and the total energy."""
    v1, er = locs(O)
    inf = np.float32(np.inf)
    v = v0.copy()
    a1 = O.ann_activity(v1, v, VTHRESH, 0.0, inf, 0.0, VWIDTH)
    rec = np.zeros(er.res_shape(), np.float32)
    state = [BASE_MIN, BASE_MAX, -1.0]
    energy = 0.0
    out = []
    for t in range(1, STEPS + 1):
        state = timescale_update(state, -1.0 if (t - 1) % DISPLAY == 0 else energy)
        dt = np.array([state[0]])
        x = frames[(t - 1) // DISPLAY].reshape(er.res_shape())
        ge = O.gsyn_accumulate(np.stack([x, rec]), [1.0, -1.0])
        ae = O.ann_activity(er, ge, -inf, -inf, inf, 0.0, 0.0)
        g1 = O.deliver_post(er, v1, NXP, NXP, w, ae)
        v = O.lca_update(v1, g1, a1, v, dt, TAU)
        a1 = O.ann_activity(v1, v, VTHRESH, 0.0, inf, 0.0, VWIDTH)
        ent, num = O.compact(a1.reshape(1, -1))
        rec = O.deliver_pre(v1, er, NXP, NXP, w, entries=ent, num_active=num)
        energy = (0.5 * O.cost_sum(er, ae, O.COST_L2)[0]
                  + float(np.float32(VTHRESH)) * O.cost_sum(v1, a1, O.COST_FIRM, VTHRESH, VWIDTH)[0])
        out.append(dict(dt=float(dt[0]), ae=ae, v=v.copy(), a1=a1.copy(), rec=rec, energy=energy))
    return out


def oracle_params(O):
    return O.lca_params(nbatch=1, inNx=IN_NX, inNy=IN_NY, inNf=1, v1Nx=V1_NX, v1Ny=V1_NY, v1Nf=V1_NF, nxp=NXP,
                        nyp=NXP, VThresh=VTHRESH, AMin=0.0, AMax=float("inf"), AShift=0.0, VWidth=VWIDTH, tau=TAU,
                        adaptive=1, baseMax=BASE_MAX, baseMin=BASE_MIN, tauFactor=TAU_FACTOR, growthFactor=GROWTH,
                        displayPeriod=DISPLAY, costKind=O.COST_FIRM, costThresh=VTHRESH, costWidth=VWIDTH)
