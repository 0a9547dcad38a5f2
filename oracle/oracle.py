"""ctypes binding of the CPU oracle (oracle/libpvoracle.so).

TEST INFRASTRUCTURE ONLY: tests/, __graft_entry__.smoke() and bench.py's
cpu_baseline / reference arm use this module as the checker.  The product path
in openpv_gb300 never imports it.

Each wrapper restates one reference loop (see pvoracle.h for the file:line each
follows) and takes numpy arrays in the reference layouts:
  activity   [nbatch][nyExt][nxExt][nf]  (extended, FP32)
  GSyn / V   [nbatch][ny][nx][nf]        (restricted, FP32)
  weights    [kernel][nyp][nxp][nfp]
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libpvoracle.so")


class Halo(C.Structure):
    _fields_ = [("lt", C.c_int), ("rt", C.c_int), ("dn", C.c_int), ("up", C.c_int)]


class Loc(C.Structure):
    _fields_ = [("nbatch", C.c_int), ("nx", C.c_int), ("ny", C.c_int), ("nf", C.c_int), ("halo", Halo)]

    @staticmethod
    def make(nbatch, nx, ny, nf, mx=0, my=None):
        my = mx if my is None else my
        return Loc(nbatch, nx, ny, nf, Halo(mx, mx, my, my))

    @property
    def nx_ext(self):
        return self.nx + self.halo.lt + self.halo.rt

    @property
    def ny_ext(self):
        return self.ny + self.halo.dn + self.halo.up

    @property
    def num_ext(self):
        return self.nx_ext * self.ny_ext * self.nf

    @property
    def num_res(self):
        return self.nx * self.ny * self.nf

    def ext_shape(self):
        return (self.nbatch, self.ny_ext, self.nx_ext, self.nf)

    def res_shape(self):
        return (self.nbatch, self.ny, self.nx, self.nf)


class Patch(C.Structure):
    _fields_ = [("nx", C.c_uint16), ("ny", C.c_uint16), ("offset", C.c_uint32)]


PATCH_DTYPE = np.dtype([("nx", np.uint16), ("ny", np.uint16), ("offset", np.uint32)])
ENTRY_DTYPE = np.dtype([("index", np.uint32), ("value", np.float32)])


class LcaParams(C.Structure):
    _fields_ = [
        ("nbatch", C.c_int),
        ("inNx", C.c_int), ("inNy", C.c_int), ("inNf", C.c_int),
        ("v1Nx", C.c_int), ("v1Ny", C.c_int), ("v1Nf", C.c_int),
        ("nxp", C.c_int), ("nyp", C.c_int),
        ("VThresh", C.c_float), ("AMin", C.c_float), ("AMax", C.c_float),
        ("AShift", C.c_float), ("VWidth", C.c_float),
        ("tau", C.c_float),
        ("selfInteract", C.c_int),
        ("errScale", C.c_float),
        ("adaptive", C.c_int),
        ("baseMax", C.c_double), ("baseMin", C.c_double),
        ("tauFactor", C.c_double), ("growthFactor", C.c_double),
        ("dtFixed", C.c_double),
        ("displayPeriod", C.c_int),
        ("l2Coeff", C.c_double),
        ("costKind", C.c_int),
        ("costThresh", C.c_double), ("costWidth", C.c_double),
        ("costCoeff", C.c_double),
    ]


_lib = None


def build():
    """Compile the oracle with its Makefile (gcc, seconds)."""
    subprocess.check_call(["make", "-s", "-C", HERE])


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        _lib = C.CDLL(LIB_PATH)
        _declare(_lib)
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def _declare(L):
    vp, i, f, d = C.c_void_p, C.c_int, C.c_float, C.c_double
    lp = C.POINTER(Loc)
    sig = {
        "pvo_required_margin": (i, [i, i, i]),
        "pvo_post_patch_size": (i, [i, i, i]),
        "pvo_patch_geometry": (i, [lp, lp, i, i, vp, vp, vp, vp]),
        "pvo_kernel_index_table": (i, [lp, lp, vp]),
        "pvo_transpose_shared": (i, [lp, lp, i, i, vp, vp]),
        "pvo_compact": (None, [vp, i, i, vp, vp]),
        "pvo_deliver_pre": (i, [lp, lp, i, i, vp, vp, vp, vp, f, vp]),
        "pvo_deliver_pre_f64": (i, [lp, lp, i, i, vp, vp, d, vp]),
        "pvo_deliver_post": (i, [lp, lp, i, i, vp, vp, f, vp]),
        "pvo_deliver_post_f64": (i, [lp, lp, i, i, vp, vp, d, vp]),
        "pvo_gsyn_accumulate": (None, [i, i, vp, vp, vp]),
        "pvo_lca_update": (None, [lp, i, vp, f, vp, vp, vp]),
        "pvo_momentum_lca_update": (None, [lp, i, f, vp, f, vp, vp, vp, vp]),
        "pvo_taus_init": (None, [vp, C.c_size_t, C.c_uint32]),
        "pvo_taus_next": (None, [vp, C.c_size_t]),
        "pvo_lif_update": (i, [C.c_char, lp, vp, f, vp, vp, vp, vp, vp, vp, vp, vp]),
        "pvo_momentum_factors": (i, [C.c_char, f, f, f, C.POINTER(f), C.POINTER(f)]),
        "pvo_momentum_update_weights": (None, [C.c_int64, f, f, vp, vp, vp]),
        "pvo_ista_update": (None, [lp, f, vp, f, vp, vp, vp]),
        "pvo_lca_update_f64": (None, [lp, i, vp, d, vp, vp, vp]),
        "pvo_ann_activity": (None, [lp, vp, f, f, f, f, f, vp]),
        "pvo_ann_activity_f64": (None, [lp, vp, d, d, d, d, d, vp]),
        "pvo_ann_vertices": (i, [f, f, f, f, f, vp, vp, vp]),
        "pvo_cost_sum": (None, [lp, vp, i, d, d, vp]),
        "pvo_cost_sum_f64": (None, [lp, vp, i, d, d, vp]),
        "pvo_adaptive_timescale": (None, [i, d, d, d, d, vp, vp]),
        "pvo_hebbian_dw": (i, [lp, lp, i, i, f, vp, vp, vp]),
        "pvo_hebbian_dw_f64": (i, [lp, lp, i, i, d, vp, vp, vp]),
        "pvo_hebbian_dw_rule": (i, [lp, lp, i, i, i, f, vp, vp, vp, vp]),
        "pvo_lca_run": (i, [C.POINTER(LcaParams), vp, vp, i, i, vp, vp, vp, vp, i]),
        "pvo_lca_run_f64": (i, [C.POINTER(LcaParams), vp, vp, i, i, vp, vp, vp, vp, i]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def _check(rc, what):
    if rc != 0:
        raise ValueError(f"oracle {what}: illegal geometry")


def required_margin(n_pre, n_post, patch):
    return lib().pvo_required_margin(n_pre, n_post, patch)


def post_patch_size(patch, n_pre, n_post):
    return lib().pvo_post_patch_size(patch, n_pre, n_post)


def patch_geometry(pre, post, nxp, nyp):
    n = pre.num_ext
    patches = np.zeros(n, PATCH_DTYPE)
    gstart = np.zeros(n, np.int64)
    apost = np.zeros(n, np.int64)
    ustart = np.zeros(n, np.int64)
    _check(lib().pvo_patch_geometry(C.byref(pre), C.byref(post), nxp, nyp, _p(patches), _p(gstart),
                                    _p(apost), _p(ustart)), "patch_geometry")
    return patches, gstart, apost, ustart


def kernel_index_table(pre, post):
    t = np.zeros(pre.num_ext, np.int32)
    nk = lib().pvo_kernel_index_table(C.byref(pre), C.byref(post), _p(t))
    return t, nk


def transpose_shared(pre, post, nxp, nyp, w_pre):
    nxp_post = post_patch_size(nxp, pre.nx, post.nx)
    nyp_post = post_patch_size(nyp, pre.ny, post.ny)
    nk_post = (post.nx // pre.nx if post.nx > pre.nx else 1) * (post.ny // pre.ny if post.ny > pre.ny else 1) * post.nf
    w_post = np.zeros((nk_post, nyp_post, nxp_post, pre.nf), np.float32)
    _check(lib().pvo_transpose_shared(C.byref(pre), C.byref(post), nxp, nyp, _p(_c(w_pre, np.float32)),
                                      _p(w_post)), "transpose_shared")
    return w_post


def compact(a_ext):
    a = _c(a_ext, np.float32)
    nb = a.shape[0]
    n = a[0].size
    ent = np.zeros((nb, n), ENTRY_DTYPE)
    num = np.zeros(nb, np.int64)
    lib().pvo_compact(_p(a), nb, n, _p(ent), _p(num))
    return ent, num


def deliver_pre(pre, post, nxp, nyp, w, a_ext=None, entries=None, num_active=None, dt_factor=1.0, gsyn=None):
    g = np.zeros(post.res_shape(), np.float32) if gsyn is None else gsyn
    assert g.dtype == np.float32 and g.flags.c_contiguous
    w = _c(w, np.float32)
    if entries is not None:
        e = np.ascontiguousarray(entries)
        n = _c(num_active, np.int64)
        rc = lib().pvo_deliver_pre(C.byref(pre), C.byref(post), nxp, nyp, _p(w), _p(e), _p(n), None,
                                   dt_factor, _p(g))
    else:
        a = _c(a_ext, np.float32)
        rc = lib().pvo_deliver_pre(C.byref(pre), C.byref(post), nxp, nyp, _p(w), None, None, _p(a),
                                   dt_factor, _p(g))
    _check(rc, "deliver_pre")
    return g


def deliver_pre_f64(pre, post, nxp, nyp, w, a_ext, dt_factor=1.0):
    g = np.zeros(post.res_shape(), np.float64)
    _check(lib().pvo_deliver_pre_f64(C.byref(pre), C.byref(post), nxp, nyp, _p(_c(w, np.float64)),
                                     _p(_c(a_ext, np.float64)), dt_factor, _p(g)), "deliver_pre_f64")
    return g


def deliver_post(src, tgt, nxp_post, nyp_post, w_post, a_ext, dt_factor=1.0, gsyn=None):
    g = np.zeros(tgt.res_shape(), np.float32) if gsyn is None else gsyn
    _check(lib().pvo_deliver_post(C.byref(src), C.byref(tgt), nxp_post, nyp_post, _p(_c(w_post, np.float32)),
                                  _p(_c(a_ext, np.float32)), dt_factor, _p(g)), "deliver_post")
    return g


def deliver_post_f64(src, tgt, nxp_post, nyp_post, w_post, a_ext, dt_factor=1.0):
    g = np.zeros(tgt.res_shape(), np.float64)
    _check(lib().pvo_deliver_post_f64(C.byref(src), C.byref(tgt), nxp_post, nyp_post,
                                      _p(_c(w_post, np.float64)), _p(_c(a_ext, np.float64)), dt_factor,
                                      _p(g)), "deliver_post_f64")
    return g


def gsyn_accumulate(gsyn, coeffs):
    """gsyn: [numChannels][...] -> G."""
    g = _c(gsyn, np.float32)
    nch = g.shape[0]
    n = g[0].size
    out = np.zeros(g.shape[1:], np.float32)
    lib().pvo_gsyn_accumulate(n, nch, _p(_c(coeffs, np.float32)), _p(g), _p(out))
    return out


def lca_update(loc, g, a_ext, v, dt_adapt, tau, self_interact=True):
    v = _c(v, np.float32).copy()
    lib().pvo_lca_update(C.byref(loc), int(self_interact), _p(_c(dt_adapt, np.float64)), tau,
                         _p(_c(g, np.float32)), _p(_c(a_ext, np.float32)), _p(v))
    return v


def momentum_lca_update(loc, g, a_ext, prev_drive, v, dt_adapt, tau, momentum_rate, self_interact=True):
    """MomentumLCAInternalStateBuffer.kpp:18-69; returns (v, prev_drive)."""
    v = _c(v, np.float32).copy()
    pd = _c(prev_drive, np.float32).copy()
    lib().pvo_momentum_lca_update(C.byref(loc), int(self_interact), momentum_rate, _p(_c(dt_adapt, np.float64)), tau,
                                  _p(_c(g, np.float32)), _p(_c(a_ext, np.float32)), _p(pd), _p(v))
    return v, pd


# LIFParams (components/LIFActivityComponent.hpp:22-45) field order and defaults
# (include/default_params.h: V_REST -70, V_EXC 0, V_INH -75, V_INHB -90, VTH_REST -55, TAU_VMEM 20,
# TAU_VTH 10, DELTA_VTH 5, DELTA_G_INHB 1, TAU_EXC 1, TAU_INH 5, TAU_INHB 10; noise amplitudes 0,
# noise frequencies 250 Hz).
LIF_FIELDS = ("Vrest", "Vexc", "Vinh", "VinhB", "VthRest", "tau", "tauVth", "deltaVth", "deltaGIB",
              "noiseAmpE", "noiseAmpI", "noiseAmpIB", "noiseFreqE", "noiseFreqI", "noiseFreqIB", "tauE", "tauI", "tauIB")
LIF_DEFAULTS = dict(Vrest=-70.0, Vexc=0.0, Vinh=-75.0, VinhB=-90.0, VthRest=-55.0, tau=20.0, tauVth=10.0, deltaVth=5.0,
                    deltaGIB=1.0, noiseAmpE=0.0, noiseAmpI=0.0, noiseAmpIB=0.0, noiseFreqE=250.0, noiseFreqI=250.0,
                    noiseFreqIB=250.0, tauE=1.0, tauI=5.0, tauIB=10.0)
TAUS_DTYPE = np.dtype([("s0", "<u4"), ("s1", "<u4"), ("s2", "<u4"), ("s3", "<u4")])


def lif_params_array(**kw):
    d = dict(LIF_DEFAULTS, **kw)
    return np.array([d[k] for k in LIF_FIELDS], np.float32)


def taus_init(count, seed):
    """cl_random_init (utils/cl_random.c): structured array of {s0, s1, s2, s3}."""
    st = np.zeros(count, TAUS_DTYPE)
    lib().pvo_taus_init(_p(st), count, seed)
    return st


def taus_next(st):
    st = st.copy()
    lib().pvo_taus_next(_p(st), st.size)
    return st


def taus_draws(count, seed, n):
    """n successive outputs (s0) of count generators seeded seed, seed + 1, ...
    (columns/Random.cpp:90-106 randomUInt): [n][count] uint32."""
    st = taus_init(count, seed)
    out = np.zeros((n, count), np.uint32)
    for i in range(n):
        st = taus_next(st)
        out[i] = st["s0"]
    return out


def uniform_random_v(nx, ny, nf, vmin, vmax, seed):
    """UniformRandomV::calcV (initv/UniformRandomV.cpp:44-60) for one batch element of a
    layer on one process: one generator per (x, y) position, seeded seed + y*nx + x
    (columns/Random.cpp:40-85 with nf = 1, restricted), drawn once per feature in feature order;
    each value min + u * (max - min) with u = s0 / (float)UINT_MAX (columns/Random.hpp:37-39,
    Random.cpp:100-103), every operation rounded to float.  Returns V [ny][nx][nf]."""
    d = taus_draws(nx * ny, seed, nf)                     # [f][xy]
    u = d.astype(np.float32) / np.float32(4294967295.0)   # (float)s0 / (float)UINT_MAX
    lo, hi = np.float32(vmin), np.float32(vmax)
    v = (lo + (u * np.float32(hi - lo)).astype(np.float32)).astype(np.float32)
    return np.ascontiguousarray(v.T.reshape(ny, nx, nf))


def uniform_random_weights(num_patches, patch_size, wmin, wmax, sparse_fraction, seed):
    """InitUniformRandomWeights::randomWeights (weightinit/InitUniformRandomWeights.cpp:63-106)
    for shared weights with minNNZ = 0: one generator per data patch, seeded seed + patch
    (InitRandomWeights::initRNGs, weightinit/InitRandomWeights.cpp:39-50); per weight, in patch
    order, one draw for the value wMin + (float)(p * draw) with p = (wMax - wMin) / 2^32 in
    double, then one draw that zeroes it when below sparseFraction * 2^32 (a float).
    Returns [num_patches][patch_size] float32."""
    d = taus_draws(num_patches, seed, 2 * patch_size)     # [draw][patch]
    p = (float(np.float32(wmax)) - float(np.float32(wmin))) / (1.0 + 4294967295.0)
    cut = float(np.float32(np.float32(sparse_fraction) * np.float32(4294967296.0)))
    w = np.zeros((num_patches, patch_size), np.float32)
    for n in range(patch_size):
        val = (np.float32(wmin) + (p * d[2 * n].astype(np.float64)).astype(np.float32)).astype(np.float32)
        w[:, n] = np.where(d[2 * n + 1].astype(np.float64) < cut, np.float32(0.0), val)
    return w


def normalize_l2(w, strength=1.0):
    """NormalizeL2::normalizeWeights (normalizers/NormalizeL2.cpp:53-155) for one connection,
    one arbor, normalizeFromPostPerspective off, no rMin / cutoff / non-negativity: per data
    patch the float sum of squares in patch order (NormalizeBase.cpp:184-193), l2 = sqrtf(sum),
    every weight multiplied by strength / l2 (NormalizeMultiply.cpp:251-254).
    w: [num_patches][...]; returns a normalised copy."""
    shp = w.shape
    w = np.ascontiguousarray(w, np.float32).reshape(shp[0], -1).copy()
    s = np.zeros(shp[0], np.float32)
    for k in range(w.shape[1]):
        s = (s + (w[:, k] * w[:, k]).astype(np.float32)).astype(np.float32)
    mult = (np.float32(strength) / np.sqrt(s)).astype(np.float32)
    return (w * mult[:, None]).astype(np.float32).reshape(shp)


def lif_update(method, loc, params, dt, state, gsyn_head, a_ext):
    """One LIF step (LIFActivityComponent.cpp:332-942).  state: dict of rnd, V, Vth, GE, GI, GIB
    (updated copies returned); gsyn_head: [3][nbatch*nx*ny*nf] EXC, INH, INHB; returns
    (state, a_ext)."""
    st = {k: (v.copy() if k == "rnd" else _c(v, np.float32).copy()) for k, v in state.items()}
    a = _c(a_ext, np.float32).copy()
    rc = lib().pvo_lif_update(method.encode()[:1], C.byref(loc), _p(_c(params, np.float32)), dt, _p(st["rnd"]),
                              _p(st["V"]), _p(st["Vth"]), _p(st["GE"]), _p(st["GI"]), _p(st["GIB"]),
                              _p(_c(gsyn_head, np.float32)), _p(a))
    _check(rc, "lif_update")
    return st, a


def momentum_factors(method, tau, decay=0.0, dw_max=1.0):
    """(dwFactor, wFactor) of MomentumUpdater::applyMomentum for momentumMethod viscosity / simple / alex."""
    a, b = C.c_float(), C.c_float()
    _check(lib().pvo_momentum_factors(method.encode()[:1], tau, decay, dw_max, C.byref(a), C.byref(b)),
           "momentum_factors")
    return a.value, b.value


def momentum_update_weights(dw, prev_dw, w, dw_factor, w_factor):
    """MomentumUpdater::updateWeights: returns (dw, prev_dw, w) after one update."""
    dw, prev_dw, w = (_c(x, np.float32).copy() for x in (dw, prev_dw, w))
    lib().pvo_momentum_update_weights(dw.size, dw_factor, w_factor, _p(dw), _p(prev_dw), _p(w))
    return dw, prev_dw, w


def ista_update(loc, g, a_ext, v, dt_adapt, tau, vthresh):
    """ISTAInternalStateBuffer.kpp:16-63."""
    v = _c(v, np.float32).copy()
    lib().pvo_ista_update(C.byref(loc), vthresh, _p(_c(dt_adapt, np.float64)), tau, _p(_c(g, np.float32)),
                          _p(_c(a_ext, np.float32)), _p(v))
    return v


def lca_update_f64(loc, g, a_ext, v, dt_adapt, tau, self_interact=True):
    v = _c(v, np.float64).copy()
    lib().pvo_lca_update_f64(C.byref(loc), int(self_interact), _p(_c(dt_adapt, np.float64)), tau,
                             _p(_c(g, np.float64)), _p(_c(a_ext, np.float64)), _p(v))
    return v


def ann_activity(loc, v, VThresh, AMin, AMax, AShift, VWidth, a_ext=None):
    a = np.zeros(loc.ext_shape(), np.float32) if a_ext is None else _c(a_ext, np.float32).copy()
    lib().pvo_ann_activity(C.byref(loc), _p(_c(v, np.float32)), VThresh, AMin, AMax, AShift, VWidth, _p(a))
    return a


def ann_activity_f64(loc, v, VThresh, AMin, AMax, AShift, VWidth, a_ext=None):
    a = np.zeros(loc.ext_shape(), np.float64) if a_ext is None else _c(a_ext, np.float64).copy()
    lib().pvo_ann_activity_f64(C.byref(loc), _p(_c(v, np.float64)), VThresh, AMin, AMax, AShift, VWidth, _p(a))
    return a


def ann_vertices(VThresh, AMin, AMax, AShift, VWidth):
    vV = np.zeros(4, np.float32)
    vA = np.zeros(4, np.float32)
    sl = np.zeros(5, np.float32)
    n = lib().pvo_ann_vertices(VThresh, AMin, AMax, AShift, VWidth, _p(vV), _p(vA), _p(sl))
    return vV[:n].copy(), vA[:n].copy(), sl[:n + 1].copy()


def apply_vertices(loc, v, vV, vA, slopes):
    """applyVerticesANNActivityBufferOnCPU (components/ANNActivityBuffer.kpp:16-77), vectorised:
    the piecewise-linear transfer function of numVertices vertices and numVertices + 1 slopes,
    restricted V -> extended A (halo zero).  float32 throughout, every product and sum rounded
    on its own (numpy does not fuse them), as the reference's CPU build computes it."""
    f = np.float32
    vV, vA, sl = (np.asarray(t, f) for t in (vV, vA, slopes))
    x = np.asarray(v, f).reshape(loc.nbatch, -1)
    n = len(vV)
    last = n - 1
    a = np.zeros_like(x)
    lo, hi = x < vV[0], x >= vV[last]
    a[lo] = vA[0] + sl[0] * (x[lo] - vV[0])
    a[hi] = vA[last] + sl[n] * (x[hi] - vV[last])
    alive = ~lo & ~hi
    for j in range(last):
        alive &= x >= vV[j]  # the loop stops at the first vertex above the potential
        eq = alive & (x == vV[j])
        a[eq] = vA[j]
        lin = alive & (x != vV[j]) & (x < vV[j + 1])
        a[lin] = vA[j] + sl[j + 1] * (x[lin] - vV[j])
    out = np.zeros(loc.ext_shape(), f)
    h = loc.halo
    out[:, h.up:h.up + loc.ny, h.lt:h.lt + loc.nx, :] = a.reshape(loc.res_shape())
    return out


COST_L2, COST_L1, COST_FIRM = 0, 1, 2


def cost_sum(loc, buf_ext, kind, p0=0.0, p1=0.0):
    out = np.zeros(loc.nbatch, np.float64)
    b = np.ascontiguousarray(buf_ext)
    if b.dtype == np.float64:
        lib().pvo_cost_sum_f64(C.byref(loc), _p(b), kind, p0, p1, _p(out))
    else:
        lib().pvo_cost_sum(C.byref(loc), _p(_c(b, np.float32)), kind, p0, p1, _p(out))
    return out


def adaptive_timescale(state, energies, base_max, base_min, tau_factor, growth_factor):
    st = _c(state, np.float64).copy()
    lib().pvo_adaptive_timescale(st.shape[0], base_max, base_min, tau_factor, growth_factor,
                                 _p(_c(energies, np.float64)), _p(st))
    return st


def hebbian_dw(pre, post, nxp, nyp, pre_ext, post_ext, dw_max=1.0, f64=False):
    nk = kernel_index_table(pre, post)[1]
    if f64:
        dw = np.zeros((nk, nyp, nxp, post.nf), np.float64)
        rc = lib().pvo_hebbian_dw_f64(C.byref(pre), C.byref(post), nxp, nyp, dw_max, _p(_c(pre_ext, np.float64)),
                                      _p(_c(post_ext, np.float64)), _p(dw))
    else:
        dw = np.zeros((nk, nyp, nxp, post.nf), np.float32)
        rc = lib().pvo_hebbian_dw(C.byref(pre), C.byref(post), nxp, nyp, dw_max, _p(_c(pre_ext, np.float32)),
                                  _p(_c(post_ext, np.float32)), _p(dw))
    _check(rc, "hebbian_dw")
    return dw


def hebbian_dw_normalized(pre, post, nxp, nyp, pre_ext, post_ext, rule=0, dw_max=1.0):
    """HebbianUpdater's dW with normalizeDw: the accumulated dW of each kernel item divided by the
    number of its contributions, 0 where there were none (HebbianUpdater.cpp:787-812).  rule 0:
    dWMax * pre * post; rule 1: pre - post (the reference's PlasticConnTest updater)."""
    nk = kernel_index_table(pre, post)[1]
    dw = np.zeros((nk, nyp, nxp, post.nf), np.float32)
    counts = np.zeros(dw.shape, np.int64)
    rc = lib().pvo_hebbian_dw_rule(C.byref(pre), C.byref(post), nxp, nyp, rule, dw_max,
                                   _p(_c(pre_ext, np.float32)), _p(_c(post_ext, np.float32)), _p(dw), _p(counts))
    _check(rc, "hebbian_dw_rule")
    out = np.zeros_like(dw)
    nz = counts != 0
    out[nz] = dw[nz] / counts[nz].astype(np.float32)
    return out, counts


def lca_params(**kw):
    """LcaParams with the LCA-tutorial defaults; keyword overrides."""
    d = dict(nbatch=1, inNx=32, inNy=32, inNf=1, v1Nx=16, v1Ny=16, v1Nf=64, nxp=8, nyp=8,
             VThresh=0.1, AMin=0.0, AMax=float("inf"), AShift=0.1, VWidth=0.0, tau=100.0,
             selfInteract=1, errScale=1.0, adaptive=0, baseMax=1.0, baseMin=1.0, tauFactor=1.0,
             growthFactor=0.0, dtFixed=1.0, displayPeriod=0, l2Coeff=0.5, costKind=COST_L1,
             costThresh=0.0, costWidth=0.0, costCoeff=None)
    d.update(kw)
    if d["costCoeff"] is None:
        d["costCoeff"] = float(np.float32(d["VThresh"]))
    return LcaParams(**d)


def lca_run(p, w, frames, num_steps, v1_init, f64=False, threads=1, want_recon=True):
    """Returns (v1_final, a_final, recon[steps][nb]..., energy[steps][nb])."""
    dt = np.float64 if f64 else np.float32
    w = _c(w, dt)
    frames = _c(frames, dt)
    nframes = frames.shape[0]
    v = _c(v1_init, dt).copy()
    nb = p.nbatch
    recon = np.zeros((num_steps, nb, p.inNy, p.inNx, p.inNf), dt) if want_recon else None
    energy = np.zeros((num_steps, nb), np.float64)
    a_final = np.zeros((nb, p.v1Ny, p.v1Nx, p.v1Nf), dt)
    fn = lib().pvo_lca_run_f64 if f64 else lib().pvo_lca_run
    rc = fn(C.byref(p), _p(w), _p(frames), nframes, num_steps, _p(v), _p(recon), _p(energy), _p(a_final), threads)
    _check(rc, "lca_run")
    return v, a_final, recon, energy
