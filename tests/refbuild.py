"""Locates (and builds on demand) oracle/_ref/libpvref.so: pieces of the reference CPU
path compiled from the reference source tree.  Only available where the reference
tree is mounted; tests that need it skip elsewhere."""
import ctypes as C
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
def reference_root():
    """The reference source tree: OPENPV_REFERENCE, else the root the oracle's build recipe
    (oracle/Makefile.ref) is configured to read."""
    env = os.environ.get("OPENPV_REFERENCE")
    if env:
        return env
    try:
        r = subprocess.run(["make", "-s", "-f", os.path.join(ROOT, "oracle", "Makefile.ref"), "print-ref"],
                           capture_output=True, text=True, timeout=30)
        return r.stdout.strip()
    except (OSError, subprocess.SubprocessError):
        return ""


REF_ROOT = reference_root()
LIB = os.path.join(ROOT, "oracle", "_ref", "libpvref.so")


class RefLoc(C.Structure):
    _fields_ = [("nbatch", C.c_int), ("nx", C.c_int), ("ny", C.c_int), ("nf", C.c_int),
                ("lt", C.c_int), ("rt", C.c_int), ("dn", C.c_int), ("up", C.c_int)]

    @staticmethod
    def of(loc):
        h = loc.halo
        return RefLoc(loc.nbatch, loc.nx, loc.ny, loc.nf, h.lt, h.rt, h.dn, h.up)


_lib = None


def available():
    return os.path.exists(LIB) or os.path.isdir(os.path.join(REF_ROOT, "src", "components"))


def lib():
    global _lib
    if _lib is None:
        if os.path.isdir(os.path.join(REF_ROOT, "src")):
            subprocess.check_call(["make", "-s", "-f", os.path.join(ROOT, "oracle", "Makefile.ref"),
                                   f"REF={REF_ROOT}"])
        _lib = C.CDLL(LIB)
        vp = C.c_void_p
        lp = C.POINTER(RefLoc)
        _lib.pvr_patch_geometry.restype = C.c_int
        _lib.pvr_patch_geometry.argtypes = [lp, lp, C.c_int, C.c_int] + [vp] * 7
        _lib.pvr_lca_update.restype = None
        _lib.pvr_lca_update.argtypes = [lp, C.c_int, vp, C.c_float, vp, vp, vp]
        _lib.pvr_momentum_lca_update.restype = None
        _lib.pvr_momentum_lca_update.argtypes = [lp, C.c_int, C.c_float, vp, C.c_float, vp, vp, vp, vp]
        _lib.pvr_ista_update.restype = None
        _lib.pvr_ista_update.argtypes = [lp, C.c_float, vp, C.c_float, vp, vp, vp]
        _lib.pvr_gsyn_accumulate.restype = None
        _lib.pvr_gsyn_accumulate.argtypes = [C.c_int, C.c_int, vp, vp, vp]
        _lib.pvr_apply_vertices.restype = None
        _lib.pvr_apply_vertices.argtypes = [lp, C.c_int, vp, vp, vp, vp, vp]
        _lib.pvr_deliver_pre.restype = C.c_int
        _lib.pvr_deliver_pre.argtypes = [lp, lp, C.c_int, C.c_int, vp, vp, vp, vp, vp]
        _lib.pvr_deliver_post.restype = C.c_int
        _lib.pvr_deliver_post.argtypes = [lp, lp, C.c_int, C.c_int, vp, vp, vp]
        _lib.pvr_lif_update.restype = C.c_int
        _lib.pvr_lif_update.argtypes = [C.c_char, lp, vp, C.c_float, C.c_float] + [vp] * 8
        _lib.pvr_taus_init.restype = None
        _lib.pvr_taus_init.argtypes = [vp, C.c_size_t, C.c_uint]
        _lib.pvr_taus_next.restype = None
        _lib.pvr_taus_next.argtypes = [vp, C.c_size_t]
        _lib.pvr_cost.restype = C.c_double
        _lib.pvr_cost.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double]
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def patch_geometry(pre, post, nxp, nyp):
    n = pre.num_ext
    nxs = np.zeros(n, np.uint16)
    nys = np.zeros(n, np.uint16)
    off = np.zeros(n, np.uint32)
    gs = np.zeros(n, np.int64)
    ap = np.zeros(n, np.int64)
    us = np.zeros(n, np.int64)
    nkx = pre.nx // post.nx if pre.nx > post.nx else 1
    nky = pre.ny // post.ny if pre.ny > post.ny else 1
    ti = np.zeros(nkx * nky * pre.nf * nxp * nyp * post.nf, np.int32)
    rc = lib().pvr_patch_geometry(C.byref(RefLoc.of(pre)), C.byref(RefLoc.of(post)), nxp, nyp, _p(nxs), _p(nys),
                                  _p(off), _p(gs), _p(ap), _p(us), _p(ti))
    if rc != 0:
        raise ValueError("reference rejected geometry")
    return nxs, nys, off, gs, ap, us, ti


def lca_update(loc, g, a_ext, v, dt_adapt, tau, self_interact=True):
    v = np.ascontiguousarray(v, np.float32).copy()
    lib().pvr_lca_update(C.byref(RefLoc.of(loc)), int(self_interact),
                         _p(np.ascontiguousarray(dt_adapt, np.float64)), tau,
                         _p(np.ascontiguousarray(g, np.float32)), _p(np.ascontiguousarray(a_ext, np.float32)), _p(v))
    return v


def momentum_lca_update(loc, g, a_ext, prev_drive, v, dt_adapt, tau, momentum_rate, self_interact=True):
    v = np.ascontiguousarray(v, np.float32).copy()
    pd = np.ascontiguousarray(prev_drive, np.float32).copy()
    lib().pvr_momentum_lca_update(C.byref(RefLoc.of(loc)), int(self_interact), momentum_rate,
                                  _p(np.ascontiguousarray(dt_adapt, np.float64)), tau,
                                  _p(np.ascontiguousarray(g, np.float32)), _p(np.ascontiguousarray(a_ext, np.float32)),
                                  _p(pd), _p(v))
    return v, pd


def ista_update(loc, g, a_ext, v, dt_adapt, tau, vthresh):
    v = np.ascontiguousarray(v, np.float32).copy()
    lib().pvr_ista_update(C.byref(RefLoc.of(loc)), vthresh, _p(np.ascontiguousarray(dt_adapt, np.float64)), tau,
                          _p(np.ascontiguousarray(g, np.float32)), _p(np.ascontiguousarray(a_ext, np.float32)), _p(v))
    return v


def gsyn_accumulate(gsyn, coeffs):
    g = np.ascontiguousarray(gsyn, np.float32)
    out = np.zeros(g.shape[1:], np.float32)
    lib().pvr_gsyn_accumulate(g[0].size, g.shape[0], _p(np.ascontiguousarray(coeffs, np.float32)), _p(g), _p(out))
    return out


def apply_vertices(loc, v, vV, vA, slopes):
    a = np.zeros(loc.ext_shape(), np.float32)
    lib().pvr_apply_vertices(C.byref(RefLoc.of(loc)), len(vV), _p(np.ascontiguousarray(vV, np.float32)),
                             _p(np.ascontiguousarray(vA, np.float32)), _p(np.ascontiguousarray(slopes, np.float32)),
                             _p(np.ascontiguousarray(v, np.float32)), _p(a))
    return a


def cost(kind, p0, p1, x):
    return lib().pvr_cost(kind, p0, p1, float(x))


def deliver_pre(pre, post, nxp, nyp, w, a_ext=None, entries=None, num_active=None, gsyn=None):
    """The reference's PresynapticPerspectiveConvolveDelivery::deliver, single-threaded."""
    g = np.zeros(post.res_shape(), np.float32) if gsyn is None else gsyn
    w = np.ascontiguousarray(w, np.float32)
    if entries is not None:
        e = np.ascontiguousarray(entries)
        n = np.ascontiguousarray(num_active, np.int64)
        rc = lib().pvr_deliver_pre(C.byref(RefLoc.of(pre)), C.byref(RefLoc.of(post)), nxp, nyp, _p(w), _p(e), _p(n),
                                   None, _p(g))
    else:
        a = np.ascontiguousarray(a_ext, np.float32)
        rc = lib().pvr_deliver_pre(C.byref(RefLoc.of(pre)), C.byref(RefLoc.of(post)), nxp, nyp, _p(w), None, None,
                                   _p(a), _p(g))
    if rc != 0:
        raise ValueError("reference rejected geometry")
    return g


def deliver_post(src, tgt, nxp_post, nyp_post, w_post, a_ext, gsyn=None):
    """The reference's PostsynapticPerspectiveConvolveDelivery::deliver, single-threaded."""
    g = np.zeros(tgt.res_shape(), np.float32) if gsyn is None else gsyn
    rc = lib().pvr_deliver_post(C.byref(RefLoc.of(src)), C.byref(RefLoc.of(tgt)), nxp_post, nyp_post,
                                _p(np.ascontiguousarray(w_post, np.float32)), _p(np.ascontiguousarray(a_ext, np.float32)),
                                _p(g))
    if rc != 0:
        raise ValueError("reference rejected geometry")
    return g


def taus_init(count, seed, dtype):
    st = np.zeros(count, dtype)
    lib().pvr_taus_init(_p(st), count, seed)
    return st


def taus_next(st):
    st = st.copy()
    lib().pvr_taus_next(_p(st), st.size)
    return st


def lif_update(method, loc, params, dt, state, gsyn_head, a_ext, sim_time=0.0):
    """The reference's LIFActivityComponent::updateActivity{Arma,Beginning,Original}."""
    st = {k: v.copy() for k, v in state.items()}
    a = np.ascontiguousarray(a_ext, dtype=np.float32).copy()
    rc = lib().pvr_lif_update(method.encode()[:1], C.byref(RefLoc.of(loc)), _p(np.ascontiguousarray(params, np.float32)),
                              sim_time, dt, _p(st["rnd"]), _p(st["V"]), _p(st["Vth"]), _p(st["GE"]), _p(st["GI"]),
                              _p(st["GIB"]), _p(np.ascontiguousarray(gsyn_head, np.float32)), _p(a))
    assert rc == 0
    return st, a
