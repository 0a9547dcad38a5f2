"""ctypes binding of libpvgpu.so (include/pvgpu.h).

This is the same C ABI a reference-side adapter binds; the Python tests and bench
call through it exactly as a C++ host would.  Device memory and streams come from
PyTorch (plumbing only): tensors are passed as raw device pointers and the current
torch stream as the cudaStream_t.

The library must exist: importing this module on a machine without libpvgpu.so
raises, there is no CPU fallback.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libpvgpu.so")

PVGPU_OK = 0
PVGPU_ERR_BAD_ARG = 1
PVGPU_ERR_TIMEOUT = 4
PVGPU_ERR_UNSUPPORTED_SHAPE = 5
DELIVER_FAST = 0
DELIVER_REFERENCE_ORDER = 1
COST_L2, COST_L1, COST_FIRM = 0, 1, 2


class PvgpuError(RuntimeError):
    def __init__(self, status, what):
        self.status = status
        super().__init__(f"{what}: {status_string(status)} ({last_error()})")


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


class ConnDesc(C.Structure):
    _fields_ = [("pre", Loc), ("post", Loc), ("nxp", C.c_int), ("nyp", C.c_int), ("dt_factor", C.c_float)]


class LcaLayerDesc(C.Structure):
    _fields_ = [("loc", Loc), ("numChannels", C.c_int), ("coeffs", C.c_float * 4), ("selfInteract", C.c_int),
                ("tau", C.c_float), ("VThresh", C.c_float), ("AMin", C.c_float), ("AMax", C.c_float),
                ("AShift", C.c_float), ("VWidth", C.c_float)]


class LcaSolverDesc(C.Structure):
    _fields_ = [("nbatch", C.c_int), ("inNx", C.c_int), ("inNy", C.c_int), ("inNf", C.c_int),
                ("v1Nx", C.c_int), ("v1Ny", C.c_int), ("v1Nf", C.c_int), ("nxp", C.c_int),
                ("VThresh", C.c_float), ("AMin", C.c_float), ("AMax", C.c_float), ("AShift", C.c_float),
                ("VWidth", C.c_float), ("tau", C.c_float), ("dt", C.c_float), ("selfInteract", C.c_int)]


class LcaGradDesc(C.Structure):
    _fields_ = [("nbatch", C.c_int), ("inNx", C.c_int), ("inNy", C.c_int), ("inNf", C.c_int), ("v1Nx", C.c_int),
                ("v1Ny", C.c_int), ("v1Nf", C.c_int), ("nxp", C.c_int), ("VThresh", C.c_float), ("lambda1", C.c_float),
                ("tau", C.c_float), ("dt", C.c_float), ("steps", C.c_int), ("checkpointEvery", C.c_int)]


class LcaSchedule(C.Structure):
    _fields_ = [("chains", C.c_int), ("reconCtas", C.c_int), ("postCtas", C.c_int), ("programmatic", C.c_int),
                ("fused", C.c_int)]


LCA_FP32 = 0
LCA_BF16 = 1

_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with openpv_gb300.build.build() "
                               "(there is no CPU fallback)")
        _lib = C.CDLL(LIB_PATH)
        _declare(_lib)
    return _lib


def _declare(L):
    vp, i, f, d, i64, sz = C.c_void_p, C.c_int, C.c_float, C.c_double, C.c_int64, C.c_size_t
    cp = C.POINTER(ConnDesc)
    lp = C.POINTER(Loc)
    sig = {
        "pvgpu_version": (C.c_char_p, []),
        "pvgpu_status_string": (C.c_char_p, [i]),
        "pvgpu_last_error": (C.c_char_p, []),
        "pvgpu_compact_scratch_bytes": (sz, [i, i64]),
        "pvgpu_compact_active": (i, [vp, i, i64, vp, vp, vp, sz, vp]),
        "pvgpu_compact_active_noalloc": (i, [vp, i, i64, vp, vp, vp]),
        "pvgpu_deliver_pre": (i, [cp, vp, vp, vp, vp, vp, i, vp]),
        "pvgpu_deliver_post": (i, [cp, vp, vp, vp, i, vp]),
        "pvgpu_transpose_weights": (i, [cp, vp, vp, vp]),
        "pvgpu_gsyn_accumulate": (i, [i64, i, vp, vp, vp, vp]),
        "pvgpu_lca_update": (i, [lp, i, vp, f, vp, vp, vp, vp]),
        "pvgpu_ann_activity": (i, [lp, vp, f, f, f, f, f, vp, vp]),
        "pvgpu_ann_vertices": (i, [lp, i, vp, vp, vp, vp, vp, vp]),
        "pvgpu_lca_layer_update": (i, [C.POINTER(LcaLayerDesc), vp, vp, vp, vp, vp]),
        "pvgpu_cost_sum": (i, [lp, vp, i, d, d, vp, vp]),
        "pvgpu_hebbian_dw": (i, [cp, f, vp, vp, vp, vp]),
        "pvgpu_tc_gemm_bf16": (i, [vp, vp, vp, i, i, i, vp, vp]),
        "pvgpu_tc_gemm_bf16_kn": (i, [vp, vp, vp, i, i, i, vp, vp]),
        "pvgpu_tc_gemm_bf16_atmem": (i, [vp, vp, vp, i, i, i, vp, vp]),
        "pvgpu_lca_solver_create": (i, [C.POINTER(LcaSolverDesc), C.POINTER(vp)]),
        "pvgpu_lca_solver_destroy": (i, [vp]),
        "pvgpu_lca_solver_set_weights": (i, [vp, vp, vp]),
        "pvgpu_lca_solver_reset": (i, [vp, vp, vp]),
        "pvgpu_lca_solver_run": (i, [vp, vp, i, i, i, vp]),
        "pvgpu_lca_solver_energy": (i, [vp, vp, d, i, d, d, d, vp, vp]),
        "pvgpu_lca_solver_state": (i, [vp, vp, vp, vp]),
        "pvgpu_lca_solver_error_flag": (i, [vp, C.POINTER(i)]),
        "pvgpu_lca_solver_profile_begin": (i, [vp, i]),
        "pvgpu_lca_solver_profile_end": (i, [vp, C.POINTER(d), C.POINTER(d), C.POINTER(i)]),
        "pvgpu_lca_solver_autotune": (i, [vp, vp, i, vp]),
        "pvgpu_lca_solver_plan_info": (i, [vp, C.POINTER(i)]),
        "pvgpu_lca_solver_set_schedule": (i, [vp, C.POINTER(LcaSchedule)]),
        "pvgpu_lca_solver_fused_plan_info": (i, [vp, C.POINTER(i)]),
        "pvgpu_lca_solver_set_fused_plan": (i, [vp, i, i, i]),
        "pvgpu_lca_solver_profile_end_fused": (i, [vp, C.POINTER(d), C.POINTER(d), C.POINTER(d), C.POINTER(i),
                                                   C.POINTER(i)]),
        "pvgpu_lca_solver_get_schedule": (i, [vp, C.POINTER(LcaSchedule)]),
        "pvgpu_deliver_ident": (i, [lp, lp, vp, vp, vp, vp, vp]),
        "pvgpu_momentum_lca_update": (i, [lp, i, f, vp, f, vp, vp, vp, vp, vp]),
        "pvgpu_ista_update": (i, [lp, f, vp, f, vp, vp, vp, vp]),
        "pvgpu_err_scale": (i, [i64, f, vp, vp]),
        "pvgpu_deliver_tc_workspace_bytes": (sz, [cp]),
        "pvgpu_deliver_post_tc": (i, [cp, vp, vp, vp, vp, sz, vp]),
        "pvgpu_deliver_pre_tc": (i, [cp, vp, vp, vp, vp, sz, vp]),
        "pvgpu_deliver_tc_check_error": (i, []),
        "pvgpu_lif_update": (i, [lp, C.c_char, vp, f, vp, vp, vp, vp, vp, vp, vp, vp, vp]),
        "pvgpu_pvp_sparse_frames": (i, [lp, vp, vp, vp, vp, vp]),
        "pvgpu_momentum_factors": (i, [C.c_char, f, f, f, C.POINTER(f), C.POINTER(f)]),
        "pvgpu_momentum_update_weights": (i, [i64, f, f, vp, vp, vp, vp]),
        "pvgpu_pvp_dense_frames": (i, [lp, vp, vp, vp]),
        "pvgpu_pvp_scatter_sparse": (i, [lp, vp, vp, vp, vp, vp]),
        "pvgpu_taus_init": (i, [vp, i64, C.c_uint32, vp]),
        "pvgpu_selftest_wait_expiry": (i, [C.c_uint64, C.POINTER(C.c_longlong), vp]),
        "pvgpu_lca_grad_create": (i, [C.POINTER(LcaGradDesc), C.POINTER(vp)]),
        "pvgpu_lca_grad_destroy": (i, [vp]),
        "pvgpu_lca_grad_run": (i, [vp, vp, vp, vp, vp, vp]),
        "pvgpu_lca_grad_info": (i, [vp, C.POINTER(i)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args


def exported_symbols(header="pvgpu.h", prefix="pvgpu"):
    """Names of the <prefix>_* functions declared in include/<header>."""
    import re
    hdr = os.path.join(os.path.dirname(HERE), "include", header)
    txt = open(hdr).read()
    return sorted(set(re.findall(r"\b(" + prefix + r"_[a-z0-9_]+)\s*\(", txt)))


def version():
    return lib().pvgpu_version().decode()


def status_string(s):
    return lib().pvgpu_status_string(s).decode()


def last_error():
    return lib().pvgpu_last_error().decode()


def check(status, what):
    if status != PVGPU_OK:
        raise PvgpuError(status, what)


# ---- torch plumbing ---------------------------------------------------------------------

def _ptr(t):
    if t is None:
        return None
    assert t.is_cuda and t.is_contiguous(), "device tensors must be contiguous CUDA tensors"
    return C.c_void_p(t.data_ptr())


def _stream(stream=None):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


def conn_desc(pre, post, nxp, nyp, dt_factor=1.0):
    return ConnDesc(pre, post, nxp, nyp, dt_factor)


def compact_active(a_ext, nbatch, num_ext, entries, num_active, scratch=None, stream=None):
    """entries: uint8/int64 tensor viewed as [nbatch][num_ext] {u32 index, f32 value}."""
    import torch
    need = lib().pvgpu_compact_scratch_bytes(nbatch, num_ext)
    if scratch is None:
        scratch = torch.empty(max(need, 1), dtype=torch.uint8, device=a_ext.device)
    check(lib().pvgpu_compact_active(_ptr(a_ext), nbatch, num_ext, _ptr(entries), _ptr(num_active), _ptr(scratch),
                                     scratch.numel() * scratch.element_size(), _stream(stream)), "compact_active")


def compact_active_noalloc(a_ext, nbatch, num_ext, entries, num_active, stream=None):
    """Compaction that allocates nothing (fixed scratch inside the library); see include/pvgpu.h."""
    check(lib().pvgpu_compact_active_noalloc(_ptr(a_ext), nbatch, num_ext, _ptr(entries), _ptr(num_active),
                                             _stream(stream)), "compact_active_noalloc")


def deliver_pre(conn, weights, gsyn, entries=None, num_active=None, a_ext=None, mode=DELIVER_FAST, stream=None):
    check(lib().pvgpu_deliver_pre(C.byref(conn), _ptr(entries), _ptr(num_active), _ptr(a_ext), _ptr(weights),
                                  _ptr(gsyn), mode, _stream(stream)), "deliver_pre")


def deliver_post(conn, a_ext, post_weights, gsyn, mode=DELIVER_FAST, stream=None):
    check(lib().pvgpu_deliver_post(C.byref(conn), _ptr(a_ext), _ptr(post_weights), _ptr(gsyn), mode,
                                   _stream(stream)), "deliver_post")


def deliver_tc_workspace_bytes(conn):
    return int(lib().pvgpu_deliver_tc_workspace_bytes(C.byref(conn)))


def _ws_nbytes(workspace):
    return workspace.numel() * workspace.element_size()


def deliver_post_tc(conn, a_ext, post_weights, gsyn, workspace, stream=None):
    """Post-perspective delivery on the tensor cores (split-TF32); see include/pvgpu.h."""
    check(lib().pvgpu_deliver_post_tc(C.byref(conn), _ptr(a_ext), _ptr(post_weights), _ptr(gsyn), _ptr(workspace),
                                      _ws_nbytes(workspace), _stream(stream)), "deliver_post_tc")


def deliver_pre_tc(conn, a_ext, weights, gsyn, workspace, stream=None):
    """Pre-perspective delivery from the dense activity on the tensor cores (split-TF32)."""
    check(lib().pvgpu_deliver_pre_tc(C.byref(conn), _ptr(a_ext), _ptr(weights), _ptr(gsyn), _ptr(workspace),
                                     _ws_nbytes(workspace), _stream(stream)), "deliver_pre_tc")


LIF_FIELDS = ("Vrest", "Vexc", "Vinh", "VinhB", "VthRest", "tau", "tauVth", "deltaVth", "deltaGIB",
              "noiseAmpE", "noiseAmpI", "noiseAmpIB", "noiseFreqE", "noiseFreqI", "noiseFreqIB", "tauE", "tauI", "tauIB")


class LifParams(C.Structure):
    """pvgpu_lif_params (LIFParams, components/LIFActivityComponent.hpp:22-45)."""
    _fields_ = [(n, C.c_float) for n in LIF_FIELDS]
    DEFAULTS = dict(Vrest=-70.0, Vexc=0.0, Vinh=-75.0, VinhB=-90.0, VthRest=-55.0, tau=20.0, tauVth=10.0,
                    deltaVth=5.0, deltaGIB=1.0, noiseAmpE=0.0, noiseAmpI=0.0, noiseAmpIB=0.0, noiseFreqE=250.0,
                    noiseFreqI=250.0, noiseFreqIB=250.0, tauE=1.0, tauI=5.0, tauIB=10.0)

    @staticmethod
    def make(**kw):
        d = dict(LifParams.DEFAULTS, **kw)
        return LifParams(*[d[n] for n in LIF_FIELDS])


def lif_update(loc, method, params, dt, rnd, v, vth, ge, gi, gib, gsyn_head, a_ext, stream=None):
    """LIF step on the device; rnd is a [n, 4] uint32 (or int32) tensor of {s0, s1, s2, s3}."""
    check(lib().pvgpu_lif_update(C.byref(loc), method.encode()[:1], C.byref(params), dt, _ptr(rnd), _ptr(v),
                                 _ptr(vth), _ptr(ge), _ptr(gi), _ptr(gib), _ptr(gsyn_head), _ptr(a_ext),
                                 _stream(stream)), "lif_update")


def taus_init(state, count, seed, stream=None):
    check(lib().pvgpu_taus_init(_ptr(state), count, seed, _stream(stream)), "taus_init")


def momentum_factors(method, tau, decay=0.0, dw_max=1.0):
    a, b = C.c_float(), C.c_float()
    check(lib().pvgpu_momentum_factors(method.encode()[:1], tau, decay, dw_max, C.byref(a), C.byref(b)),
          "momentum_factors")
    return a.value, b.value


def momentum_update_weights(dw, prev_dw, w, dw_factor, w_factor, stream=None):
    check(lib().pvgpu_momentum_update_weights(dw.numel(), dw_factor, w_factor, _ptr(dw), _ptr(prev_dw), _ptr(w),
                                              _stream(stream)), "momentum_update_weights")


def deliver_tc_check_error():
    return int(lib().pvgpu_deliver_tc_check_error())


def transpose_weights(conn, w_pre, w_post, stream=None):
    check(lib().pvgpu_transpose_weights(C.byref(conn), _ptr(w_pre), _ptr(w_post), _stream(stream)), "transpose")


def gsyn_accumulate(n, coeffs, gsyn, g, stream=None):
    c = (C.c_float * len(coeffs))(*coeffs)
    check(lib().pvgpu_gsyn_accumulate(n, len(coeffs), c, _ptr(gsyn), _ptr(g), _stream(stream)), "gsyn_accumulate")


def lca_update(loc, self_interact, dt_adapt, tau, g, a_ext, v, stream=None):
    check(lib().pvgpu_lca_update(C.byref(loc), int(self_interact), _ptr(dt_adapt), tau, _ptr(g), _ptr(a_ext), _ptr(v),
                                 _stream(stream)), "lca_update")


def momentum_lca_update(loc, self_interact, momentum_rate, dt_adapt, tau, g, a_ext, prev_drive, v, stream=None):
    check(lib().pvgpu_momentum_lca_update(C.byref(loc), int(self_interact), momentum_rate, _ptr(dt_adapt), tau,
                                          _ptr(g), _ptr(a_ext), _ptr(prev_drive), _ptr(v), _stream(stream)),
          "momentum_lca_update")


def ista_update(loc, vthresh, dt_adapt, tau, g, a_ext, v, stream=None):
    check(lib().pvgpu_ista_update(C.byref(loc), vthresh, _ptr(dt_adapt), tau, _ptr(g), _ptr(a_ext), _ptr(v),
                                  _stream(stream)), "ista_update")


def ann_activity(loc, v, VThresh, AMin, AMax, AShift, VWidth, a_ext, stream=None):
    check(lib().pvgpu_ann_activity(C.byref(loc), _ptr(v), VThresh, AMin, AMax, AShift, VWidth, _ptr(a_ext),
                                   _stream(stream)), "ann_activity")


def ann_vertices(loc, vertices_v, vertices_a, slopes, v, a_ext, stream=None):
    check(lib().pvgpu_ann_vertices(C.byref(loc), vertices_v.numel(), _ptr(vertices_v), _ptr(vertices_a), _ptr(slopes),
                                   _ptr(v), _ptr(a_ext), _stream(stream)), "ann_vertices")


def lca_layer_update(desc, gsyn, dt_adapt, v, a_ext, stream=None):
    check(lib().pvgpu_lca_layer_update(C.byref(desc), _ptr(gsyn), _ptr(dt_adapt), _ptr(v), _ptr(a_ext),
                                       _stream(stream)), "lca_layer_update")


def cost_sum(loc, buf_ext, kind, p0, p1, out, stream=None):
    check(lib().pvgpu_cost_sum(C.byref(loc), _ptr(buf_ext), kind, p0, p1, _ptr(out), _stream(stream)), "cost_sum")


def hebbian_dw(conn, dw_max, pre_ext, post_ext, dw, stream=None):
    check(lib().pvgpu_hebbian_dw(C.byref(conn), dw_max, _ptr(pre_ext), _ptr(post_ext), _ptr(dw), _stream(stream)),
          "hebbian_dw")


def selftest_wait_expiry(limit_ns, stream=None):
    """(status, expired, ns waited) of a bounded device wait that nothing satisfies."""
    out = (C.c_longlong * 2)()
    st = lib().pvgpu_selftest_wait_expiry(int(limit_ns), out, _stream(stream))
    return st, int(out[0]), int(out[1])


def tc_gemm_bf16(A, B, C, M, N, K, err, stream=None):
    check(lib().pvgpu_tc_gemm_bf16(_ptr(A), _ptr(B), _ptr(C), M, N, K, _ptr(err), _stream(stream)), "tc_gemm_bf16")


def tc_gemm_bf16_atmem(A, B, C, M, N, K, err, stream=None):
    """C = A @ B^T with A read by the MMA from tensor memory."""
    check(lib().pvgpu_tc_gemm_bf16_atmem(_ptr(A), _ptr(B), _ptr(C), M, N, K, _ptr(err), _stream(stream)),
          "tc_gemm_bf16_atmem")


def tc_gemm_bf16_kn(A, B, C, M, N, K, err, stream=None):
    """C = A @ B with B [K][N] read as the MN-major tcgen05 operand."""
    check(lib().pvgpu_tc_gemm_bf16_kn(_ptr(A), _ptr(B), _ptr(C), M, N, K, _ptr(err), _stream(stream)),
          "tc_gemm_bf16_kn")


ENTRY_DTYPE = np.dtype([("index", np.uint32), ("value", np.float32)])


class LcaSolver:
    """The batched LCA module (pvgpu_lca_solver_*): input -> error <-> V1, two fused kernels per
    timestep.  Inputs, weights and state are device tensors in the OpenPV layouts."""

    def __init__(self, nbatch, in_shape, v1_shape, nxp, VThresh, AMin=0.0, AMax=float("inf"), AShift=None,
                 VWidth=0.0, tau=100.0, dt=1.0, self_interact=True):
        iny, inx, inf_ = in_shape
        vy, vx, vf = v1_shape
        self.desc = LcaSolverDesc(nbatch, inx, iny, inf_, vx, vy, vf, nxp, VThresh, AMin, AMax,
                                  VThresh if AShift is None else AShift, VWidth, tau, dt, int(self_interact))
        h = C.c_void_p()
        check(lib().pvgpu_lca_solver_create(C.byref(self.desc), C.byref(h)), "lca_solver_create")
        self.h = h
        self.nbatch = nbatch
        self.v1_shape = (nbatch, vy, vx, vf)

    def close(self):
        if self.h:
            lib().pvgpu_lca_solver_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_weights(self, w, stream=None):
        check(lib().pvgpu_lca_solver_set_weights(self.h, _ptr(w), _stream(stream)), "lca_solver_set_weights")

    def reset(self, v0=None, stream=None):
        check(lib().pvgpu_lca_solver_reset(self.h, _ptr(v0), _stream(stream)), "lca_solver_reset")

    def run(self, x, steps, x3_steps=0, precision=LCA_BF16, stream=None):
        check(lib().pvgpu_lca_solver_run(self.h, _ptr(x), steps, x3_steps, precision, _stream(stream)),
              "lca_solver_run")

    def energy(self, x, out, l2_coeff=0.5, cost_kind=COST_L1, cost_thresh=0.0, cost_width=0.0, cost_coeff=None,
               stream=None):
        cc = float(np.float32(self.desc.VThresh)) if cost_coeff is None else cost_coeff
        check(lib().pvgpu_lca_solver_energy(self.h, _ptr(x), l2_coeff, cost_kind, cost_thresh, cost_width, cc,
                                            _ptr(out), _stream(stream)), "lca_solver_energy")

    def state(self, v=None, a=None, stream=None):
        check(lib().pvgpu_lca_solver_state(self.h, _ptr(v), _ptr(a), _stream(stream)), "lca_solver_state")

    def autotune(self, x, trial_steps=6, stream=None):
        """Pick the fastest kernel shapes for this geometry (state undefined afterwards: reset)."""
        check(lib().pvgpu_lca_solver_autotune(self.h, _ptr(x), trial_steps, _stream(stream)), "lca_solver_autotune")

    def plan_info(self):
        """{"bf16"|"bf16x3": {FT, nV, nW, stageA, reconStages}} of the shapes in use."""
        out = (C.c_int * 10)()
        check(lib().pvgpu_lca_solver_plan_info(self.h, out), "lca_solver_plan_info")
        keys = ("feature_tile", "v_slots", "w_slots", "a_staged", "recon_stages")
        return {form: dict(zip(keys, out[5 * i:5 * i + 5])) for i, form in enumerate(("bf16", "bf16x3"))}

    def set_schedule(self, chains=1, recon_ctas=0, post_ctas=0, programmatic=True, fused=True):
        """Layout of BF16 runs: fused single-launch timesteps or kernels R + P on every step; one
        chain over the batch or two half-batch chains on parallel graph branches; caps on the
        persistent grids; early launch within a chain."""
        sc = LcaSchedule(chains, recon_ctas, post_ctas, int(programmatic), int(fused))
        check(lib().pvgpu_lca_solver_set_schedule(self.h, C.byref(sc)), "lca_solver_set_schedule")

    def schedule(self):
        sc = LcaSchedule()
        check(lib().pvgpu_lca_solver_get_schedule(self.h, C.byref(sc)), "lca_solver_get_schedule")
        return {"chains": sc.chains, "recon_ctas": sc.reconCtas, "post_ctas": sc.postCtas,
                "programmatic": bool(sc.programmatic), "fused": bool(sc.fused)}

    def fused_plan_info(self):
        """{feature_tile, v_slots, w_slots} of the fused kernel (zeros: no fused form here)."""
        out = (C.c_int * 3)()
        check(lib().pvgpu_lca_solver_fused_plan_info(self.h, out), "lca_solver_fused_plan_info")
        return {"feature_tile": out[0], "v_slots": out[1], "w_slots": out[2]}

    def set_fused_plan(self, feature_tile, v_slots, w_slots=2):
        check(lib().pvgpu_lca_solver_set_fused_plan(self.h, feature_tile, v_slots, w_slots), "lca_solver_set_fused_plan")

    def profile_end_fused(self):
        """(recon ms, post ms, fused ms, steps, fused steps) over the profiled timesteps."""
        r, p, f, n, nf = C.c_double(), C.c_double(), C.c_double(), C.c_int(), C.c_int()
        check(lib().pvgpu_lca_solver_profile_end_fused(self.h, C.byref(r), C.byref(p), C.byref(f), C.byref(n),
                                                       C.byref(nf)), "lca_solver_profile_end_fused")
        return r.value, p.value, f.value, n.value, nf.value

    def profile_begin(self, max_steps):
        check(lib().pvgpu_lca_solver_profile_begin(self.h, max_steps), "lca_solver_profile_begin")

    def profile_end(self):
        """(recon ms, post ms, steps) summed over the profiled timesteps."""
        r, p, n = C.c_double(), C.c_double(), C.c_int()
        check(lib().pvgpu_lca_solver_profile_end(self.h, C.byref(r), C.byref(p), C.byref(n)), "lca_solver_profile_end")
        return r.value, p.value, n.value

    def error_flag(self):
        f = C.c_int(0)
        check(lib().pvgpu_lca_solver_error_flag(self.h, C.byref(f)), "lca_solver_error_flag")
        return f.value


class LcaGrad:
    """dL/dW of unrolled LCA (pvgpu_lca_grad_*): L = 0.5 ||x - W^T a_T||^2 + lam ||a_T||_1 after
    `steps` timesteps from V = 0, checkpointed every `checkpoint_every`; device tensors in the
    OpenPV layouts (W [F][P][P][C], x [nb][ny][nx][C])."""

    def __init__(self, nbatch, in_shape, v1_shape, nxp, VThresh, lam, steps, checkpoint_every=10, tau=100.0,
                 dt=1.0):
        iny, inx, inf_ = in_shape
        vy, vx, vf = v1_shape
        self.desc = LcaGradDesc(nbatch, inx, iny, inf_, vx, vy, vf, nxp, VThresh, lam, tau, dt, steps,
                                checkpoint_every)
        h = C.c_void_p()
        check(lib().pvgpu_lca_grad_create(C.byref(self.desc), C.byref(h)), "lca_grad_create")
        self.h = h

    def close(self):
        if self.h:
            lib().pvgpu_lca_grad_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def run(self, w, x, dw, loss, stream=None):
        check(lib().pvgpu_lca_grad_run(self.h, _ptr(w), _ptr(x), _ptr(dw), _ptr(loss), _stream(stream)),
              "lca_grad_run")

    def emulated_fp32(self):
        f = C.c_int(0)
        check(lib().pvgpu_lca_grad_info(self.h, C.byref(f)), "lca_grad_info")
        return bool(f.value)


# ---- libpvhost.so: the C++ host side (params file -> column of layers and connections) ----------

HOST_LIB_PATH = os.path.join(HERE, "libpvhost.so")
_host = None


def host_lib():
    global _host
    if _host is None:
        lib()  # libpvgpu.so first (libpvhost.so links it)
        if not os.path.exists(HOST_LIB_PATH):
            raise RuntimeError(f"{HOST_LIB_PATH} is missing: build it with openpv_gb300.build.build()")
        _host = C.CDLL(HOST_LIB_PATH)
        vp, i, i64, sz, cs = C.c_void_p, C.c_int, C.c_int64, C.c_size_t, C.c_char_p
        sig = {
            "pvhost_last_error": (cs, []),
            "pvhost_params_dump": (i, [cs, C.c_char_p, sz]),
            "pvhost_column_create": (i, [cs, C.POINTER(vp)]),
            "pvhost_column_destroy": (i, [vp]),
            "pvhost_set_weights": (i, [vp, cs, vp, i64]),
            "pvhost_set_input": (i, [vp, cs, vp, i]),
            "pvhost_set_state": (i, [vp, cs, vp]),
            "pvhost_advance": (i, [vp, i]),
            "pvhost_read_layer": (i, [vp, cs, i, vp, i64]),
            "pvhost_layer_info": (i, [vp, cs, C.POINTER(i)]),
            "pvhost_delivery_keyword": (i, [vp, cs, C.c_char_p, sz]),
            "pvhost_delivery_engine": (i, [vp, cs, C.c_char_p, sz]),
            "pvhost_pvp_writer_open": (i, [cs, i, i, i, i, C.POINTER(vp)]),
            "pvhost_pvp_write_sparse_device": (i, [vp, C.POINTER(Loc), vp, vp, C.c_double, vp]),
            "pvhost_pvp_write_dense_device": (i, [vp, C.POINTER(Loc), vp, C.c_double, vp]),
            "pvhost_pvp_write_sparse_host": (i, [vp, vp, C.c_int32, C.c_double]),
            "pvhost_pvp_write_dense_host": (i, [vp, vp, C.c_double]),
            "pvhost_pvp_writer_close": (i, [vp]),
            "pvhost_pvp_reader_open": (i, [cs, C.POINTER(vp)]),
            "pvhost_pvp_reader_info": (i, [vp, vp, C.POINTER(C.c_double), C.POINTER(i)]),
            "pvhost_pvp_read_dense": (i, [vp, i, vp, C.c_int64, C.POINTER(C.c_double)]),
            "pvhost_pvp_read_sparse": (i, [vp, i, vp, C.c_int64, C.POINTER(C.c_int32), C.POINTER(C.c_double)]),
            "pvhost_pvp_read_to_device": (i, [vp, i, C.POINTER(Loc), vp, vp]),
            "pvhost_pvp_reader_close": (i, [vp]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(_host, name)
            fn.restype = res
            fn.argtypes = args
    return _host


class PvhostError(RuntimeError):
    def __init__(self, status, what):
        self.status = status
        super().__init__(f"{what}: {status_string(status)} ({host_lib().pvhost_last_error().decode()})")


def host_check(status, what):
    if status != PVGPU_OK:
        raise PvhostError(status, what)


def params_dump(text):
    """Canonical listing of a params file's groups and parameters (no GPU needed)."""
    buf = C.create_string_buffer(1 << 20)
    host_check(host_lib().pvhost_params_dump(text.encode(), buf, len(buf)), "params_dump")
    return buf.value.decode()


PVP_HEADER_FIELDS = ("headerSize", "numParams", "fileType", "nx", "ny", "nf", "numRecords", "recordSize", "dataSize",
                     "dataType", "nxProcs", "nyProcs", "nxExtended", "nyExtended", "kx0", "ky0", "nBatch", "nBands")


def pvp_sparse_frames(loc, entries, num_active, out, counts, stream=None):
    check(lib().pvgpu_pvp_sparse_frames(C.byref(loc), _ptr(entries), _ptr(num_active), _ptr(out), _ptr(counts),
                                        _stream(stream)), "pvp_sparse_frames")


def pvp_dense_frames(loc, a_ext, out, stream=None):
    check(lib().pvgpu_pvp_dense_frames(C.byref(loc), _ptr(a_ext), _ptr(out), _stream(stream)), "pvp_dense_frames")


def pvp_scatter_sparse(loc, file_entries, counts, a_ext, bad, stream=None):
    check(lib().pvgpu_pvp_scatter_sparse(C.byref(loc), _ptr(file_entries), _ptr(counts), _ptr(a_ext), _ptr(bad),
                                         _stream(stream)), "pvp_scatter_sparse")


class PvpWriter:
    """A .pvp activity file being written (libpvhost.so)."""

    def __init__(self, path, nx, ny, nf, sparse):
        h = C.c_void_p()
        host_check(host_lib().pvhost_pvp_writer_open(str(path).encode(), nx, ny, nf, int(sparse), C.byref(h)),
                   "pvp_writer_open")
        self.h = h

    def write_sparse_device(self, loc, entries, num_active, t, stream=None):
        host_check(host_lib().pvhost_pvp_write_sparse_device(self.h, C.byref(loc), _ptr(entries), _ptr(num_active),
                                                             float(t), _stream(stream)), "pvp_write_sparse_device")

    def write_dense_device(self, loc, a_ext, t, stream=None):
        host_check(host_lib().pvhost_pvp_write_dense_device(self.h, C.byref(loc), _ptr(a_ext), float(t),
                                                            _stream(stream)), "pvp_write_dense_device")

    def write_sparse(self, indices, values, t):
        e = np.zeros(len(indices), ENTRY_DTYPE)
        e["index"] = indices
        e["value"] = values
        host_check(host_lib().pvhost_pvp_write_sparse_host(self.h, e.ctypes.data_as(C.c_void_p) if len(e) else None,
                                                           len(e), float(t)), "pvp_write_sparse_host")

    def write_dense(self, values, t):
        v = np.ascontiguousarray(values, dtype=np.float32)
        host_check(host_lib().pvhost_pvp_write_dense_host(self.h, v.ctypes.data_as(C.c_void_p), float(t)),
                   "pvp_write_dense_host")

    def close(self):
        if self.h:
            host_check(host_lib().pvhost_pvp_writer_close(self.h), "pvp_writer_close")
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class PvpReader:
    """A .pvp activity file (types 2, 4, 6) read by libpvhost.so."""

    def __init__(self, path):
        h = C.c_void_p()
        host_check(host_lib().pvhost_pvp_reader_open(str(path).encode(), C.byref(h)), "pvp_reader_open")
        self.h = h
        v = (C.c_int32 * 18)()
        t = C.c_double()
        n = C.c_int()
        host_check(host_lib().pvhost_pvp_reader_info(self.h, v, C.byref(t), C.byref(n)), "pvp_reader_info")
        self.header = dict(zip(PVP_HEADER_FIELDS, list(v)))
        self.header["timestamp"] = t.value
        self.num_frames = n.value
        self.shape = (self.header["ny"], self.header["nx"], self.header["nf"])

    def read_dense(self, frame):
        out = np.zeros(self.shape, np.float32)
        t = C.c_double()
        host_check(host_lib().pvhost_pvp_read_dense(self.h, frame, out.ctypes.data_as(C.c_void_p), out.size,
                                                    C.byref(t)), "pvp_read_dense")
        return out, t.value

    def read_sparse(self, frame):
        cap = int(np.prod(self.shape))
        e = np.zeros(cap, ENTRY_DTYPE)
        n = C.c_int32()
        t = C.c_double()
        host_check(host_lib().pvhost_pvp_read_sparse(self.h, frame, e.ctypes.data_as(C.c_void_p), cap, C.byref(n),
                                                     C.byref(t)), "pvp_read_sparse")
        return e[:n.value].copy(), t.value

    def read_to_device(self, first_frame, loc, a_ext, stream=None):
        host_check(host_lib().pvhost_pvp_read_to_device(self.h, first_frame, C.byref(loc), _ptr(a_ext),
                                                        _stream(stream)), "pvp_read_to_device")

    def close(self):
        if self.h:
            host_lib().pvhost_pvp_reader_close(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class Column:
    """An OpenPV column built from params text by libpvhost.so; host numpy arrays in and out."""

    def __init__(self, params_text):
        self.h = C.c_void_p()
        host_check(host_lib().pvhost_column_create(params_text.encode(), C.byref(self.h)), "column_create")

    def __del__(self):
        if getattr(self, "h", None) and _host is not None:
            _host.pvhost_column_destroy(self.h)
            self.h = None

    def layer_info(self, name):
        out = (C.c_int * 6)()
        host_check(host_lib().pvhost_layer_info(self.h, name.encode(), out), "layer_info")
        return dict(zip(("nbatch", "nx", "ny", "nf", "halo", "phase"), out))

    def delivery(self, conn):
        buf = C.create_string_buffer(128)
        host_check(host_lib().pvhost_delivery_keyword(self.h, conn.encode(), buf, len(buf)), "delivery_keyword")
        return buf.value.decode()

    def delivery_engine(self, conn):
        buf = C.create_string_buffer(64)
        host_check(host_lib().pvhost_delivery_engine(self.h, conn.encode(), buf, len(buf)), "delivery_engine")
        return buf.value.decode()

    def set_weights(self, conn, w):
        w = np.ascontiguousarray(w, dtype=np.float32)
        host_check(host_lib().pvhost_set_weights(self.h, conn.encode(), w.ctypes.data_as(C.c_void_p), w.size),
                   "set_weights")

    def set_input(self, layer, frames):
        f = np.ascontiguousarray(frames, dtype=np.float32)
        host_check(host_lib().pvhost_set_input(self.h, layer.encode(), f.ctypes.data_as(C.c_void_p), f.shape[0]),
                   "set_input")

    def set_state(self, layer, v):
        v = np.ascontiguousarray(v, dtype=np.float32)
        host_check(host_lib().pvhost_set_state(self.h, layer.encode(), v.ctypes.data_as(C.c_void_p)), "set_state")

    def advance(self, steps):
        host_check(host_lib().pvhost_advance(self.h, steps), "advance")

    def read(self, layer, which):
        i = self.layer_info(layer)
        out = np.zeros((i["nbatch"], i["ny"], i["nx"], i["nf"]), np.float32)
        host_check(host_lib().pvhost_read_layer(self.h, layer.encode(), 0 if which == "V" else 1,
                                                out.ctypes.data_as(C.c_void_p), out.size), "read_layer")
        return out
