"""The drop-in adapters of adapters/ -- the replacement bodies of the reference's GPU delivery and
update translation units -- compiled unchanged against stand-ins of the framework classes
(tests/adapter_standins; a GPU host need not have the reference's source tree) and driven through the framework's
life cycle (communicateInitInfo, setCudaDevice, allocateDataStructures, copyInitialStateToGPU,
deliver / runKernel) on device buffers, against the oracle (whose loops are pinned bit for bit
to the reference's own compiled code):
  * PresynapticPerspectiveGPUDelivery: sparse and dense presynaptic layers, the channel offset
    into a two-channel GSyn (the other channel untouched), two arbors with their own weights, a
    datastore the host has updated (copied to the device by the adapter), non-shared weights
    refused -- GSyn within 1e-5 of max|GSyn| (FAST delivery order);
  * PostsynapticPerspectiveGPUDelivery: the LCA error -> V1 connection (FP32 kernel) and a
    one-to-one connection (tensor-core entry, workspace allocated by the adapter), within 1e-5;
  * HyPerLCAInternalStateBuffer / ANNActivityBuffer / GSynAccumulator runKernel(): bit for bit."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SI = os.path.join(ROOT, "tests", "adapter_standins")
AD = os.path.join(ROOT, "adapters")


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from openpv_gb300 import build
    build.build()
    from openpv_gb300 import capi
    capi.lib()
    out = os.path.join(SI, "_build")
    os.makedirs(out, exist_ok=True)
    so = os.path.join(out, "libadapters_standin.so")
    pkg = os.path.join(ROOT, "openpv_gb300")
    srcs = [os.path.join(SI, "harness.cpp"),
            os.path.join(AD, "delivery", "PresynapticPerspectiveGPUDelivery.cpp"),
            os.path.join(AD, "delivery", "PostsynapticPerspectiveGPUDelivery.cpp"),
            os.path.join(AD, "components", "HyPerLCAInternalStateBuffer.cu"),
            os.path.join(AD, "components", "ANNActivityBuffer.cu"),
            os.path.join(AD, "components", "GSynAccumulator.cu")]
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    cmd = [nvcc, "-std=c++17", "-shared", "-Xcompiler", "-fPIC", "-gencode", "arch=compute_103a,code=sm_103a",
           "-I", SI, "-I", AD, "-I", os.path.join(ROOT, "include")] + srcs + \
          ["-L", pkg, "-lpvgpu", "-Xlinker", f"-rpath,{pkg}", "-o", so]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    lib = C.CDLL(so)
    lib.standin_last_error.restype = C.c_char_p
    return torch, capi, lib


def l8(loc):
    h = loc.halo
    return (C.c_int * 8)(loc.nbatch, loc.nx, loc.ny, loc.nf, h.lt, h.rt, h.dn, h.up)


def ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def stream(torch):
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def OL(O, loc):
    return O.Loc.make(loc.nbatch, loc.nx, loc.ny, loc.nf, loc.halo.lt, loc.halo.dn)


def sparse_activity(rng, loc, p):
    a = np.zeros(loc.ext_shape(), np.float32)
    h = loc.halo
    a[:, h.up:h.up + loc.ny, h.lt:h.lt + loc.nx, :] = (rng.random(loc.res_shape()) < p) * rng.uniform(0.1, 1.0,
                                                                                                  loc.res_shape())
    return a


def run_pre(env, oracle, pre, post, nxp, nyp, *, sparse, arbors=1, stale=False, shared=True, channel=1):
    torch, capi, lib = env
    rng = np.random.default_rng(pre.nx * 31 + post.nf)
    a = sparse_activity(rng, pre, 0.15)
    nk = (pre.nx // post.nx if pre.nx > post.nx else 1) * (pre.ny // post.ny if pre.ny > post.ny else 1) * pre.nf
    w = rng.normal(0, 0.05, (arbors, nk, nyp, nxp, post.nf)).astype(np.float32)
    ent, num = oracle.compact(a.reshape(pre.nbatch, -1))
    ref = np.zeros(post.res_shape(), np.float32)
    for ar in range(arbors):
        ref = oracle.deliver_pre(OL(oracle, pre), OL(oracle, post), nxp, nyp, w[ar], a_ext=a, gsyn=ref)
    gsyn = torch.full((2,) + post.res_shape(), 0.0, device="cuda")
    gsyn[1 - channel] = 3.25  # the other channel must stay as it is
    dev = lambda t: torch.from_numpy(np.ascontiguousarray(t)).cuda()
    if stale:  # the host holds the new activity; the device copies are out of date
        ad = torch.zeros(pre.ext_shape(), device="cuda")
        ed = torch.zeros((pre.nbatch, pre.num_ext, 2), dtype=torch.int32, device="cuda")
        nd = torch.zeros(pre.nbatch, dtype=torch.int64, device="cuda")
    else:
        ad = dev(a)
        ed = dev(ent.view(np.uint8)).view(torch.int32).reshape(pre.nbatch, pre.num_ext, 2)
        nd = dev(num)
    ha = np.ascontiguousarray(a)
    hn = np.ascontiguousarray(num)
    he = np.ascontiguousarray(ent)
    wd = dev(w)  # every device tensor stays referenced until the call has returned
    rc = lib.standin_pre_delivery(l8(pre), l8(post), nxp, nyp, nk, int(sparse), int(shared), channel, arbors,
                                  C.c_float(1.0), int(stale), ptr(ad), ptr(ed), ptr(nd), ptr(wd), ptr(gsyn),
                                  ha.ctypes.data_as(C.c_void_p), hn.ctypes.data_as(C.c_void_p),
                                  he.ctypes.data_as(C.c_void_p), stream(torch))
    torch.cuda.synchronize()
    return rc, gsyn.cpu().numpy(), ref


@pytest.mark.parametrize("case", [
    # (pre nb,nx,ny,nf,halo), (post nx,ny,nf,halo), nxp, nyp, sparse, arbors, stale
    ((2, 16, 16, 64, 2), (32, 32, 1, 3), 8, 8, True, 1, False),   # LCA reconstruction V1 -> error
    ((2, 16, 16, 64, 2), (32, 32, 1, 3), 8, 8, False, 1, False),  # the same from the dense datastore
    ((1, 24, 20, 16, 3), (24, 20, 64, 0), 7, 7, True, 2, False),  # one-to-one, two arbors
    ((2, 16, 16, 24, 2), (32, 32, 3, 3), 8, 8, True, 1, True),    # datastore updated on the host
])
def test_presynaptic_adapter_matches_oracle(env, oracle, case):
    torch, capi, lib = env
    (nb, nx, ny, nf, h), (qx, qy, qf, qh), nxp, nyp, sparse, arbors, stale = case
    pre, post = capi.Loc.make(nb, nx, ny, nf, h), capi.Loc.make(nb, qx, qy, qf, qh)
    rc, g, ref = run_pre(env, oracle, pre, post, nxp, nyp, sparse=sparse, arbors=arbors, stale=stale)
    assert rc == 0, lib.standin_last_error()
    assert np.all(g[0] == 3.25)
    assert np.abs(g[1] - ref).max() <= 1e-5 * np.abs(ref).max()


def test_presynaptic_adapter_refuses_non_shared_weights(env, oracle):
    torch, capi, lib = env
    pre, post = capi.Loc.make(1, 16, 16, 8, 2), capi.Loc.make(1, 32, 32, 1, 3)
    rc, g, _ = run_pre(env, oracle, pre, post, 8, 8, sparse=True, shared=False)
    assert rc == 1 and b"shared weights only" in lib.standin_last_error()
    assert np.all(g[1] == 0.0)


@pytest.mark.parametrize("case", [
    # (pre nb,nx,ny,nf,halo), (post nx,ny,nf,halo), nxp, nyp (presynaptic patch), tensor-core entry
    ((2, 32, 32, 1, 3), (16, 16, 64, 2), 4, 4, False),  # error -> V1 (TransposeConn of the LCA module)
    ((1, 24, 24, 32, 3), (24, 24, 32, 0), 7, 7, True),  # one-to-one
])
def test_postsynaptic_adapter_matches_oracle(env, oracle, case):
    torch, capi, lib = env
    (nb, nx, ny, nf, h), (qx, qy, qf, qh), nxp, nyp, tc = case
    pre, post = capi.Loc.make(nb, nx, ny, nf, h), capi.Loc.make(nb, qx, qy, qf, qh)
    rng = np.random.default_rng(qf + nx)
    a = rng.normal(size=pre.ext_shape()).astype(np.float32)
    nk = (nx // qx if nx > qx else 1) * (ny // qy if ny > qy else 1) * nf
    w = rng.normal(0, 0.05, (nk, nyp, nxp, qf)).astype(np.float32)
    w_post = oracle.transpose_shared(OL(oracle, pre), OL(oracle, post), nxp, nyp, w)
    nkp, nyp_post, nxp_post = w_post.shape[:3]
    ref = oracle.deliver_post(OL(oracle, pre), OL(oracle, post), nxp_post, nyp_post, w_post, a)
    dev = lambda t: torch.from_numpy(np.ascontiguousarray(t)).cuda()
    gsyn = torch.zeros((1,) + post.res_shape(), device="cuda")
    used = C.c_int(-1)
    ad, wd = dev(a), dev(w_post)
    rc = lib.standin_post_delivery(l8(pre), l8(post), nxp, nyp, nxp_post, nyp_post, nkp, 0, 1, C.c_float(1.0),
                                   ptr(ad), ptr(wd), ptr(gsyn), C.byref(used), stream(torch))
    torch.cuda.synchronize()
    assert rc == 0, lib.standin_last_error()
    assert used.value == int(tc)
    g = gsyn.cpu().numpy()[0]
    assert np.abs(g - ref).max() <= 1e-5 * np.abs(ref).max()


def test_update_components_bitexact(env, oracle):
    torch, capi, lib = env
    rng = np.random.default_rng(5)
    loc = capi.Loc.make(2, 16, 16, 64, 2)
    oloc = OL(oracle, loc)
    dev = lambda t: torch.from_numpy(np.ascontiguousarray(t)).cuda()
    # GSynAccumulator: G = 1*ch0 - 1*ch1 (the error layer's coefficients), and three channels
    for coeffs in ([1.0, -1.0], [0.5, -2.0, 0.25]):
        gs = rng.normal(size=(len(coeffs),) + loc.res_shape()).astype(np.float32)
        g = torch.zeros(loc.res_shape(), device="cuda")
        cf = np.array(coeffs, np.float32)
        gsd = dev(gs)
        rc = lib.standin_gsyn_accumulate(l8(loc), len(coeffs), cf.ctypes.data_as(C.c_void_p), ptr(gsd), ptr(g),
                                         stream(torch))
        torch.cuda.synchronize()
        assert rc == 0, lib.standin_last_error()
        assert np.array_equal(g.cpu().numpy().view(np.uint32), oracle.gsyn_accumulate(gs, cf).view(np.uint32))
    # HyPerLCAInternalStateBuffer: V = e V + (1 - e)(G + A), per-image time steps
    v0 = rng.normal(0, 0.2, loc.res_shape()).astype(np.float32)
    a_ext = oracle.ann_activity(oloc, v0, 0.1, 0.0, np.inf, 0.1, 0.0)
    gin = rng.normal(size=loc.res_shape()).astype(np.float32)
    dt = np.array([1.0, 0.5])
    v, dtd, gd, ad = dev(v0), dev(dt), dev(gin), dev(a_ext)
    rc = lib.standin_lca_update(l8(loc), 1, C.c_double(100.0), ptr(dtd), ptr(gd), ptr(ad), ptr(v), stream(torch))
    torch.cuda.synchronize()
    assert rc == 0, lib.standin_last_error()
    ref = oracle.lca_update(oloc, gin, a_ext, v0, dt, 100.0)
    assert np.array_equal(v.cpu().numpy().view(np.uint32), ref.view(np.uint32))
    # ANNActivityBuffer: the soft threshold's vertices
    vV, vA, sl = oracle.ann_vertices(np.float32(0.1), np.float32(0.0), np.float32(np.inf), np.float32(0.1),
                                     np.float32(0.0))
    a = torch.zeros(loc.ext_shape(), device="cuda")
    vVd, vAd, sld, v0d = dev(vV), dev(vA), dev(sl), dev(v0)
    rc = lib.standin_ann_vertices(l8(loc), len(vV), ptr(vVd), ptr(vAd), ptr(sld), ptr(v0d), ptr(a), stream(torch))
    torch.cuda.synchronize()
    assert rc == 0, lib.standin_last_error()
    ref = oracle.apply_vertices(oloc, v0, vV, vA, sl)
    assert np.array_equal(a.cpu().numpy().view(np.uint32), ref.view(np.uint32))
