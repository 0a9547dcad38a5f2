"""The drop-in adapters (adapters/: the replacement bodies of the reference's GPU delivery and
update translation units, a CudaKernel.hpp without cuDNN, and its launcher) compile against the
OpenPV reference's own headers with the CUDA build on, reach no cuDNN header, and call the C ABI
of libpvgpu for their work.  Needs the reference source tree (the oracle recipe's root);
skipped where it is absent."""
import os
import shutil
import subprocess

import pytest

from tests.refbuild import REF_ROOT

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
AD = os.path.join(ROOT, "adapters")
OBJS = {
    "PresynapticPerspectiveGPUDelivery": ["pvgpu_deliver_pre"],
    "PostsynapticPerspectiveGPUDelivery": ["pvgpu_deliver_post", "pvgpu_deliver_post_tc",
                                           "pvgpu_deliver_tc_workspace_bytes"],
    "HyPerLCAInternalStateBuffer": ["pvgpu_lca_update"],
    "MomentumLCAInternalStateBuffer": ["pvgpu_momentum_lca_update"],
    "ISTAInternalStateBuffer": ["pvgpu_ista_update"],
    "ANNActivityBuffer": ["pvgpu_ann_vertices"],
    "GSynAccumulator": ["pvgpu_gsyn_accumulate"],
    "CudaKernel": [],
}

CUDA_INC = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"))),
                        "include")

pytestmark = pytest.mark.skipif(not os.path.isdir(os.path.join(REF_ROOT, "src", "delivery")),
                                reason="reference source tree not present")


@pytest.fixture(scope="module")
def built():
    r = subprocess.run(["make", "-s", "-f", os.path.join(AD, "Makefile"), f"REF={REF_ROOT}"], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return os.path.join(AD, "_build")


@pytest.mark.parametrize("tu", sorted(OBJS))
def test_adapter_compiles_and_calls_the_library(built, tu):
    obj = os.path.join(built, tu + ".o")
    assert os.path.exists(obj)
    undefined = subprocess.run(["nm", "-u", "-C", obj], capture_output=True, text=True).stdout
    for sym in OBJS[tu]:
        assert sym in undefined, (tu, sym)
    # every method the reference header declares is defined here (no leftover of the old body)
    defined = subprocess.run(["nm", "-C", "--defined-only", obj], capture_output=True, text=True).stdout
    if tu.endswith("Delivery"):
        for m in ("::deliver(float*)", "::deliverUnitInput(float*)", "::allocateDataStructures()",
                  "::communicateInitInfo(", "::setCudaDevice(", "::initializeRecvKernelArgs()"):
            assert f"PV::{tu}{m}" in defined, (tu, m)


def test_no_translation_unit_reaches_cudnn():
    inc = ["-I", AD, "-I", os.path.join(AD, "config"), "-I", os.path.join(REF_ROOT, "src"),
           "-I", os.path.join(ROOT, "include"), "-I", CUDA_INC]
    for src in ("delivery/PresynapticPerspectiveGPUDelivery.cpp", "delivery/PostsynapticPerspectiveGPUDelivery.cpp",
                "arch/cuda/CudaKernel.cpp"):
        r = subprocess.run(["g++", "-std=c++17", "-fopenmp", "-M"] + inc + [os.path.join(AD, src)],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        deps = r.stdout
        assert "cudnn" not in deps, src
        assert os.path.join(AD, "arch", "cuda", "CudaKernel.hpp") in deps, src
        assert os.path.join(REF_ROOT, "src", "arch", "cuda", "CudaKernel.hpp") not in deps, src
