"""Builds libpvgpu.so in-tree from openpv_gb300/csrc with nvcc for sm_103a.

Every translation unit is compiled in parallel (one nvcc per .cu/.cpp), then linked
into openpv_gb300/libpvgpu.so with the CUDA runtime linked statically, so the library
loads next to any PyTorch build without a runtime-library path.  Only the
translation units whose source (or any header) changed are recompiled.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libpvgpu.so")
HOST = os.path.join(HERE, "host")
HOST_LIB = os.path.join(HERE, "libpvhost.so")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
                     "--expt-relaxed-constexpr", "-I", INCLUDE, "-I", CSRC]


def nvcc():
    cand = [os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"]
    for c in cand:
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: libpvgpu.so cannot be built")


def _headers_mtime():
    hs = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + \
        glob.glob(os.path.join(INCLUDE, "*.h")) + glob.glob(os.path.join(HOST, "*.hpp"))
    return max((os.path.getmtime(h) for h in hs), default=0.0)


def _compile(src, obj, hdr_mtime, extra):
    if os.path.exists(obj):
        om = os.path.getmtime(obj)
        if om >= os.path.getmtime(src) and om >= hdr_mtime:
            return obj, None
    cmd = [nvcc()] + NVCC_FLAGS + extra + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return obj, f"{' '.join(cmd)}\n{r.stdout}\n{r.stderr}"
    return obj, None


def build(verbose=False, extra=()):
    os.makedirs(OBJ, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))
    hm = _headers_mtime()
    jobs = []
    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        for s in srcs:
            o = os.path.join(OBJ, os.path.splitext(os.path.basename(s))[0] + ".o")
            jobs.append(ex.submit(_compile, s, o, hm, list(extra)))
        results = [j.result() for j in jobs]
    errs = [e for _, e in results if e]
    if errs:
        raise RuntimeError("libpvgpu build failed:\n" + "\n".join(errs))
    objs = [o for o, _ in results]
    if not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-ldl"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"libpvgpu link failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose:
        print("built", LIB)
    build_host(verbose)
    return LIB


def build_host(verbose=False):
    """libpvhost.so: the C++ host side (params reader, column, delivery classes) over libpvgpu.so."""
    srcs = sorted(glob.glob(os.path.join(HOST, "*.cpp")))
    if not srcs:
        return None
    hm = _headers_mtime()
    flags = ["-I", HOST]
    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        jobs = [ex.submit(_compile, s, os.path.join(OBJ, "host_" + os.path.splitext(os.path.basename(s))[0] + ".o"),
                          hm, flags) for s in srcs]
        results = [j.result() for j in jobs]
    errs = [e for _, e in results if e]
    if errs:
        raise RuntimeError("libpvhost build failed:\n" + "\n".join(errs))
    objs = [o for o, _ in results]
    if not os.path.exists(HOST_LIB) or any(os.path.getmtime(o) > os.path.getmtime(HOST_LIB) for o in objs) or \
            os.path.getmtime(LIB) > os.path.getmtime(HOST_LIB):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", HOST_LIB] + objs + ["-L", HERE, "-lpvgpu", "-Xlinker",
                                                                       "-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"libpvhost link failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose:
        print("built", HOST_LIB)
    return HOST_LIB


if __name__ == "__main__":
    build(verbose=True, extra=sys.argv[1:])
