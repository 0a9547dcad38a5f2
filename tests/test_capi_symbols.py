"""CPU checks of the C ABI: libpvgpu.so builds, loads and exports every entry point
include/pvgpu.h declares (no compute call: there is no GPU here)."""
import ctypes as C
import os

import pytest


@pytest.fixture(scope="module")
def built():
    from openpv_gb300 import build
    try:
        build.nvcc()
    except RuntimeError:
        pytest.skip("nvcc not available")
    return build.build()


def test_library_exports_every_declared_symbol(built):
    from openpv_gb300 import capi
    lib = C.CDLL(built)
    declared = capi.exported_symbols()
    assert len(declared) >= 10
    missing = [s for s in declared if not hasattr(lib, s)]
    assert not missing, f"declared in include/pvgpu.h but not exported: {missing}"


def test_status_strings_and_version(built):
    from openpv_gb300 import capi
    assert "sm_103a" in capi.version()
    assert capi.status_string(0) == "ok"
    for s in range(1, 7):
        assert capi.status_string(s) != "unknown status"


def test_bad_arguments_rejected_without_gpu(built):
    """Argument checks run on the host before any CUDA call."""
    from openpv_gb300 import capi
    L = capi.lib()
    pre = capi.Loc.make(1, 16, 16, 4, 2)
    post = capi.Loc.make(1, 32, 32, 1, 3)
    bad = capi.ConnDesc(pre, post, 8, 8, 1.0)
    # null weights / gsyn
    assert L.pvgpu_deliver_pre(C.byref(bad), None, None, None, None, None, 0, None) == 1
    # a geometry OpenPV rejects: one-to-many with a patch that is not a multiple of the ratio
    illegal = capi.ConnDesc(pre, post, 7, 7, 1.0)
    dummy = C.c_void_p(16)
    assert L.pvgpu_deliver_pre(C.byref(illegal), None, None, dummy, dummy, dummy, 0, None) == 6
    assert L.pvgpu_compact_active(None, 1, 10, None, None, None, 0, None) == 1
    assert L.pvgpu_cost_sum(None, None, 0, 0.0, 0.0, None, None) == 1


def test_host_library_exports_every_declared_symbol(built):
    """libpvhost.so (the C++ host side over the C ABI) loads and exports include/pvhost.h."""
    from openpv_gb300 import build, capi
    lib = C.CDLL(build.HOST_LIB)
    declared = capi.exported_symbols("pvhost.h", "pvhost")
    assert len(declared) >= 8
    missing = [s for s in declared if not hasattr(lib, s)]
    assert not missing, f"declared in include/pvhost.h but not exported: {missing}"


def test_struct_layouts_match_the_header(tmp_path):
    """Every struct the Python bindings pass across the C ABI has the size and field offsets the
    header gives it (a C program compiled against include/pvgpu.h prints them)."""
    import shutil
    import subprocess
    from openpv_gb300 import capi
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    structs = {
        "pvgpu_halo": capi.Halo,
        "pvgpu_loc": capi.Loc,
        "pvgpu_conn_desc": capi.ConnDesc,
        "pvgpu_lca_layer_desc": capi.LcaLayerDesc,
        "pvgpu_lca_solver_desc": capi.LcaSolverDesc,
        "pvgpu_lca_schedule": capi.LcaSchedule,
        "pvgpu_lca_grad_desc": capi.LcaGradDesc,
        "pvgpu_lif_params": capi.LifParams,
    }
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "pvgpu.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append(f'   printf("{cname} size %zu\\n", sizeof({cname}));')
        for field, _ in py._fields_:
            lines.append(f'   printf("{cname} {field} %zu\\n", offsetof({cname}, {field}));')
    lines.append('   printf("pvgpu_entry size %zu index %zu value %zu\\n", sizeof(pvgpu_entry), '
                 'offsetof(pvgpu_entry, index), offsetof(pvgpu_entry, value));')
    lines.append('   printf("pvgpu_taus size %zu\\n", sizeof(pvgpu_taus));')
    lines += ["   return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    subprocess.run([cc, "-std=c99", "-I", inc, str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines()
    got = {}
    for line in out:
        parts = line.split()
        if parts[0] == "pvgpu_entry":
            got["pvgpu_entry"] = tuple(int(v) for v in parts[2::2])
        else:
            got[(parts[0], parts[1])] = int(parts[2])
    for cname, py in structs.items():
        assert got[(cname, "size")] == C.sizeof(py), cname
        for field, _ in py._fields_:
            assert got[(cname, field)] == getattr(py, field).offset, (cname, field)
    e = capi.ENTRY_DTYPE
    assert got["pvgpu_entry"] == (e.itemsize, e.fields["index"][1], e.fields["value"][1])
    assert got[("pvgpu_taus", "size")] == 16  # the bindings hand over 4 x uint32 per neuron
