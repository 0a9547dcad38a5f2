"""CPU tests of the host side's params reader (the grammar of io/parser/params.l / params.y)
through libpvhost.so's pvhost_params_dump; no GPU needed."""
import os

import pytest

from tests.lca_params import lca_params


@pytest.fixture(scope="module")
def capi():
    from openpv_gb300 import build
    try:
        build.nvcc()
    except RuntimeError:
        pytest.skip("nvcc not available")
    build.build()
    from openpv_gb300 import capi
    return capi


def groups(dump):
    out, cur = {}, None
    for line in dump.splitlines():
        if not line.startswith("  "):
            kw, name = line.split(" ", 1)
            key = name.strip('"') if kw != "ParameterSweep" else "sweep:" + name.strip('"')
            cur = out.setdefault(key, {"keyword": kw})
        elif cur is not None:
            k, v = line.strip().split(" = ", 1)
            cur[k] = v
    return out


def test_lca_module_params(capi):
    g = groups(capi.params_dump(lca_params()))
    assert g["column"]["keyword"] == "HyPerCol" and g["column"]["nbatch"] == "2"
    assert g["V1"]["keyword"] == "HyPerLCALayer" and g["V1"]["nxScale"] == "0.5"
    assert float(g["V1"]["AMax"]) == pytest.approx(3.40282347e38)  # infinity = FLT_MAX
    assert g["V1"]["sparseLayer"] == "1" and g["V1"]["InitVType"] == '"ZeroV"'
    assert g["ResidualToV1"]["originalConnName"] == '"V1ToResidual"'
    assert g["InputToResidual"]["delay"] == "[0]"
    assert float(g["Residual"]["VThresh"]) == pytest.approx(-3.40282347e38)


def test_grammar_features(capi):
    text = """
    randomSeed = 12345;   // a directive
    HyPerCol "c" = { nx = 8; ny = 8; dt = 1.0e0; };
    ANNLayer "base" = { nf = 3; VThresh = 0.25; AMin = -1.5; flag = true; off = false; name = NULL;
                        vec = [1, -2.5, 3e-1]; empty = []; };
    ANNLayer "derived" = { #include "base"; @VThresh = +0.5; extra = -infinity; };
    ParameterSweep "derived":VThresh = { 0.1; 0.2; };
    """
    g = groups(capi.params_dump(text))
    assert g["base"]["vec"] == "[1, -2.5, 0.3]" and g["base"]["empty"] == "[]"
    assert g["base"]["flag"] == "1" and g["base"]["off"] == "0" and g["base"]["name"] == "NULL"
    d = g["derived"]
    assert d["nf"] == "3" and d["VThresh"] == "0.5" and d["AMin"] == "-1.5"  # included, then overridden
    assert float(d["extra"]) == pytest.approx(-3.40282347e38)
    assert g["sweep:derived"]["VThresh"] == "[0.1, 0.2]"
    assert "randomSeed = 12345" in capi.params_dump(text)


@pytest.mark.parametrize("bad, where", [
    ('HyPerCol "c" = { nx = 8 ny = 8; };', "line 1"),
    ('HyPerCol "c" = { nx = 8; };\nANNLayer "a" = { @VThresh = 1; };', "line 2"),    # override of nothing
    ('ANNLayer "a" = { nf = 1; #include "b"; };', "line 1"),                           # include not first
    ('ANNLayer "a" = { nf = 1; nf = 2; };', "line 1"),                                  # duplicate
])
def test_syntax_errors_name_the_line(capi, bad, where):
    with pytest.raises(RuntimeError, match=where):
        capi.params_dump(bad)


def test_reference_lca_test_params_parse(capi):
    """The reference's own GPU LCA test params file parses, with its delivery switches (read as
    text from the reference tree when it is present)."""
    from tests.refbuild import REF_ROOT
    path = os.path.join(REF_ROOT, "tests", "GPULCATest", "input", "GPULCATest.params")
    if not os.path.exists(path):
        pytest.skip("reference tree not present")
    g = groups(capi.params_dump(open(path).read()))
    kws = {v["keyword"] for v in g.values()}
    assert "HyPerCol" in kws and "HyPerLCALayer" in kws
    assert any(v.get("receiveGpu") is not None for v in g.values())
