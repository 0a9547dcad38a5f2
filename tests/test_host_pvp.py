""".pvp activity files through libpvhost.so on the CPU: the reader against the reference's own
known-answer files (tests/BufferUtilsPvpTest of the OpenPV tree, read where they lie) and against
fixtures written by the reference's Python writer (tests/golden, made by make_pvp_fixtures.py);
the writer's header and frames against LayerIO / SparseLayerIO (io/LayerIO.cpp,
io/SparseLayerIO.cpp) and read back by both readers."""
import os
import struct

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden")
from tests.refbuild import REF_ROOT as REF
KAT = os.path.join(REF, "tests", "BufferUtilsPvpTest", "input")


@pytest.fixture(scope="module")
def capi():
    from openpv_gb300 import build
    build.build()
    from openpv_gb300 import capi
    return capi


def test_reads_reference_writer_fixtures(capi):
    fx = np.load(os.path.join(GOLD, "pvp_fixtures.npz"))
    with capi.PvpReader(os.path.join(GOLD, "dense_6x5x4_x3.pvp")) as r:
        assert r.header["fileType"] == 4 and r.num_frames == 3 and r.shape == (5, 6, 4)
        for i in range(3):
            v, t = r.read_dense(i)
            assert t == fx["dense_t"][i]
            assert np.array_equal(v.view(np.uint32), fx["dense"][i].view(np.uint32))
    with capi.PvpReader(os.path.join(GOLD, "sparse_7x6x3_x4.pvp")) as r:
        assert r.header["fileType"] == 6 and r.num_frames == 4 and r.shape == (6, 7, 3)
        for i in range(4):
            v, t = r.read_dense(i)
            assert t == fx["sparse_t"][i]
            assert np.array_equal(v, fx["sparse"][i])
            e, _ = r.read_sparse(i)
            flat = fx["sparse"][i].reshape(-1)
            assert np.array_equal(e["index"], np.nonzero(flat)[0])  # ascending restricted index
            assert np.array_equal(e["value"], flat[flat != 0])


@pytest.mark.skipif(not os.path.isdir(KAT), reason="reference source tree not mounted")
def test_reference_known_answer_files(capi):
    """BufferUtilsPvpTest (tests/BufferUtilsPvpTest/src/main.cpp): dense 8x4x2, three frames holding
    0, 1, 2, ... continuing across frames; sparse 5x5x1, five frames of 13 values 1, 2, ... at the
    even positions; binary 3x2x1, three frames with (1 + i + frame) % 2; frame f at time f + 1."""
    with capi.PvpReader(os.path.join(KAT, "input_8x4x2_x3.pvp")) as r:
        val = 0.0
        for f in range(3):
            v, t = r.read_dense(f)
            assert t == f + 1
            assert np.array_equal(v.reshape(-1), np.arange(val, val + 64, dtype=np.float32))
            val += 64
    with capi.PvpReader(os.path.join(KAT, "sparse_5x5x1_x5.pvp")) as r:
        val = 1.0
        for f in range(5):
            e, t = r.read_sparse(f)
            assert t == f + 1 and len(e) == 13
            assert np.array_equal(e["index"], np.arange(0, 25, 2))
            assert np.array_equal(e["value"], np.arange(val, val + 13, dtype=np.float32))
            val += 13
    with capi.PvpReader(os.path.join(KAT, "binary_3x2x1_x3.pvp")) as r:
        assert r.header["fileType"] == 2
        for f in range(3):
            v, t = r.read_dense(f)
            assert t == f + 1
            assert np.array_equal(v.reshape(-1), np.array([(1 + i + f) % 2 for i in range(6)], np.float32))


def test_writer_follows_layer_io(capi, tmp_path):
    """Header as SparseLayerIO::writeHeader / LayerIO::writeHeader (80 bytes, numParams 20, FLOAT
    data type, nBatch 1, timestamp 0) with nBands counting the frames; frames as
    {double t, int count, {uint32, float} x count} and {double t, float x nx*ny*nf}."""
    fx = np.load(os.path.join(GOLD, "pvp_fixtures.npz"))
    sp_path, de_path = tmp_path / "s.pvp", tmp_path / "d.pvp"
    with capi.PvpWriter(sp_path, 7, 6, 3, True) as w:
        for i in range(4):
            flat = fx["sparse"][i].reshape(-1)
            idx = np.nonzero(flat)[0]
            w.write_sparse(idx, flat[idx], fx["sparse_t"][i])
    with capi.PvpWriter(de_path, 6, 5, 4, False) as w:
        for i in range(3):
            w.write_dense(fx["dense"][i], fx["dense_t"][i])
    raw = open(sp_path, "rb").read()
    h = struct.unpack("<18id", raw[:80])
    assert h[:18] == (80, 20, 6, 7, 6, 3, 1, 0, 8, 3, 1, 1, 7, 6, 0, 0, 1, 4) and h[18] == 0.0
    pos = 80
    for i in range(4):
        t, n = struct.unpack("<di", raw[pos:pos + 12])
        flat = fx["sparse"][i].reshape(-1)
        assert t == fx["sparse_t"][i] and n == np.count_nonzero(flat)
        e = np.frombuffer(raw[pos + 12:pos + 12 + 8 * n], dtype=capi.ENTRY_DTYPE)
        assert np.array_equal(e["index"], np.nonzero(flat)[0]) and np.array_equal(e["value"], flat[flat != 0])
        pos += 12 + 8 * n
    assert pos == len(raw)
    raw = open(de_path, "rb").read()
    h = struct.unpack("<18id", raw[:80])
    assert h[:18] == (80, 20, 4, 6, 5, 4, 1, 120, 4, 3, 1, 1, 6, 5, 0, 0, 1, 3) and h[18] == 0.0
    assert len(raw) == 80 + 3 * (8 + 120 * 4)
    for i in range(3):
        off = 80 + i * (8 + 480)
        assert struct.unpack("<d", raw[off:off + 8])[0] == fx["dense_t"][i]
        assert raw[off + 8:off + 488] == fx["dense"][i].astype("<f4").tobytes()
    # and our reader reads both back
    with capi.PvpReader(sp_path) as r:
        assert r.num_frames == 4
        assert np.array_equal(r.read_dense(1)[0], fx["sparse"][1])


def test_reference_reader_reads_our_files(capi, tmp_path):
    """The reference's Python reader (pvtools) reads what the writer wrote."""
    if not os.path.isdir(os.path.join(REF, "python", "pvtools")):
        pytest.skip("reference source tree not mounted")
    pytest.importorskip("scipy")
    import sys
    import types
    pkg = types.ModuleType("pvtools")
    pkg.__path__ = [os.path.join(REF, "python", "pvtools")]
    sys.modules.setdefault("pvtools", pkg)
    from pvtools import pvpFile
    fx = np.load(os.path.join(GOLD, "pvp_fixtures.npz"))
    p = tmp_path / "s.pvp"
    with capi.PvpWriter(p, 7, 6, 3, True) as w:
        for i in range(4):
            flat = fx["sparse"][i].reshape(-1)
            idx = np.nonzero(flat)[0]
            w.write_sparse(idx, flat[idx], fx["sparse_t"][i])
    f = pvpFile.pvpOpen(str(p), "r")
    d = f.read()
    f.close()
    assert np.array_equal(np.asarray(d["values"].todense()).reshape(4, 6, 7, 3), fx["sparse"])
    assert np.array_equal(np.asarray(d["time"]), fx["sparse_t"])


def test_reader_rejects_bad_files(capi, tmp_path):
    p = tmp_path / "bad.pvp"
    p.write_bytes(b"\x00" * 40)
    with pytest.raises(capi.PvhostError):
        capi.PvpReader(p)
    # a sparse frame whose count runs past the end of the file
    q = tmp_path / "trunc.pvp"
    with capi.PvpWriter(q, 4, 4, 1, True) as w:
        w.write_sparse(np.array([1, 5]), np.array([1.0, 2.0], np.float32), 1.0)
    raw = bytearray(open(q, "rb").read())
    raw[88:92] = struct.pack("<i", 1000)
    q.write_bytes(bytes(raw))
    with pytest.raises(capi.PvhostError):
        capi.PvpReader(q)
