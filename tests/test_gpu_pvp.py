"""Device side of the .pvp activity files: frame payloads packed on the GPU (pvgpu_pvp_*) equal
the file semantics (SparseList cropped to restricted indices in order, halo entries dropped; the
restricted activity for dense frames), and files written from device buffers hold what the
reference's Python writer put in the committed fixtures (tests/golden)."""
import os

import numpy as np
import pytest

from tests.test_gpu_kernels import H, T

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from openpv_gb300 import build
    build.build()
    from openpv_gb300 import capi
    capi.lib()
    capi.host_lib()
    return torch


def crop_ref(a_ext, h):
    """SparseList::crop of the compacted extended activity, per batch element."""
    nb, nyE, nxE, nf = a_ext.shape
    res = a_ext[:, h:nyE - h, h:nxE - h, :].reshape(nb, -1)
    return [(np.nonzero(r)[0].astype(np.uint32), r[r != 0]) for r in res]


@pytest.mark.parametrize("nb, nx, ny, nf, h, p", [(3, 17, 9, 5, 2, 0.3), (2, 40, 33, 8, 0, 0.05), (1, 5, 4, 3, 3, 1.0),
                                                  (2, 8, 8, 2, 1, 0.0)])
def test_sparse_and_dense_frames(cuda, nb, nx, ny, nf, h, p):
    torch = cuda
    from openpv_gb300 import capi
    loc = capi.Loc.make(nb, nx, ny, nf, h)
    rng = np.random.default_rng(nx * ny + nf)
    a = ((rng.random(loc.ext_shape()) < p) * rng.normal(size=loc.ext_shape())).astype(np.float32)  # halo too
    ad = T(torch, a)
    ent = torch.zeros((nb, loc.num_ext, 2), dtype=torch.int32, device="cuda")
    num = torch.zeros(nb, dtype=torch.int64, device="cuda")
    capi.compact_active(ad, nb, loc.num_ext, ent, num)
    nres = nx * ny * nf
    out = torch.zeros((nb, nres, 2), dtype=torch.int32, device="cuda")
    cnt = torch.full((nb,), -1, dtype=torch.int32, device="cuda")
    capi.pvp_sparse_frames(loc, ent, num, out, cnt)
    got = H(out).view(np.uint8).reshape(nb, nres, 8).view(capi.ENTRY_DTYPE).reshape(nb, nres)
    for b, (idx, val) in enumerate(crop_ref(a, h)):
        c = int(H(cnt)[b])
        assert c == len(idx)
        assert np.array_equal(got[b, :c]["index"], idx)
        assert np.array_equal(got[b, :c]["value"].view(np.uint32), val.view(np.uint32))
    dense = torch.zeros((nb, ny, nx, nf), device="cuda")
    capi.pvp_dense_frames(loc, ad, dense)
    assert np.array_equal(H(dense), a[:, h:h + ny, h:h + nx, :])
    # back into a (zeroed) extended activity: the restricted part returns, the halo stays 0
    back = T(torch, np.full(loc.ext_shape(), 7.0, np.float32))
    bad = torch.zeros(1, dtype=torch.int32, device="cuda")
    capi.pvp_scatter_sparse(loc, out, cnt, back, bad)
    want = np.zeros_like(a)
    want[:, h:h + ny, h:h + nx, :] = a[:, h:h + ny, h:h + nx, :]
    assert np.array_equal(H(back), want) and int(H(bad)[0]) == 0


def test_scatter_flags_out_of_layer_index(cuda):
    torch = cuda
    from openpv_gb300 import capi
    loc = capi.Loc.make(1, 4, 4, 1, 1)
    e = np.zeros((1, 16), capi.ENTRY_DTYPE)
    e["index"][0, :2] = [3, 99]
    e["value"][0, :2] = [1.5, 2.0]
    ed = T(torch, e.view(np.int32).reshape(1, 16, 2))
    cnt = T(torch, np.array([2], np.int32))
    a = torch.zeros(loc.ext_shape(), device="cuda")
    bad = torch.zeros(1, dtype=torch.int32, device="cuda")
    capi.pvp_scatter_sparse(loc, ed, cnt, a, bad)
    assert int(H(bad)[0]) == 1
    assert H(a)[0, 1, 4, 0] == 1.5 and np.count_nonzero(H(a)) == 1


def test_files_written_from_the_device_hold_the_reference_fixture_frames(cuda, tmp_path):
    """The fixture frames (written by the reference's Python writer) laid into a batch of
    extended activities with nonzero halos, written from the device by the library: every frame
    reads back equal to the reference writer's file, frame by frame."""
    torch = cuda
    from openpv_gb300 import capi
    fx = np.load(os.path.join(GOLD, "pvp_fixtures.npz"))
    h = 2
    rng = np.random.default_rng(3)
    # sparse layer 7x6x3, batch of 4 = the 4 fixture frames
    loc = capi.Loc.make(4, 7, 6, 3, h)
    a = (rng.random(loc.ext_shape()) < 0.3).astype(np.float32) * 9.0  # halo junk, dropped by the crop
    a[:, h:h + 6, h:h + 7, :] = fx["sparse"]
    ad = T(torch, a)
    ent = torch.zeros((4, loc.num_ext, 2), dtype=torch.int32, device="cuda")
    num = torch.zeros(4, dtype=torch.int64, device="cuda")
    capi.compact_active(ad, 4, loc.num_ext, ent, num)
    p = tmp_path / "s.pvp"
    with capi.PvpWriter(p, 7, 6, 3, True) as w:
        w.write_sparse_device(loc, ent, num, 2.0)
    with capi.PvpReader(p) as mine, capi.PvpReader(os.path.join(GOLD, "sparse_7x6x3_x4.pvp")) as ref:
        assert mine.num_frames == 4 and mine.header["nBands"] == 4
        for i in range(4):
            e1, t1 = mine.read_sparse(i)
            e2, _ = ref.read_sparse(i)
            assert t1 == 2.0
            assert np.array_equal(e1["index"], e2["index"]) and np.array_equal(e1["value"], e2["value"])
        # and back to the device, four frames into a batch of four
        back = torch.zeros(loc.ext_shape(), device="cuda")
        mine.read_to_device(0, loc, back)
        assert np.array_equal(H(back)[:, h:h + 6, h:h + 7, :], fx["sparse"])
        assert np.count_nonzero(H(back)) == np.count_nonzero(fx["sparse"])
    # dense layer 6x5x4, batch of 3
    loc = capi.Loc.make(3, 6, 5, 4, 1)
    a = rng.normal(size=loc.ext_shape()).astype(np.float32)
    a[:, 1:6, 1:7, :] = fx["dense"]
    q = tmp_path / "d.pvp"
    with capi.PvpWriter(q, 6, 5, 4, False) as w:
        w.write_dense_device(loc, T(torch, a), 1.0)
    with capi.PvpReader(q) as mine, capi.PvpReader(os.path.join(GOLD, "dense_6x5x4_x3.pvp")) as ref:
        for i in range(3):
            assert np.array_equal(mine.read_dense(i)[0].view(np.uint32), ref.read_dense(i)[0].view(np.uint32))
