"""Writes the .pvp fixtures of tests/test_host_pvp.py and tests/test_gpu_pvp.py with the
reference's own Python writer (python/pvtools/pvpFile.py of the OpenPV tree), together with the
arrays they hold (pvp_fixtures.npz).  Run once where the reference tree is mounted:

    python tests/golden/make_pvp_fixtures.py /path/to/OpenPV

The package's __init__ (which needs matplotlib) is bypassed; only pvpFile and readpvpheader load.
"""
import os
import sys
import types

import numpy as np


def load_pvtools(ref_root):
    pkg = types.ModuleType("pvtools")
    pkg.__path__ = [os.path.join(ref_root, "python", "pvtools")]
    sys.modules["pvtools"] = pkg
    from pvtools import pvpFile  # noqa: E402
    return pvpFile


def main(ref_root):
    here = os.path.dirname(os.path.abspath(__file__))
    pvpFile = load_pvtools(ref_root)
    import scipy.sparse as sp
    rng = np.random.default_rng(2024)
    # dense: 3 frames of 5 (y) x 6 (x) x 4 (f), times 1, 2, 3
    dense = rng.normal(size=(3, 5, 6, 4)).astype(np.float32)
    dense_t = np.array([1.0, 2.0, 3.0])
    f = pvpFile.pvpOpen(os.path.join(here, "dense_6x5x4_x3.pvp"), "w")
    f.write({"values": dense, "time": dense_t})
    f.close()
    # sparse values: 4 frames of 6 (y) x 7 (x) x 3 (f), about 20 % nonzero, one empty frame
    sparse = ((rng.random((4, 6 * 7 * 3)) < 0.2) * rng.uniform(0.1, 2.0, (4, 6 * 7 * 3))).astype(np.float32)
    sparse[2] = 0.0
    sparse_t = np.array([0.5, 1.5, 2.5, 3.5])
    f = pvpFile.pvpOpen(os.path.join(here, "sparse_7x6x3_x4.pvp"), "w")
    f.write({"values": sp.csr_matrix(sparse), "time": sparse_t}, shape=(6, 7, 3))
    f.close()
    np.savez(os.path.join(here, "pvp_fixtures.npz"), dense=dense, dense_t=dense_t,
             sparse=sparse.reshape(4, 6, 7, 3), sparse_t=sparse_t)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("OPENPV_REFERENCE", "/root/reference"))
