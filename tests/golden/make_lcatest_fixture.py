"""Writes the known-answer fixtures of the reference's LCA system tests (OpenPV tree):
  tests/golden/lcatest_correct.npz from tests/LCATest/input (LCATest.params): the two input
  frames the test's PvpLayer "Input" shows (inputImages.pvp) and the frames of the known-answer
  reconstruction (correct.pvp, 40 frames, compared by the test with the Reconstruction layer at
  every timestep to 1e-6) at the timesteps listed in STEPS;
  tests/golden/momentumlcatest_correct.npz from tests/MomentumLCATest/input
  (MomentumLCATest.params): the test image and all 10 known-answer reconstruction frames.
Run once where the reference tree is mounted:

    python tests/golden/make_lcatest_fixture.py /path/to/OpenPV
"""
import os
import sys

import numpy as np

STEPS = (1, 2, 20, 21, 40)  # first step, the adaptive time step's first growth, both sides of the frame change, last


def read_dense_pvp(path):
    """A non-spiking activity file (PVP_NONSPIKING_ACT_FILE_TYPE, float data): an 80-byte header
    of 18 int32 and a double, then per frame a double timestamp and nx*ny*nf floats."""
    raw = open(path, "rb").read()
    h = np.frombuffer(raw, np.int32, 18)
    hsize, ftype, nx, ny, nf, dtype = int(h[0]), int(h[2]), int(h[3]), int(h[4]), int(h[5]), int(h[9])
    assert hsize == 80 and ftype == 4 and dtype == 3, (hsize, ftype, dtype)
    n = nx * ny * nf
    rec = 8 + 4 * n
    nframes = (len(raw) - hsize) // rec
    assert hsize + nframes * rec == len(raw)
    times = np.zeros(nframes)
    frames = np.zeros((nframes, ny, nx, nf), np.float32)
    for i in range(nframes):
        off = hsize + i * rec
        times[i] = np.frombuffer(raw, np.float64, 1, off)[0]
        frames[i] = np.frombuffer(raw, np.float32, n, off + 8).reshape(ny, nx, nf)
    return frames, times


def momentum_fixture(ref_root):
    """tests/MomentumLCATest/input: the 60x60 test image and all 10 known-answer frames."""
    d = os.path.join(ref_root, "tests", "MomentumLCATest", "input")
    x, xt = read_dense_pvp(os.path.join(d, "testimage.pvp"))
    c, ct = read_dense_pvp(os.path.join(d, "correct.pvp"))
    assert x.shape == (1, 60, 60, 1) and c.shape == (10, 60, 60, 1)
    assert np.array_equal(ct, np.arange(1, 11, dtype=np.float64))
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "momentumlcatest_correct.npz")
    np.savez_compressed(out, input_frame=x, correct=c)
    print("wrote", out)


def main(ref_root):
    momentum_fixture(ref_root)
    d = os.path.join(ref_root, "tests", "LCATest", "input")
    x, xt = read_dense_pvp(os.path.join(d, "inputImages.pvp"))
    c, ct = read_dense_pvp(os.path.join(d, "correct.pvp"))
    assert x.shape == (2, 64, 128, 1) and c.shape == (40, 64, 128, 1)
    assert np.array_equal(ct, np.arange(1, 41, dtype=np.float64))
    idx = np.array(STEPS) - 1
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lcatest_correct.npz")
    np.savez_compressed(out, input_frames=x, input_times=xt, steps=np.array(STEPS, np.int32), correct=c[idx])
    print("wrote", out)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ["OPENPV_REFERENCE"])
