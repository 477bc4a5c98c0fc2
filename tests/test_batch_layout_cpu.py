"""hcc_batch_layout (host only): the packing of a batched ensemble. Shifted clouds keep a gap of at least two
support radii on some axis between every pair of bounding boxes (so no particle can see another cloud), the canvas
is the union box, shifts are pure translations, and bad inputs are rejected."""
import ctypes as C
import sys

import numpy as np
import pytest


def _layout(lib, clouds, radius):
    D = clouds[0].shape[1]
    offs = np.zeros(len(clouds) + 1, dtype=np.int64)
    offs[1:] = np.cumsum([c.shape[0] for c in clouds])
    pos = np.ascontiguousarray(np.concatenate(clouds), dtype=np.float64)
    shifts = np.zeros((len(clouds), D))
    canvas = np.zeros(2 * D)
    st = lib.hcc_batch_layout(D, radius, len(clouds), offs.ctypes.data_as(C.POINTER(C.c_int64)),
                              pos.ctypes.data_as(C.POINTER(C.c_double)), shifts.ctypes.data_as(C.POINTER(C.c_double)),
                              canvas.ctypes.data_as(C.POINTER(C.c_double)))
    return st, shifts, canvas


@pytest.mark.parametrize("D", [1, 2, 3])
def test_packed_clouds_keep_two_radii_apart(hcc, cuda_lib, D):
    rng = np.random.default_rng(D)
    radius = 0.05
    clouds = []
    for k in range(23):
        lo = rng.uniform(-3, 3, D)
        ext = rng.uniform(0.0, 1.5, D) * (k % 5 != 0)         # some single-point / flat clouds
        clouds.append(lo + rng.random((int(rng.integers(1, 60)), D)) * ext)
    st, shifts, canvas = _layout(cuda_lib, clouds, radius)
    assert st == 0
    boxes = []
    for c, s in zip(clouds, shifts):
        p = c + s
        assert np.all(p >= canvas[:D] - 1e-12) and np.all(p <= canvas[D:] + 1e-12)
        boxes.append((p.min(axis=0), p.max(axis=0)))
    for a in range(len(boxes)):
        for b in range(a + 1, len(boxes)):
            (la, ha), (lb, hb) = boxes[a], boxes[b]
            sep = np.maximum(lb - ha, la - hb)                # per-axis separation (negative: overlap)
            assert sep.max() >= 2 * radius - 1e-12, (a, b, sep)


def test_layout_rejects_bad_input(hcc, cuda_lib):
    one = [np.zeros((3, 2))]
    assert _layout(cuda_lib, one, 0.0)[0] == hcc._abi.HCC_ERR_INVALID
    bad = [np.array([[0.0, np.nan]])]
    assert _layout(cuda_lib, bad, 0.1)[0] == sys.modules["hcc_gb300._abi"].HCC_ERR_NONFINITE
