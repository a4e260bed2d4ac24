"""Loading and checking the golden fixtures of tests/golden/ (made by
tests/golden/make_golden.py, an independent binary64 restatement)."""
import glob
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
POS_TOL_VOXEL = 1e-5
NRM_TOL = 1e-4
NRM_MIN_GRAD = 1e-3   # normals compared where the unnormalised gradient is not tiny


def cases():
    return sorted(glob.glob(os.path.join(GOLDEN, "*.npz")))


def load(path):
    d = np.load(path)
    return {k: d[k] for k in d.files}


def check_mesh(g, soup_pos, normals, tri_cube):
    """soup_pos/normals in canonical order (cube id, slot)."""
    cell = float(g["cell"])
    assert np.array_equal(tri_cube, g["tri_cube"])
    assert soup_pos.shape == g["pos"].shape
    err = np.abs(soup_pos.astype(np.float64) - g["pos"]).max(initial=0.0) / cell
    assert err <= POS_TOL_VOXEL, err
    good = g["nlen"] > NRM_MIN_GRAD
    nerr = np.abs(normals[good].astype(np.float64) - g["nrm"][good]).max(initial=0.0)
    assert nerr <= NRM_TOL, nerr
    assert (normals[g["nlen"] == 0] == 0).all()
