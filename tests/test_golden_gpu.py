"""The CUDA extraction (through the C ABI) reproduces the golden fixtures."""
import os

import numpy as np
import pytest

from golden_util import cases, check_mesh, load
from mc_util import gpu_extract

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("path", cases(), ids=lambda p: os.path.basename(p))
def test_gpu_matches_golden(mcg, path):
    g = load(path)
    out = gpu_extract(mcg, g["vol"], float(g["cell"]))
    check_mesh(g, out["soup"]["pos"], out["normals"], out["tri_cube"])
