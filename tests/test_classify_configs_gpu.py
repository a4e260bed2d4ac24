"""Every classify configuration (item width, in-box or separate halo box,
stage ring and CTA size; MCG_CLS_CFG, read once per process) gives the
oracle's counts, on volumes that take the TMA path with and without the
halo column inside the volume, the plain-copy path, and float2."""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import json, sys
import numpy as np
import torch
sys.path.insert(0, sys.argv[1])
import marching_cube_gb300 as mcg
import oracle
from marching_cube_gb300 import synthetic
out = []
for shape, seed in [((20, 33, 300), 1), ((17, 40, 130), 2), ((11, 13, 45), 3), ((24, 24, 128), 4)]:
    vol = synthetic.random_volume(shape, seed=seed)
    m = mcg.extract(torch.from_numpy(vol).cuda(), 0.01, normals=True, tri_cube=True)
    torch.cuda.synchronize()
    occ, tri = oracle.mc_count(vol)
    o = oracle.mc_extract(vol, 0.01)
    tc = m.tri_cube.cpu().numpy()
    order = np.argsort(tc, kind="stable")
    idx = (order[:, None] * 3 + np.arange(3)[None, :]).reshape(-1)
    soup = m.soup.cpu().numpy().reshape(-1, 28)[idx]
    same = (m.counts["occupied"] == occ and m.counts["triangles"] == tri and
            np.array_equal(soup.reshape(-1), o["soup"].view(np.uint8).reshape(-1)))
    out.append(bool(same))
rng = np.random.default_rng(5)
f2 = np.stack([rng.standard_normal((14, 20, 200)).astype(np.float32),
               (rng.random((14, 20, 200)) > 0.03).astype(np.float32)], axis=-1)
m = mcg.extract(torch.from_numpy(f2).cuda(), 0.5, normals=False)
torch.cuda.synchronize()
occ, tri = oracle.mc_count(f2)
out.append(bool(m.counts["occupied"] == occ and m.counts["triangles"] == tri))
print(json.dumps(out))
"""


@pytest.mark.parametrize("cfg", [0, 1, 2, 3, 4, 5])
def test_classify_config_matches_oracle(cfg):
    env = dict(os.environ, MCG_CLS_CFG=str(cfg))
    r = subprocess.run([sys.executable, "-c", CHILD, REPO], env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    res = json.loads(r.stdout.strip().splitlines()[-1])
    assert all(res), res
