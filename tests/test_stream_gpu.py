"""ExtractStream: a sequence of host volumes extracted with the copies in
both directions overlapped gives, volume by volume, the soup and normals of
the plain extraction."""
import numpy as np
import pytest
import torch

from marching_cube_gb300 import synthetic

pytestmark = pytest.mark.gpu


def test_stream_matches_plain(mcg):
    vols = [synthetic.sphere_volume(96, radius=r, seed=i) for i, r in enumerate((20.0, 30.0, 35.0, 25.0, 40.0))]
    cap = 400000
    hv = [torch.from_numpy(v).pin_memory() for v in vols]
    outs = [{"soup": torch.zeros((cap, 28), dtype=torch.uint8).pin_memory(),
             "normals": torch.zeros((cap, 3), dtype=torch.float32).pin_memory()} for _ in vols]
    st = mcg.ExtractStream((96, 96, 96), 0.01, cap)
    res = st.run(hv, outs)
    for v, r, o in zip(vols, res, outs):
        m = mcg.extract(torch.from_numpy(v).cuda(), 0.01, soup=True, normals=True)
        n = m.num_vertices
        assert r["vertices"] == n and r["status"] == 0
        assert np.array_equal(o["soup"][:n].numpy(), m.soup.cpu().numpy())
        assert np.array_equal(o["normals"][:n].numpy().view(np.uint32), m.normals.cpu().numpy().view(np.uint32))
    # a capacity too small for the largest volume: cut soup, status reported
    st2 = mcg.ExtractStream((96, 96, 96), 0.01, 1000)
    small = [{"soup": torch.zeros((1000, 28), dtype=torch.uint8).pin_memory(), "normals": None}] * 2
    r2 = st2.run(hv[:2], small)
    assert all(r["status"] == mcg.MCG_ERR_CAPACITY for r in r2)
