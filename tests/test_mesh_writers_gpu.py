"""Mesh writers on the GPU (mcg_mesh_ply / mcg_mesh_obj / mcg_mesh_write)
against the oracle (the reference's writers over glibc stdio): the same
bytes for PLY, OBJ and the qi_volume listing."""
import numpy as np
import pytest
import torch

import oracle
from marching_cube_gb300 import synthetic
from mesh_cases import crafted, soup

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mcg():
    import marching_cube_gb300 as m
    return m


def as_mesh(mcg, s, n):
    s = torch.from_numpy(np.ascontiguousarray(s)).cuda()
    n = torch.from_numpy(np.ascontiguousarray(n, np.float32)).cuda()
    return mcg.Mesh(s, n, counts={"vertices": s.shape[0], "triangles": s.shape[0] // 3})


def check(mcg, s, n):
    m = as_mesh(mcg, s, n)
    assert mcg.mesh_ply(m) == oracle.mesh_ply(s, n)
    assert mcg.mesh_obj(m) == oracle.mesh_obj(s, n)


def test_crafted(mcg):
    s, n = crafted()
    check(mcg, s, n)
    check(mcg, s[:0], n[:0])
    check(mcg, s[:7], n[:7])  # a soup that does not end on a triangle


def test_key_collisions(mcg):
    """Positions on a 10^-4 grid plus offsets that stay inside or cross the
    rounding boundary: many different floats per printed key."""
    rng = np.random.default_rng(3)
    base = rng.integers(0, 3000, size=(30000, 3)) / 1e4
    off = rng.choice([0.0, 2e-5, -2e-5, 4.9e-5, -4.9e-5, 5.1e-5, 1e-7], size=(30000, 3))
    p = (base + off).astype(np.float32)
    p[rng.random(30000) < 0.01] *= -1
    nrm = rng.normal(size=(30000, 3)).astype(np.float32)
    nrm[rng.random((30000, 3)) < 0.05] = -0.0
    vox = rng.integers(-5, 600, size=(30000, 3))
    s = soup(p, vox, rng.integers(-32767, 32768, 30000), rng.integers(-32768, 32768, 30000))
    check(mcg, s, nrm)


def test_extracted_meshes(mcg):
    """Soups and normals of real extractions: the C1 sphere (128^3, 1 cm) and
    a 160^3 stress volume (spheres + gradient noise, 3 mm voxels)."""
    for data, cell in ((torch.from_numpy(synthetic.sphere_volume(128)).cuda(), 0.01),
                       (synthetic.stress_volume(160, seed=4, n_spheres=30), 0.003)):
        mesh = mcg.extract(data, cell, soup=True, normals=True)
        nv = mesh.num_vertices
        assert nv > 1000
        s = mesh.soup[:nv].cpu().numpy()
        n = mesh.normals[:nv].cpu().numpy()
        assert mcg.mesh_ply(mesh) == oracle.mesh_ply(s, n)
        assert mcg.mesh_obj(mesh) == oracle.mesh_obj(s, n)


def test_files_and_errors(mcg, tmp_path):
    s, n = crafted()
    m = as_mesh(mcg, s, n)
    mcg.mesh_write(m, str(tmp_path / "a.ply"))
    mcg.mesh_write(m, str(tmp_path / "a.obj"), qi_path=str(tmp_path / "qi_volume.txt"))
    assert (tmp_path / "a.ply").read_bytes() == oracle.mesh_ply(s, n)
    obj, qi = oracle.mesh_obj(s, n)
    assert (tmp_path / "a.obj").read_bytes() == obj and (tmp_path / "qi_volume.txt").read_bytes() == qi
    with pytest.raises(mcg.MCGError) as e:
        mcg.mesh_write(m, str(tmp_path / "a.stl"))
    assert e.value.status == mcg.MCG_ERR_INVALID_ARG
    far = soup(np.array([[200.0, 1.0, 1.0]] * 3, np.float32))
    with pytest.raises(mcg.MCGError) as e:
        mcg.mesh_obj(as_mesh(mcg, far, np.zeros((3, 3), np.float32)))
    assert e.value.status == mcg.MCG_ERR_TOO_LARGE
