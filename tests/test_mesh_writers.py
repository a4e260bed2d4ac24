"""Mesh writers: the oracle (the reference's writers over glibc stdio,
kf.cu:3394-3424 and 3625-3726) against known answers.  No GPU needed."""
import numpy as np

import oracle
from mesh_cases import crafted, soup


def test_obj_known_answer():
    s, n = crafted()
    obj, qi = oracle.mesh_obj(s, n)
    lines = obj.decode().splitlines()
    v = [l for l in lines if l.startswith("v ")]
    vn = [l for l in lines if l.startswith("vn ")]
    f = [l for l in lines if l.startswith("f ")]
    # keys: 0.1000_0.2000_0.3000 (x2), 1.0000_2.0000_3.0000, 0.0312_0.0078_1.5000 (x2),
    # 2.0000_2.0000_2.0000, -0.0000_0.5000_0.5000 (x2: -0.00001 and -0.0), 0.0000_0.5000_0.5000,
    # 100.0000_12.3456_0.0000 and 99.9999_12.3457_0.0001 ... distinct
    assert v[0] == "v 0.100000 0.200000 0.300000"
    assert v[2] == "v 0.031250 0.007812 1.500000"  # 1/128 prints with the tie to even
    assert v[4] == "v -0.000010 0.500000 0.500000" and v[5] == "v 0.000000 0.500000 0.500000"
    assert len(v) == len(vn) == 9
    assert vn[0] == "vn 0.000000 -0.000000 1.000000"
    assert vn[1] == "vn -0.600000 0.800000 0.000000"  # the normal of soup vertex 2
    assert vn[2] == "vn 0.007812 -0.023438 0.039062"  # 7812.5 -> 7812, 23437.5 -> 23438, 39062.5 -> 39062
    # triangles 0-2 have two equal ids and are dropped: 0.1 / 0.10001 share
    # "0.1000", 0.03125 / 0.0312 share "0.0312" (312.5 ties to even), -0.00001
    # and -0.0 share "-0.0000"; triangle 3 keeps three keys ("99.9999" twice in
    # x but 12.3456 / 12.3457 in y)
    assert f == ["f 7 8 9", "f 1 2 4"]
    assert qi.decode().splitlines()[0] == "qi tsdf w vx vy vz"
    assert qi.decode().splitlines()[1] == "1 -32766 0 -7 -6 -5"
    assert qi.decode().splitlines()[4] == "4 5 3 8 9 10"


def test_ply_known_answer():
    s, n = crafted()
    ply = oracle.mesh_ply(s, n)
    head, body = ply.split(b"end_header\n", 1)
    assert head.startswith(b"ply\nformat binary_little_endian 1.0\nelement vertex 15\n")
    assert b"element face 5\nproperty list uint8 int32 vertex_indices\n" in head
    assert len(body) == 15 * 24 + 5 * 13
    vb = np.frombuffer(body[:15 * 24], np.float32).reshape(15, 6)
    assert np.array_equal(vb[:, :3].view(np.uint32), s[:, :12].copy().view(np.float32).reshape(15, 3).view(np.uint32))
    assert np.array_equal(vb[:, 3:].view(np.uint32), n.view(np.uint32))
    fb = np.frombuffer(body[15 * 24:], np.uint8).reshape(5, 13)
    assert (fb[:, 0] == 3).all()
    assert np.array_equal(fb[:, 1:].copy().view(np.int32).reshape(5, 3), np.arange(15).reshape(5, 3))


def test_empty_soup():
    obj, qi = oracle.mesh_obj(soup(np.zeros((0, 3))), np.zeros((0, 3), np.float32))
    assert obj == b"" and qi == b"qi tsdf w vx vy vz\n"
