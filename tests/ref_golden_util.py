"""Loading the fixtures that the reference's own source produced
(tests/golden/ref/, made by tests/golden/make_ref_golden.py)."""
import glob
import os

import numpy as np

REF_GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref")


def load(name):
    d = np.load(os.path.join(REF_GOLDEN, name))
    return {k: d[k] for k in d.files}


def mesh_cases():
    return sorted(os.path.basename(p) for p in glob.glob(os.path.join(REF_GOLDEN, "*.npz")))


def poses(g):
    return [(p[:9].reshape(3, 3), p[9:]) for p in g["poses"]]


def rle_body(img, nz):
    """Per-slice sizes and the concatenated slice bytes of an RLE volume image
    (40-byte header, then per slice a 4-byte size and the records)."""
    b = bytes(img)
    o, sizes, body = 40, [], []
    for _ in range(nz):
        s = int.from_bytes(b[o:o + 4], "little")
        sizes.append(s)
        body.append(b[o + 4:o + 4 + s])
        o += 4 + s
    assert o == len(b)
    return np.array(sizes, np.int64), np.frombuffer(b"".join(body), np.uint8)
