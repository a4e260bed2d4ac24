"""Text-record volume loader on the GPU (mcg_text_records_*) against the
oracle (the reference loop over libstdc++ streams, kf.cu:3289-3361):
bit-exact volumes, the same stored count, and MCG_ERR_FORMAT exactly where
the reference's loop would never end."""
import numpy as np
import pytest
import torch

import oracle
from text_cases import DIM, KAT, ORIGIN

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mcg():
    import marching_cube_gb300 as m
    return m


def gpu_load(mcg, source, dim, origin, **kw):
    stats = {}
    try:
        v = mcg.load_text_records(source, dim, origin, stats=stats, **kw)
        return v.data.cpu().numpy(), stats, 0
    except mcg.MCGError as e:
        assert e.status == mcg.MCG_ERR_FORMAT, e
        return None, stats, 1


def check(mcg, text, dim, origin, variants=("host", "device")):
    want, st = oracle.text_load(text, dim, origin)
    for how in variants:
        if how == "host":
            src = text
        elif how == "device":
            src = torch.frombuffer(bytearray(text), dtype=torch.uint8).cuda() if text else \
                torch.zeros(0, dtype=torch.uint8, device="cuda")
        else:  # device, 16-byte misaligned start
            buf = torch.zeros(len(text) + 3, dtype=torch.uint8, device="cuda")
            if text:
                buf[3:] = torch.frombuffer(bytearray(text), dtype=torch.uint8).cuda()
            src = buf[3:]
        got, stats, status = gpu_load(mcg, src, dim, origin)
        assert status == st["status"], (how, text[:200])
        assert stats["stored"] == st["stored"], (how, stats, st)
        if got is not None:
            assert np.array_equal(got, want), (how, text[:200])


@pytest.mark.parametrize("case", range(len(KAT)))
def test_known_answers(mcg, case):
    check(mcg, KAT[case][0], DIM, ORIGIN, ("host", "device", "misaligned"))


def _random_text(rng, n_records, dim, origin, p_bad=0.0):
    """Records around the window with every white-space byte, signs, leading
    zeros, long digit runs and (optionally) malformed fields."""
    ws = [b" ", b"\t", b"\n", b"\r\n", b"  ", b"\v", b"\f"]
    out = []
    for _ in range(n_records):
        rec = []
        for f in range(5):
            if f < 3:
                v = int(origin[f] + rng.integers(-2, dim + 2))
            elif f == 3:
                v = int(rng.integers(-40000, 40000))
            else:
                v = int(rng.integers(-5, 70000))
            s = str(v).encode()
            r = rng.random()
            if r < 0.03:
                s = (b"+" + s) if v >= 0 else s
            elif r < 0.06:
                s = (b"-" if v < 0 else b"") + b"000" + str(abs(v)).encode()
            if p_bad and rng.random() < p_bad:
                s = rng.choice([b"x", b"+", b"-", b"1.5", b"99999999999", b"--3", b"7a"])
            rec.append(s)
        for i, s in enumerate(rec):
            out.append(s)
            if i == 4:
                out.append(b"\n" if rng.random() < 0.9 else ws[int(rng.integers(len(ws)))])
            elif rng.random() < 0.02 and rec[i + 1][:1] in (b"-", b"+") and s[-1:].isdigit():
                pass  # no separator: the sign starts the next field
            else:
                out.append(ws[int(rng.integers(len(ws)))] if rng.random() < 0.2 else b" ")
    text = b"".join(out)
    cut = rng.random()
    if cut < 0.2:
        text = text.rstrip()
    elif cut < 0.3:
        text = text[: int(rng.integers(0, len(text) + 1))]
    return text


def test_random_texts(mcg):
    rng = np.random.default_rng(11)
    for it in range(120):
        dim = int(rng.integers(1, 6))
        origin = tuple(int(v) for v in rng.integers(-3, 600, size=3))
        n = int(rng.integers(0, 3 * dim ** 3 + 4))
        text = _random_text(rng, n, dim, origin, p_bad=0.02 if it % 3 == 0 else 0.0)
        check(mcg, text, dim, origin)


def test_segment_boundaries(mcg):
    """Texts of several 16 KiB segments: fields straddle 64-byte slices and
    segment ends; leading-zero runs longer than a slice."""
    rng = np.random.default_rng(12)
    for it in range(12):
        dim = 12
        origin = (100, 200, 300)
        text = _random_text(rng, 3000 + 997 * it, dim, origin, p_bad=0.0005 if it % 2 else 0.0)
        if it == 5:
            text = b"100 200 300 " + b"0" * 200 + b"7 8\n" + text
        check(mcg, text, dim, origin, ("host", "device", "misaligned"))


def test_file_tail(mcg, tmp_path):
    rng = np.random.default_rng(13)
    dim, origin = 6, (512, 512, 0)
    text = _random_text(rng, 2000, dim, origin)
    p = tmp_path / "dump.vol"
    p.write_bytes(text)
    n = len(text)
    for tail in (n + 10, n, n - 1, n - 7, n // 2, 40, 3, 1):
        want, st = oracle.text_load_file(str(p), dim, origin, tail_bytes=tail)
        got, stats, status = gpu_load(mcg, str(p), dim, origin, tail_bytes=tail)
        assert status == st["status"] and stats["stored"] == st["stored"], tail
        if got is not None:
            assert np.array_equal(got, want), tail
    # tail_bytes=None: the whole file
    want, st = oracle.text_load(text, dim, origin)
    got, stats, status = gpu_load(mcg, str(p), dim, origin, tail_bytes=None)
    assert np.array_equal(got, want)
    with pytest.raises(mcg.MCGError) as e:
        mcg.load_text_records(str(tmp_path / "missing.vol"), dim, origin)
    assert e.value.status == mcg.MCG_ERR_IO


def test_dump_128_against_oracle(mcg):
    """A 128^3 window inside a 136 x 132 x 140 dump (out-of-window records on
    every side), ~2.5M records, through host memory."""
    from marching_cube_gb300 import synthetic
    g = torch.Generator(device="cuda").manual_seed(3)
    box = (140, 132, 136)  # nz, ny, nx
    vals = torch.randint(-32767, 32768, box + (2,), generator=g, device="cuda", dtype=torch.int32).to(torch.int16)
    origin = (512, 512, 0)
    box_origin = (origin[0] - 3, origin[1] - 2, origin[2] - 5)
    text = synthetic.text_dump(vals, box_origin).cpu().numpy().tobytes()
    want, st = oracle.text_load(text, 128, origin)
    got, stats, status = gpu_load(mcg, text, 128, origin)
    assert status == 0 and stats["stored"] == st["stored"] == 128 ** 3
    assert np.array_equal(got, want)
    # the window of the source volume, voxel for voxel
    ref = vals[5:133, 2:130, 3:131].cpu().numpy()
    assert np.array_equal(got, ref)


def test_dump_512_round_trip(mcg):
    """Full size: a 512^3 window dump (134M records, ~3 GB of text) loads
    back to its source volume (no oracle: size-independent property)."""
    from marching_cube_gb300 import synthetic
    n = 512
    g = torch.Generator(device="cuda").manual_seed(4)
    vals = torch.randint(-32767, 32768, (n, n, n, 2), generator=g, device="cuda", dtype=torch.int32)
    vals = vals.to(torch.int16)
    text = synthetic.text_dump(vals, (512, 512, 0))
    stats = {}
    v = mcg.load_text_records(text, n, stats=stats)
    assert stats["stored"] == n ** 3 and stats["fail_offset"] == -1
    assert torch.equal(v.data, vals)
    host = text.cpu().numpy()
    del text
    v2 = mcg.load_text_records(host, n, out=v.data)
    assert torch.equal(v2.data, vals)


def test_chunk_pipeline(mcg, tmp_path):
    """Texts longer than the 64 MiB copy/parse chunks: records straddling
    chunk ends, a field longer than a whole chunk (parsed again once the
    text is resident), and a failure two chunks in; host memory and file."""
    chunk = 64 << 20
    filler = b"9 20 0 1 1\n"  # x = 9: outside the window
    a = filler * (chunk // len(filler) + 1001)
    big = b"10 20 1 " + b"0" * (chunk + 12345) + b"7 8\n"
    text = a + b"10 20 0 3 4\n" + big + filler * 999 + b"11 21 1 -5 6"
    check(mcg, text, DIM, ORIGIN, ("host",))
    p = tmp_path / "long.vol"
    p.write_bytes(text)
    want, st = oracle.text_load(text, DIM, ORIGIN)
    got, stats, status = gpu_load(mcg, str(p), DIM, ORIGIN, tail_bytes=None)
    assert status == 0 and stats["stored"] == st["stored"] and np.array_equal(got, want)
    bad = a + filler * 600000 + b"10 20 0 3 4\n10 20 1 7x 8\n" + filler * 10
    check(mcg, bad, DIM, ORIGIN, ("host",))
