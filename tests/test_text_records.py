"""Text-record volume loader: the oracle (the reference loop over libstdc++
streams, kf.cu:3289-3361) against known answers written from the C++ rules
for `is >> int` (C++11 [istream.formatted.arithmetic], [facet.num.get.virtuals]):

  * white space is skipped first; reaching end of file there sets eofbit and
    failbit and leaves the value unchanged;
  * a field is an optional sign and decimal digits; no digits -> value 0 and
    failbit; outside int -> INT_MAX / INT_MIN and failbit; a field that runs
    into end of file sets eofbit;
  * once the stream is not good, the remaining extractions leave their values
    unchanged;
  * the loop evaluates the record after every five extractions and stops at
    eofbit; a failed stream that never reaches end of file repeats the same
    record forever (it fills the window when the record lies inside it).

Window of these cases: dim 2 at origin (10, 20, 0), i.e. x in [10, 12),
y in [20, 22), z in [0, 2); eight slots in arrival order (z fastest).
No GPU needed.
"""
import numpy as np
import pytest

import oracle

from text_cases import DIM, I32_MAX, KAT, ORIGIN, i16, slots  # noqa: F401


@pytest.mark.parametrize("case", range(len(KAT)))
def test_oracle_known_answers(case):
    text, want, status = KAT[case]
    vol, st = oracle.text_load(text, DIM, ORIGIN)
    got = slots(vol)
    assert got[:len(want)] == want, (text, got)
    assert all(v == (0, 0) for v in got[len(want):])
    assert st["stored"] == len(want)
    assert st["status"] == status


def test_oracle_file_tail(tmp_path):
    text = b"10 20 0 1 1\n10 20 1 2 2\n10 21 0 3 3\n"
    p = tmp_path / "dump.txt"
    p.write_bytes(text)
    n = len(text)
    # tail at least the file: the whole file, no line skipped
    vol, st = oracle.text_load_file(str(p), DIM, ORIGIN, tail_bytes=n)
    assert slots(vol)[:4] == [(1, 1), (2, 2), (3, 3), (3, 3)]
    # a tail starting inside line 1 skips the rest of that line
    vol, st = oracle.text_load_file(str(p), DIM, ORIGIN, tail_bytes=n - 3)
    assert slots(vol)[:3] == [(2, 2), (3, 3), (3, 3)] and st["stored"] == 3
    # a tail starting exactly at a line start skips that whole line
    vol, st = oracle.text_load_file(str(p), DIM, ORIGIN, tail_bytes=n - 12)
    assert slots(vol)[:2] == [(3, 3), (3, 3)] and st["stored"] == 2
    # the cut line reaches end of file: the loop does not run
    p.write_bytes(b"10 20 0 1 1\n10 20 1 2 2")
    vol, st = oracle.text_load_file(str(p), DIM, ORIGIN, tail_bytes=5)
    assert st["stored"] == 0 and st["iterations"] == 0


def test_oracle_arrival_order():
    """Window records fill z fastest, then y, then x (kf.cu:3330-3352)."""
    d = 3
    recs = []
    rng = np.random.default_rng(5)
    vals = rng.integers(-32767, 32768, size=d ** 3)
    for i, (x, y, z) in enumerate((x, y, z) for x in range(d) for y in range(d) for z in range(d)):
        recs.append(b"%d %d %d %d %d\n" % (100 + x, 200 + y, 7 + z, vals[i], i))
    vol, st = oracle.text_load(b"".join(recs), d, (100, 200, 7))
    assert st["stored"] == d ** 3
    for i, (x, y, z) in enumerate((x, y, z) for x in range(d) for y in range(d) for z in range(d)):
        assert tuple(vol[z, y, x]) == (vals[i], i)
