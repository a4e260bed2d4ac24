"""Known-answer cases of the text-record loader, shared by the oracle and
GPU tests.  Window: dim 2 at origin (10, 20, 0), i.e. x in [10, 12),
y in [20, 22), z in [0, 2); eight slots in arrival order (z fastest)."""

DIM = 2
ORIGIN = (10, 20, 0)
I32_MAX = 2 ** 31 - 1


def slots(vol):
    """(sdf, w) per arrival slot s: zi = s % dim, yi = s / dim % dim, xi = s / dim^2."""
    d = vol.shape[0]
    out = []
    for s in range(d ** 3):
        zi, yi, xi = s % d, (s // d) % d, s // (d * d)
        out.append((int(vol[zi, yi, xi, 0]), int(vol[zi, yi, xi, 1])))
    return out


def i16(v):
    return ((v + 2 ** 15) % 2 ** 16) - 2 ** 15


# text -> (stored (sdf, w) in arrival order, status)
KAT = [
    # trailing newline: the loop runs once more, all extractions fail at end
    # of file and the last record is evaluated again
    (b"10 20 0 5 6\n10 20 1 7 8\n", [(5, 6), (7, 8), (7, 8)], 0),
    # no trailing white space: the last field sets eofbit, no repeat
    (b"10 20 0 5 6\n10 20 1 7 8", [(5, 6), (7, 8)], 0),
    # a repeated record outside the window stores nothing
    (b"10 20 0 5 6\n9 20 0 7 8\n", [(5, 6)], 0),
    # trailing spaces only
    (b"10 20 0 5 6 \t ", [(5, 6), (5, 6)], 0),
    # partial last record: x, y fresh, z, sdf, w kept from the record before
    (b"10 20 0 5 6\n11 21", [(5, 6), (5, 6)], 0),
    (b"10 20 0 5 6\n11 21 \n", [(5, 6), (5, 6)], 0),
    (b"10 20 0 5 6\n11 21 1 9", [(5, 6), (9, 6)], 0),
    # records outside the window are skipped
    (b"9 20 0 1 1\n10 20 0 2 2\n10 22 0 3 3\n10 21 2 9 9\n10 21 1 4 4", [(2, 2), (4, 4)], 0),
    # signs, every white-space character, fields split only by a sign
    (b"+10 20 0 -5 6 10\t20\r1 +7\v8", [(-5, 6), (7, 8)], 0),
    (b"10 20 0 5 6 10 20 1-3 4\f", [(5, 6), (-3, 4), (-3, 4)], 0),
    (b"010 020 00 0005 06", [(5, 6)], 0),
    # short / ushort conversion of the int fields
    (b"10 20 0 40000 70000 10 20 1 -40000 -1", [(i16(40000), i16(70000)), (i16(-40000), -1)], 0),
    (b"10 20 0 -2147483648 2147483647", [(0, -1)], 0),
    # a bad character inside the window: weight 0, the record repeats into
    # every remaining slot
    (b"10 20 0 5 6\n10 20 1 7x 8\n", [(5, 6)] + [(7, 0)] * 7, 0),
    # "--5": the sdf field has no digits -> 0; weight keeps its value (0)
    (b"10 20 0 --5 6", [(0, 0)] * 8, 0),
    # int overflow inside the window: INT_MAX as weight, repeats
    (b"10 20 0 5 99999999999 10 20 1 1 1", [(5, -1)] * 8, 0),
    # overflow running into end of file: evaluated once
    (b"10 20 0 5 6\n10 20 1 3 -99999999999", [(5, 6), (3, 0)], 0),
    # a sign at end of file: no digits (0), end of file, evaluated once
    (b"10 20 0 5 6\n10 20 1 3 -", [(5, 6), (3, 0)], 0),
    # a bad character that leaves the record outside the window: the
    # reference never leaves its loop (status 1)
    (b"10 20 0 5 6\nabc 1 2 3 4\n", [(5, 6)], 1),
    (b"2147483648 20 0 1 1\n", [], 1),
    # empty and white-space-only texts: one iteration over zeros
    (b"", [], 0),
    (b" \n\n ", [], 0),
    # more records than slots: the loop ends after the eighth
    (b"".join(b"10 20 0 %d %d\n" % (i, i + 1) for i in range(12)), [(i, i + 1) for i in range(8)], 0),
]
