"""Pattern set and synthetic evaluator weights for the think-mode fixtures.

The reference's think mode reads a feature file and a value file (main.cu:74,
eval.cu:12-60) whose trained values are not published, so the fixtures use a
pattern set of this project's own choosing, written in the reference's
feature-file format (a count, then 8 rows of 8 binary digits per feature,
each row read as a std::bitset<8> and shifted to byte j, eval.cu:15-24), and
weights drawn from a fixed integer generator (splitmix64), written in the
reference's value-file format (per feature 3^popcount doubles, then one
double offset, native byte order, eval.cu:30-51).  The generator is plain
integer arithmetic, so the same bytes come out on every machine.
"""
import struct

import numpy as np


def _diagonal():
    return ["".join("1" if c == r else "0" for c in range(8)) for r in range(8)]


# feature masks as 8 row strings (row j is byte j of the mask)
PATTERNS = [
    ["11111111"] + ["00000000"] * 7,                      # row 1
    ["00000000", "11111111"] + ["00000000"] * 6,          # row 2
    ["00000000"] * 2 + ["11111111"] + ["00000000"] * 5,   # row 3
    ["00000000"] * 3 + ["11111111"] + ["00000000"] * 4,   # row 4
    ["11100000"] * 3 + ["00000000"] * 5,                  # 3x3 corner
    ["11110000", "11110000", "11000000"] + ["00000000"] * 5,  # 10-square corner
    _diagonal(),                                          # main diagonal
    ["01111110", "00111100"] + ["00000000"] * 6,          # edge wedge
    ["00100000", "00010000", "00001000", "00000100", "00000010", "00000001",
     "00000000", "00000000"],                             # 6-square diagonal
    ["11000000", "10000000"] + ["00000000"] * 6,          # 3-square corner
]

SEED = 20261203
SCALE = 5.0
OFFSET = 0.3752


def mask_of(rows):
    """The reference's reading of 8 rows: row j is a std::bitset<8> built
    from the string (first character = bit 7), shifted left by 8j."""
    m = 0
    for j, s in enumerate(rows):
        m |= int(s, 2) << (8 * j)
    return m


def features():
    return [mask_of(r) for r in PATTERNS]


def splitmix64_stream(seed, n):
    out = np.zeros(n, np.uint64)
    x = seed & 0xFFFFFFFFFFFFFFFF
    mask = 0xFFFFFFFFFFFFFFFF
    for i in range(n):
        x = (x + 0x9E3779B97F4A7C15) & mask
        z = x
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & mask
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & mask
        out[i] = z ^ (z >> 31)
    return out


def values(feats=None, seed=SEED, scale=SCALE):
    """All tables in feature order: uniform in [-scale, scale), 53-bit
    fractions of splitmix64 outputs."""
    feats = features() if feats is None else feats
    total = sum(3 ** bin(f).count("1") for f in feats)
    z = splitmix64_stream(seed, total)
    u = (z >> np.uint64(11)).astype(np.float64) * (1.0 / (1 << 53))
    return (u * 2.0 - 1.0) * scale


def write_features(path, rows_list=None):
    rows_list = PATTERNS if rows_list is None else rows_list
    with open(path, "w") as f:
        f.write("%d\n" % len(rows_list))
        for rows in rows_list:
            f.write("\n".join(rows) + "\n\n")


def write_values(path, vals=None, offset=OFFSET):
    vals = values() if vals is None else vals
    with open(path, "wb") as f:
        f.write(np.asarray(vals, np.float64).tobytes())
        f.write(struct.pack("=d", offset))


def edge_boards():
    """Hand-made positions: the start, a root that must pass, a finished
    game with empty squares, full boards, and a near-full board."""
    start = (0x0000000810000000, 0x0000001008000000)
    must_pass = (1 << 9, 1 << 0)           # B2 vs A1: only the opponent can move
    over = (1 << 0, (1 << 62) | (1 << 63))  # nobody can move, 61 empties
    full_a = (0x00000000FFFFFFFF, 0xFFFFFFFF00000000)
    full_b = (0xFFFFFFFFFFFF0000, 0x000000000000FFFF)
    near = (0xFFFFFFFFFFFFFF00 & ~(1 << 63), 0x00000000000000FC)
    return [start, must_pass, over, full_a, full_b, near]
