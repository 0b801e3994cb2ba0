"""base81 board codec and board files (Python side, for tests and tools).

Same format as the C++ host layer (host/boardfile.cpp): character i covers
squares 4i..4i+3; square j adds w_j for the side to move and 2*w_j for the
other side, w = (1, 3, 9, 32), plus 33 (test.cpp:7-19, to_board.cpp:15-39).
"""
import numpy as np

_W = (1, 3, 9, 32)


def encode(p, o):
    out = []
    for i in range(16):
        v = 33
        for j in range(4):
            sq = 4 * i + j
            if (p >> sq) & 1:
                v += _W[j]
            if (o >> sq) & 1:
                v += 2 * _W[j]
        out.append(chr(v))
    return "".join(out)


def decode(s):
    if len(s) < 16:
        raise ValueError("board string shorter than 16 characters")
    p = o = 0
    for i in range(16):
        v = ord(s[i]) - 33
        if v < 0 or v > 90:
            raise ValueError("character %r outside the base81 alphabet" % s[i])
        hi, lo = v >> 5, v & 31
        if hi > 2 or lo > 26:
            raise ValueError("character %r outside the base81 alphabet" % s[i])
        for j, d in enumerate((lo % 3, (lo // 3) % 3, lo // 9, hi)):
            if d == 1:
                p |= 1 << (4 * i + j)
            elif d == 2:
                o |= 1 << (4 * i + j)
    return p, o


def read_board_file(path):
    """Boards of a board file in file order (no sort/dedup), as uint64 arrays."""
    with open(path) as f:
        n = int(f.readline().split()[0])
        lines = [f.readline() for _ in range(n)]
    p = np.zeros(n, np.uint64)
    o = np.zeros(n, np.uint64)
    for i, ln in enumerate(lines):
        p[i], o[i] = decode(ln)
    return p, o


def write_board_file(path, p, o):
    with open(path, "w") as f:
        f.write("%d\n" % len(p))
        for a, b in zip(p, o):
            f.write(encode(int(a), int(b)) + "\n")


def read_result_file(path):
    """{board string: (score, extra columns...)} from "<board> <score> ..." lines."""
    out = {}
    with open(path) as f:
        for ln in f:
            parts = ln.split()
            if parts:
                out[parts[0]] = tuple(int(x) for x in parts[1:])
    return out


def empties(p, o):
    x = np.asarray(p, np.uint64) | np.asarray(o, np.uint64)
    return 64 - np.array([bin(int(v)).count("1") for v in x], np.int64)
