"""Regenerates the golden fixtures in this directory from the reference itself.

Runs in a checkout that has the reference sources (it builds them with
oracle/ref_build.sh into oracle/_ref/) on an x86-64 host; nothing at test
time runs it.  Inputs come from the oracle's seeded random-playout generator
(oracle.c, orc_generate), so the board files also pin the generator.

Fixtures (all board files use the reference's input format: a count line,
then one 16-char base81 board per line; *.ref files are the reference's
output lines "<base81> <score> <loop steps>", one per unique board, in the
reference's ascending (player, opponent) order, from `refsolve --per-board`):

  c1_seed0_e10.txt / .ref    4,096 positions, seed 0, 10 empties, DEPTH 10
  c3_seed2_mixed.txt / .ref  first 256 positions of seed 2 (8..16 empties),
                             DEPTH 16
  c4_seed4_e18.txt / .ref    first 16 positions of seed 4 (18 empties),
                             DEPTH 18
  c5_seed5_e20_22.txt / .ref first 4 positions of seed 5 (20..22 empties),
                             DEPTH 22
  readme9.txt / .ref         the 9 board lines shown in the reference
                             README (README.md:11-19), DEPTH 10
  lop_seed21_e11_12.txt/.ref 48 lopsided positions of seed 21 (11..12
                             empties): the first whose score the oracle's
                             alpha-beta puts at |score| >= 40 in under
                             100,000 nodes (games where one side passes
                             again and again), DEPTH 12; the scores in the
                             .ref file are the reference's own
  codec_vectors.txt          2,000 random disjoint boards encoded by the
                             reference's fromBoard ("<p hex> <o hex> <str>")

Think mode (reference's eval.cu + thinker.cu, `refthink --per-board`), with
the pattern set and synthetic weights of think_data.py; *.ref lines are
"<base81> <score> <best move> <loop steps>":

  think_seed6_e24_34_d6      240 positions, seed 6, 24..34 empties, depth 6
  think_seed7_e6_12_d4       400 positions, seed 7, 6..12 empties, depth 4
  think_seed8_e20_28_d8      24 positions, seed 8, 20..28 empties, depth 8
  think_edge_d5              think_data.edge_boards(), depth 5
  eval_vectors.txt           Evaluator::eval of 2,000 positions of seed 9
                             (4..60 empties) and the edge boards,
                             "<p hex> <o hex> <float bits hex>"

Usage: python tests/golden/make_golden.py [--only NAME ...]
"""
import argparse
import ctypes
import os
import subprocess
import sys
import tempfile
from concurrent.futures import ThreadPoolExecutor

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

README9 = None  # read from the reference README at run time (lines 11-19)

THINK_FIXTURES = {
    # name: (seed, count, min_empties, max_empties, think depth)
    "think_seed6_e24_34_d6": (6, 240, 24, 34, 6),
    "think_seed7_e6_12_d4": (7, 400, 6, 12, 4),
    "think_seed8_e20_28_d8": (8, 24, 20, 28, 8),
}

FIXTURES = {
    # name: (seed, count, min_empties, max_empties, depth)
    "c1_seed0_e10": (0, 4096, 10, 10, 10),
    "c3_seed2_mixed": (2, 256, 8, 16, 16),
    "c4_seed4_e18": (4, 16, 18, 18, 18),
    "c5_seed5_e20_22": (5, 4, 20, 22, 22),
}


def _oracle():
    from gpuothello2_gb300 import build as B

    B.build_oracle()
    lib = ctypes.CDLL(B.ORACLE_LIB)
    u64 = ctypes.c_uint64
    lib.orc_generate.argtypes = [u64, u64, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                 ctypes.c_void_p, ctypes.c_void_p]
    lib.orc_encode.argtypes = [u64, u64, ctypes.c_char_p]
    return lib


def write_boards(path, lines):
    with open(path, "w") as f:
        f.write("%d\n" % len(lines))
        for s in lines:
            f.write(s + "\n")


def generate_lines(lib, seed, count, lo, hi):
    p = np.zeros(count, np.uint64)
    o = np.zeros(count, np.uint64)
    lib.orc_generate(seed, 0, count, lo, hi, p.ctypes.data, o.ctypes.data)
    buf = ctypes.create_string_buffer(17)
    out = []
    for i in range(count):
        lib.orc_encode(int(p[i]), int(o[i]), buf)
        out.append(buf.value.decode())
    return out


def lopsided_lines(lib, seed, lo, hi, count):
    """The first `count` positions of the stream whose score the oracle's
    alpha-beta puts at |score| >= 40 within 100,000 nodes (selection only;
    the fixture's scores come from the reference)."""
    from tests.oracle_lib import Oracle
    from gpuothello2_gb300 import build as B

    orc = Oracle(B.ORACLE_LIB)
    p, o = orc.generate(seed, 20000, lo, hi)
    sc, _, nodes, _ = orc.solve_batch(p, o, mode=1)
    pick = np.nonzero((np.abs(sc.astype(int)) >= 40) & (nodes < 100000))[0][:count]
    buf = ctypes.create_string_buffer(17)
    out = []
    for i in pick:
        lib.orc_encode(int(p[i]), int(o[i]), buf)
        out.append(buf.value.decode())
    return out


def run_reference(refsolve, lines, depth, jobs, prefix=()):
    """Runs the reference per board on `jobs` processes; returns its lines
    re-sorted into the reference's (player, opponent) order.  `prefix` goes
    before the board-file arguments (refthink's feature and value files)."""
    chunks = [lines[i::jobs] for i in range(jobs) if lines[i::jobs]]
    with tempfile.TemporaryDirectory() as td:
        def one(k):
            inp = os.path.join(td, "in%d.txt" % k)
            out = os.path.join(td, "out%d.txt" % k)
            write_boards(inp, chunks[k])
            subprocess.run([refsolve, *prefix, inp, out, str(depth), "--per-board"],
                           check=True, stderr=subprocess.DEVNULL)
            return open(out).read().splitlines()

        with ThreadPoolExecutor(jobs) as ex:
            results = [ln for part in ex.map(one, range(len(chunks))) for ln in part]
    from gpuothello2_gb300 import codec

    uniq = {}
    for ln in results:
        uniq[ln.split()[0]] = ln
    return sorted(uniq.values(), key=lambda ln: codec.decode(ln.split()[0]))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", nargs="*")
    ap.add_argument("--jobs", type=int, default=os.cpu_count())
    args = ap.parse_args()
    subprocess.run([os.path.join(ROOT, "oracle", "ref_build.sh")], check=True)
    refsolve = os.path.join(ROOT, "oracle", "_ref", "refsolve")
    lib = _oracle()
    want = set(args.only) if args.only else None
    for name, (seed, count, lo, hi, depth) in FIXTURES.items():
        if want and name not in want:
            continue
        lines = generate_lines(lib, seed, count, lo, hi)
        write_boards(os.path.join(HERE, name + ".txt"), lines)
        ref = run_reference(refsolve, lines, depth, args.jobs)
        with open(os.path.join(HERE, name + ".ref"), "w") as f:
            f.write("\n".join(ref) + "\n")
        print(name, len(lines), "boards,", len(ref), "unique")
    if not want or "lop_seed21_e11_12" in want:
        lines = lopsided_lines(lib, 21, 11, 12, 48)
        write_boards(os.path.join(HERE, "lop_seed21_e11_12.txt"), lines)
        ref = run_reference(refsolve, lines, 12, args.jobs)
        with open(os.path.join(HERE, "lop_seed21_e11_12.ref"), "w") as f:
            f.write("\n".join(ref) + "\n")
        print("lop_seed21_e11_12", len(lines), "boards,", len(ref), "unique")
    if not want or "readme9" in want:
        readme = open("/root/reference/README.md").read().splitlines()
        lines = [ln.strip() for ln in readme[10:19]]
        write_boards(os.path.join(HERE, "readme9.txt"), lines)
        ref = run_reference(refsolve, lines, 10, 1)
        with open(os.path.join(HERE, "readme9.ref"), "w") as f:
            f.write("\n".join(ref) + "\n")
        print("readme9", len(ref))
    if not want or want & (set(THINK_FIXTURES) | {"think_edge_d5", "eval_vectors"}):
        make_think(lib, want, args.jobs)
    if not want or "codec" in want:
        out = subprocess.run([refsolve, "--codec", "2000", "20261203"], check=True,
                             capture_output=True, text=True).stdout
        with open(os.path.join(HERE, "codec_vectors.txt"), "w") as f:
            f.write(out)
        print("codec_vectors", len(out.splitlines()))


def make_think(lib, want, jobs):
    from tests.golden import think_data as T

    refthink = os.path.join(ROOT, "oracle", "_ref", "refthink")
    with tempfile.TemporaryDirectory() as td:
        feat, val = os.path.join(td, "features.txt"), os.path.join(td, "values.bin")
        T.write_features(feat)
        T.write_values(val)
        buf = ctypes.create_string_buffer(17)

        def encode(pairs):
            out = []
            for p, o in pairs:
                lib.orc_encode(int(p), int(o), buf)
                out.append(buf.value.decode())
            return out

        cases = {name: (generate_lines(lib, seed, count, lo, hi), depth)
                 for name, (seed, count, lo, hi, depth) in THINK_FIXTURES.items()}
        cases["think_edge_d5"] = (encode(T.edge_boards()), 5)
        for name, (lines, depth) in cases.items():
            if want and name not in want:
                continue
            write_boards(os.path.join(HERE, name + ".txt"), lines)
            ref = run_reference(refthink, lines, depth, jobs, prefix=(feat, val))
            with open(os.path.join(HERE, name + ".ref"), "w") as f:
                f.write("\n".join(ref) + "\n")
            print(name, len(lines), "boards,", len(ref), "unique")
        if not want or "eval_vectors" in want:
            lines = generate_lines(lib, 9, 2000, 4, 60) + encode(T.edge_boards())
            inp = os.path.join(td, "eval_in.txt")
            write_boards(inp, lines)
            out = subprocess.run([refthink, "--eval", feat, val, inp], check=True,
                                 capture_output=True, text=True).stdout
            with open(os.path.join(HERE, "eval_vectors.txt"), "w") as f:
                f.write(out)
            print("eval_vectors", len(out.splitlines()))


if __name__ == "__main__":
    main()
