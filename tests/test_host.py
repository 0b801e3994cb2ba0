"""Host-side checks that need no GPU: the C ABI library loads and exports
every function include/gpuothello2.h declares, argument validation, and the
CLI's argument and file errors (main.cu:175-185, 49-67 semantics)."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from tests.conftest import GOLDEN, ROOT


def declared_functions():
    text = open(os.path.join(ROOT, "include", "gpuothello2.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*([a-z_0-9]+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol(built):
    import gpuothello2_gb300 as g

    names = declared_functions()
    assert len(names) >= 9
    lib = ctypes.CDLL(built.LIB)
    for name in names:
        assert hasattr(lib, name), name
    assert set(names) == set(g.EXPORTED_SYMBOLS)


def test_argument_validation_needs_no_device(built):
    import gpuothello2_gb300 as g

    L = g.lib()
    p = np.zeros(4, np.uint64)
    s = np.zeros(4, np.int8)
    assert L.solve_batch(p.ctypes.data, p.ctypes.data, -1, 10, s.ctypes.data) == g.GPO_ERR_ARG
    assert L.solve_batch(None, p.ctypes.data, 4, 10, s.ctypes.data) == g.GPO_ERR_ARG
    assert L.solve_batch(p.ctypes.data, p.ctypes.data, 4, 0, s.ctypes.data) == g.GPO_ERR_DEPTH
    assert L.solve_batch(p.ctypes.data, p.ctypes.data, 4, 33, s.ctypes.data) == g.GPO_ERR_DEPTH
    assert L.solve_batch(p.ctypes.data, p.ctypes.data, 0, 10, s.ctypes.data) == g.GPO_OK
    bad = g.options(method=7)
    assert L.solve_batch_ex(p.ctypes.data, p.ctypes.data, 4, 10, s.ctypes.data, None, None,
                            ctypes.byref(bad), None) == g.GPO_ERR_ARG
    assert L.gpo_generate(0, 0, 4, 10, 61, p.ctypes.data, p.ctypes.data) == g.GPO_ERR_ARG
    assert L.gpo_generate(1 << 40, 0, 4, 10, 10, p.ctypes.data, p.ctypes.data) == g.GPO_ERR_ARG
    assert g.strerror(g.GPO_ERR_DEPTH).startswith("depth")


def run_cli(args, cwd=None):
    from gpuothello2_gb300 import build

    return subprocess.run([build.SOLVER_BIN] + args, capture_output=True, text=True, cwd=cwd,
                          timeout=120)


def test_cli_usage_and_think_mode(built):
    r = run_cli([])
    assert r.returncode == 1 and "usage:" in r.stderr
    r = run_cli(["a", "b", "10", "3"])
    assert r.returncode == 1 and "THINK_DEPTH" in r.stderr
    r = run_cli(["a", "b", "x"])
    assert r.returncode == 1


def test_cli_think_mode_needs_the_evaluator_files(built, tmp_path):
    boards = tmp_path / "boards.txt"
    boards.write_text("1\n" + "!" * 16 + "\n")
    r = subprocess.run([built.SOLVER_BIN, str(boards), str(tmp_path / "out.txt"), "60", "5"],
                       cwd=str(tmp_path), capture_output=True, text=True, timeout=60)
    assert r.returncode != 0
    assert "subboard.txt" in r.stderr and "value/value52" in r.stderr


def test_cli_file_errors(built, tmp_path):
    r = run_cli([str(tmp_path / "missing.txt"), str(tmp_path / "o.txt"), "10"])
    assert r.returncode != 0 and "cannot open" in r.stderr
    short = tmp_path / "short.txt"
    short.write_text("3\n!!%[nNNNNNnNNNNN\n")
    r = run_cli([str(short), str(tmp_path / "o.txt"), "10"])
    assert r.returncode != 0 and "Failed to load boards" in r.stderr
    bad = tmp_path / "bad.txt"
    bad.write_text("1\n!!%[nNNN NnNNNNN\n")
    r = run_cli([str(bad), str(tmp_path / "o.txt"), "10"])
    assert r.returncode != 0 and "bad board" in r.stderr
    trunc = tmp_path / "trunc.txt"
    trunc.write_text("1\n!!%[nNNNN\n")
    r = run_cli([str(trunc), str(tmp_path / "o.txt"), "10"])
    assert r.returncode != 0 and "bad board" in r.stderr


def test_python_board_file_roundtrip(tmp_path):
    from gpuothello2_gb300 import codec

    p, o = codec.read_board_file(os.path.join(GOLDEN, "c1_seed0_e10.txt"))
    path = tmp_path / "b.txt"
    codec.write_board_file(str(path), p, o)
    assert path.read_text() == open(os.path.join(GOLDEN, "c1_seed0_e10.txt")).read()


def test_ctypes_mirrors_match_the_header_layout(tmp_path):
    """The Python Options/Stats structures have the C structs' size and field
    offsets (compiled from include/gpuothello2.h with the host compiler)."""
    import gpuothello2_gb300 as g

    structs = {"gpo_options": g.Options, "gpo_stats": g.Stats}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "gpuothello2.h"',
             "int main(void) {"]
    for cname, py in structs.items():
        lines.append('  printf("%s size %%zu\\n", sizeof(%s));' % (cname, cname))
        for field, _ in py._fields_:
            lines.append('  printf("%s %s %%zu\\n", offsetof(%s, %s));' %
                         (cname, field, cname, field))
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o",
                    str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    c_layout = {}
    for ln in out.splitlines():
        cname, field, value = ln.split()
        c_layout[(cname, field)] = int(value)
    for cname, py in structs.items():
        assert c_layout[(cname, "size")] == ctypes.sizeof(py), cname
        for field, _ in py._fields_:
            assert c_layout[(cname, field)] == getattr(py, field).offset, (cname, field)


def test_result_differ_matches_by_board(built, tmp_path):
    """diff_results compares result files by board: order and duplicates do
    not matter; a changed score, a missing board and a board listed with two
    scores are reported."""
    import random
    import subprocess

    ref = [ln.split()[:2] for ln in open(os.path.join(GOLDEN, "c1_seed0_e10.ref"))][:300]
    a = tmp_path / "a.txt"
    a.write_text("".join("%s %s\n" % (b, v) for b, v in ref))
    lines = ref + ref[:17]  # duplicates
    random.Random(5).shuffle(lines)
    b = tmp_path / "b.txt"
    b.write_text("".join("%s %s\n" % (x, v) for x, v in lines))
    run = lambda x, y: subprocess.run([built.DIFF_BIN, str(x), str(y)], capture_output=True,
                                      text=True)
    r = run(a, b)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "0 differ, 0 only in A, 0 only in B" in r.stdout
    changed = [list(x) for x in ref]
    changed[10][1] = str(int(changed[10][1]) + 2)
    c = tmp_path / "c.txt"
    c.write_text("".join("%s %s\n" % (x, v) for x, v in changed[1:]))  # board 0 missing
    r = run(a, c)
    assert r.returncode == 1
    assert ("differs: %s %s %s" % (ref[10][0], ref[10][1], changed[10][1])) in r.stdout
    assert ("only in A: %s %s" % (ref[0][0], ref[0][1])) in r.stdout
    bad = tmp_path / "bad.txt"
    bad.write_text("%s %s\n%s %d\n" % (ref[3][0], ref[3][1], ref[3][0], int(ref[3][1]) + 2))
    assert run(a, bad).returncode == 2
