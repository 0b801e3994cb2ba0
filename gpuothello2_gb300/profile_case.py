"""Small, self-contained solver runs for profiling (ncu) and peak probes.

  python -m gpuothello2_gb300.profile_case [N] [EMPTIES]
      generates N positions (seed 1) with EMPTIES empties and solves them
      twice with the default batched method (the second launch is the one
      to capture: `ncu ... -k regex:batched_kernel -s 1 -c 1 ...`)
  python -m gpuothello2_gb300.profile_case --int-peak
      prints the INT32 issue rates measured by libgpo_intpeak.so
  python -m gpuothello2_gb300.profile_case --think [N] [DEPTH]
      think mode: loads an evaluator of 13 patterns (5 to 12 squares) with
      seeded random weights, runs N positions (seed 6, 24..34 empties) to
      DEPTH plies twice and prints the second run's kernel time, positions/s
      and nodes/s
"""
import ctypes
import os
import sys


def int_peak():
    from . import build

    lib = ctypes.CDLL(build.INTPEAK_LIB)
    lib.gpo_int_peak.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                 ctypes.POINTER(ctypes.c_double)]
    for op, name in ((0, "lop3.b32"), (1, "add.u32")):
        v, ms = ctypes.c_double(), ctypes.c_double()
        rc = lib.gpo_int_peak(op, ctypes.byref(v), ctypes.byref(ms))
        if rc != 0:
            raise RuntimeError("gpo_int_peak failed")
        print("int peak %s: %.3f Tops/s (%.3f ms per launch)" % (name, v.value / 1e12, ms.value),
              flush=True)


def think_case(n, depth):
    import numpy as np

    import gpuothello2_gb300 as g

    # 4 rows, 2 diagonals, corner blocks, an edge with its X squares and
    # shorter lines: 13 patterns of 5 to 12 squares
    rows = [0xFF << (8 * r) for r in range(4)]
    masks = rows + [0x8040201008040201, 0x0102040810204080, 0x1F1F, 0x070707, 0x42FF,
                    0x0F0F0F, 0x1F, 0x804020100804, 0x3C3C]
    rng = np.random.default_rng(1)
    total = sum(3 ** bin(m).count("1") for m in masks)
    g.eval_load(masks, rng.uniform(-4, 4, total), 0.5)
    p, o = g.generate(6, n, 24, 34)
    for _ in range(2):
        _, _, nodes, st, _ = g.think(p, o, depth)
    sec = st.kernel_ms / 1e3
    print("think ok n=%d depth=%d kernel_ms=%.3f positions/s=%.4g nodes/s=%.4g" %
          (n, depth, st.kernel_ms, n / sec, st.nodes / sec), flush=True)


def main(argv):
    if argv and argv[0] == "--int-peak":
        int_peak()
        return
    if argv and argv[0] == "--think":
        think_case(int(argv[1]) if len(argv) > 1 else 65536, int(argv[2]) if len(argv) > 2 else 6)
        return
    import gpuothello2_gb300 as g

    n = int(argv[0]) if argv else 131072
    e = int(argv[1]) if len(argv) > 1 else 10
    p, o = g.generate(1, n, e, e)
    for _ in range(2):
        _, _, _, st, _ = g.solve(p, o, e)
    print("ok", n, e, st.nodes, st.kernel_ms, flush=True)


if __name__ == "__main__":
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    main(sys.argv[1:])
