"""Small, self-contained solver runs for profiling (ncu) and peak probes.

  python -m gpuothello2_gb300.profile_case [N] [EMPTIES]
      generates N positions (seed 1) with EMPTIES empties and solves them
      twice with the default batched method (the second launch is the one
      to capture: `ncu ... -k regex:batched_kernel -s 1 -c 1 ...`)
  python -m gpuothello2_gb300.profile_case --int-peak
      prints the INT32 issue rates measured by libgpo_intpeak.so
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


def main(argv):
    if argv and argv[0] == "--int-peak":
        int_peak()
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
