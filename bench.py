#!/usr/bin/env python
"""Benchmark: exact-solved positions/s on a mixed 8-16-empty batch.

Workload (one "step" = one exact solve of the whole batch): 1,048,576
positions from the seeded random-playout stream, seed 2, empty count uniform
in 8..16 per position, DEPTH 16 -- the batched-uneven configuration the
headline metric is quoted on.  Inputs are generated on the GPU once, outside
the timed region.

  value  positions/s of the batched solver with inputs resident in HBM
         (solve_batch_device; per-step CUDA events on the launching stream;
         a 256 MiB write flushes L2 between steps, untimed)
  e2e    the same metric through solve_batch_ex with pinned HOST buffers,
         host->device copies and the device->host score read inside the
         wall-clock timed region (the last warm-up step runs this way, so a
         default run costs W + K solves)
  plain  the plain thread-per-board kernel on the same batch (the
         denominator of the batched-vs-plain ratio)
  roofline  integer-ALU bound: 418 INT32 ops per node (mobility + flip +
         make-move of the reference arithmetic) x nodes / batched-kernel
         time, against the INT32 issue rate measured live by
         libgpo_intpeak.so (the HBM and BF16 peaks do not bound integer code)
  cpu_baseline  the oracle's restatement of the reference tree on all host
         cores, on a bounded sample of the same stream

The transposition table is always on; the line reports its size, probes,
hits, updates and 32-byte-sector traffic rate.  A stratified sample of the
scores is checked against the oracle outside the timed region
(`parity_sample`).  The top of the search (nodes with >= 12 empties in the
first two plies) is ordered by the learned move orderer, whose weights were
trained by the library's own GPU kernels and are loaded from a file
(`--no-learned`: fastest-first only).  Options: `--tuned` autotunes the launch and search parameters on
a sample of the batch first (untimed); `--plain` also times the plain kernel
on the same batch; `--table-bits` sets the table size.

`--impl reference` times the reference algorithm on the host cores instead
(the oracle port of the reference tree; the reference's own search only
exists as GPU code), printing the same metric with "impl": "reference".
Multi-GPU (torchrun): every rank solves its own 1,048,576-position slice of
the stream (weak scaling, no collective on the data path).
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

W_NODE = 418  # INT32 ops per node: mobility + flip + make-move of the reference arithmetic
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per search node
# of one batched-kernel launch, from one ncu capture of a smaller launch
# (profiles/batched_kernel_ncu.md), scaled to this launch by its node count:
# the traffic is the transposition table's, which grows with the nodes.
TRAFFIC_BYTES_PER_NODE = (6.700996e9 + 3.144086e9) / 3303996693
TRAFFIC_SOURCE = ("ncu capture of 131,072 positions x 12 empties (9.85 GB in 3.30e9 nodes, "
                  "profiles/batched_kernel_ncu.md; table from 7 empties there, from 9 now, "
                  "so an upper estimate), scaled by nodes")
SEED, N_POS, LO, HI, DEPTH = 2, 1 << 20, 8, 16, 16
METRIC = "exact-solved positions/s at 8\u201316 empties: batched+learned vs plain, same GB300"
WORKLOAD = ("1,048,576 positions, random playouts seed 2, empties uniform 8..16, DEPTH 16")
CPU_SAMPLE = 1536
SMI_FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def slice_first(rank, n):
    """First stream index of a rank's slice: rank r solves positions
    [r*n, (r+1)*n) of the workload stream, so the ranks' slices are disjoint
    and together form the first world*n positions (weak scaling)."""
    return rank * n


def max_over_ranks(seconds, world, device=None):
    """The slowest rank's time (the job ends when every rank has finished);
    a float64 all-reduce on the process group's backend."""
    if world == 1:
        return seconds
    import torch
    import torch.distributed as dist

    t = torch.tensor([seconds], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_value(world, n, steps, seconds):
    """Whole-job positions/s: every rank's positions over the slowest time."""
    return world * n * steps / seconds


class ClockSampler:
    """nvidia-smi sampling during the timed region (read-only queries)."""

    def __init__(self, device):
        self.device = device
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + SMI_FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [ln for ln in out.splitlines() if ln.strip()]

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in getattr(self, "lines", []):
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_reference_rate(sample, threads=0, max_seconds=20.0):
    """Oracle restatement of the reference tree (orc_solve_ref) on the host
    cores over the first `sample` positions of the workload stream; stops
    early after max_seconds.  Returns (positions/s, positions, seconds,
    threads)."""
    import numpy as np
    from gpuothello2_gb300 import build as B
    from tests.oracle_lib import Oracle

    B.build_oracle()
    orc = Oracle(B.ORACLE_LIB)
    threads = threads or orc.L.orc_num_cores()
    p, o = orc.generate(SEED, sample, LO, HI)
    chunk = max(threads * 8, 64)
    done, t0 = 0, time.perf_counter()
    while done < sample:
        k = min(chunk, sample - done)
        orc.solve_batch(p[done:done + k], o[done:done + k], DEPTH, mode=0, threads=threads)
        done += k
        if time.perf_counter() - t0 > max_seconds:
            break
    dt = time.perf_counter() - t0
    return done / dt, done, dt, threads


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    rates, total_done, total_t, thr = [], 0, 0.0, 0
    for step in range(args.warmup + args.steps):
        r, done, dt, thr = cpu_reference_rate(512, max_seconds=15.0)
        if step >= args.warmup:
            rates.append(r)
            total_done += done
            total_t += dt
    value = total_done / total_t
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "positions/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * total_t / max(1, args.steps), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "sample_per_step": 512},
        "cpu_baseline": {"value": value, "unit": "positions/s", "cores": thr, "kind": "port",
                         "sample": "first 512 positions of the workload stream per step; "
                                   "oracle restatement of the reference tree (reference "
                                   "order, no table), %d host threads" % thr},
        "e2e": {"value": value, "unit": "positions/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def parity_sample(p, o, scores, threads=0):
    """Scores of a stratified sample of the batch against the oracle's own
    alpha-beta solver (orc_solve_fast: a different tree, same exact values),
    outside the timed region: every 512th position of the batch (all empty
    counts in proportion) plus the first 256 positions with 16 empties (the
    hardest searches)."""
    import numpy as np
    from gpuothello2_gb300 import build as B
    from tests.oracle_lib import Oracle

    B.build_oracle()
    orc = Oracle(B.ORACLE_LIB)
    empties = 64 - np.array([bin(int(a) | int(b)).count("1") for a, b in zip(p[:1 << 16], o[:1 << 16])])
    hard = np.nonzero(empties == HI)[0][:256]
    idx = np.unique(np.concatenate([np.arange(0, len(p), 512), hard]))
    t0 = time.perf_counter()
    want, _, _, _ = orc.solve_batch(p[idx], o[idx], DEPTH, mode=1, threads=threads)
    mism = int(np.sum(want.astype(int) != scores[idx].astype(int)))
    return {"n": int(len(idx)), "mismatches": mism, "hard_16_empties": int(len(hard)),
            "seconds": time.perf_counter() - t0,
            "how": "every 512th position + the first 256 with 16 empties, against the oracle's "
                   "own alpha-beta (orc_solve_fast), outside the timed region"}


def profile_cases(args):
    """Small runs for profiling (ncu) and peak probes; no JSON line.
    --profile-solve N E: N positions (seed 1) at E empties, solved twice with the
    library defaults and the learned orderer (capture the second launch:
    `ncu ... -k regex:batched_kernel -s 1 -c 1 ...`); --profile-think N D: think
    mode with 13 patterns of 5-12 squares and seeded random weights, N positions
    (seed 6, 24..34 empties) to D plies, twice; --int-peak: the INT32 issue rates
    measured by libgpo_intpeak."""
    import numpy as np

    import __graft_entry__

    __graft_entry__.build()
    import gpuothello2_gb300 as g
    from gpuothello2_gb300 import build as B

    if args.int_peak:
        lib = ctypes.CDLL(B.INTPEAK_LIB)
        lib.gpo_int_peak.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                     ctypes.POINTER(ctypes.c_double)]
        for op, name in ((0, "lop3.b32"), (1, "add.u32")):
            v, ms = ctypes.c_double(), ctypes.c_double()
            if lib.gpo_int_peak(op, ctypes.byref(v), ctypes.byref(ms)) != 0:
                raise RuntimeError("gpo_int_peak failed")
            print("int peak %s: %.3f Tops/s (%.3f ms per launch)" % (name, v.value / 1e12,
                                                                     ms.value), flush=True)
    if args.profile_solve:
        n, e = args.profile_solve
        g.mlp_load(np.fromfile(args.weights, dtype=np.float32))
        p, o = g.generate(1, n, e, e)
        for _ in range(2):
            _, _, _, st, _ = g.solve(p, o, e)
        print("solve n=%d empties=%d nodes=%d kernel_ms=%.1f" % (n, e, st.nodes, st.kernel_ms),
              flush=True)
    if args.profile_think:
        n, depth = args.profile_think
        # 4 rows, 2 diagonals, corner blocks, an edge with its X squares and
        # shorter lines: 13 patterns of 5 to 12 squares
        masks = [0xFF << (8 * r) for r in range(4)] + [
            0x8040201008040201, 0x0102040810204080, 0x1F1F, 0x070707, 0x42FF, 0x0F0F0F, 0x1F,
            0x804020100804, 0x3C3C]
        rng = np.random.default_rng(1)
        g.eval_load(masks, rng.uniform(-4, 4, sum(3 ** bin(m).count("1") for m in masks)), 0.5)
        p, o = g.generate(6, n, 24, 34)
        for _ in range(2):
            _, _, _, st, _ = g.think(p, o, depth)
        sec = st.kernel_ms / 1e3
        print("think n=%d depth=%d kernel_ms=%.3f positions/s=%.4g nodes/s=%.4g" %
              (n, depth, st.kernel_ms, n / sec, st.nodes / sec), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--plain", action="store_true",
                    help="also time the plain kernel on the same batch (minutes)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-parity", action="store_true")
    ap.add_argument("--n", type=int, default=N_POS)
    ap.add_argument("--table-bits", type=int, default=0,
                    help="transposition table of 2^bits entries (0 = library default: 2^28 on "
                         "a device with >= 64 GiB)")
    ap.add_argument("--no-learned", dest="learned", action="store_false",
                    help="fastest-first ordering only (by default the top of the search is "
                         "ordered by the learned move orderer, weights from --weights)")
    ap.add_argument("--weights", default=os.path.join(ROOT, "gpuothello2_gb300", "data",
                                                      "orderer.f32"))
    ap.add_argument("--tuned", action="store_true",
                    help="autotune launch/search parameters on a 4,096-position sample of the "
                         "batch first (untimed; cached per GPU, depth and empties range)")
    ap.add_argument("--profile-solve", type=int, nargs=2, metavar=("N", "EMPTIES"))
    ap.add_argument("--profile-think", type=int, nargs=2, metavar=("N", "DEPTH"))
    ap.add_argument("--int-peak", action="store_true")
    args = ap.parse_args()
    if args.profile_solve or args.profile_think or args.int_peak:
        profile_cases(args)
        return
    if args.impl == "reference":
        run_reference(args)
        return

    import numpy as np
    import torch

    import __graft_entry__

    __graft_entry__.build()
    import gpuothello2_gb300 as g

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    L = g.lib()
    n = args.n
    dev = torch.device("cuda", local)
    dp = torch.empty(n, dtype=torch.int64, device=dev)
    do = torch.empty(n, dtype=torch.int64, device=dev)
    ds = torch.empty(n, dtype=torch.int8, device=dev)
    stream = torch.cuda.current_stream(dev)
    rc = L.gpo_generate_device(SEED, slice_first(rank, n), n, LO, HI, dp.data_ptr(),
                               do.data_ptr(), stream.cuda_stream)
    assert rc == 0, g.strerror(rc)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    learned_info = None
    if args.learned:
        w = np.fromfile(args.weights, dtype=np.float32)
        g.mlp_load(w)
        learned_info = {"weights": os.path.relpath(args.weights, ROOT), "min_empties": 12}
    tuned, tuned_src = {}, None
    if args.tuned:
        from gpuothello2_gb300 import autotune

        params, tuned_src = autotune.tune_batch(dp.cpu().numpy().view(np.uint64),
                                                do.cpu().numpy().view(np.uint64), DEPTH)
        tuned = autotune.to_options(params)

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize(dev)

    def batched_options():
        return g.options(method=g.METHOD_BATCHED, use_learned=1 if args.learned else 0,
                         table_bits=args.table_bits, **tuned)

    def solve_device(method):
        st = g.Stats()
        opt = batched_options() if method == g.METHOD_BATCHED else g.options(method=method)
        rc = L.solve_batch_device(dp.data_ptr(), do.data_ptr(), n, DEPTH, ds.data_ptr(), None,
                                  None, ctypes.byref(opt), ctypes.byref(st), stream.cuda_stream)
        if rc != 0:
            raise g.SolverError(rc, "solve_batch_device")
        return st

    hp = torch.empty(n, dtype=torch.int64, pin_memory=True)
    ho = torch.empty(n, dtype=torch.int64, pin_memory=True)
    hs = torch.empty(n, dtype=torch.int8, pin_memory=True)
    hp.copy_(dp.cpu())
    ho.copy_(do.cpu())

    def solve_host():
        """One step through the host-buffer entry point (pinned buffers):
        host->device copies, solve, device->host scores, wall clock."""
        opt = batched_options()
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        rc = L.solve_batch_ex(hp.data_ptr(), ho.data_ptr(), n, DEPTH, hs.data_ptr(), None, None,
                              ctypes.byref(opt), None)
        t1 = time.perf_counter()
        if rc != 0:
            raise g.SolverError(rc, "solve_batch_ex")
        return t1 - t0

    def timed(method, warmup, steps, sampler=None, e2e=None):
        # warm-up steps are untimed for `value`; the last one goes through
        # the host-buffer entry point and is the end-to-end measurement
        for w in range(warmup):
            flush.zero_()
            if e2e is not None and w == warmup - 1:
                e2e.append(solve_host())
            else:
                solve_device(method)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(steps)]
        stats = []
        barrier()
        if sampler:
            sampler.__enter__()
        for k in range(steps):
            flush.zero_()
            ev[k][0].record(stream)
            stats.append(solve_device(method))
            ev[k][1].record(stream)
        barrier()
        if sampler:
            sampler.__exit__(None, None, None)
        step_ms = [a.elapsed_time(b) for a, b in ev]
        return step_ms, stats

    sampler = ClockSampler(local)
    e2e_t = []
    step_ms, stats = timed(g.METHOD_BATCHED, args.warmup, args.steps, sampler, e2e_t)
    kern_ms = [st.kernel_ms for st in stats]
    nodes = [st.nodes for st in stats]
    total_s = max_over_ranks(sum(step_ms) / 1000.0, world, dev)
    value = job_value(world, n, args.steps, total_s)
    scores = ds.cpu().numpy()
    e2e_value = job_value(world, n, 1, max_over_ranks(e2e_t[0], world, dev)) if e2e_t else None
    if e2e_t:
        assert np.array_equal(hs.numpy(), scores), "host and device entry points disagree"
    kern_s = sum(kern_ms) / 1000.0
    probes = sum(st.table_probes for st in stats)
    updates = sum(st.table_updates for st in stats)
    # a probe reads the two 16-byte entries of a bucket (one 32-byte sector);
    # an update reads the bucket and writes one entry
    table_stats = {"entries": 1 << int(stats[0].table_bits), "probes": probes,
                   "hits": sum(st.table_hits for st in stats), "updates": updates,
                   "sector_bytes": 32 * (probes + 2 * updates),
                   "gbs": 32 * (probes + 2 * updates) / kern_s / 1e9 if kern_s > 0 else None,
                   "min_empties": 9}

    plain = None
    if args.plain:
        p_ms, p_stats = timed(g.METHOD_PLAIN, 1, 1)
        plain = {"value": n / (p_ms[0] / 1000.0), "unit": "positions/s", "ms_per_step": p_ms[0],
                 "nodes_per_step": p_stats[0].nodes, "kernel_ms": p_stats[0].kernel_ms}
        assert np.array_equal(ds.cpu().numpy(), scores), "plain and batched kernels disagree"

    peak = ctypes.c_double(0.0)
    ipk = ctypes.CDLL(os.path.join(ROOT, "gpuothello2_gb300", "lib", "libgpo_intpeak.so"))
    ipk.gpo_int_peak.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                 ctypes.POINTER(ctypes.c_double)]
    peaks = []
    for op in (0, 1):
        ipk.gpo_int_peak(op, ctypes.byref(peak), None)
        peaks.append(peak.value)
    int_peak = max(peaks)
    mean_kern_s = statistics.mean(kern_ms) / 1000.0
    mean_nodes = statistics.mean(nodes)
    achieved = mean_nodes * W_NODE / mean_kern_s

    parity = None
    cpu = None
    if rank == 0:
        pos_p = dp.cpu().numpy().view(np.uint64)
        pos_o = do.cpu().numpy().view(np.uint64)
        if not args.no_parity:
            parity = parity_sample(pos_p, pos_o, scores)
        if not args.no_cpu:
            r, done, dt, thr = cpu_reference_rate(CPU_SAMPLE)
            cpu = {"value": r, "unit": "positions/s", "cores": thr, "kind": "port",
                   "sample": "first %d positions of the workload stream (%.1f s), oracle "
                             "restatement of the reference tree, %d threads" % (done, dt, thr)}

    launches = int(sum(st.launches for st in stats))
    line = {
        "metric": METRIC, "value": value, "unit": "positions/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * total_s / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
        "data": "synthetic: seeded random playouts (xoshiro256**, seed 2), generated on device",
        "config": {"workload": WORKLOAD, "positions_per_gpu": n, "depth": DEPTH,
                   "l2": "flushed between steps (256 MiB write, untimed); the table clear "
                         "(16 B x entries) at the start of every solve also evicts it",
                   "method": ("batched: empties-bucketed persistent queue, per-lane "
                              "principal-variation search with transposition table and "
                              "stability cutoff, warp-local helping on hard positions, the "
                              "last unfinished positions handed back and finished by a root "
                              "split over the whole GPU; learned ordering %s"
                              % ("on" if args.learned else "off")),
                   "table_entries": table_stats["entries"],
                   "tuned": ({"params": tuned, "source": tuned_src} if args.tuned else None),
                   "learned": learned_info},
        "e2e": {"value": e2e_value, "unit": "positions/s", "h2d_bytes_per_step": 16 * n,
                "d2h_bytes_per_step": n,
                "how": "last warm-up step through solve_batch_ex, pinned host buffers, wall clock"},
        "roofline": {"bound": "int32-alu", "achieved": achieved / 1e12, "peak": int_peak / 1e12,
                     "unit": "TOPS (INT32)", "frac": achieved / int_peak,
                     "traffic": TRAFFIC_BYTES_PER_NODE * mean_nodes,
                     "traffic_source": TRAFFIC_SOURCE,
                     "peak_source": "measured live: lop3.b32/add.u32 issue rate (libgpo_intpeak)",
                     "kernel": "batched_kernel", "ops_per_node": W_NODE,
                     "nodes_per_launch": mean_nodes, "kernel_ms": 1000.0 * mean_kern_s},
        "nodes_per_s": mean_nodes / mean_kern_s,
        "nodes_per_position": mean_nodes / n,
        "splits_per_step": statistics.mean(st.splits for st in stats),
        "tail_handoff": {"positions_per_step": statistics.mean(st.tail_positions for st in stats),
                         "frontier_per_step": statistics.mean(st.root_split_positions
                                                              for st in stats)},
        "table": table_stats,
        "parity_sample": parity,
        "cpu_baseline": cpu,
        "clocks": sampler.summary(),
        # counted by the library per call: bucketing (3) and the search (1),
        # and the same again for the root split that finishes the tail
        "gpu_launches": launches,
        "plain": plain,
        "speedup_vs_plain": (value / plain["value"]) if plain else None,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
