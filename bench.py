"""Benchmark of the canonicity-check hot path on one GB300.

Workload (one "step"): the exact canonicity check of 1,048,576 STS(15)
incidence matrices (15 x 35, one uint64 per row): item i is a random STS(15)
(Stinson hill-climbing, seed 20241203 + splitmix stream i) under a uniform row
and column permutation; odd items are replaced by their canonical form
(CanonizeMatrix).  Per matrix the check reports the canonical flag, the first
rejecting row permutation (witness) and |Aut| (for a rejected matrix taken from
its canonical form, reached as CanonizeMatrix does).  The batch is generated on the GPU once, before
timing.

  value : checks/s with the batch resident in HBM (canon_check_bibd_device),
          CUDA events on the launching stream, L2 flushed between steps.
  e2e   : checks/s through the public batch API with host buffers
          (canon_submit_bibd + canon_sync: pinned staging, H2D, kernel, D2H of
          every result array), host wall clock.

`--impl reference` times the CPU restatement of the reference checker (the
oracle) on all host cores over a bounded sample of the same workload.
"""
import argparse
import concurrent.futures as cf
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "incidence-system-enumeration_gb300"))

N_ITEMS = 1 << 20
V, B = 15, 35
SEED = 20241203
FLAGS_NAME = "COMPLETE|RAW|AUT_CANON"
METRIC = "exact canonicity checks/sec (STS(15) 15x35, plain order)"
WORKLOAD = ("1,048,576 STS(15) 15x35 bit-packed matrices, seed %d, odd items canonical; "
            "outputs canonical flag + first rejecting permutation + |Aut|" % SEED)
IN_BYTES = V * 8          # packed rows read per check
OUT_BYTES = 1 + 16 + 16   # flag + witness + |Aut| written per check
# DRAM bytes per check of the converged lex-max pass: dram__bytes_read.sum + dram__bytes_write.sum
# of one ncu capture of 65,536 checks (8,426,496 B + 0 B; profiles/bibd_conv_kernel_sts15_65k.md),
# scaled by the checks of a launch (traffic grows with the number of matrices read).
TRAFFIC_PER_CHECK = 8426496.0 / 65536
# Integer work of the lex-max search (the check's roofline): a node compares the best
# arrangement of every candidate row with the bound, one bit-sliced step per column of
# the matrix: the column's row mask ANDed with the tied rows, a 6-plane carry chain
# (AND + XOR per plane) and the final XOR -- 12 lane operations per column and node.
INT_OPS_PER_NODE_COLUMN = 12
MEASURED_PEAKS = os.path.join(REPO, "MEASURED_PEAKS.json")
CPU_NOTE = ("the oracle: a C restatement of the reference's checker (TestCanonicity + CanonizeMatrix), "
            "not the reference binary, which does not build on this platform")


def peaks():
    try:
        with open(MEASURED_PEAKS) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(), "ise_gb300_clocks_%d.csv" % os.getpid())

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def remove(self):
        try:
            os.remove(self.path)
        except OSError:
            pass

    def summary(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        try:
            rows = [l.split(",") for l in open(self.path).read().splitlines() if l.strip()]
        except Exception:
            return out
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except (ValueError, IndexError):
                continue
            for k, name in enumerate(names):
                if len(r) > 5 + k and "Active" in r[5 + k] and "Not" not in r[5 + k]:
                    reasons.add(name)
        if sm:
            out = {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                   "samples": len(sm)}
        self.remove()
        return out


def dist_setup(n_gpus):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return rank, world, local, dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, x):
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def cpu_sample_rows(n):
    """The first n items of the workload, built on the CPU by the oracle's
    restatement of the generator and canonizer (same streams as the device)."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    rows = np.stack([oracle.sts_random_rows(V, SEED, i) for i in range(n)])

    def canon(i):
        M = oracle.rows_to_matrix(rows[i], B)
        C, _, _ = oracle.bibd_canonize(M)
        return i, (C.astype(np.uint64) << np.arange(B, dtype=np.uint64)).sum(axis=1, dtype=np.uint64)

    with cf.ThreadPoolExecutor(os.cpu_count() or 1) as ex:
        for i, r in ex.map(canon, range(1, n, 2)):
            rows[i] = r
    return rows


def cpu_check_rate(rows, threads, budget_s):
    """Oracle checks/s over `rows` on `threads` host threads (ctypes releases the GIL)."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    flags = oracle.SAVE_ROW_PERM | oracle.SAVE_ROW_TO_CHANGE

    def one(i):
        M = oracle.bibd_normalize(oracle.rows_to_matrix(rows[i], B))
        res = oracle.bibd_test(M, flags)
        if not res["canonical"]:
            oracle.bibd_canonize(M)          # |Aut| from the canonical form
        return res["canonical"]

    done = 0
    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(threads) as ex:
        idx = 0
        while idx < len(rows):
            chunk = list(range(idx, min(len(rows), idx + 4 * threads)))
            list(ex.map(one, chunk))
            done += len(chunk)
            idx += len(chunk)
            if time.perf_counter() - t0 > budget_s:
                break
    dt = time.perf_counter() - t0
    return done / dt, done, dt


def run_reference(args, rank, world, dist):
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    sample = 256 * threads
    rows = cpu_sample_rows(sample)
    for _ in range(args.warmup):
        cpu_check_rate(rows[: 2 * threads], threads, 60)
    rates = []
    t_all = 0.0
    n_all = 0
    for _ in range(args.steps):
        rate, done, dt = cpu_check_rate(rows, threads, 30)
        rates.append(rate)
        t_all += dt
        n_all += done
    value = n_all / t_all
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "checks/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * t_all / max(1, args.steps), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u8/u64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "ordering": "plain", "l2": "n/a (host CPU)"},
        "cpu_baseline": {"value": value, "unit": "checks/s", "cores": threads, "kind": "port",
                         "sample": "first %d items of the workload per step (%d checks/step)"
                                   % (len(rows), len(rows)), "note": CPU_NOTE},
        "e2e": {"value": value, "unit": "checks/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_gpu(args, rank, world, local, dist):
    import ise_gb300 as G
    n = args.items
    ctx = G.Context(device=local, max_items=n, max_words=n * V, aut_cap=1)
    flags = G.COMPLETE | G.RAW | (G.AUT_CANON if args.mode == "autcanon" else 0)
    d_rows = ctx.alloc(n * V * 8)
    d_can = ctx.alloc(n)
    d_wit = ctx.alloc(n * 16)
    d_aut = ctx.alloc(n * 16)
    d_st = ctx.alloc(n)
    # rank r checks its own shard of the N x 1M items: the seeded stream SEED + r (rank 0's
    # shard is the single-GPU batch)
    ctx.generate_sts_device(n, V, SEED + rank, True, d_rows)
    ctx.stream_sync()
    # the autotuner picks the check variant for this shape on a sample (setup, untimed)
    variant, tune_ms = ctx.tune_bibd(min(n, 1 << 16), V, B, flags, d_rows)
    l2_flush = ctx.alloc(512 << 20)
    zeros = np.zeros(512 << 20, np.uint8)

    def flush_l2():
        ctx.h2d(l2_flush, zeros)

    for _ in range(args.warmup):
        ctx.check_bibd_device(n, V, B, flags, d_rows, d_can, d_wit, d_aut, d_st)
        ctx.stream_sync()
    launches0 = ctx.kernel_launches()
    times = []
    barrier(dist)
    ctx.stream_sync()
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush_l2()
            ctx.check_bibd_device(n, V, B, flags, d_rows, d_can, d_wit, d_aut, d_st)
            ctx.stream_sync()
            times.append(ctx.last_kernel_ms())
    barrier(dist)
    launches = ctx.kernel_launches() - launches0
    t_total = max_over_ranks(dist, sum(times) / 1e3)
    st = ctx.d2h(np.zeros(n, np.uint8), d_st)
    can = ctx.d2h(np.zeros(n, np.uint8), d_can)
    if st.any():
        raise SystemExit("bench: %d items reported a bad status" % int((st != 0).sum()))
    value = world * n * args.steps / t_total
    ms_step = 1e3 * t_total / args.steps
    hbm, src = peaks()
    roofline, roofline_hbm = integer_roofline(ctx, args, n, flags, variant, d_rows, d_can, d_aut, d_st, flush_l2,
                                              hbm, src, times)

    # end to end through the batch API with host buffers
    host_rows = ctx.d2h(np.zeros(n * V, np.uint64), d_rows)
    e2e_dt = None
    if not args.no_e2e:
        e2e_steps = max(1, min(args.steps, 3))
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            ctx.submit_bibd(host_rows, V, B, flags)
            res = ctx.sync(raw=True, copy=False)   # the result buffers as the C API returns them
        e2e_dt = (time.perf_counter() - t0) / e2e_steps
        assert res["n"] == n and np.array_equal(res["canonical"], can)
    if e2e_dt is not None:
        e2e_dt = max_over_ranks(dist, e2e_dt)
    h2d = n * V * 8 + n * 16
    d2h = n * (1 + 1 + 1 + 1 + 4 + 16 + 16 + 8 + 2 + 1)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        sample = min(n, 4096 * threads)
        rows_s = host_rows.reshape(n, V)[:sample]
        rate, done, dt = cpu_check_rate(rows_s, threads, 20)
        cpu = {"value": rate, "unit": "checks/s", "cores": threads, "kind": "port",
               "sample": "first %d items of the same batch (%d checked in %.1f s)" % (sample, done, dt),
               "note": CPU_NOTE}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "checks/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "u64 bit rows / u8", "data": "synthetic",
            "config": {"workload": WORKLOAD if n == N_ITEMS else "%d items of: %s" % (n, WORKLOAD),
                       "ordering": "plain", "flags": FLAGS_NAME if args.mode == "autcanon" else "COMPLETE|RAW",
                       "items_per_step": n, "canonical_fraction": float(can.mean()),
                       "variant": G.VARIANT_NAMES[variant],
                       "tune_ms_65536": [round(x, 2) for x in tune_ms],
                       "l2": "flushed between steps (512 MiB write)",
                       "parallelism": ("replicas: rank r checks its own 1M items (seed %d + r)" % SEED)
                                      if world > 1 else "single GPU"},
            "e2e": None if e2e_dt is None else {"value": world * n / e2e_dt, "unit": "checks/s",
                                                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "roofline": roofline,
            "roofline_hbm": roofline_hbm,
            "cpu_baseline": cpu,
            "gpu_launches": launches,
            "clocks": clk.summary(),
        }
        print(json.dumps(line), flush=True)
    for p in (d_rows, d_can, d_wit, d_aut, d_st, l2_flush):
        ctx.free(p)
    ctx.close()


def integer_roofline(ctx, args, n, flags, variant, d_rows, d_can, d_aut, d_st, flush_l2, hbm, src, times):
    """The integer roofline of the dominant kernel (the lex-max pass of the two-pass
    check, or the one-pass kernel): algorithmic integer operations per launch --
    lex-max nodes (counted exactly on the device for this batch) x columns x 12 --
    over that kernel's own CUDA-event time, against the integer lane-operation rate
    this GPU sustains (canon_measure_int_peak).  HBM is reported beside it."""
    import ise_gb300 as G
    d_nodes = ctx.alloc(8 * n)
    ctx.lexmax_nodes_bibd(n, V, B, flags, d_rows, d_nodes)
    nodes = ctx.d2h(np.zeros(n, np.uint64), d_nodes)
    ctx.free(d_nodes)
    ops = float(nodes.sum()) * B * INT_OPS_PER_NODE_COLUMN
    conv_names = {G.VARIANT_CONVERGED: "bibd_conv_kernel<35, 15> (lex-max pass, converged layout)",
                  G.VARIANT_CONVERGED_D2: "bibd_conv_kernel<35, 15, 2> (lex-max pass, converged layout, "
                                          "loads staged 2 ahead)",
                  G.VARIANT_CONVERGED_D8: "bibd_conv_kernel<35, 15, 8> (lex-max pass, converged layout, "
                                          "loads staged 8 ahead)"}
    if variant == G.VARIANT_TWO_PASS or variant in conv_names:
        # the first pass alone: without witness and trials outputs only it is launched
        ms = []
        for _ in range(2):
            flush_l2()
            ctx.check_bibd_device(n, V, B, flags, d_rows, d_can, None, d_aut, d_st)
            ctx.stream_sync()
            ms.append(ctx.last_kernel_ms())
        kname = conv_names.get(variant, "bibd_max_kernel<35, 15> (lex-max pass)")
    else:
        ms = list(times)
        kname = "the one-pass check kernel"
    k_s = sum(ms) / len(ms) / 1e3
    peak = ctx.measure_int_peak()
    roof = {"bound": "int", "achieved": ops / k_s / 1e12, "peak": peak / 1e12, "unit": "Tops/s",
            "frac": ops / k_s / peak, "traffic": TRAFFIC_PER_CHECK * n,
            "kernel": kname, "kernel_ms": 1e3 * k_s,
            "ops_per_launch": ops, "nodes_per_check_mean": float(nodes.mean()),
            "ops_model": "lex-max nodes x %d columns x %d lane ops (bit-sliced count per column and node)"
                         % (B, INT_OPS_PER_NODE_COLUMN),
            "peak_source": "measured on this GPU: independent 32-bit XOR/ADD/shift chains (canon_measure_int_peak)"}
    achieved_hbm = (IN_BYTES + OUT_BYTES) * n / k_s / 1e9
    roof_hbm = {"bound": "hbm", "achieved": achieved_hbm, "peak": hbm, "unit": "GB/s",
                "frac": achieved_hbm / hbm, "peak_source": src,
                "note": "secondary: %d algorithmic bytes per check (rows in, flag + witness + |Aut| out)"
                        % (IN_BYTES + OUT_BYTES)}
    return roof, roof_hbm


ENUM_WORKLOADS = {
    "enum-sts13": ("bibd", (13, 26, 6, 3, 1), "config 1: all BIBD(13,26,6,3,1) (STS(13)) by orderly generation"),
    "enum-sts15": ("bibd", (15, 35, 7, 3, 1), "all BIBD(15,35,7,3,1) (STS(15)) by orderly generation"),
    "enum-k10": ("ksys", (10,), "config 5: all 1-factorizations of K10, every round checked"),
    # larger families of the reference's result files (their published run times are
    # 11.04 s and 1.10 s); the oracle's depth-first enumeration of them takes minutes,
    # so they carry no CPU leg
    "enum-12-22": ("bibd", (12, 22, 11, 6, 5), "all BIBD(12,22,11,6,5) (11,603 designs) by orderly generation"),
    "enum-9-36": ("bibd", (9, 36, 12, 3, 3), "all BIBD(9,36,12,3,3) (22,521 designs) by orderly generation"),
    "enum-16-24": ("bibd", (16, 24, 9, 6, 3), "all BIBD(16,24,9,6,3) (18,920 designs) by orderly generation"),
    # k-systems with groups of 3 and 4 (the reference's 15x7x3 run: 7 matrices, 2.44 s on 10
    # threads from its 26 start matrices of 4 rounds); the oracle has no enumeration for them
    "enum-kts15": ("kgroups", (15, 3), "all k-systems of 15 players in groups of 3: the 7 Kirkman triple systems"),
    "enum-ag24": ("kgroups", (16, 4), "all k-systems of 16 players in groups of 4: the resolution of AG(2,4)"),
}
ENUM_NO_CPU = {"enum-12-22", "enum-9-36", "enum-16-24", "enum-kts15", "enum-ag24"}


def run_enum(args):
    """Whole enumerations with every level checked on the GPU (configs 1 and 5)."""
    import ise_gb300 as G
    kind, params, desc = ENUM_WORKLOADS[args.workload]
    ctx = G.Context(max_items=1 << 20)
    runs = []
    l0 = None
    for i in range(args.warmup + args.steps):
        if i == args.warmup:
            l0 = ctx.kernel_launches()
        if kind == "bibd":
            found, st = ctx.enumerate_bibd(*params)
        elif kind == "kgroups":
            found, st = ctx.enumerate_ksys_groups(*params)
        else:
            found, st = ctx.enumerate_ksys(*params)
        runs.append((len(found), st.checks, st.seconds, st.kernel_ms, st.batches,
                     [int(x) for x in st.level_checks], [round(float(x), 3) for x in st.level_kernel_ms],
                     st.gen_seconds, int(st.trials), [round(float(x), 3) for x in st.level_gen_ms]))
    launches = ctx.kernel_launches() - l0
    timed = runs[args.warmup:]
    secs = sum(r[2] for r in timed)
    checks = sum(r[1] for r in timed)
    designs = sum(r[0] for r in timed)
    cpu = None
    if not args.no_cpu and args.workload not in ENUM_NO_CPU:
        import time as _t
        sys.path.insert(0, os.path.join(REPO, "oracle"))
        import oracle
        t0 = _t.perf_counter()
        if kind == "bibd":
            ref, nchk = oracle.bibd_enumerate(*params)
        else:
            ref, nchk = oracle.ksys_enumerate(*params)
        dt = _t.perf_counter() - t0
        assert len(ref) == timed[0][0]
        cpu = {"value": len(ref) / dt, "unit": "designs/s", "cores": 1, "kind": "port",
               "sample": "one whole enumeration (%d checks, %.1f s)" % (nchk, dt)}
    line = {"metric": "designs/sec (%s)" % args.workload, "value": designs / secs, "unit": "designs/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * secs / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64 bit rows / u8",
            "data": "exhaustive", "config": {"workload": desc, "designs": timed[0][0],
                                             "checks_per_step": timed[0][1], "batches_per_step": timed[0][4],
                                             "level_checks": timed[0][5], "level_kernel_ms": timed[-1][6],
                                             "level_gen_ms": timed[-1][9]},
            "checks_per_s": checks / secs, "kernel_ms_per_step": sum(r[3] for r in timed) / args.steps,
            "gen_ms_per_step": 1e3 * sum(r[7] for r in timed) / args.steps,
            "cpu_baseline": cpu, "gpu_launches": launches}
    if kind in ("ksys", "kgroups"):
        # relabelings the checks tried (cnvCheckNew candidates), the k-system check's unit of work
        line["relabelings_tried_per_step"] = timed[0][8]
    print(json.dumps(line), flush=True)
    ctx.close()


def run_mix(args):
    """Config 3: one persistent launch over the uneven 2M mix of partial matrices, each
    made by seeded random backtracking of its filled rows (ise_gb300.workloads)."""
    import ise_gb300 as G
    from ise_gb300 import workloads
    n_total = args.items if args.items != N_ITEMS else workloads.MIX_ITEMS
    t0 = time.perf_counter()
    batches = workloads.config3_mix(n_total, SEED + 3)
    gen_s = time.perf_counter() - t0
    n = sum(len(bt["nrows"]) for bt in batches)
    # a level-keeping caller reads only the verdicts: canon_sync returns canonical + status
    ctx = G.Context(max_items=n + 16, max_words=16 * n, aut_cap=1, options=G.OPT_VERDICT_SYNC)
    for _ in range(args.warmup):
        workloads.submit_mix(ctx, batches)
        ctx.sync(raw=True)
    l0 = ctx.kernel_launches()
    kms, walls = [], []
    with ClockSampler(0) as clk:
        for _ in range(args.steps):
            t0 = time.perf_counter()
            workloads.submit_mix(ctx, batches)
            r = ctx.sync(raw=True, copy=False)      # the result buffers as the C API returns them
            walls.append(time.perf_counter() - t0)
            kms.append(r["kernel_ms"])
    launches = ctx.kernel_launches() - l0
    r = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in r.items()}
    if r["n"] != n or r["status"].any():
        raise SystemExit("bench: mix reported %d bad status items" % int((r["status"] != 0).sum()))
    kinds, off = [], 0
    for bt in batches:
        cnt = len(bt["nrows"])
        can = r["canonical"][off:off + cnt].astype(np.float64)
        kinds.append({"shape": bt["name"], "items": cnt, "rows_filled": [int(bt["nrows"].min()),
                                                                          int(bt["nrows"].max())],
                      "canonical_fraction": float(can.mean()),
                      "from_complete_design": int(bt["from_complete"])})
        off += cnt
    h2d = sum(int(bt["data"].nbytes) for bt in batches) + 16 * n    # rows / rounds + work descriptors
    d2h = 2 * n         # canonical + status (CANON_OPT_VERDICT_SYNC)
    line = {"metric": "exact canonicity checks/sec (config 3 uneven mix, one persistent launch)",
            "value": n * args.steps / (sum(kms) / 1e3), "unit": "checks/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": sum(kms) / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u64 bit rows / u8", "data": "synthetic",
            "config": {"workload": "%d partial matrices by seeded random backtracking of their filled rows "
                                   "(seed %d): 40%% STS(15) 5-15 rows, 30%% BIBD(8,14,7,4,3) 4-8, "
                                   "20%% BIBD(11,11,5,5,2) 4-11, 10%% K10 3-9 rounds" % (n, SEED + 3),
                       "kinds": kinds,
                       "canonical_fraction": float(r["canonical"].astype(np.float64).mean()),
                       "generation_s": gen_s},
            "e2e": {"value": n * args.steps / sum(walls), "unit": "checks/s",
                    "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "gpu_launches": launches, "clocks": clk.summary()}
    print(json.dumps(line), flush=True)
    ctx.close()


def run_learned(args):
    """Config 4: the learned first-row order against the plain order."""
    import ise_gb300 as G
    n_train = 333_334                       # x 15 rows = 5.0M (features, label) pairs
    n_eval = args.items
    ctx = G.Context(max_items=16, aut_cap=1)
    t0 = time.perf_counter()
    d_rows = ctx.alloc(n_train * V * 8)
    ctx.generate_sts_device(n_train, V, SEED, True, d_rows)
    d_lab = ctx.alloc(2 * n_train)
    d_nodes = ctx.alloc(8 * n_train)
    ctx.label_first_rows(n_train, V, B, G.RAW, d_rows, d_lab, d_nodes)
    lab = ctx.d2h(np.zeros(n_train, np.uint16), d_lab)
    labels = ((lab[:, None] >> np.arange(V, dtype=np.uint16)) & 1).astype(np.float32).reshape(-1)
    d_feat = ctx.alloc(n_train * V * 64 * 2)
    ctx.mlp_features(n_train, V, B, d_rows, d_feat)
    d_y = ctx.alloc(labels.nbytes)
    ctx.h2d(d_y, labels)
    params0 = G.init_mlp_params(SEED)
    params, losses = ctx.mlp_train(n_train * V, d_feat, d_y, params0, epochs=3, batch=65536, lr=1e-3)
    train_s = time.perf_counter() - t0
    for p_ in (d_rows, d_lab, d_nodes, d_feat, d_y):
        ctx.free(p_)

    # evaluation on a fresh batch
    d_rows = ctx.alloc(n_eval * V * 8)
    ctx.generate_sts_device(n_eval, V, SEED + 1, True, d_rows)
    flags = G.COMPLETE | G.RAW | G.AUT_CANON
    res = {}
    for name, prm in (("plain", None), ("learned", params)):
        ctx.set_ordering(prm)
        bufs = [ctx.alloc(n_eval), ctx.alloc(16 * n_eval), ctx.alloc(16 * n_eval), ctx.alloc(n_eval)]
        for _ in range(args.warmup):
            ctx.check_bibd_device(n_eval, V, B, flags, d_rows, *bufs)
            ctx.stream_sync()
        ms = []
        for _ in range(args.steps):
            ctx.check_bibd_device(n_eval, V, B, flags, d_rows, *bufs)
            ctx.stream_sync()
            ms.append(ctx.last_kernel_ms())
        outs = [ctx.d2h(np.zeros(n_eval * k, np.uint8), b) for b, k in zip(bufs, (1, 16, 16, 1))]
        res[name] = (n_eval * args.steps / (sum(ms) / 1e3), outs)
        for b in bufs:
            ctx.free(b)
    identical = all(np.array_equal(a, b) for a, b in zip(res["plain"][1], res["learned"][1]))
    canon_mask = res["plain"][1][0].astype(bool)
    # lex-max nodes of the check's search (the first pass) in both orders, split by verdict
    d_nodes = ctx.alloc(8 * n_eval)
    node_stats = {}
    for name, prm in (("plain", None), ("learned", params)):
        ctx.set_ordering(prm)
        ctx.lexmax_nodes_bibd(n_eval, V, B, flags, d_rows, d_nodes)
        nd = ctx.d2h(np.zeros(n_eval, np.uint64), d_nodes).astype(np.float64)
        node_stats[name] = {"mean": float(nd.mean()), "canonical_mean": float(nd[canon_mask].mean()),
                            "noncanonical_mean": float(nd[~canon_mask].mean())}
    ctx.set_ordering(None)
    # the first rows that reach the canonical form, and the top-1 hit rate of the network
    d_lab = ctx.alloc(2 * n_eval)
    ctx.label_first_rows(n_eval, V, B, G.RAW, d_rows, d_lab)
    lab = ctx.d2h(np.zeros(n_eval, np.uint16), d_lab)
    # the bound on what any first-row order can save: the exact labels as the order
    # (the rows that start a labeling of the canonical form first, as a perfect network
    # would rank them)
    bits = ((lab[:, None] >> np.arange(V, dtype=np.uint16)) & 1).astype(np.int64)
    rank = np.argsort(-bits * 16 + np.arange(V)[None, :], axis=1, kind="stable").astype(np.uint64)
    perfect = (rank << (np.uint64(4) * np.arange(V, dtype=np.uint64))[None, :]).sum(axis=1, dtype=np.uint64)
    perfect |= np.uint64(0xF) << np.uint64(4 * V)      # nibble 15: the unused position
    d_ord = ctx.alloc(8 * n_eval)
    ctx.h2d(d_ord, perfect)
    ctx.lexmax_nodes_bibd(n_eval, V, B, flags, d_rows, d_nodes, d_ord)
    nd = ctx.d2h(np.zeros(n_eval, np.uint64), d_nodes).astype(np.float64)
    node_stats["exact labels as the order"] = {"mean": float(nd.mean()), "canonical_mean": float(nd[canon_mask].mean()),
                                               "noncanonical_mean": float(nd[~canon_mask].mean())}
    ctx.free(d_ord)
    d_feat = ctx.alloc(65536 * V * 64 * 2)
    d_log = ctx.alloc(65536 * V * 4)
    ctx.mlp_features(65536, V, B, d_rows, d_feat)
    ctx.mlp_forward(65536 * V, d_feat, params, d_log)
    logit = ctx.d2h(np.zeros(65536 * V, np.float32), d_log).reshape(65536, V)
    top1 = float(np.mean((lab[:65536] >> np.argmax(logit, axis=1).astype(np.uint16)) & 1))
    for p_ in (d_lab, d_nodes, d_feat, d_log, d_rows):
        ctx.free(p_)
    line = {"metric": "exact canonicity checks/sec, learned-ordered vs plain (config 4)",
            "value": res["learned"][0], "unit": "checks/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "bf16 MLP / u64 bit rows", "data": "synthetic",
            "config": {"workload": "train: %d STS(15) (seed %d, %d rows, labels from the exact search); eval: "
                                   "%d fresh STS(15) (seed %d)" % (n_train, SEED, n_train * V, n_eval, SEED + 1),
                       "mlp": "64-128-128-1 BF16, FP32 accumulate, Adam 3 epochs, batch 65536"},
            "plain_checks_per_s": res["plain"][0], "learned_over_plain": res["learned"][0] / res["plain"][0],
            "outputs_identical": identical, "train_loss_per_epoch": [float(x) for x in losses],
            "train_seconds": train_s, "top1_hit_rate": top1,
            "lexmax_nodes": node_stats,
            "lexmax_nodes_learned_over_plain": node_stats["learned"]["mean"] / node_stats["plain"]["mean"]}
    print(json.dumps(line), flush=True)
    ctx.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-baseline leg")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end leg")
    ap.add_argument("--items", type=int, default=N_ITEMS,
                    help="matrices per step (default: the full 1,048,576; smaller only for profiling)")
    ap.add_argument("--workload", default="check-sts15",
                    choices=["check-sts15", "mix", "learned"] + sorted(ENUM_WORKLOADS),
                    help="check-sts15 (default, the metric's configuration) or a whole enumeration")
    ap.add_argument("--mode", default="autcanon", choices=["autcanon", "plain"],
                    help="autcanon: |Aut| of rejected matrices via canonization (the workload); "
                         "plain: the reference's TestCanonicity outputs only")
    args = ap.parse_args()
    rank, world, local, dist = dist_setup(args.gpus)
    if args.workload == "mix":
        if rank == 0:
            run_mix(args)
    elif args.workload == "learned":
        if rank == 0:
            run_learned(args)
    elif args.workload != "check-sts15":
        if rank == 0:
            run_enum(args)
    elif args.impl == "reference":
        run_reference(args, rank, world, dist)
    else:
        run_gpu(args, rank, world, local, dist)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
