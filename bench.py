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
# DRAM bytes per check of the check kernel: dram__bytes_read.sum + dram__bytes_write.sum of one ncu
# capture of 131,072 checks (15,918,592 B + 0 B; profiles/bibd_uniform_kernel_sts15_131k.md),
# scaled by the checks of a launch (traffic grows with the number of matrices read).
TRAFFIC_PER_CHECK = 15918592.0 / 131072
MEASURED_PEAKS = os.path.join(REPO, "MEASURED_PEAKS.json")


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
        self.path = os.path.join(REPO, "gpurun_out", "clocks_%d.csv" % os.getpid())

    def __enter__(self):
        os.makedirs(os.path.dirname(self.path), exist_ok=True)
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
                                   % (len(rows), len(rows))},
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
    ctx.generate_sts_device(n, V, SEED, True, d_rows)
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
    achieved = (IN_BYTES + OUT_BYTES) * n / (sum(times) / len(times) / 1e3) / 1e9

    # end to end through the batch API with host buffers
    host_rows = ctx.d2h(np.zeros(n * V, np.uint64), d_rows)
    e2e_dt = None
    if not args.no_e2e:
        e2e_steps = max(1, min(args.steps, 3))
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            ctx.submit_bibd(host_rows, V, B, flags)
            res = ctx.sync(raw=True)
        e2e_dt = (time.perf_counter() - t0) / e2e_steps
        assert res["n"] == n and np.array_equal(res["canonical"], can)
    h2d = n * V * 8 + n * 16
    d2h = n * (1 + 1 + 1 + 1 + 4 + 16 + 16 + 8 + 2 + 1)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        sample = min(n, 4096 * threads)
        rows_s = host_rows.reshape(n, V)[:sample]
        rate, done, dt = cpu_check_rate(rows_s, threads, 20)
        cpu = {"value": rate, "unit": "checks/s", "cores": threads, "kind": "port",
               "sample": "first %d items of the same batch (%d checked in %.1f s)" % (sample, done, dt)}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "checks/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "u64 bit rows / u8", "data": "synthetic",
            "config": {"workload": WORKLOAD if n == N_ITEMS else "%d items of: %s" % (n, WORKLOAD),
                       "ordering": "plain", "flags": FLAGS_NAME if args.mode == "autcanon" else "COMPLETE|RAW",
                       "items_per_step": n, "canonical_fraction": float(can.mean()),
                       "variant": ["one pass", "two passes", "split by first row"][variant],
                       "tune_ms_65536": [round(x, 2) for x in tune_ms],
                       "l2": "flushed between steps (512 MiB write)",
                       "parallelism": "replicas" if world > 1 else "single GPU"},
            "e2e": None if e2e_dt is None else {"value": world * n / e2e_dt, "unit": "checks/s",
                                                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                         "frac": achieved / hbm, "traffic": TRAFFIC_PER_CHECK * n,
                         "note": "peak %s; the check is an integer search (ALU/issue bound), HBM "
                                 "traffic is %d B per check" % (src, IN_BYTES + OUT_BYTES)},
            "cpu_baseline": cpu,
            "gpu_launches": launches,
            "clocks": clk.summary(),
        }
        print(json.dumps(line), flush=True)
    for p in (d_rows, d_can, d_wit, d_aut, d_st, l2_flush):
        ctx.free(p)
    ctx.close()


ENUM_WORKLOADS = {
    "enum-sts13": ("bibd", (13, 26, 6, 3, 1), "config 1: all BIBD(13,26,6,3,1) (STS(13)) by orderly generation"),
    "enum-sts15": ("bibd", (15, 35, 7, 3, 1), "all BIBD(15,35,7,3,1) (STS(15)) by orderly generation"),
    "enum-k10": ("ksys", (10,), "config 5: all 1-factorizations of K10, every round checked"),
    # larger families of the reference's result files (their published run times are
    # 11.04 s and 1.10 s); the oracle's depth-first enumeration of them takes minutes,
    # so they carry no CPU leg
    "enum-12-22": ("bibd", (12, 22, 11, 6, 5), "all BIBD(12,22,11,6,5) (11,603 designs) by orderly generation"),
    "enum-9-36": ("bibd", (9, 36, 12, 3, 3), "all BIBD(9,36,12,3,3) (22,521 designs) by orderly generation"),
}
ENUM_NO_CPU = {"enum-12-22", "enum-9-36"}


def run_enum(args):
    """Whole enumerations with every level checked on the GPU (configs 1 and 5)."""
    import ise_gb300 as G
    kind, params, desc = ENUM_WORKLOADS[args.workload]
    ctx = G.Context(max_items=1 << 20)
    runs = []
    for _ in range(args.warmup + args.steps):
        if kind == "bibd":
            found, st = ctx.enumerate_bibd(*params)
        else:
            found, st = ctx.enumerate_ksys(*params)
        runs.append((len(found), st.checks, st.seconds, st.kernel_ms, st.batches,
                     [int(x) for x in st.level_checks], [round(float(x), 3) for x in st.level_kernel_ms],
                     st.gen_seconds))
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
                                             "level_checks": timed[0][5], "level_kernel_ms": timed[-1][6]},
            "checks_per_s": checks / secs, "kernel_ms_per_step": sum(r[3] for r in timed) / args.steps,
            "gen_ms_per_step": 1e3 * sum(r[7] for r in timed) / args.steps,
            "cpu_baseline": cpu}
    print(json.dumps(line), flush=True)
    ctx.close()


MIX_SHAPES = [  # (share, kind, (v, b, r, k, lambda) or np, min filled rows, max filled rows)
    (0.40, "bibd", (15, 35, 7, 3, 1), 5, 15),
    (0.30, "bibd", (8, 14, 7, 4, 3), 4, 8),
    (0.20, "bibd", (11, 11, 5, 5, 2), 4, 11),
    (0.10, "ksys", 10, 3, 9),
]


def _permute_bits(words, perm):
    """Column permutation of packed rows: new column c = old column perm[c]."""
    bits = (words[..., None] >> perm.astype(np.uint64)) & np.uint64(1)
    return (bits << np.arange(perm.shape[-1], dtype=np.uint64)).sum(axis=-1, dtype=np.uint64)


def build_mix(ctx, n_total, seed):
    """Seeded stand-in for the uneven batch of config 3: partial matrices that are
    prefixes of randomly relabelled designs (so every one is a valid partial design)."""
    import ise_gb300 as G
    rng = np.random.default_rng(seed)
    batches = []
    for share, kind, params, lo, hi in MIX_SHAPES:
        cnt = int(round(share * n_total))
        nr = rng.integers(lo, hi + 1, size=cnt).astype(np.uint8)
        if kind == "bibd" and params[0] == 15:
            d = ctx.alloc(cnt * 15 * 8)
            ctx.generate_sts_device(cnt, 15, seed + 1, False, d)
            rows = ctx.d2h(np.zeros(cnt * 15, np.uint64), d).reshape(cnt, 15)
            ctx.free(d)
            batches.append(("bibd", 15, 35, rows, nr))
        elif kind == "bibd":
            v, b = params[0], params[1]
            designs, _ = ctx.enumerate_bibd(*params)
            base = np.stack([G.pack_rows(M) for M, _ in designs])
            pick = rng.integers(len(base), size=cnt)
            rp = np.argsort(rng.random((cnt, v)), axis=1)
            rows = np.take_along_axis(base[pick], rp, axis=1)
            cp = np.argsort(rng.random((cnt, b)), axis=1)
            rows = _permute_bits(rows, cp[:, None, :].repeat(v, axis=1))
            batches.append(("bibd", v, b, rows, nr))
        else:
            found, _ = ctx.enumerate_ksys(params)
            base = np.stack([R for R, _ in found])                       # 396 x 9 x 10
            pick = rng.integers(len(base), size=cnt)
            R = base[pick].astype(np.int64)
            # relabel so that a random round becomes round 0 = (0 1)(2 3)...
            d = rng.integers(9, size=cnt)
            src = R[np.arange(cnt), d]                                   # cnt x 10 players in pair order
            gperm = np.argsort(rng.random((cnt, 5)), axis=1)
            flip = rng.integers(2, size=(cnt, 5))
            lab = np.zeros((cnt, 10), np.int64)
            for g in range(5):
                a_ = src[np.arange(cnt), 2 * gperm[:, g]]
                b_ = src[np.arange(cnt), 2 * gperm[:, g] + 1]
                x_ = np.where(flip[:, g] == 1, b_, a_)
                y_ = np.where(flip[:, g] == 1, a_, b_)
                lab[np.arange(cnt), x_] = 2 * g
                lab[np.arange(cnt), y_] = 2 * g + 1
            X = np.take_along_axis(lab[:, None, :].repeat(9, axis=1), R, axis=2)   # relabelled rounds
            pa, pb = X[..., 0::2], X[..., 1::2]
            lo_, hi_ = np.minimum(pa, pb), np.maximum(pa, pb)
            order = np.argsort(lo_, axis=2)
            lo_ = np.take_along_axis(lo_, order, axis=2)
            hi_ = np.take_along_axis(hi_, order, axis=2)
            rounds = np.stack([lo_, hi_], axis=3).reshape(cnt, 9, 10)
            rorder = np.argsort(rounds[:, :, 1], axis=1)
            rounds = np.take_along_axis(rounds, rorder[:, :, None], axis=1).astype(np.uint8)
            batches.append(("ksys", 10, 9, rounds, nr))
    return batches


def run_mix(args):
    """Config 3: one persistent launch over the uneven 2M mix."""
    import ise_gb300 as G
    n_total = args.items if args.items != N_ITEMS else 2_097_152
    ctx = G.Context(max_items=n_total + 16, max_words=16 * n_total, aut_cap=1)
    batches = build_mix(ctx, n_total, SEED + 3)
    n = sum(len(b[4]) for b in batches)

    def submit():
        for kind, v, b, rows, nr in batches:
            if kind == "bibd":
                ctx.submit_bibd(rows, v, b, G.RAW, nr)
            else:
                ctx.submit_ksys(rows, v, b, 0, nr)

    for _ in range(args.warmup):
        submit()
        ctx.sync()
    l0 = ctx.kernel_launches()
    kms, walls = [], []
    with ClockSampler(0) as clk:
        for _ in range(args.steps):
            t0 = time.perf_counter()
            submit()
            r = ctx.sync(raw=True)
            walls.append(time.perf_counter() - t0)
            kms.append(r["kernel_ms"])
    assert r["n"] == n and not r["status"].any()
    line = {"metric": "exact canonicity checks/sec (config 3 uneven mix, one persistent launch)",
            "value": n * args.steps / (sum(kms) / 1e3), "unit": "checks/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": sum(kms) / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u64 bit rows / u8", "data": "synthetic",
            "config": {"workload": "%d partial matrices: 40%% STS(15) 5-15 rows, 30%% BIBD(8,14,7,4,3) 4-8, "
                                   "20%% BIBD(11,11,5,5,2) 4-11, 10%% K10 3-9 rounds; prefixes of randomly "
                                   "relabelled designs, seed %d" % (n, SEED + 3),
                       "canonical_fraction": float(r["canonical"].astype(np.float64).mean())},
            "e2e": {"value": n * args.steps / sum(walls), "unit": "checks/s",
                    "h2d_bytes_per_step": int(sum(b[3].nbytes for b in batches) + 16 * n),
                    "d2h_bytes_per_step": 51 * n},
            "gpu_launches": ctx.kernel_launches() - l0, "clocks": clk.summary()}
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
    # lex-max nodes in both orders and the top-1 hit rate of the network
    d_lab = ctx.alloc(2 * n_eval)
    d_nodes = ctx.alloc(8 * n_eval)
    ctx.set_ordering(None)
    ctx.label_first_rows(n_eval, V, B, G.RAW, d_rows, d_lab, d_nodes)
    nodes_plain = ctx.d2h(np.zeros(n_eval, np.uint64), d_nodes).astype(np.float64)
    lab = ctx.d2h(np.zeros(n_eval, np.uint16), d_lab)
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
            "lexmax_nodes_plain_mean": float(nodes_plain.mean())}
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
