"""Benchmark of the device Mehrotra IPM on the block-angular LP (family 1:
40 blocks of 500x1200 + 2000 linking rows, m=22000, n=48000, 288k nnz).

A step is one complete solve to 1e-8 relative primal / dual infeasibility and
duality gap, mixed precision (FP32 fronts, FP64 residuals and refinement, FP64
switch near convergence). value = LPs/s with the LP resident in device memory
(CUDA events around sk_solver_run on the solver stream); e2e = LPs/s through the
one-shot C ABI call sk_ipm_solve_csc from host arrays (analysis, upload, solve
and download inside the timed region).

--impl reference times the CPU restatement of the reference algorithm (oracle/,
plain C, FP64, dense Cholesky) on all host cores over a bounded sample of the
same LP family (see cpu_sample()).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "soverign-gpu-accelerator-_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

METRIC = "time-to-1e-8 gap & LPs/sec: mixed+learned vs plain FP64 IPM, same GB300"
WORKLOAD = "block-angular LP, 40 blocks of 500x1200 + 2000 linking rows (m=22000, n=48000, 6 nnz/col), seed 0xC1"
FULL_NNZ = 288000


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), d.get("bf16_tflops", 1900.0), "measured"
    return 6800.0, 1900.0, "fallback"


def ensure_built():
    import sankhya_gb300 as sk
    if not os.path.exists(sk.LIB_PATH):
        import __graft_entry__ as g
        g.build()
    return sk


def cpu_sample(sk):
    """Bounded CPU sample of the workload: one block of the same family
    (500x1200 block + 50 linking rows, m=550, n=1200, 7200 nnz = 1/40 of the full
    LP's nonzeros). CPU LPs/s on the full LP is reported as the sample rate x
    7200/288000 (linear in nnz, which favours the CPU: its dense factorisation
    grows as m^3)."""
    return sk.block_angular(0xC1, 1, 500, 1200, 50, 5)


class Clocks:
    def __init__(self):
        self.p = None
        import tempfile
        # nvidia-smi samples of the timed region (path overridable for keeping the record)
        self.path = os.environ.get("SK_BENCH_CLOCKS", os.path.join(tempfile.gettempdir(), "sk_bench_clocks.csv"))

    def start(self):
        try:
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if not self.p:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.p.terminate()
        self.p.wait()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        dev = os.environ.get("LOCAL_RANK", "0")
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax.append(float(parts[2]))
                except ValueError:
                    continue
                for nm, v in zip(names, parts[5:9]):
                    if v.lower() == "active":
                        reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def count_kernel_launches(fn):
    """Kernels launched by one call of fn() (which launches only this library's
    kernels), counted from a CUPTI trace (torch.profiler); graph-launched kernels
    are included. Returns None if the profiler is unavailable."""
    import tempfile
    try:
        import torch
        from torch.profiler import ProfilerActivity, profile
        acts = [ProfilerActivity.CPU, ProfilerActivity.CUDA]
        with profile(activities=acts):       # the first session of a process records no kernels
            torch.zeros(1, device="cuda").add_(1)
            torch.cuda.synchronize()
        with profile(activities=acts) as prof:
            fn()
            torch.cuda.synchronize()
        with tempfile.NamedTemporaryFile(suffix=".json", delete=False) as f:
            path = f.name
        prof.export_chrome_trace(path)
        with open(path) as f:
            trace = json.load(f)
        os.unlink(path)
        return sum(1 for e in trace.get("traceEvents", []) if e.get("cat") == "kernel")
    except Exception:
        return None


WEIGHTS = os.path.join(ROOT, "soverign-gpu-accelerator-_gb300", "weights", "learned_start_family3.npy")


def batch_comparison(sk, nlps, dist=None, rank=0, world=1):
    """LPs/s on the first `nlps` members of the 512-LP uneven batch (family 3),
    solved as one batch: mixed precision + learned start (falling back per LP to
    Mehrotra's start), mixed precision + Mehrotra's start, and the plain FP64 IPM
    (unit start); device time of the second of two runs of each. Then the plain
    FP64 IPM on the same LPs one at a time (sequential solves). With several ranks
    the LPs are sharded (sharding.shard_lps): each rank solves its own LPs as one
    batch, the time is the slowest rank's and the per-LP results are gathered to
    rank 0 once per arm; no other communication."""
    import sharding
    lps_all = [sk.generate(3, k) for k in range(nlps)]
    shards = sharding.shard_lps([sharding.lp_cost(lp.m, lp.n, lp.nnz) for lp in lps_all], world)
    mine = shards[rank]
    lps = [lps_all[k] for k in mine]
    net = None
    if os.path.exists(WEIGHTS):
        net = sk.Gnn(1)
        net.load(WEIGHTS)
    out = {"lps": nlps, "members": "family-3 instances 0..%d (m %d..%d)" % (
        nlps - 1, min(lp.m for lp in lps_all), max(lp.m for lp in lps_all))}
    if world > 1:
        out["sharding"] = {"ranks": world, "lps_per_rank": [len(sh) for sh in shards]}
    arms = [("mixed_learned", sk.PREC_MIXED, sk.START_LEARNED), ("mixed_mehrotra", sk.PREC_MIXED, sk.START_MEHROTRA),
            ("plain_fp64", sk.PREC_FP64, sk.START_UNIT)]
    for name, prec, start in arms:
        if start == sk.START_LEARNED and net is None:   # the same weights file on every rank
            continue
        infos, ms = [], 0.0
        if lps:
            s = sk.Solver(lps, precision=prec, start=start)
            if start == sk.START_LEARNED:
                s.set_gnn(net)
            s.run()
            s.run()
            infos = [s.result(k, want_vectors=False)[0] for k in range(len(lps))]
            s.close()
            ms = infos[0]["device_ms"]
        ms = barrier_max(dist, ms)
        per_lp = sharding.gather_results({mine[q]: {"status": i["status"], "iterations": i["iterations"],
                                                    "learned_start": i["learned_start"]}
                                          for q, i in enumerate(infos)}, dist, rank, world)
        if per_lp is None:
            continue
        vals = [per_lp[k] for k in range(nlps)]
        out[name] = {"ms": ms, "lps_per_s": 1000.0 * nlps / ms, "all_optimal": all(v["status"] == 0 for v in vals),
                     "mean_iterations": sum(v["iterations"] for v in vals) / nlps}
        if start == sk.START_LEARNED:
            out[name]["learned_used"] = sum(v["learned_start"] for v in vals)
    if net is not None:
        net.close()
    if "plain_fp64" in out:
        base = out["plain_fp64"]["lps_per_s"]
        for name in ("mixed_learned", "mixed_mehrotra"):
            if name in out:
                out[name]["speedup_vs_plain_fp64"] = out[name]["lps_per_s"] / base
    # the same LPs solved one after another by the plain FP64 IPM, one LP per solver (how the
    # reference's device IPM is used); device time of the second of two runs of each
    try:
        seq_ms, seq_ok = 0.0, True
        for lp in lps:
            s = sk.Solver([lp], precision=sk.PREC_FP64, start=sk.START_UNIT)
            s.run()
            s.run()
            info, *_ = s.result(0, want_vectors=False)
            s.close()
            seq_ms += info["device_ms"]
            seq_ok = seq_ok and info["status"] == 0
        seq_ms = barrier_max(dist, seq_ms)
        oks = sharding.gather_results({rank: seq_ok}, dist, rank, world)
        if oks is not None:
            out["sequential_plain_fp64"] = {"ms": seq_ms, "lps_per_s": 1000.0 * nlps / seq_ms,
                                            "all_optimal": all(oks.values())}
            for name in ("mixed_learned", "mixed_mehrotra", "plain_fp64"):
                if name in out:
                    out[name]["speedup_vs_sequential_plain_fp64"] = out[name]["lps_per_s"] / (1000.0 * nlps / seq_ms)
    except Exception as e:          # the comparison is auxiliary: report, do not lose the bench line
        out["sequential_plain_fp64"] = {"error": "%s: %s" % (type(e).__name__, e)}
    return out


def family2_comparison(sk, unit_start_arm=False):
    """Time-to-1e-8 on the family-2 staircase LP (m=200000, n=500000): mixed precision with
    the learned start (falling back to Mehrotra's start), mixed precision with the plain
    method's unit start, and the plain FP64 IPM. One solve per arm (each solve is tens of
    seconds); host analysis (ordering, plan) is timed separately from the device solve."""
    lp = sk.generate(2, 0)
    ref = None
    fixture = os.path.join(ROOT, "tests", "golden", "highs_large_objectives.json")
    if os.path.exists(fixture):
        with open(fixture) as f:
            for c in json.load(f)["cases"]:
                if c["name"] == "family2_0" and c["digest"]["nnz"] == lp.nnz:
                    ref = c["objective"]
    net = None
    if os.path.exists(WEIGHTS):
        net = sk.Gnn(1)
        net.load(WEIGHTS)
    out = {"workload": "staircase transportation LP, 50 stages (m=200000, n=500000, 4 nnz/col), seed 0xC2",
           "objective_reference": "HiGHS (tests/golden/highs_large_objectives.json)" if ref is not None else None}
    arms = [("mixed_learned", sk.PREC_MIXED, sk.START_LEARNED), ("mixed_unit_start", sk.PREC_MIXED, sk.START_UNIT),
            ("plain_fp64", sk.PREC_FP64, sk.START_UNIT)]
    if not unit_start_arm:
        arms = [a for a in arms if a[0] != "mixed_unit_start"]
    for name, prec, start in arms:
        if start == sk.START_LEARNED and net is None:
            continue
        t0 = time.perf_counter()
        s = sk.Solver([lp], precision=prec, start=start)
        t1 = time.perf_counter()
        if start == sk.START_LEARNED:
            s.set_gnn(net)
        s.run()
        info, *_ = s.result(0, want_vectors=False)
        t2 = time.perf_counter()
        if name == "mixed_learned":
            # instrumented replay of one FP32 factorisation at the final iterate (not part of the solve time)
            out["profile_fp32"] = s.profile(fp32=True)
        s.close()
        arm = {"status": info["status"], "iterations": info["iterations"], "device_ms": info["device_ms"],
               "analysis_s": t1 - t0, "wall_s": t2 - t0, "objective": info["objective"],
               "rel_pinf": info["rel_pinf"], "rel_dinf": info["rel_dinf"], "rel_gap": info["rel_gap"],
               "precision_path": info["precision_path"], "switch_iteration": info["switch_iteration"],
               "factorizations": info["factorizations"], "solves": info["solves"],
               "nnz_factor": info["nnz_factor"], "flops_per_factorization": info["flops_factor"]}
        if start == sk.START_LEARNED:
            arm["learned_used"] = info["learned_start"]
        if ref is not None:
            arm["rel_obj_err_vs_highs"] = abs(info["objective"] - ref) / (1.0 + abs(ref))
        out[name] = arm
    if net is not None:
        net.close()
    base = out["plain_fp64"]
    for name in ("mixed_learned", "mixed_unit_start"):
        if name in out:
            out[name]["speedup_device_vs_plain_fp64"] = base["device_ms"] / out[name]["device_ms"]
            out[name]["speedup_wall_vs_plain_fp64"] = base["wall_s"] / out[name]["wall_s"]
    return out


def _block_diag_csr(parts, col_offsets):
    """Concatenates per-LP CSR arrays (row_ptrs, col_idx, vals) into the CSR of the
    block-diagonal matrix, shifting each block's columns by its offset."""
    import numpy as np
    rps, cis, vs, base = [], [], [], 0
    for (rp, ci, v), co in zip(parts, col_offsets):
        rps.append(rp[:-1].astype(np.int64) + base)
        cis.append(ci.astype(np.int64) + co)
        vs.append(v)
        base += len(v)
    rps.append(np.array([base], dtype=np.int64))
    if base >= 2 ** 31:
        raise ValueError("batch too large for int32 indices")
    return (np.concatenate(rps).astype(np.int32), np.concatenate(cis).astype(np.int32),
            np.ascontiguousarray(np.concatenate(vs)))


def spmv_rooflines(sk, hbm, src, nlps=512, warm=3, reps=10):
    """HBM roofline of the solver's SpMV kernel (autotuned plan, sk_spmv_plan_*) for
    y = A x and y = A^T x on the block-diagonal matrix of the family-3 batch (512
    LPs: 61 M nonzeros, 0.73 GB of CSR indices and values per product, several times
    the 129 MB L2). A 256 MB buffer is written before each timed launch; each launch
    sits between CUDA events on the launching stream (torch's current stream).
    Algorithmic bytes: 12 nnz + 4 (rows + 1) + 8 cols + 8 rows (CSR read once, x read
    once, y written once). The same product through torch's CSR matmul (cuSPARSE)
    is timed the same way for comparison, and the two results are compared."""
    import numpy as np
    import torch
    lps = [sk.generate(3, k) for k in range(nlps)]
    roff = np.cumsum([0] + [lp.m for lp in lps])[:-1]
    coff = np.cumsum([0] + [lp.n for lp in lps])[:-1]
    M, N = sum(lp.m for lp in lps), sum(lp.n for lp in lps)
    mats = [("A x", M, N, _block_diag_csr([lp.csr() for lp in lps], coff)),
            ("A^T y", N, M, _block_diag_csr([(lp.col_ptrs, lp.row_idx, lp.vals) for lp in lps], roff))]
    del lps
    stream = torch.cuda.current_stream()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    out = []
    for name, rows, cols, (rp, ci, v) in mats:
        nnz = len(v)
        d_rp, d_ci, d_v = (torch.from_numpy(a).cuda() for a in (rp, ci, v))
        x = torch.randn(cols, dtype=torch.float64, device="cuda")
        y = torch.zeros(rows, dtype=torch.float64, device="cuda")
        plan = sk.SpmvPlan(rows, cols, nnz, d_rp.data_ptr(), d_ci.data_ptr(), d_v.data_ptr(),
                           stream=stream.cuda_stream)
        tune = plan.info()

        def timed(fn):
            for _ in range(warm):
                fn()
            evs = []
            for _ in range(reps):
                flush.zero_()
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                fn()
                b.record(stream)
                evs.append((a, b))
            torch.cuda.synchronize()
            return statistics.mean(a.elapsed_time(b) for a, b in evs)

        ms = timed(lambda: plan.execute(x.data_ptr(), y.data_ptr(), stream=stream.cuda_stream))
        lib_ms, max_rel = None, None
        try:
            A = torch.sparse_csr_tensor(d_rp, d_ci, d_v, size=(rows, cols))
            xc = x.view(-1, 1)
            z = A.matmul(xc)
            lib_ms = timed(lambda: A.matmul(xc))
            torch.cuda.synchronize()
            scale = torch.sparse_csr_tensor(d_rp, d_ci, d_v.abs(), size=(rows, cols)).matmul(x.abs().view(-1, 1))
            max_rel = float(((z.view(-1) - y).abs() / (1.0 + scale.view(-1))).max())
        except Exception as e:      # torch build without CUDA CSR matmul: comparison left out
            lib_ms = "unavailable: %s" % type(e).__name__
        nbytes = 12.0 * nnz + 4.0 * (rows + 1) + 8.0 * cols + 8.0 * rows
        a = nbytes / (ms / 1000.0) / 1e9
        kname = "k_spmv_win" if tune["windowed"] else "k_spmv"
        out.append({"kernel": "%s<%d, EpiAxpby> (%s, family-3 batch of %d LPs as one block-diagonal matrix)"
                              % (kname, tune["group"], name, nlps),
                    "bound": "hbm", "achieved": a, "peak": hbm, "unit": "GB/s", "frac": a / hbm,
                    "peak_source": "%s copy bandwidth (MEASURED_PEAKS.json hbm_gbs)" % src, "traffic": None,
                    "rows": rows, "cols": cols, "nnz": nnz, "algorithmic_bytes": nbytes, "ms_per_launch": ms,
                    "launches_timed": reps, "l2": "256 MB written before each launch",
                    "lanes_per_row": tune["group"], "rule_lanes_per_row": tune["heuristic_group"],
                    "shared_memory_windows": tune["windowed"],
                    "autotune_ms_per_width": tune["ms_per_group"],
                    "autotune_ms_per_width_windowed": tune["ms_windowed_per_group"],
                    "cusparse_ms_per_launch": lib_ms, "max_rel_diff_vs_cusparse": max_rel})
        plan.close()
        del d_rp, d_ci, d_v, x, y
    del flush
    torch.cuda.empty_cache()
    return out


def assembly_roofline(prof, hbm, src, workload, note):
    """Assembly class of an instrumented replay (sk_solver_profile): algorithmic bytes of
    one assembly over its event-timed duration (both assembly kernels)."""
    a_ms, a_b = prof["assembly"]["ms"], prof.get("assembly_bytes")
    if not a_b or a_ms <= 0:
        return None
    a = a_b / (a_ms / 1000.0) / 1e9
    return {"kernel": "k_asm_diag_* + k_asm_slots_sparse / k_asm_cols_dense (assembly of D A Theta A^T D + "
                      "delta I, %s)" % workload,
            "bound": "hbm", "achieved": a, "peak": hbm, "unit": "GB/s", "frac": a / hbm,
            "peak_source": "%s copy bandwidth (MEASURED_PEAKS.json hbm_gbs)" % src, "traffic": None,
            "ms_total": a_ms, "launches": prof["assembly"]["launches"], "algorithmic_bytes": a_b, "note": note}


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl" if args.impl == "ours" else "gloo")
        return rank, world, dist
    return rank, world, None


def barrier_max(dist, v):
    """Max of v over all ranks (v itself without a process group)."""
    if dist is None:
        return v
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_ours(args):
    rank, world, dist = dist_setup(args)
    sk = ensure_built()
    import numpy as np
    import torch
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    os.environ.setdefault("CUDA_VISIBLE_DEVICES", os.environ.get("CUDA_VISIBLE_DEVICES", ""))
    lp = sk.generate(1, 0)
    solver = sk.Solver([lp], precision=sk.PREC_MIXED)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")   # 256 MB > 129 MB L2
    for _ in range(args.warmup):
        solver.run()
    info0, *_ = solver.result(0, want_vectors=False)
    if info0["status"] != 0:
        raise SystemExit("warm-up solve did not converge: %s" % info0)
    clocks = Clocks()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    dev_ms = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        solver.run()
        info, *_ = solver.result(0, want_vectors=False)
        assert info["status"] == 0, info
        dev_ms.append(info["device_ms"])
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    total_ms = barrier_max(dist, sum(dev_ms))
    value = world * args.steps / (total_ms / 1000.0)
    # kernels per solve, counted on one more (untimed) run of the same solve
    per_run = count_kernel_launches(solver.run)
    launches = per_run * args.steps if per_run is not None else None
    # kernel-class breakdown (instrumented replay of one factorisation + solve at the final iterate)
    prof = solver.profile(fp32=True)                 # tensor-core FP32 updates
    prof_simt = solver.profile(fp32=True, tensor=False)
    solver.close()
    # plain FP64 solve of the same LP for the comparison the metric names
    fp64 = sk.Solver([lp], precision=sk.PREC_FP64)
    fp64.run()
    info64, *_ = fp64.result(0, want_vectors=False)
    fp64.run()
    info64b, *_ = fp64.result(0, want_vectors=False)
    prof64 = fp64.profile(fp32=False)
    fp64.close()
    batch = batch_comparison(sk, args.batch_lps, dist, rank, world) if args.batch_lps > 0 else None
    family2 = None if args.no_family2 else family2_comparison(sk, args.family2_unit_start)
    # end to end through the C ABI (host arrays in, host solution out)
    e2e_t = []
    for _ in range(max(1, args.steps)):
        flush.zero_()
        torch.cuda.synchronize()
        t = time.perf_counter()
        infoe, x, y, s = sk.solve(lp, precision=sk.PREC_MIXED)
        e2e_t.append(time.perf_counter() - t)
        assert infoe["status"] == 0
    e2e_total = barrier_max(dist, sum(e2e_t))
    e2e_value = world * len(e2e_t) / e2e_total
    h2d = lp.nbytes()
    d2h = (2 * lp.n + lp.m) * 8
    hbm, bf16, src = peaks()
    fp64_peak = 1.25   # TFLOP/s, nominal dense FP64 of a GB300 (no FP64 entry in MEASURED_PEAKS.json)
    note = ("event-timed replay of one factorisation and one triangular solve at the final iterate; "
            "the update class includes the diagonal-tile Cholesky fused into it")

    def upd_roof(p, kernel, peak, peak_src, bound):
        u = p["update"]
        a = p["update_flops"] / (u["ms"] / 1000.0) / 1e12 if u["ms"] > 0 else 0.0
        return {"kernel": kernel, "bound": bound, "achieved": a, "peak": peak, "unit": "TFLOP/s", "frac": a / peak,
                "peak_source": peak_src, "traffic": None, "launches": u["launches"], "ms_total": u["ms"],
                "algorithmic_flops": p["update_flops"], "note": note}

    def solve_roof(p, kernel, elem):
        ms = p["fwd_solve"]["ms"] + p["bwd_solve"]["ms"]
        nbytes = 2.0 * elem * info["nnz_factor"]          # each factor entry read once per direction
        a = nbytes / (ms / 1000.0) / 1e9 if ms > 0 else 0.0
        return {"kernel": kernel, "bound": "hbm", "achieved": a, "peak": hbm, "unit": "GB/s", "frac": a / hbm,
                "peak_source": "%s copy bandwidth (MEASURED_PEAKS.json hbm_gbs)" % src, "traffic": None,
                "ms_total": ms, "algorithmic_bytes": nbytes, "note": note}

    # The dominant kernel of the mixed solve (launch list in profiles/): the FP64 trailing update of
    # the last factorisations, an FP64-pipe-bound SIMT kernel.
    roof = upd_roof(prof64, "k_update<double> (FP64 frontal trailing update)", fp64_peak,
                    "nominal GB300 dense FP64 1.25 TFLOP/s (of nominal; MEASURED_PEAKS.json has no FP64 entry)",
                    "fp64")
    # DRAM bytes of one captured launch (ncu, profiles/k_update_fp64_family1.md): 15.1 MB read, 0 written,
    # against 59.5 MB of operand bytes for that launch's 465 tiles (panels and C are L2 hits)
    roof["traffic"] = 15.1e6
    roof["traffic_note"] = ("dram__bytes_read.sum + dram__bytes_write.sum of one captured launch (465 output "
                            "tiles; operand bytes 59.5 MB), profiles/k_update_fp64_family1.md")
    rooflines = [roof,
                 upd_roof(prof, "k_update_tc (FP32 frontal trailing update, tcgen05 TF32 x3; flops counted once)",
                          bf16, "%s bf16 dense tensor peak (MEASURED_PEAKS.json bf16_tflops)" % src, "tensor"),
                 upd_roof(prof_simt, "k_update<float> (FP32 frontal trailing update, SIMT)", bf16,
                          "%s bf16 dense tensor peak (MEASURED_PEAKS.json bf16_tflops)" % src, "tensor"),
                 solve_roof(prof, "k_fwd_tasks<float> + k_bwd_tasks<float> (one triangular solve pair)", 4),
                 solve_roof(prof64, "k_fwd_tasks<double> + k_bwd_tasks<double> (one triangular solve pair)", 8)]
    rooflines.append(assembly_roofline(prof, hbm, src, "family-1 LP, FP32 fronts", note))
    if family2 is not None and "profile_fp32" in family2:
        rooflines.append(assembly_roofline(family2.pop("profile_fp32"), hbm, src,
                                           "family-2 staircase LP, FP32 fronts", note))
    if args.spmv_lps > 0:
        rooflines.extend(spmv_rooflines(sk, hbm, src, nlps=args.spmv_lps))
    rooflines = [r for r in rooflines if r is not None]
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(sk, cores=1)
    line = {"metric": METRIC, "value": value, "unit": "LPs/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64+f32",
            "data": "synthetic, seeded generator (family 1)",
            "config": {"workload": WORKLOAD, "precision": "mixed (FP32 fronts, FP64 residuals/refinement)",
                       "tolerance": "rel pinf, dinf, gap <= 1e-8", "l2": "256 MB buffer written between steps",
                       "parallelism": "replicas" if world > 1 else "single GPU",
                       "iterations": info["iterations"], "precision_path": info["precision_path"],
                       "switch_iteration": info["switch_iteration"], "factorizations": info["factorizations"],
                       "solves": info["solves"], "nnz_factor": info["nnz_factor"],
                       "supernodes": info["num_supernodes"], "flops_per_factorization": info["flops_factor"]},
            "batch_family3": batch,
            "staircase_family2": family2,
            "plain_fp64": {"ms_per_solve": info64b["device_ms"], "iterations": info64b["iterations"],
                           "lps_per_s": 1000.0 / info64b["device_ms"] if info64b["device_ms"] > 0 else None,
                           "speedup_mixed_vs_fp64": info64b["device_ms"] / (total_ms / args.steps)},
            "kernel_breakdown_ms": {"mixed": {k: v for k, v in prof.items() if isinstance(v, dict)},
                                    "mixed_simt_update": {k: v for k, v in prof_simt.items() if isinstance(v, dict)},
                                    "fp64": {k: v for k, v in prof64.items() if isinstance(v, dict)}},
            "wall_s_timed_region": wall,
            "gpu_launches": launches,
            "gpu_launches_note": "kernels of libsankhya_gb300 per solve (CUPTI trace of one extra run) x steps",
            "roofline": roof, "kernel_rooflines": rooflines, "cpu_baseline": cpu, "clocks": clk,
            "e2e": {"value": e2e_value, "unit": "LPs/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "ms_per_step": 1000.0 * e2e_total / len(e2e_t)}}
    if rank == 0:
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


def _cpu_worker(args):
    import sk_oracle as so
    import sankhya_gb300 as sk
    lp = cpu_sample(sk)
    t = time.perf_counter()
    r, *_ = so.ipm_solve(lp)
    return time.perf_counter() - t, r["status"], r["objective"]


def cpu_baseline(sk, cores=1, rounds=12):
    """Oracle port (FP64 CPU restatement of the reference algorithm) on the
    bounded sample; `cores` processes each solve their own copy."""
    import multiprocessing as mp
    import sk_oracle as so
    so.oracle()
    lp = cpu_sample(sk)
    t0 = time.perf_counter()
    if cores == 1:
        res = [_cpu_worker(None) for _ in range(rounds)]
    else:
        ctx = mp.get_context("spawn")
        with ctx.Pool(cores) as pool:
            res = pool.map(_cpu_worker, range(cores * rounds))
    wall = time.perf_counter() - t0
    n = len(res)
    assert all(r[1] == 0 for r in res), res[:2]
    sample_rate = n / wall
    return {"value": sample_rate * lp.nnz / FULL_NNZ, "unit": "LPs/s", "cores": cores, "kind": "port",
            "sample": "%d solves of the one-block member of the family (m=%d, n=%d, nnz=%d) on %d core(s), "
                      "%.1f s; full-LP rate = sample rate x %d/%d nnz" % (n, lp.m, lp.n, lp.nnz, cores, wall,
                                                                       lp.nnz, FULL_NNZ),
            "sample_lps_per_s": sample_rate}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    sk = ensure_built()
    import sk_oracle as so
    so.oracle()
    cores = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_baseline(sk, cores=cores, rounds=1)
    vals = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        vals.append(cpu_baseline(sk, cores=cores, rounds=1))
    wall = time.perf_counter() - t0
    v = statistics.mean(x["value"] for x in vals)
    line = {"metric": METRIC, "impl": "reference", "value": v, "unit": "LPs/s", "n_gpus": 0, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * wall / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic, seeded generator (family 1)",
            "config": {"workload": WORKLOAD, "implementation": "CPU restatement of the reference's Mehrotra IPM "
                       "(oracle/sk_oracle.c, dense FP64 Cholesky); the reference's own CPU code cannot be built "
                       "on the GPU host (its sources are not there)"},
            "cpu_baseline": {"value": v, "unit": "LPs/s", "cores": cores, "kind": "port", "sample": vals[0]["sample"]},
            "e2e": {"value": v, "unit": "LPs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--batch-lps", type=int, default=32,
                    help="family-3 batch members for the mixed+learned vs plain FP64 batch comparison (0: skip)")
    ap.add_argument("--spmv-lps", type=int, default=512,
                    help="family-3 members in the block-diagonal matrix of the SpMV roofline (0: skip)")
    ap.add_argument("--no-family2", action="store_true",
                    help="skip the family-2 staircase LP (m=200000) comparison (about 3 minutes)")
    ap.add_argument("--family2-unit-start", action="store_true",
                    help="add a mixed-precision unit-start arm to the family-2 comparison")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
