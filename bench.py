"""Benchmark of the device Mehrotra IPM: mixed precision + learned start against the
plain FP64 IPM, on one GB300.

Headline workload: the uneven batch of 512 independent LPs (family 3:
m ~ logUniform[200, 5000], n = ceil(m U[2, 3]), density 0.5-2 %, instances
0..511; 763,585 rows, 1,925,793 columns, 61 M nonzeros in all), solved as one
batch to 1e-8 relative primal / dual infeasibility and duality gap per LP.

A step is one complete batched solve of the 512 LPs in mixed precision (FP32
fronts with TF32 x3 tensor-core updates while the directions pass the accuracy
check, FP64 fronts after the switch with FP64-accurate tensor-core updates; FP64
residuals, operator and PCG throughout) started from the learned point (the
bipartite network's prediction, falling back per LP to Mehrotra's start).
value = LPs/s with the batch resident in device memory (CUDA events around
sk_solver_run on the solver stream); the A matrices of the batch (0.73 GB of CSR
and CSC arrays) exceed the 129 MB L2 and a 256 MB buffer is written before every
step. e2e = the same LPs/s through the C ABI from host arrays (sk_solver_create:
host analysis and upload; sk_solver_run; sk_solver_result: download of x, y, s of
every LP), all inside the timed region.

The line also carries the plain FP64 IPM on the same batch (unit start, FP64
fronts on the FP64 pipe: the comparison the metric names), the 512 LPs solved
one at a time by the plain FP64 IPM (config 3's "sequential plain solves"), the
precision-only gain (mixed vs FP64, both from the unit start), the family-2
staircase LP's time-to-1e-8 (m=200000), the family-1 block-angular LP, the
learned start on held-out seeds (config 4), kernel rooflines and a CPU baseline.
The compact comparison blocks are printed last in the line.

--impl reference times a CPU implementation of the path on the host cores over a
bounded, stratified sample of the same 512-LP batch, built by the oracle's own copy
of the generator (no product code is loaded): the reference's own CPU simplex
(oracle/_ref, built from the reference sources) where that library exists, else the
CPU restatement of the reference's Mehrotra IPM (oracle/sk_oracle.c, FP64 dense
Cholesky); `kind` says which ran.
"""
import argparse
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "soverign-gpu-accelerator-_gb300")
ORACLE = os.path.join(ROOT, "oracle")
for _p in (PKG, ORACLE):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "time-to-1e-8 gap & LPs/sec: mixed+learned vs plain FP64 IPM, same GB300"
BATCH = 512
WORKLOAD = ("uneven batch of 512 independent LPs solved as one batch (family 3: m ~ logUniform[200,5000], "
            "n = ceil(m U[2,3]), density 0.5-2%, instances 0..511; 763585 rows, 1925793 cols, 61.0 M nnz)")
WEIGHTS = os.path.join(PKG, "weights", "learned_start_family3.npy")
HELDOUT0 = 200100          # first held-out family-3 seed (training: 100000..; tuning: 200000..200099)


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


def spmv_rooflines(sk, lps, hbm, src, warm=3, reps=10):
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
    nlps = len(lps)
    roff = np.cumsum([0] + [lp.m for lp in lps])[:-1]
    coff = np.cumsum([0] + [lp.n for lp in lps])[:-1]
    M, N = sum(lp.m for lp in lps), sum(lp.n for lp in lps)
    mats = [("A x", M, N, _block_diag_csr([lp.csr() for lp in lps], coff)),
            ("A^T y", N, M, _block_diag_csr([(lp.col_ptrs, lp.row_idx, lp.vals) for lp in lps], roff))]
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


def load_net(sk):
    if not os.path.exists(WEIGHTS):
        raise SystemExit("learned-start weights missing: %s" % WEIGHTS)
    net = sk.Gnn(1)
    net.load(WEIGHTS)
    return net


def batch_stats(solver, nlps):
    infos = [solver.result(k, want_vectors=False)[0] for k in range(nlps)]
    its = [i["iterations"] for i in infos]
    return infos, {"all_optimal": all(i["status"] == 0 for i in infos),
                   "optimal": sum(1 for i in infos if i["status"] == 0),
                   "mean_iterations": sum(its) / nlps, "max_iterations": max(its),
                   "max_rel_gap": max(i["rel_gap"] for i in infos),
                   "max_rel_pinf": max(i["rel_pinf"] for i in infos),
                   "max_rel_dinf": max(i["rel_dinf"] for i in infos)}


def batch_arm(sk, lps, prec, start, net=None, runs=1, **opts):
    """`runs` batched solves of `lps` on one solver; device time of the last run and
    per-LP statistics of the last run (the kernels are already loaded and tuned by
    earlier solves in the process, so one run is a warm measurement)."""
    t0 = time.perf_counter()
    s = sk.Solver(lps, precision=prec, start=start, **opts)
    setup = time.perf_counter() - t0
    if start == sk.START_LEARNED:
        s.set_gnn(net)
    ms = []
    for _ in range(runs):
        s.run()
        ms.append(s.result(0, want_vectors=False)[0]["device_ms"])
    infos, st = batch_stats(s, len(lps))
    s.close()
    out = {"ms": ms[-1], "lps_per_s": 1000.0 * len(lps) / ms[-1], "setup_s": setup}
    out.update(st)
    if start == sk.START_LEARNED:
        used = sum(i["learned_start"] for i in infos)
        out["learned_used"] = used
        out["fallback_rate"] = 1.0 - used / len(lps)
    return out, infos


def sequential_plain(sk, lps):
    """The LPs solved one after another by the plain FP64 IPM (unit start), one LP per
    solver, as the reference's device IPM is used: sum of the device times of one
    solve each (after a warm-up solve of the first LP); host set-up timed apart."""
    w = sk.Solver([lps[0]], precision=sk.PREC_FP64, start=sk.START_UNIT)
    w.run()
    w.close()
    tot, ok, setup, its = 0.0, 0, 0.0, 0
    for lp in lps:
        t = time.perf_counter()
        s = sk.Solver([lp], precision=sk.PREC_FP64, start=sk.START_UNIT)
        setup += time.perf_counter() - t
        s.run()
        info, *_ = s.result(0, want_vectors=False)
        s.close()
        tot += info["device_ms"]
        ok += info["status"] == 0
        its += info["iterations"]
    return {"ms": tot, "lps_per_s": 1000.0 * len(lps) / tot, "optimal": ok, "all_optimal": ok == len(lps),
            "mean_iterations": its / len(lps), "host_setup_s": setup}


def family2_comparison(sk, net):
    """Time-to-1e-8 on the family-2 staircase LP (m=200000, n=500000): mixed precision
    with the learned start (falling back to Mehrotra's start) against the plain FP64
    IPM (unit start); one solve per arm; host analysis (ordering, plan) timed apart
    from the device solve."""
    lp = sk.generate(2, 0)
    out = {}
    prof = None
    for name, prec, start in (("mixed_learned", sk.PREC_MIXED, sk.START_LEARNED),
                              ("plain_fp64", sk.PREC_FP64, sk.START_UNIT)):
        t0 = time.perf_counter()
        s = sk.Solver([lp], precision=prec, start=start)
        t1 = time.perf_counter()
        if start == sk.START_LEARNED:
            s.set_gnn(net)
        s.run()
        info, *_ = s.result(0, want_vectors=False)
        t2 = time.perf_counter()
        if name == "mixed_learned":
            prof = s.profile(fp32=True)      # instrumented replay, not part of the solve time
        s.close()
        out[name] = {"status": info["status"], "iterations": info["iterations"], "device_s": info["device_ms"] / 1e3,
                     "analysis_s": t1 - t0, "wall_s": t2 - t0, "objective": info["objective"],
                     "rel_gap": info["rel_gap"], "switch_iteration": info["switch_iteration"]}
        if start == sk.START_LEARNED:
            out[name]["learned_used"] = info["learned_start"]
    m, p = out["mixed_learned"], out["plain_fp64"]
    out["speedup_device"] = p["device_s"] / m["device_s"]
    out["speedup_wall"] = p["wall_s"] / m["wall_s"]
    out["rel_obj_diff"] = abs(m["objective"] - p["objective"]) / (1.0 + abs(p["objective"]))
    return out, prof


def family1_comparison(sk):
    """Family-1 block-angular LP (m=22000, n=48000): mixed precision vs plain FP64, device
    time of the second of two solves each."""
    lp = sk.generate(1, 0)
    out, profs = {}, {}
    for name, prec in (("mixed", sk.PREC_MIXED), ("plain_fp64", sk.PREC_FP64)):
        s = sk.Solver([lp], precision=prec, start=sk.START_UNIT)
        s.run()
        s.run()
        info, *_ = s.result(0, want_vectors=False)
        profs[name] = s.profile(fp32=(prec == sk.PREC_MIXED))
        s.close()
        out[name] = {"ms": info["device_ms"], "iterations": info["iterations"], "status": info["status"],
                     "switch_iteration": info["switch_iteration"]}
    out["speedup"] = out["plain_fp64"]["ms"] / out["mixed"]["ms"]
    return out, profs


def heldout_comparison(sk, net, count, batch):
    """The learned start on held-out family-3 seeds (instances 200100.., never used in
    training or tuning), solved in batches of `batch`: mixed + learned against mixed
    + Mehrotra's start (the fallback); iterations, fallback rate and time-to-1e-8."""
    agg = {"mixed_learned": [0.0, 0, 0, 0, 0], "mixed_mehrotra": [0.0, 0, 0, 0, 0]}   # ms, iters, optimal, used, n
    for b0 in range(0, count, batch):
        lps = [sk.generate(3, HELDOUT0 + k) for k in range(b0, min(count, b0 + batch))]
        for name, start in (("mixed_learned", sk.START_LEARNED), ("mixed_mehrotra", sk.START_MEHROTRA)):
            r, infos = batch_arm(sk, lps, sk.PREC_MIXED, start, net)
            a = agg[name]
            a[0] += r["ms"]
            a[1] += sum(i["iterations"] for i in infos)
            a[2] += r["optimal"]
            a[3] += sum(i["learned_start"] for i in infos)
            a[4] += len(lps)
    out = {"lps": count, "seeds": "family-3 instances %d..%d" % (HELDOUT0, HELDOUT0 + count - 1),
           "batch": batch}
    for name, a in agg.items():
        out[name] = {"s": a[0] / 1e3, "lps_per_s": 1000.0 * a[4] / a[0], "mean_iterations": a[1] / a[4],
                     "optimal": a[2]}
    out["mixed_learned"]["fallback_rate"] = 1.0 - agg["mixed_learned"][3] / count
    out["iterations_saved"] = out["mixed_mehrotra"]["mean_iterations"] - out["mixed_learned"]["mean_iterations"]
    out["time_ratio_learned_vs_mehrotra"] = out["mixed_learned"]["s"] / out["mixed_mehrotra"]["s"]
    return out


def update_roofline(prof, kernel, peak, src, workload):
    u = prof["update"]
    ach = prof["update_flops"] / (u["ms"] / 1000.0) / 1e12 if u["ms"] > 0 else 0.0
    out = {"kernel": "%s (%s)" % (kernel, workload), "bound": "tensor", "achieved": ach, "peak": peak,
           "unit": "TFLOP/s", "frac": ach / peak,
           "peak_source": "%s bf16 dense tensor peak (MEASURED_PEAKS.json bf16_tflops)" % src, "traffic": None,
           "launches": u["launches"], "ms_total": u["ms"], "algorithmic_flops": prof["update_flops"],
           "note": "FP64 flops of the trailing updates (sum over fronts of 2 w t(t+1)/2 per tile step) over the "
                   "update class's event-timed duration in an instrumented replay of one factorisation"}
    mma = prof.get("mma_flops")
    if mma and u["ms"] > 0:
        # the work the tensor cores run for those flops: TF32 x3 three products, the emulated FP64
        # update 28 BF16 digit-pair products, over 128 x 64 blocks with K padded to 64
        out["executed_tflops"] = mma / (u["ms"] / 1000.0) / 1e12
        out["executed_frac"] = out["executed_tflops"] / peak
        out["executed_flops"] = mma
    return out


def solve_roofline(prof, nnz_factor, elem, hbm, src, workload, kernel):
    """Triangular solve (forward + backward) of an instrumented replay: each factor entry is
    read once per direction (algorithmic bytes = 2 nnz(L) x element size)."""
    ms = prof["fwd_solve"]["ms"] + prof["bwd_solve"]["ms"]
    nbytes = 2.0 * nnz_factor * elem
    ach = nbytes / (ms / 1000.0) / 1e9 if ms > 0 else 0.0
    return {"kernel": "%s (%s)" % (kernel, workload), "bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s",
            "frac": ach / hbm, "peak_source": "%s copy bandwidth (MEASURED_PEAKS.json hbm_gbs)" % src,
            "traffic": None, "ms_total": ms, "algorithmic_bytes": nbytes,
            "launches": prof["fwd_solve"]["launches"] + prof["bwd_solve"]["launches"]}


def run_ours(args):
    rank, world, dist = dist_setup(args)
    sk = ensure_built()
    import sharding
    import torch
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    lps_all = [sk.generate(3, k) for k in range(args.batch)]
    shards = sharding.shard_lps([sharding.lp_cost(lp.m, lp.n, lp.nnz) for lp in lps_all], world)
    lps = [lps_all[k] for k in shards[rank]]
    net = load_net(sk)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")   # 256 MB > 129 MB L2
    t0 = time.perf_counter()
    solver = sk.Solver(lps, precision=sk.PREC_MIXED, start=sk.START_LEARNED)
    setup_s = time.perf_counter() - t0
    solver.set_gnn(net)
    for _ in range(args.warmup):
        solver.run()
    _, st0 = batch_stats(solver, len(lps))
    if not st0["all_optimal"]:
        raise SystemExit("warm-up batch solve left LPs unsolved: %s" % st0)
    clocks = Clocks()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    dev_ms = []
    torch.cuda.nvtx.range_push("sk_timed")      # the timed steps, for a profiler's NVTX filter
    t0 = time.perf_counter()
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        solver.run()
        dev_ms.append(solver.result(0, want_vectors=False)[0]["device_ms"])
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    torch.cuda.nvtx.range_pop()
    clk = clocks.stop()
    infos, st = batch_stats(solver, len(lps))
    total_ms = barrier_max(dist, sum(dev_ms))
    value = args.batch * args.steps / (total_ms / 1000.0)
    per_run = count_kernel_launches(solver.run)
    launches = per_run * args.steps if per_run is not None else None
    prof = solver.profile(fp32=True)                 # instrumented replay of one FP32 factorisation + solve
    prof64 = solver.profile(fp32=False)              # same, FP64 fronts (tensor-core FP64 updates)
    nnz_factor = infos[0]["nnz_factor"]
    solver.close()
    headline = {"ms_per_batch": total_ms / args.steps, "lps_per_s": value, "setup_s": setup_s,
                "learned_used": sum(i["learned_start"] for i in infos),
                "fallback_rate": 1.0 - sum(i["learned_start"] for i in infos) / len(lps)}
    headline.update(st)

    # the comparison the metric names: the plain FP64 IPM (unit start) on the same batch; the
    # precision-only gain (mixed vs FP64 from the same unit start); Mehrotra's start in mixed precision
    arms = {}
    if not args.quick:
        for name, prec, start in (("plain_fp64", sk.PREC_FP64, sk.START_UNIT),
                                  ("mixed_unit_start", sk.PREC_MIXED, sk.START_UNIT),
                                  ("mixed_mehrotra", sk.PREC_MIXED, sk.START_MEHROTRA)):
            a, _ = batch_arm(sk, lps, prec, start)
            a["ms"] = barrier_max(dist, a["ms"])
            a["lps_per_s"] = 1000.0 * args.batch / a["ms"]
            arms[name] = a
    seq = sequential_plain(sk, lps) if (args.sequential and world == 1 and not args.quick) else None

    # end to end through the C ABI: host arrays in, x, y, s of every LP out
    e2e_steps = max(1, min(args.steps, args.e2e_steps))
    e2e_t = []
    h2d = sum(lp.nbytes() for lp in lps)
    d2h = sum((2 * lp.n + lp.m) * 8 for lp in lps)
    for _ in range(e2e_steps):
        flush.zero_()
        torch.cuda.synchronize()
        t = time.perf_counter()
        s = sk.Solver(lps, precision=sk.PREC_MIXED, start=sk.START_LEARNED)
        s.set_gnn(net)
        s.run()
        res = [s.result(k) for k in range(len(lps))]
        s.close()
        e2e_t.append(time.perf_counter() - t)
        if not all(r[0]["status"] == 0 for r in res):
            raise SystemExit("end-to-end batch solve left LPs unsolved")
    e2e_total = barrier_max(dist, sum(e2e_t))
    e2e_value = args.batch * len(e2e_t) / e2e_total

    hbm, bf16, src = peaks()
    wl = "512-LP family-3 batch, dense normal matrices"
    classes = {}
    for tag, pr in (("fp32", prof), ("fp64", prof64)):
        for k, v in pr.items():
            if isinstance(v, dict):
                classes["%s %s" % (k, tag)] = v["ms"]
    rooflines = [
        solve_roofline(prof64, nnz_factor, 8, hbm, src, wl + ", FP64 factor",
                       "k_fwd_tasks<double> + k_bwd_tasks<double> (triangular solves)"),
        solve_roofline(prof, nnz_factor, 4, hbm, src, wl + ", FP32 factor",
                       "k_fwd_tasks<float> + k_bwd_tasks<float> (triangular solves)"),
        update_roofline(prof64, "k_oz_digits + k_update_oz (FP64-accurate trailing update on the tensor cores, "
                        "BF16 digit products; FP64 flops counted)", bf16, src, wl + ", FP64 fronts"),
        update_roofline(prof, "k_update_tc (FP32 trailing update, tcgen05 TF32 x3; FP32 flops counted once)", bf16,
                        src, wl + ", FP32 fronts"),
        assembly_roofline(prof, hbm, src, wl + ", FP32 fronts", "event-timed replay of one assembly")]
    # the dominant kernel class of one FP64 factorisation + triangular solve
    dominant = max(rooflines[:3], key=lambda r: r["ms_total"])
    extra = {}
    if not args.quick:
        if args.spmv:
            rooflines.extend(spmv_rooflines(sk, lps_all, hbm, src))
        f1, f1prof = family1_comparison(sk)
        extra["family1"] = f1
        rooflines.append(assembly_roofline(f1prof["mixed"], hbm, src, "family-1 LP, FP32 fronts",
                                           "event-timed replay of one assembly"))
        if args.family2:
            f2, f2prof = family2_comparison(sk, net)
            extra["family2"] = f2
            if f2prof is not None:
                rooflines.append(assembly_roofline(f2prof, hbm, src, "family-2 staircase LP, FP32 fronts",
                                                   "event-timed replay of one assembly"))
        if args.heldout > 0:
            extra["family4"] = heldout_comparison(sk, net, args.heldout, args.batch)
    net.close()
    rooflines = [r for r in rooflines if r is not None]
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_sample_run(args.cpu_cap)
        cpu["value"] = cpu.pop("lps_per_s")

    line = {"metric": METRIC, "value": value, "unit": "LPs/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64+f32",
            "data": "synthetic, seeded generator (family 3, instances 0..%d)" % (args.batch - 1),
            "config": {"workload": WORKLOAD, "lps": args.batch, "precision": "mixed (FP32/TF32x3 fronts, FP64 "
                       "residuals/PCG, FP64 fronts with tensor-core FP64-accurate updates after the switch)",
                       "start": "learned (per-LP fallback to Mehrotra's start)",
                       "tolerance": "per LP rel pinf, dinf, gap <= 1e-8",
                       "l2": "inputs 0.73 GB > L2; 256 MB buffer written before every step",
                       "parallelism": ("LP-sharded batch over %d ranks" % world) if world > 1 else "single GPU",
                       "mean_iterations": st["mean_iterations"], "max_iterations": st["max_iterations"],
                       "plain_fp64_lps_per_s": arms["plain_fp64"]["lps_per_s"] if arms else None},
            "gpu_launches": launches,
            "roofline": dominant, "cpu_baseline": cpu, "clocks": clk,
            "e2e": {"value": e2e_value, "unit": "LPs/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "ms_per_step": 1000.0 * e2e_total / len(e2e_t), "steps": len(e2e_t),
                    "path": "sk_solver_create (host analysis + upload) + sk_solver_run + sk_solver_result for "
                            "every LP (pageable host arrays)"},
            "kernel_rooflines": rooflines,
            "kernel_breakdown_ms": classes,
            "gpu_launches_note": "kernels of libsankhya_gb300 per batch solve (CUPTI trace of one extra run) x steps",
            "wall_s_timed_region": wall,
            "detail": {"mixed_learned": headline, "arms": arms, "sequential_plain_fp64": seq}}
    # compact comparison blocks last (the end of the line is what a log tail keeps)
    if arms:
        p = arms["plain_fp64"]
        line["config3"] = {
            "mixed_learned_lps_per_s": value, "plain_fp64_lps_per_s": p["lps_per_s"],
            "speedup_vs_plain_fp64": value / p["lps_per_s"],
            "time_ratio_vs_plain_fp64": (total_ms / args.steps) / p["ms"],
            "mixed_mehrotra_lps_per_s": arms["mixed_mehrotra"]["lps_per_s"],
            "precision_only_speedup_unit_start": arms["mixed_unit_start"]["lps_per_s"] / p["lps_per_s"],
            "sequential_plain_fp64_lps_per_s": seq["lps_per_s"] if seq else None,
            "speedup_vs_sequential_plain_fp64": value / seq["lps_per_s"] if seq else None,
            "mean_iterations": st["mean_iterations"], "plain_fp64_mean_iterations": p["mean_iterations"],
            "all_optimal": st["all_optimal"] and p["all_optimal"], "learned_used": headline["learned_used"]}
    if "family1" in extra:
        f1 = extra["family1"]
        line["config1"] = {"mixed_ms": f1["mixed"]["ms"], "plain_fp64_ms": f1["plain_fp64"]["ms"],
                           "speedup": f1["speedup"], "iterations": f1["mixed"]["iterations"],
                           "plain_fp64_iterations": f1["plain_fp64"]["iterations"],
                           "status": [f1["mixed"]["status"], f1["plain_fp64"]["status"]]}
    if "family2" in extra:
        f2 = extra["family2"]
        line["config2"] = {"mixed_learned_device_s": f2["mixed_learned"]["device_s"],
                           "plain_fp64_device_s": f2["plain_fp64"]["device_s"],
                           "speedup_device": f2["speedup_device"], "speedup_wall": f2["speedup_wall"],
                           "mixed_learned_wall_s": f2["mixed_learned"]["wall_s"],
                           "plain_fp64_wall_s": f2["plain_fp64"]["wall_s"],
                           "iterations": [f2["mixed_learned"]["iterations"], f2["plain_fp64"]["iterations"]],
                           "learned_used": f2["mixed_learned"].get("learned_used"),
                           "rel_obj_diff": f2["rel_obj_diff"],
                           "status": [f2["mixed_learned"]["status"], f2["plain_fp64"]["status"]]}
    if "family4" in extra:
        f4 = extra["family4"]
        line["config4"] = {"heldout_lps": f4["lps"], "mean_iterations_learned": f4["mixed_learned"]["mean_iterations"],
                           "mean_iterations_mehrotra": f4["mixed_mehrotra"]["mean_iterations"],
                           "fallback_rate": f4["mixed_learned"]["fallback_rate"],
                           "time_to_1e8_s_learned": f4["mixed_learned"]["s"],
                           "time_to_1e8_s_mehrotra": f4["mixed_mehrotra"]["s"],
                           "optimal": [f4["mixed_learned"]["optimal"], f4["mixed_mehrotra"]["optimal"]]}
    if rank == 0:
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


# ---- CPU baseline -----------------------------------------------------------------------

def cpu_sample_members(count=16):
    """A stratified sample of the 512-LP batch: the members at every (512 / count)-th
    position of the batch sorted by row count (from the smallest), so the sample spans
    the batch's size range. Sizes come from the oracle's copy of the generator."""
    import sk_oracle as so
    sizes = sorted(range(BATCH), key=lambda k: (so.generate_dims(3, k)[0], k))
    stride = BATCH // count
    return [sizes[stride // 2 + stride * q] for q in range(count)]


def _cpu_kind():
    import sk_oracle as so
    return "reference" if so.have_reference() else "port"


def _cpu_one(k, q, kind):
    import sk_oracle as so
    lp = so.generate(3, k)
    t = time.perf_counter()
    if kind == "reference":
        st, obj, _ = so.ref_simplex(lp)
    else:
        r, *_ = so.ipm_solve(lp)
        st = r["status"]
    q.put((k, lp.m, st, time.perf_counter() - t))


def cpu_sample_run(cap, members=None, kind=None):
    """CPU implementation of the path on the stratified sample, one LP per host core, all
    cores at once: the reference's own CPU simplex (oracle/_ref) where it was built
    from the reference sources, else the oracle's FP64 dense-Cholesky restatement of
    the reference's Mehrotra IPM. A member still running after `cap` seconds is
    stopped and counted as not finished (DNF). LPs/s = finished LPs / wall seconds of
    the whole sample."""
    members = members or cpu_sample_members()
    kind = kind or _cpu_kind()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    cores = os.cpu_count() or 1
    t0 = time.perf_counter()
    procs, done, pending = {}, {}, list(members)
    while pending or procs:
        while pending and len(procs) < cores:
            k = pending.pop(0)
            p = ctx.Process(target=_cpu_one, args=(k, q, kind))
            p.start()
            procs[k] = (p, time.perf_counter())
        try:
            k, m, stt, dt = q.get(timeout=0.05)
            done[k] = {"m": m, "status": stt, "seconds": dt}
            procs[k][0].join()
            del procs[k]
        except Exception:
            pass
        now = time.perf_counter()
        for k in [k for k, (p, ts) in procs.items() if now - ts > cap]:
            procs[k][0].terminate()
            procs[k][0].join()
            del procs[k]
            done[k] = {"status": "DNF"}
    wall = time.perf_counter() - t0
    fin = [k for k in members if done.get(k, {}).get("status") == 0]
    what = ("reference CPU Phase-I + primal simplex (oracle/_ref, src/simplex/phase1.cpp:124-449)"
            if kind == "reference" else "oracle/sk_oracle.c FP64 dense-Cholesky restatement of the reference's "
                                        "Mehrotra IPM")
    return {"lps_per_s": len(fin) / wall, "unit": "LPs/s", "cores": min(cores, len(members)), "kind": kind,
            "nproc": cores, "wall_s": wall, "finished": len(fin), "dnf": [k for k in members if k not in fin],
            "per_lp_1core_s": {str(k): round(done[k]["seconds"], 3) for k in fin},
            "sample": ("stratified sample of the 512-LP batch: %d members (every %d-th by row count), one LP per "
                       "core on %d cores, per-LP cap %.0f s (DNF beyond); %s"
                       % (len(members), BATCH // len(members), min(cores, len(members)), cap, what))}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import sk_oracle as so
    so.oracle()
    kind = _cpu_kind()
    members = cpu_sample_members()
    for _ in range(args.warmup):
        cpu_sample_run(args.cpu_cap, members, kind)
    vals = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        vals.append(cpu_sample_run(args.cpu_cap, members, kind))
    wall = time.perf_counter() - t0
    v = statistics.mean(x["lps_per_s"] for x in vals)
    last = vals[-1]
    line = {"metric": METRIC, "impl": "reference", "value": v, "unit": "LPs/s", "n_gpus": 0, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * wall / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic, seeded generator (family 3, oracle copy)",
            "config": {"workload": WORKLOAD, "sample": last["sample"],
                       "implementation": "reference's own CPU simplex" if kind == "reference" else
                       "CPU restatement of the reference's Mehrotra IPM (the reference's own CPU code needs its "
                       "sources, which are not on the GPU host)"},
            "cpu_baseline": {"value": v, "unit": "LPs/s", "cores": last["cores"], "kind": kind,
                             "nproc": last["nproc"], "sample": last["sample"], "finished": last["finished"],
                             "dnf": last["dnf"], "per_lp_1core_s": last["per_lp_1core_s"]},
            "e2e": {"value": v, "unit": "LPs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--batch", type=int, default=BATCH, help="family-3 members in the batch (instances 0..batch-1)")
    ap.add_argument("--e2e-steps", type=int, default=3, help="end-to-end steps (at most --steps)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-cap", type=float, default=6.0, help="per-LP time cap of the CPU baseline (s)")
    ap.add_argument("--quick", action="store_true", help="headline only (no other arms, families or rooflines)")
    ap.add_argument("--no-sequential", dest="sequential", action="store_false",
                    help="skip the LPs solved one at a time by the plain FP64 IPM")
    ap.add_argument("--no-family2", dest="family2", action="store_false",
                    help="skip the family-2 staircase LP (m=200000) comparison")
    ap.add_argument("--heldout", type=int, default=512, help="held-out family-3 seeds for the learned start (0: skip)")
    ap.add_argument("--no-spmv", dest="spmv", action="store_false")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
