#!/usr/bin/env python
"""Benchmark of the SHCI hot path on GB300: Hamiltonian build + Davidson.

Workload (the largest configuration of the metric): synthetic FCIDUMP, n = 40 orbitals,
10 alpha + 10 beta electrons, no symmetry; heat-bath schedule 1e-3, 5e-4, 2e-4, 1e-4, 5e-5
(one iteration each, as the reference's eps_vars_schedule), then the first eps_var = 2e-5
iteration: its selection gives the determinant list (~4.5M dets) the timed step works on.

One step = Hamiltonian<S>::update (two-hole core join index + single fill pass, mixed storage:
FP32 value + FP32 residual, rows then sorted by column) + one full Davidson::diagonalize call (the reference's maximum of
9 H*v products, tol = 0 so every step does the same work, FP64 vectors, float-pair products
and 64-bit fixed-point sums in H*v) + the FP64-accurate Rayleigh-quotient correction of the
Ritz vector (a pass over the FP32 residual store).  value = device seconds per step
(inputs resident in HBM); e2e = the same through the public API with the det list and start
vector copied from pinned host memory each step and the energy read back.

Also in the line: the three PT2 stages on the step's wavefunction, timed over the same
warm-up and step counts (`pt2`), the all-FP64 step and its PT2 (`fp64`,
`pt2_fp64_wavefunction`, `totals`), the whole variational stage to the converged eps_var =
2e-5 space and a step on it (`converged`), the oracle checks (`parity`: the oracle's own det
list and sampled rows), full device and oracle runs of the n = 16 and n = 26 configurations
(`small_configs`) and the 256-instance batched workload (`batched`).

--impl reference times the CPU restatement of the reference's algorithm (oracle/) on a
strided sample of the same step's rows with every host thread, scaled to the full step.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "H-build+Davidson s and PT2 s at ~2e7 dets, mixed vs FP64 on GPU, |dE|<1e-6 Ha"
# workload -> (eps_vars_schedule iterations, eps_var of the timed iteration)
WORKLOADS = {
    3: ([1e-3, 5e-4, 2e-4, 1e-4, 5e-5], 2e-5),   # n=40 10a10b: the metric's configuration
    2: ([1e-3, 5e-4, 2e-4, 1e-4], 5e-5),         # n=26 7a7b: small case (profiling)
    1: ([], 2e-4),                               # n=16 5a5b
}
WORKLOAD = 3
SCHEDULE, EPS_VAR = WORKLOADS[WORKLOAD]
TARGET_ERROR = 5e-5
DAVIDSON_MATVECS = 9


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d["hbm_gbs"], "measured"
    return 6800.0, "fallback"


class Clocks:
    """Samples nvidia-smi clocks and throttle reasons during the timed region."""

    def __init__(self, device):
        self.device = device
        self.samples = []
        self.proc = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 7:
                self.samples.append(f)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4) if s[3 + k] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.samples)}


def dist_info():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


def max_over_ranks(value, device):
    """The job's clock for N independent replicas: the largest per-rank value (identity on
    one rank or without an initialised process group)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return value
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def make_workload(data_dir):
    from shci_gb300 import synthetic
    return synthetic.workload_fcidump(WORKLOAD, data_dir), synthetic.WORKLOADS[WORKLOAD]


def gpu_setup(ctx, fcidump, w):
    """Schedule iterations on the device, then the first eps_var selection: returns the det
    list and the start vector of the timed step (host arrays)."""
    import shci_gb300 as S
    ctx.load_fcidump(fcidump, w["n_up"], w["n_dn"])
    ctx.build_queues()
    for eps in SCHEDULE:
        ctx.select(eps)
        ctx.update_hamiltonian(S.PREC_MIXED)
        ctx.davidson(TARGET_ERROR / 50)
    ctx.select(EPS_VAR)
    return ctx.dets()


def sample_stride(n, target_rows=20000):
    return max(1, n // target_rows)


def cpu_sample(fcidump, w, up, dn, target_rows=20000, keep=None):
    """Oracle (CPU restatement) timing of one step on a strided row sample, scaled.  keep (a
    dict, optional) receives the oracle's sampled rows."""
    from oracle.oracle import Oracle
    o = Oracle(fcidump, w["n_up"], w["n_dn"])
    o.set_dets(up, dn)
    n = len(up)
    stride = sample_stride(n, target_rows)
    r = o.hbuild_sample(stride, 0)
    if keep is not None:
        keep["rows"] = o.sample_rows()
    scale = n / max(1, r["rows"])
    step = r["index_s"] + scale * (r["rows_s"] + DAVIDSON_MATVECS * r["spmv_s"])
    return step, {"value": step, "unit": "s", "cores": Oracle.threads(), "kind": "port",
                  "sample": "rows i = 0 mod %d (%d of %d rows, %d upper nnz) of the step's "
                            "Hamiltonian; full det index built; H-build and %d H*v scaled by %.1f"
                            % (stride, r["rows"], n, r["nnz"], DAVIDSON_MATVECS, scale),
                  "index_s": r["index_s"], "rows_s": r["rows_s"], "spmv_s": r["spmv_s"]}


def run_reference(args):
    rank, world, _ = dist_info()
    if rank != 0:
        return
    from oracle import oracle as orc
    orc.build(ref=False)
    fcidump, w = make_workload(args.data)
    o = orc.Oracle(fcidump, w["n_up"], w["n_dn"])
    t0 = time.time()
    for eps in SCHEDULE:
        o.run_variation_step(eps, False, TARGET_ERROR)
    o.select(EPS_VAR)
    up, dn, _ = o.dets()
    setup_s = time.time() - t0
    del o  # the setup's matrices and selection state are not part of the timed sample
    vals, walls = [], []
    info = None
    for k in range(args.warmup + args.steps):
        t1 = time.time()
        v, info = cpu_sample(fcidump, w, up, dn)
        if k >= args.warmup:
            vals.append(v)
            walls.append(time.time() - t1)
    value = statistics.median(vals)
    info["value"] = value
    # a step of this arm is the bounded sample: ms_per_step is its measured wall time; value is
    # the metric for the whole step (the sample scaled by the row fraction, as `sample` says)
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": "s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": statistics.median(walls) * 1e3, "value_is_scaled_sample": True,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": {"workload": workload_name(len(up)), "n_dets": len(up)},
        "cpu_baseline": info, "setup_s": setup_s,
        "e2e": {"value": value, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))


def workload_name(n):
    from shci_gb300 import synthetic
    w = synthetic.WORKLOADS[WORKLOAD]
    return ("synthetic n=%d %da%db C1, schedule %s then first eps_var=%g iteration "
            "(%d dets): H-build + Davidson (9 H*v)"
            % (w["n"], w["n_up"], w["n_dn"], SCHEDULE, EPS_VAR, n))


PT2 = {  # workload -> (eps_pt_dtm, eps_pt_psto, eps_pt, psto batches, sto batches, samples)
    3: (1e-6, 2e-7, 1e-8, 16, 64, 200000),
    2: (1e-6, 1e-7, 5e-8, 16, 64, 20000),
    1: (1e-6, 1e-6, 1e-6, 16, 64, 2000),
}


def run_pt2(ctx, stream, e_var):
    """Solver<S>::run_perturbation's three stages on the context's wavefunction, each timed
    with CUDA events on the context stream."""
    import torch
    eps_dtm, eps_psto, eps_pt, nb_psto, nb_sto, n_samples = PT2[WORKLOAD]
    out = {"eps_pt_dtm": eps_dtm, "eps_pt_psto": eps_psto, "eps_pt": eps_pt}
    try:
        t = []
        for _ in range(4):
            ev = torch.cuda.Event(enable_timing=True)
            t.append(ev)
        ctx.profile(True)
        t[0].record(stream)
        dtm, _, n_dtm = ctx.pt2_dtm(e_var, eps_dtm, 0)
        t[1].record(stream)
        psto = (0.0, 0.0, 0, 0)
        if eps_psto < eps_dtm:
            psto = ctx.pt2_psto(e_var, eps_dtm, eps_psto, nb_psto, TARGET_ERROR, eps_pt)
        t[2].record(stream)
        sto, sto_u, loops = ctx.pt2_sto(e_var, eps_psto, eps_pt, nb_sto, n_samples, 347634253,
                                        100, TARGET_ERROR, psto[1], semisto=False)
        t[3].record(stream)
        torch.cuda.synchronize()
        prof = ctx.profile_get()
        ctx.profile(False)
        ms = [t[k].elapsed_time(t[k + 1]) for k in range(3)]
        # device time per stage kind over all three PT2 stages; the rest of the wall time is
        # host work (sampling, batch bookkeeping) and small launches
        out["device_ms"] = {k: round(v[0], 2) for k, v in prof.items() if k.startswith("pt2")}
        e2 = dtm + psto[0] + sto
        out.update({"s": sum(ms) / 1e3, "dtm_s": ms[0] / 1e3, "psto_s": ms[1] / 1e3,
                    "sto_s": ms[2] / 1e3, "n_pt_dets_dtm": n_dtm, "psto_batches": psto[3],
                    "n_pt_dets_psto": psto[2], "sto_iterations": len(loops),
                    "sto_batches": nb_sto, "sto_samples": n_samples,
                    "correction": e2, "uncert": (psto[1] ** 2 + sto_u ** 2) ** 0.5,
                    "energy_total": e_var + e2})
    except Exception as e:  # report, do not lose the H-build / Davidson line
        out["error"] = str(e)
    return out


def run_pt2_timed(ctx, stream, e_var, warmup, steps):
    """The three PT2 stages, warmup untimed runs and steps timed runs (CUDA events on the
    context stream per run); the last run's full record plus the per-run seconds."""
    secs = []
    out = None
    for k in range(warmup + steps):
        out = run_pt2(ctx, stream, e_var)
        if "error" in out:
            return out
        if k >= warmup:
            secs.append(out["s"])
    out["s_runs"] = secs
    out["s"] = statistics.median(secs)
    out["warmup"], out["steps"] = warmup, steps
    return out


def parity_n40(fcidump, w, up, dn):
    """The oracle's own selection schedule on the CPU gives the step's det list independently;
    it must equal the device's bit for bit (the sampled rows are compared by compare_rows)."""
    import numpy as np
    from oracle.oracle import Oracle
    t0 = time.time()
    o = Oracle(fcidump, w["n_up"], w["n_dn"])
    for eps in SCHEDULE:
        o.run_variation_step(eps, False, TARGET_ERROR)
    o.select(EPS_VAR)
    oup, odn, _ = o.dets()
    del o
    out = {"oracle_select_s": time.time() - t0, "n_dets_oracle": int(len(oup)),
           "dets_equal": bool(len(oup) == len(up) and np.array_equal(oup, up)
                              and np.array_equal(odn, dn))}
    return out


def compare_rows(o_rows, g_rows, mixed):
    """Oracle sample rows vs device rows: (all columns equal, all values equal)."""
    import numpy as np
    _, ooff, ocols, ovals = o_rows
    goff, gcols, gvals = g_rows
    if not (np.array_equal(ooff, goff) and np.array_equal(ocols, gcols)):
        return False, False
    if mixed:
        hi = ovals.astype(np.float32)
        lo = (ovals - hi.astype(np.float64)).astype(np.float32)
        want = hi.astype(np.float64) + lo.astype(np.float64)
    else:
        want = ovals
    return True, bool(np.array_equal(gvals, want))


SMALL = {  # workload -> (eps_vars, schedule, eps_pt_dtm or None)
    1: ([2e-4, 1e-4], [], 1e-6),
    2: ([5e-5], [1e-3, 5e-4, 2e-4, 1e-4], None),
}


def run_converged(fcidump, w, device, warmup, steps):
    """The whole variational stage of the workload as Solver::run_all_variations runs it
    (schedule iterations, then eps_var iterations until the det list and Davidson converge,
    the Hamiltonian updated incrementally), timed end to end on the host clock; then the step
    (H build + Davidson with 9 H*v + the FP64 energy correction) on the converged det list,
    timed like the headline step."""
    import torch
    import shci_gb300 as S
    ctx = S.Context(device)
    ctx.load_fcidump(fcidump, w["n_up"], w["n_dn"])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e = ctx.run_variation([EPS_VAR], SCHEDULE, TARGET_ERROR, precision=S.PREC_MIXED)
    torch.cuda.synchronize()
    var_s = time.perf_counter() - t0
    nd, nz, en = ctx.var_trace()
    up, dn, c_conv = ctx.dets()
    n = int(nd[-1])
    stream = torch.cuda.ExternalStream(ctx.stream())
    c_dev = torch.from_numpy(c_conv).to("cuda:%d" % device)
    # the step rebuilds the whole matrix of the converged list
    ctx.set_dets(up, dn, c_conv)

    def step():
        ctx.set_coefs_dev(c_dev.data_ptr(), n)
        ctx.update_hamiltonian(S.PREC_MIXED)
        ctx.davidson(0.0)
        return ctx.energy_fp64()

    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ctx.profile(True)
    ev0.record(stream)
    for _ in range(steps):
        e_step = step()
    ev1.record(stream)
    torch.cuda.synchronize()
    prof = ctx.profile_get()
    ctx.profile(False)
    st = ctx.hamiltonian_stats()
    peak = ctx.memory_stats()[1]
    _, peak_live = ctx.memory_cached()
    ctx.close()
    return {"variation_stage_s": var_s, "energy_var": float(e[0]),
            "iterations": [{"n_dets": int(a), "nnz_sym": int(b), "energy": float(c)}
                           for a, b, c in zip(nd, nz, en)],
            "n_dets": n, "nnz_upper": st["nnz"], "ms_per_step": ev0.elapsed_time(ev1) / steps,
            "steps": steps, "warmup": warmup, "energy_step": e_step, "peak_device_bytes": peak_live,
            "peak_device_bytes_with_cache": peak,
            "build": {"one_pass": st.get("one_pass"), "path": st["path"]},
            "stage_ms_per_step": {k: round(v[0] / steps, 2) for k, v in prof.items()}}


def run_small_configs(data_dir, device, repeats=3):
    """The benchmark's first two configurations run in full, on the device and by the oracle
    on every host thread (median of `repeats` runs each, no sampling or scaling): n = 16
    (variation at 2e-4 then 1e-4, deterministic PT2 at 1e-6) and n = 26 (schedule 1e-3 ...
    1e-4, variation at 5e-5).  Phases: variation (selection + Hamiltonian + Davidson
    iterations) and deterministic PT2."""
    import shci_gb300 as S
    from oracle.oracle import Oracle
    from shci_gb300 import synthetic
    out = {}
    for k, (eps_vars, sched, eps_dtm) in SMALL.items():
        wk = synthetic.WORKLOADS[k]
        f = synthetic.workload_fcidump(k, data_dir)
        g_var, g_pt, c_var, c_pt = [], [], [], []
        res = {}
        for r in range(repeats):
            ctx = S.Context(device)
            ctx.load_fcidump(f, wk["n_up"], wk["n_dn"])
            t0 = time.perf_counter()
            e = ctx.run_variation(eps_vars, sched, TARGET_ERROR, precision=S.PREC_MIXED)
            t1 = time.perf_counter()
            g_var.append(t1 - t0)
            nd, _, _ = ctx.var_trace()
            res.update(n_dets=int(nd[-1]), energy_var_gpu=float(e[-1]))
            if eps_dtm:
                ctx.build_queues()
                t2 = time.perf_counter()
                v, _, n_pt = ctx.pt2_dtm(e[-1], eps_dtm, 1)
                g_pt.append(time.perf_counter() - t2)
                res.update(pt_dtm_gpu=v, n_pt_dets=int(n_pt))
            ctx.close()
            o = Oracle(f, wk["n_up"], wk["n_dn"])
            t0 = time.perf_counter()
            eo = o.run_all_variations(eps_vars, sched, TARGET_ERROR)
            c_var.append(time.perf_counter() - t0)
            res["energy_var_cpu"] = float(eo[-1])
            if eps_dtm:
                t2 = time.perf_counter()
                vo, _, _ = o.pt_dtm(eps_dtm, 1)
                c_pt.append(time.perf_counter() - t2)
                res["pt_dtm_cpu"] = vo
            del o
        med = statistics.median
        res.update({"variation": {"gpu_s": med(g_var), "cpu_s": med(c_var)},
                    "cpu_cores": Oracle.threads(), "cpu_kind": "port", "repeats": repeats,
                    "workload": "synthetic n=%d %da%db, eps_vars %s, schedule %s"
                                % (wk["n"], wk["n_up"], wk["n_dn"], eps_vars, sched)})
        if eps_dtm:
            res["pt_dtm"] = {"eps_pt_dtm": eps_dtm, "gpu_s": med(g_pt), "cpu_s": med(c_pt)}
        out["n%d" % wk["n"]] = res
    return out


def run_batched(data_dir, n_instances=256, cpu_sample=8):
    """Workload 5: n_instances synthetic FCIDUMPs (n ~ U[12,20], electrons per spin ~
    U[3, n/2-1], seeds 20261203 + 1000 + i), eps_var 1e-4, deterministic PT2 at 1e-6, solved
    by the concurrent batch runner; CPU baseline = the oracle on the first cpu_sample
    instances, scaled."""
    import shci_gb300
    from shci_gb300 import synthetic
    inst = []
    for i in range(n_instances):
        path, n, ne = synthetic.batch_instance(i, os.path.join(data_dir, "batch"))
        inst.append((path, ne, ne))
    t0 = time.perf_counter()
    res, used = shci_gb300._lib.batch_solve(inst, [1e-4], [], (1e-6, 1e-6, 1e-6), n_workers=0)
    t = time.perf_counter() - t0
    out = {"instances": n_instances, "s": t, "instances_per_s": n_instances / t,
           "workers": used, "total_dets": int(sum(r["n_dets"] for r in res)),
           "max_dets": int(max(r["n_dets"] for r in res))}
    if cpu_sample:
        from oracle.oracle import Oracle
        tc = time.perf_counter()
        for path, nu, nd in inst[:cpu_sample]:
            o = Oracle(path, nu, nd)
            o.run_all_variations([1e-4], [], TARGET_ERROR)
            o.pt_dtm(1e-6, 1)
        tc = time.perf_counter() - tc
        share = sum(r["seconds"] for r in res[:cpu_sample]) / max(1e-9, sum(r["seconds"] for r in res))
        out["cpu_baseline"] = {"value": tc / max(share, 1e-9), "unit": "s",
                               "cores": Oracle.threads(), "kind": "port",
                               "sample": "oracle solves of the first %d instances scaled by their "
                                         "share of the GPU per-instance solve time" % cpu_sample}
    return out


def run_ours(args):
    import numpy as np
    import torch
    import shci_gb300 as S
    rank, world, local = dist_info()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    fcidump, w = make_workload(args.data)
    ctx = S.Context(local)
    t0 = time.time()
    up, dn, c0 = gpu_setup(ctx, fcidump, w)
    setup_s = time.time() - t0
    n = len(up)
    stream = torch.cuda.ExternalStream(ctx.stream())
    c0_dev = torch.from_numpy(c0).to(f"cuda:{local}")
    torch.cuda.synchronize()

    def step(prec):
        ctx.set_coefs_dev(c0_dev.data_ptr(), n)
        ctx.update_hamiltonian(prec)
        e, conv, tr = ctx.davidson(0.0)
        return ctx.energy_fp64(), e

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        step(S.PREC_MIXED)
    barrier()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ctx.profile(True)
    l0 = ctx.launches()
    with Clocks(local) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            e_mixed, e_dav = step(S.PREC_MIXED)
        ev1.record(stream)
        barrier()
    launches = ctx.launches() - l0
    prof = ctx.profile_get()
    ctx.profile(False)
    ms = ev0.elapsed_time(ev1) / args.steps
    stats = ctx.hamiltonian_stats()
    ms = max_over_ranks(ms, f"cuda:{local}")

    # PT2 on the step's wavefunction (the metric's "PT2 s"): dtm, psto, sto stages, timed over
    # the same warm-up and step counts
    pt2 = run_pt2_timed(ctx, stream, e_mixed, args.warmup, args.steps) if args.pt2 else None
    batched = run_batched(args.data) if args.batched else None

    # all-FP64 form of the same step, timed over the same step count
    ev2, ev3 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    step(S.PREC_FP64)
    barrier()
    ev2.record(stream)
    for _ in range(args.steps):
        e_fp64, _ = step(S.PREC_FP64)
    ev3.record(stream)
    barrier()
    ms_fp64 = ev2.elapsed_time(ev3) / args.steps
    sample = np.arange(0, n, sample_stride(n), dtype=np.uint64)
    rows_fp64 = ctx.hamiltonian_rows(sample) if args.parity else None
    pt2_fp64 = run_pt2(ctx, stream, e_fp64) if args.pt2 else None

    # end to end through the public API with pinned host buffers
    pin_up = torch.from_numpy(up).pin_memory()
    pin_dn = torch.from_numpy(dn).pin_memory()
    pin_c = torch.from_numpy(c0).pin_memory()
    e2e_ms = []
    for k in range(args.warmup + args.steps):
        barrier()
        ta = time.perf_counter()
        ctx.set_dets(pin_up.numpy(), pin_dn.numpy(), pin_c.numpy())
        ctx.update_hamiltonian(S.PREC_MIXED)
        ctx.davidson(0.0)
        e_e2e = ctx.energy_fp64()
        tb = time.perf_counter()
        if k >= args.warmup:
            e2e_ms.append((tb - ta) * 1e3)
    e2e = statistics.median(e2e_ms)
    rows_mixed = ctx.hamiltonian_rows(sample) if args.parity else None
    # the whole variational stage, and the step on its converged det list (after the headline
    # context has released its memory, before the host-side oracle work)
    converged = None
    if args.converged:
        ctx.close()
        converged = run_converged(fcidump, w, local, 1, args.steps)

    if rank != 0:
        return
    # roofline of the dominant kernel (per-launch averages over the timed region)
    hbm, peak_kind = peaks()
    per = {k: (v[0] / max(1, v[1]), v[1]) for k, v in prof.items()}
    dom = max(prof, key=lambda k: prof[k][0])
    nnz, cand = stats["nnz"], stats["candidates"]
    m = stats.get("core_entries", 0)
    # Algorithmic HBM bytes per launch.  H build: read the det list (16 B/det), write counts /
    # read row offsets and the diagonal (8 B/det), write the store (12 B per stored element:
    # u32 column + FP32 value + FP32 residual).  Core join: each row reads its entries' bucket
    # spans (8 B per entry) and the det id of each candidate (4 B); the candidates' spin
    # strings are gathered from the L2-resident det list.  Building the join writes keys and
    # entry ids (4 B keys + 4 B ids per entry), sorts them (4 passes; each reads the keys for
    # the histogram, then reads and writes keys and ids: 20 B/entry) and writes spans and det
    # ids (read 8 B, write 12 B per entry).  Row sort: read and write each stored element
    # (u32 column + FP32 value + FP32 residual: 24 B) and read each row's offset and length.
    # Energy correction: read the store's columns and residuals once (8 B/element), row
    # offsets and lengths, the Ritz vector, and write the row sums.
    # H*v: read the store once (col + FP32 value = 8 B/element), row offsets, x (twice), y
    # read-modify-write and the diagonal.
    alg = {
        "hbuild_count": 16.0 * n + 4 * n + 8 * n + 8.0 * m + 4.0 * cand * (m > 0),
        "hbuild_fill": 16.0 * n + 8 * (n + 1) + 12.0 * nnz + (8.0 * m + 4.0 * cand) * (m > 0),
        "join_keys": 16.0 * n + 8.0 * m,
        "join_sort": 4 * 20.0 * m,
        "join_buckets": 20.0 * m,
        "hbuild_rowsort": 24.0 * nnz + 12.0 * n,
        "spmv_res_rows": 8.0 * nnz + 12.0 * n + 8.0 * n + 8.0 * n,
        "spmv": 8.0 * nnz + 8 * (n + 1) + 4 * n + 16 * n + 16 * n + 8 * n,
    }
    # DRAM bytes per launch measured by ncu (dram__bytes_read.sum + dram__bytes_write.sum) for
    # one full-size H*v launch of the n=26 workload: 1.2964e9 B for 152,895,046 stored
    # elements = 8.479 B per element, scaled here by the step's element count (the store is
    # read once; x, y and the diagonal stay in L2).
    measured_traffic = {"spmv": 8.479 * nnz}
    kernels = {}
    for k, (ms_l, cnt) in per.items():
        b = alg.get(k)
        g = (b / (ms_l * 1e-3) / 1e9) if b else None
        kernels[k] = {"ms_per_launch": ms_l, "launches": cnt,
                      "gbs": g, "frac": (g / hbm) if g else None}
        if k in ("hbuild_count", "hbuild_fill"):
            kernels[k]["candidates_per_s"] = cand / (ms_l * 1e-3)
    dk = kernels[dom]
    roof = {"kernel": dom, "bound": "hbm", "achieved": dk["gbs"], "peak": hbm, "unit": "GB/s",
            "frac": dk["frac"], "traffic": measured_traffic.get(dom), "peak_kind": peak_kind,
            "alg_bytes_per_launch": alg.get(dom)}
    cpu = None
    keep = {}
    if not args.no_cpu_baseline or args.parity:
        _, cpu = cpu_sample(fcidump, w, up, dn, keep=keep)
    parity = None
    if args.parity:
        parity = parity_n40(fcidump, w, up, dn)
        o_rows = keep["rows"]
        parity["sample_rows"] = int(len(sample))
        parity["sample_elements"] = int(len(o_rows[2]))
        parity["rows_equal_oracle"] = bool(np.array_equal(o_rows[0], sample))
        c64, v64 = compare_rows(o_rows, rows_fp64, False)
        cmx, vmx = compare_rows(o_rows, rows_mixed, True)
        parity.update({"fp64_columns_equal": c64, "fp64_values_equal": v64,
                       "mixed_columns_equal": cmx, "mixed_split_equal": vmx})
    if args.no_cpu_baseline:
        cpu = None
    small = run_small_configs(args.data, local) if args.small else None
    pt2_total = None
    if pt2 and pt2_fp64 and "error" not in pt2 and "error" not in pt2_fp64:
        pt2_total = {"energy_total_mixed": e_mixed + pt2["correction"],
                     "energy_total_fp64": e_fp64 + pt2_fp64["correction"],
                     "dE_pt2_mixed_vs_fp64": abs(pt2["correction"] - pt2_fp64["correction"]),
                     "dE_total_mixed_vs_fp64": abs(e_mixed + pt2["correction"]
                                                   - e_fp64 - pt2_fp64["correction"])}
    line = {
        "metric": METRIC, "value": ms / 1e3, "unit": "s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "storage": "f32 value + f32 residual",
        "data": "synthetic",
        "config": {"workload": workload_name(n), "n_dets": n, "nnz_upper": nnz,
                   "nnz_sym": 2 * (nnz + n) - n, "l2": "inputs larger than L2 (H store %.0f GB)"
                   % (12 * nnz / 1e9), "setup_s": setup_s},
        "roofline": roof, "kernels": kernels, "cpu_baseline": cpu, "hamiltonian": stats,
        "e2e": {"value": e2e / 1e3, "unit": "s", "h2d_bytes_per_step": 24 * n,
                "d2h_bytes_per_step": 8},
        "gpu_launches": launches // args.steps,
        "clocks": clk.summary(),
        "pt2": pt2,
        "pt2_fp64_wavefunction": pt2_fp64,
        "totals": pt2_total,
        "parity": parity,
        "converged": converged,
        "small_configs": small,
        "batched": batched,
        "fp64": {"ms_per_step": ms_fp64, "steps": args.steps, "energy": e_fp64},
        "energy_mixed_fp64corrected": e_mixed, "energy_davidson_mixed": e_dav,
        "dE_mixed_vs_fp64": abs(e_mixed - e_fp64),
        "speedup_mixed_vs_fp64": ms_fp64 / ms,
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--data", default=os.environ.get("SHCI_BENCH_DATA", "/tmp/shci_bench_data"))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", type=int, default=3, choices=sorted(WORKLOADS))
    ap.add_argument("--no-pt2", dest="pt2", action="store_false",
                    help="skip the PT2 measurement")
    ap.add_argument("--no-converged", dest="converged", action="store_false",
                    help="skip the whole variational stage and the converged-space step")
    ap.add_argument("--no-small", dest="small", action="store_false",
                    help="skip the full device and oracle runs of the two small configurations")
    ap.add_argument("--no-parity", dest="parity", action="store_false",
                    help="skip the oracle checks (independent det list, sampled rows)")
    ap.add_argument("--no-batched", dest="batched", action="store_false",
                    help="skip workload 5 (256 small instances, concurrent batch runner)")
    args = ap.parse_args()
    global WORKLOAD, SCHEDULE, EPS_VAR
    WORKLOAD = args.workload
    SCHEDULE, EPS_VAR = WORKLOADS[WORKLOAD]
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
