"""Benchmark: converged minimisations per second on one GB300.

Headline workload (the single-GPU plain-method configuration): a binary
PhaseField on a periodic 192^3 grid (resolution 1, interface width 1,
surface tension 1), concentration 0 + U[-0.05, 0.05] (seed 0), minimised by
L-BFGS (m = 10) to gradient RMS < 1e-7 with FP32 fields, FP64 reductions
and an FP64 polishing stage.  One step = one complete minimisation from the
initial field.  Inputs are resident in HBM before the timed region; each
step's working set (x, g, 2 x 11 history vectors: ~0.8 GB) exceeds the
129 MB L2, so no flush is needed between steps.

Also reported (keys "batched" and "plain"): 4096 Lennard-Jones clusters,
N ~ U{13..400}, half FIRE (dtMax 0.1, no line search) and half L-BFGS
(m = 5) to RMS < 1e-6, run by the persistent batch kernels, against the same
instances minimised one at a time with the whole GPU (a sample) and against
the CPU oracle on a stratified sample (one process per host core); counts
are converged instances.  Keys "mixed_batch" and "serving": the mixed
phase-field / mesh batch and the Poisson serving stream.

Also reported (key "rows"): Anneal on a batch of LJ clusters and
PhaseFieldUnstructured on a batch of three-fluid grids, each against the CPU
oracle on a sample.

--impl reference times one complete minimisation of the headline workload
by the CPU restatement of the reference algorithm (oracle/, or the reference
library itself when it was built on this host) on all host threads.
--only SECTIONS runs selected sections alone (batched, mixed, serve, rows),
e.g. the mixed batch and the serving stream at their stated sizes
(--mixed-full --mixed-grids 512 --mixed-sheets 256, --serve-full).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

GRID = (192, 192, 192)
TOL = 1e-7
METRIC = "converged minimisations/s batched vs plain on GB300 at ΔE/E<1e-8; p50/p99 ms"
# DRAM bytes per algorithmic byte of the PhaseField 192^3 minimisation's
# FP32 stage (the stepped graph), from one ncu capture of a graph launch
# running 19 iterations: dram__bytes_read.sum + dram__bytes_write.sum =
# 24.20 GB against the kernels' own count of 21.52 GB.  Traffic per step =
# this ratio x the step's algorithmic bytes.
PF_TRAFFIC_PER_ALGO_BYTE = 24.20 / 21.52


def _peaks():
    try:
        with open(os.path.join(HERE, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """nvidia-smi clock/throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.rows = []
        self._stop = threading.Event()
        self._t = None

    def start(self):
        def run():
            while not self._stop.is_set():
                try:
                    out = subprocess.run(["nvidia-smi", "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                                          "-i", os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0]],
                                         capture_output=True, text=True, timeout=5).stdout
                    for line in out.strip().splitlines():
                        self.rows.append([c.strip() for c in line.split(",")])
                except Exception:
                    pass
                self._stop.wait(0.2)
        self._t = threading.Thread(target=run, daemon=True)
        self._t.start()

    def stop(self):
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)
        sm = [float(r[1]) for r in self.rows if len(r) > 2 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 2 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for k, nm in enumerate(names):
                if len(r) > 5 + k and r[5 + k].lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def pf_setup():
    from minim_gb300 import abi
    from tests.workloads import pf_noise
    p = abi.phase_field(GRID, interface_size=1.0, surface_tension=1.0)
    x0 = pf_noise(GRID, seed=0, amp=0.05)
    mp = abi.minimiser("lbfgs", m=10, tol=TOL, precision="mixed")
    return p, x0, mp


def lj_batch_setup(count=4096):
    from minim_gb300 import abi
    from tests.workloads import Rng, lj_cluster
    rng = Rng(12345)
    sizes = 13 + (rng.uniform(count) * (400 - 13 + 1)).astype(int)
    items = []
    for i, n in enumerate(sizes):
        x0 = lj_cluster(int(n), seed=i)
        if i < count // 2:
            mp = abi.minimiser("fire", dt_max=0.1, tol=1e-6)  # Fire(0.1): no line search
        else:
            mp = abi.minimiser("lbfgs", m=5, tol=1e-6)
        items.append((x0, mp))
    return abi.lj(), items


def run_gpu(args):
    import torch  # device plumbing only (pinned host buffers)
    from minim_gb300 import abi, runtime
    from oracle.oracle import Oracle

    p, x0, mp = pf_setup()
    runtime.load()
    # warm-up (W full minimisations)
    insts = [runtime.Instance(p, x0) for _ in range(args.steps)]
    warm = runtime.Instance(p, x0)
    for _ in range(args.warmup):
        warm.coords = x0
        r = warm.minimise(mp)
    del warm

    clocks = Clocks()
    clocks.start()
    launches0 = runtime.launch_count()
    kernel_ms, abytes, results = 0.0, 0.0, []
    t0 = time.perf_counter()
    for inst in insts:
        r = inst.minimise(mp)
        st = runtime.last_run_stats()
        kernel_ms += st["kernel_ms"]
        abytes += st["abytes"]
        results.append(r)
    t1 = time.perf_counter()
    launches = runtime.launch_count() - launches0
    clk = clocks.stop()
    ok = all(r.status == abi.RES_CONVERGED for r in results)
    value = args.steps / (kernel_ms / 1e3)
    ms_per_step = kernel_ms / args.steps
    lat = [runtime.last_run_stats()["kernel_ms"]]

    # parity of the last result under the FP64 checker (energy and RMS at x)
    xg = insts[-1].coords
    ora = Oracle(p, x0)
    e_chk, g_chk = ora.energy_gradient(xg)
    e_init = ora.energy(x0)
    rel_err = abs(results[-1].energy - e_chk) / max(abs(e_chk), 1e-300)
    floor_err = abs(results[-1].energy - e_chk) / max(abs(e_chk), abs(e_init))
    rms_chk = float(np.sqrt(np.mean(g_chk ** 2)))
    # the FP32 stage's kernels, one evaluation each at the start against the
    # checker at the same FP32 point: the quad sweep (whole GPU) and the
    # stepped graph's two-trial line stencil
    e0, g0 = ora.energy_gradient(x0)
    x32 = np.asarray(x0, np.float32).astype(np.float64)
    eo32, go32 = ora.energy_gradient(x32)
    e_k, g_k = insts[-1].eval_kernel(abi.EVAL_FP32_GRID, x0)
    d = -g0 * 0.1
    e_l, g_l, pts = insts[-1].eval_kernel(abi.EVAL_LINES, x0, d, 1.0, points=True)
    eo_l, go_l = ora.energy_gradient(pts[0])
    gscale = lambda g: max(np.max(np.abs(g)), 1e-300)
    fp32_stage = {"sweep_grad_rel_err": float(np.max(np.abs(g_k - go32)) / gscale(go32)),
                  "sweep_energy_rel_err": abs(e_k - eo32) / abs(eo32),
                  "lines_grad_rel_err": float(np.max(np.abs(g_l[0] - go_l)) / gscale(go_l)),
                  "lines_energy_rel_err": abs(e_l[0] - eo_l) / abs(eo_l)}
    del insts

    # end to end through the C ABI with host buffers: H2D of x0 from pinned
    # host memory (instance creation), minimise, D2H of the result into pinned
    # host memory, every step
    x_pin = torch.empty(x0.size, dtype=torch.float64, pin_memory=True)
    x_pin.numpy()[:] = x0
    out_pin = torch.empty(x0.size, dtype=torch.float64, pin_memory=True)
    e2e_times = []
    for _ in range(args.steps):
        ta = time.perf_counter()
        inst = runtime.Instance(p, x_pin.numpy())
        inst.minimise(mp)
        inst.get_coords(out_pin.numpy())
        e2e_times.append(time.perf_counter() - ta)
        inst.close()
    e2e_value = args.steps / sum(e2e_times)

    hbm_peak, peak_kind = _peaks()
    achieved = abytes / (kernel_ms / 1e3) / 1e9
    traffic = PF_TRAFFIC_PER_ALGO_BYTE * abytes / args.steps
    roofline = {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                "frac": achieved / hbm_peak, "traffic": traffic, "traffic_unit": "bytes/step",
                "algorithmic_bytes_per_step": abytes / args.steps, "peak_source": peak_kind,
                "kernel": "stepped graph of phase kernels (FP32 L-BFGS stage) + grid_kernel<K_PF1> "
                          "(set-up iteration, FP64 stage)"}

    out = {
        "metric": METRIC, "value": value, "unit": "minimisations/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32+fp64",
        "data": "synthetic (seeded noise field)",
        "config": {"workload": "PhaseField binary 192^3 periodic, Lbfgs m=10, RMS<1e-7, mixed FP32/FP64",
                   "grid": list(GRID), "ndof": int(np.prod(GRID)), "l2": "working set > L2, no flush"},
        "iterations": results[-1].iter, "fp64_iters": results[-1].fp64_iters,
        "converged": ok, "energy": results[-1].energy,
        "parity": {"energy_rel_err": rel_err, "energy_err_vs_max_E_Einit": floor_err,
                   "oracle_rms_at_x": rms_chk, "fp32_stage": fp32_stage},
        "e2e": {"value": e2e_value, "unit": "minimisations/s",
                "h2d_bytes_per_step": int(x0.size * 8), "d2h_bytes_per_step": int(x0.size * 8)},
        "gpu_launches": int(launches), "roofline": roofline, "clocks": clk,
        "wall_s_timed": t1 - t0,
    }
    if not args.no_batched:
        out.update(run_batched(args))
    if args.mixed > 0 or args.mixed_grids > 0 or args.mixed_sheets > 0:
        out.update(run_mixed(args))
    if args.serve > 0:
        out.update(run_serving(args))
    if args.rows:
        out["rows"] = run_rows(args)
    if not args.no_cpu:
        out["cpu_baseline"] = cpu_baseline(results[-1].iter, budget_s=args.cpu_budget)
    return out


def _fp32_peak():
    """Nominal FP32 rate of this GPU in TFLOP/s: 128 FP32 lanes per SM x 2
    flops per fused multiply-add x SMs x the maximum SM clock (the measured
    peaks file's `sm_max_mhz`, else 2070 MHz)."""
    import torch
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    mhz = 2070.0
    try:
        with open(os.path.join(HERE, "MEASURED_PEAKS.json")) as f:
            mhz = float(json.load(f).get("sm_max_mhz", mhz))
    except Exception:
        pass
    return 128 * 2 * sms * mhz * 1e6 / 1e12


def _oracle_lj_job(job):
    """One CPU oracle minimisation of a batched Lennard-Jones instance (run in
    a worker process): (index, status, iterations, energy, seconds)."""
    i, n, fire = job
    from minim_gb300 import abi
    from oracle.oracle import Oracle
    from tests.workloads import lj_cluster
    mp = abi.minimiser("fire", dt_max=0.1, tol=1e-6) if fire else abi.minimiser("lbfgs", m=5, tol=1e-6)
    t = time.perf_counter()
    r = Oracle(abi.lj(), lj_cluster(n, seed=i)).minimise(mp)
    return i, int(r.status), int(r.iter), float(r.energy), time.perf_counter() - t


def _stratified(sizes, idx, per_bucket, rng, edges=(13, 113, 213, 313, 401)):
    out = []
    for lo, hi in zip(edges[:-1], edges[1:]):
        cand = [i for i in idx if lo <= sizes[i] < hi]
        if cand:
            out += list(rng.choice(cand, size=min(per_bucket, len(cand)), replace=False))
    return sorted(int(i) for i in out)


def run_batched(args):
    """The batched Lennard-Jones workload: 4096 clusters, N ~ U{13..400},
    half Fire(0.1) and half Lbfgs(m = 5) to RMS < 1e-6, in one batch run
    (the persistent batch kernels, autotuned launch shapes).  Throughput
    counts converged instances only.  Beside it: the same instances one at a
    time on the whole GPU (a sample), and the CPU oracle on a stratified
    sample of both halves (one process per host core, one thread each),
    whose per-instance times are extrapolated to the whole batch; the FIRE
    half's statuses are compared with the oracle's on that sample."""
    from minim_gb300 import abi, runtime
    p, items = lj_batch_setup(args.batch)
    sizes = [x0.size // 3 for x0, _ in items]
    insts = [runtime.Instance(p, x0) for x0, _ in items]
    b = runtime.Batch()
    for inst, (_, mp) in zip(insts, items):
        b.add(inst, mp)
    # warm-up: a short batch of both methods (module load, workspace pool,
    # the autotuner's first measurements)
    wb = runtime.Batch()
    half = len(items) // 2
    warm = [runtime.Instance(p, x0) for x0, _ in items[max(half - 32, 0):half + 32]]
    for inst, (_, mp) in zip(warm, items[max(half - 32, 0):half + 32]):
        wm = abi.MinimiserParams.from_buffer_copy(mp)
        wm.max_iter = 500
        wb.add(inst, wm)
    wb.run()
    del wb, warm
    res = b.run()
    st = runtime.last_run_stats()
    conv = sum(r.status == abi.RES_CONVERGED for r in res)
    status = [int(r.status) for r in res]
    batched = conv / (st["kernel_ms"] / 1e3)
    by_method = {}
    for name, sl in (("fire", slice(0, half)), ("lbfgs", slice(half, None))):
        rs = res[sl]
        by_method[name] = {"instances": len(rs), "converged": sum(r.status == abi.RES_CONVERGED for r in rs),
                           "maxiter": sum(r.status == abi.RES_MAXITER for r in rs),
                           "nan": sum(r.status == abi.RES_NAN for r in rs)}
    # plain: the same instances one at a time on the whole GPU (sample)
    rng = np.random.default_rng(0)
    idx = rng.choice(len(items), size=min(args.plain_sample, len(items)), replace=False)
    plain_ms, plain_conv = 0.0, 0
    for i in idx:
        inst = runtime.Instance(p, items[i][0])
        r = inst.minimise(items[i][1])
        plain_ms += runtime.last_run_stats()["kernel_ms"]
        plain_conv += r.status == abi.RES_CONVERGED
    plain = plain_conv / (plain_ms / 1e3)
    flops32 = st["pairs32"] * 20
    out = {
        "batched": {"value": batched, "unit": "converged minimisations/s", "instances": len(items),
                    "converged": int(conv), "kernel_ms": st["kernel_ms"], "tune_ms": st["tune_ms"],
                    "by_method": by_method, "iterations": st["iterations"],
                    "fp64_iteration_share": st["fp64_iterations"] / max(st["iterations"], 1),
                    "fp32_tflops": flops32 / (st["kernel_ms"] / 1e3) / 1e12,
                    "fp32_peak_tflops": _fp32_peak(),
                    "fp32_frac": flops32 / (st["kernel_ms"] / 1e3) / 1e12 / _fp32_peak(),
                    "launch_shapes": [t for t in runtime.tune_table() if t["kind"] == "lj"],
                    "workload": f"{len(items)} LJ clusters N~U{{13..400}}, half Fire(0.1) half Lbfgs(m=5), "
                                f"RMS<1e-6"},
        "plain": {"value": plain, "unit": "converged minimisations/s", "sample": int(len(idx)),
                  "converged": int(plain_conv), "kernel_ms": plain_ms},
        "batched_vs_plain": batched / plain if plain > 0 else None,
    }
    out["batched"]["iteration_cost_fit"] = _iteration_cost_fit(sizes[:half], res[:half])
    # MIXED against FP64 throughout on every 8th cluster of the Lbfgs half
    # (the FIRE half's 100000-iteration runs take minutes in FP64)
    sample = [("lj", p, items[i][0], None) for i in range(half, len(items), 8)]
    out["batched"]["mixed_vs_fp64"] = dict(_precision_compare(sample, items[half][1]),
                                           sample=f"{len(sample)} Lbfgs clusters (every 8th)")
    if args.cpu_sample > 0 and not args.no_cpu:
        out["batched"]["cpu_baseline"], out["batched"]["fire_vs_oracle"] = \
            _batched_cpu(items, sizes, status, res, args)
    return out


def _iteration_cost_fit(sizes, res):
    """Device time of one FIRE iteration in each precision stage, from the
    per-instance results of the runs that reached the iteration limit (every
    one runs the same number of iterations, split between the stages):
    run_ms = a32 N^2 n32 + b32 n32 + a64 N^2 n64 + b64 n64 by least squares,
    with n64 the FP64-stage iterations.  Times are per instance while it
    shares its SM with the batch's other resident instances."""
    from minim_gb300 import abi
    rows = [(n, r.iter - r.fp64_iters, r.fp64_iters, r.run_ms) for n, r in zip(sizes, res)
            if r.status == abi.RES_MAXITER]
    if len(rows) < 8:
        return None
    a = np.array(rows, dtype=float)
    n2 = a[:, 0] ** 2
    X = np.stack([n2 * a[:, 1], a[:, 1], n2 * a[:, 2], a[:, 2]], 1)
    c, *_ = np.linalg.lstsq(X, a[:, 3] * 1e3, rcond=None)  # microseconds
    at = lambda n, k: float(c[k] * n * n + c[k + 1])
    return {"instances": len(rows), "us_per_n2_fp32": float(c[0]), "us_fixed_fp32": float(c[1]),
            "us_per_n2_fp64": float(c[2]), "us_fixed_fp64": float(c[3]),
            "us_per_iteration_n390": {"fp32": at(390, 0), "fp64": at(390, 2)},
            "fp64_share_of_instance_time": float((X[:, 2:] @ c[2:]).sum() / (X @ c).sum())}


def _batched_cpu(items, sizes, status, res, args):
    import concurrent.futures as cf
    import multiprocessing as mpc
    from minim_gb300 import abi
    half = len(items) // 2
    rng = np.random.default_rng(1)
    per = max(1, args.cpu_sample // 8)
    fire_idx = _stratified(sizes, range(half), per, rng)
    lb_idx = _stratified(sizes, range(half, len(items)), per, rng)
    jobs = [(i, sizes[i], i < half) for i in fire_idx + lb_idx]
    cores = os.cpu_count() or 1
    t0 = time.perf_counter()
    with cf.ProcessPoolExecutor(max_workers=cores, mp_context=mpc.get_context("spawn")) as ex:
        outs = list(ex.map(_oracle_lj_job, jobs))
    wall = time.perf_counter() - t0
    got = {o[0]: o for o in outs}
    # per-instance CPU seconds, extrapolated by size bucket and method to the
    # whole batch; converged fraction likewise
    edges = (13, 113, 213, 313, 401)
    total_s, total_conv = 0.0, 0.0
    for fire, rng_idx in ((True, range(half)), (False, range(half, len(items)))):
        for lo, hi in zip(edges[:-1], edges[1:]):
            members = [i for i in rng_idx if lo <= sizes[i] < hi]
            samp = [got[i] for i in got if (i < half) == fire and lo <= sizes[i] < hi]
            if not members or not samp:
                continue
            total_s += len(members) * float(np.mean([o[4] for o in samp]))
            total_conv += len(members) * float(np.mean([o[1] == abi.RES_CONVERGED for o in samp]))
    cpu_rate = total_conv / (total_s / cores)
    fire_s = [got[i] for i in fire_idx]
    agree = [status[i] == o[1] for i, o in zip(fire_idx, fire_s)]
    both = [(res[i].energy, o[3]) for i, o in zip(fire_idx, fire_s)
            if status[i] == abi.RES_CONVERGED and o[1] == abi.RES_CONVERGED]
    same_e = [abs(a - c) <= 1e-6 * abs(c) for a, c in both]
    cpu = {"value": cpu_rate, "unit": "converged minimisations/s", "cores": cores, "kind": "port",
           "sample": f"{len(jobs)} instances ({len(fire_idx)} Fire, {len(lb_idx)} Lbfgs) stratified by N, "
                     f"one process per core, {wall:.1f} s wall; per-instance times extrapolated to "
                     f"{len(items)} instances"}
    fire = {"sample": len(fire_idx), "status_matches_oracle": float(np.mean(agree)) if agree else None,
            "oracle_statuses": {abi.RES_NAMES[k]: sum(o[1] == k for o in fire_s) for k in (0, 1, 2)},
            "gpu_statuses": {abi.RES_NAMES[k]: sum(status[i] == k for i in fire_idx) for k in (0, 1, 2)},
            "both_converged": len(both), "same_minimum_1e-6": int(sum(same_e))}
    return cpu, fire


def mixed_items(n_grids, n_sheets, full, seed=11):
    """Instances of the mixed phase-field / mesh batch.  full: the stated
    distribution -- 2-D three-fluid PhaseField grids (hard density
    constraint, fixed volumes, a random point on the simplex per node) with
    sides uniform in {64, 128, 256, 512}, and BarAndHinge sheets of V = k^2
    vertices with V uniform in [1000, 100000] (flat jittered rest shape,
    Gaussian out-of-plane start of amplitude 0.1); otherwise the capped
    version (sides 64 / 128, sheets of 32^2 .. 64^2 vertices).  All Lbfgs
    (m = 5) to RMS < 1e-7."""
    from minim_gb300 import abi
    from tests.workloads import Rng, pf_simplex, sheet
    rng = Rng(seed)
    u = rng.uniform(n_grids + n_sheets)
    items = []
    for i in range(n_grids):
        side = (64, 128, 256, 512)[min(int(u[i] * 4), 3)] if full else (64 if u[i] < 0.5 else 128)
        grid = (side, side, 1)
        items.append(("pf", abi.phase_field(grid, nfluid=3, volume_fixed=True),
                      pf_simplex(grid, 3, seed=5000 + i), None))
    for i in range(n_sheets):
        if full:
            k = int(round(np.sqrt(1000 + u[n_grids + i] * 99000)))
        else:
            k = 32 + int(u[n_grids + i] * 33)
        flat, tris, pert = sheet(k, seed=6000 + i)
        items.append(("bah", abi.bar_and_hinge(triangulation=tris, rigidity=(1, 0.01)), flat, pert))
    return items


def _oracle_rate(jobs, strata):
    """CPU oracle baseline of a set of minimisations: `jobs` maps a stratum
    to its sampled (potential, start coordinates, minimiser parameters);
    `strata` maps each stratum to the number of instances it stands for.
    The sampled minimisations run on one host thread each, all host threads
    at once (the oracle's C calls release the interpreter lock), each timed
    from its first iteration (set-up excluded, as on the GPU side); the mean
    time and converged fraction of each stratum's sample are extrapolated to
    its instances.  Returns (converged minimisations/s on all threads,
    threads, sample description)."""
    import concurrent.futures as cf
    from minim_gb300 import abi
    from oracle.oracle import Oracle

    def one(job):
        p, x0, start, mp = job
        o = Oracle(p, x0)
        if start is not None:
            o.coords = start
        t = time.perf_counter()
        r = o.minimise(mp)
        return int(r.status), time.perf_counter() - t

    cores = os.cpu_count() or 1
    flat = [(k, j) for k, js in jobs.items() for j in js]
    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(max_workers=cores) as ex:
        outs = list(ex.map(lambda kj: (kj[0],) + one(kj[1]), flat))
    wall = time.perf_counter() - t0
    total_s, total_conv = 0.0, 0.0
    for k, count in strata.items():
        samp = [o for o in outs if o[0] == k]
        if not samp or not count:
            continue
        total_s += count * float(np.mean([o[2] for o in samp]))
        total_conv += count * float(np.mean([o[1] == abi.RES_CONVERGED for o in samp]))
    rate = total_conv / (total_s / cores) if total_s > 0 else None
    desc = (f"{len(flat)} instances in {len(jobs)} strata, one host thread each, {cores} threads, "
            f"{wall:.1f} s wall; per-instance times extrapolated to {sum(strata.values())} instances")
    return rate, cores, desc


def _mixed_cpu(items, mp, per):
    """The oracle baseline of the mixed batch: `per` instances of each
    stratum (PhaseField grid side; BarAndHinge sheet size, split at the
    median vertex count)."""
    rng = np.random.default_rng(2)
    key = {}
    sheets = sorted(np.size(x0) for kind, _, x0, _ in items if kind == "bah")
    split = sheets[len(sheets) // 2] if sheets else 0
    for j, (kind, p, x0, start) in enumerate(items):
        k = f"pf{int(round(np.sqrt(np.size(x0) / 3)))}" if kind == "pf" else \
            ("bah_small" if np.size(x0) < split else "bah_large")
        key.setdefault(k, []).append(j)
    strata = {k: len(v) for k, v in key.items()}
    jobs = {}
    for k, v in key.items():
        pick = rng.choice(v, size=min(per, len(v)), replace=False)
        jobs[k] = [(items[j][1], items[j][2], items[j][3], mp) for j in sorted(int(i) for i in pick)]
    return _oracle_rate(jobs, strata)


def _serving_cpu(reqs, per):
    """The oracle baseline of a serving stream's requests (their throughput
    with every host thread busy, arrivals ignored): `per` requests of each
    stratum (LJ below / above 100 particles, 2-D and 3-D PhaseField,
    BarAndHinge)."""
    rng = np.random.default_rng(3)
    key = {}
    for j, (_, kind, p, x0, mp) in enumerate(reqs):
        if kind == "lj":
            k = "lj_small" if np.size(x0) < 300 else "lj_large"
        elif kind == "pf":
            k = "pf3d" if p.struct.grid[2] > 1 else "pf2d"
        else:
            k = "bah"
        key.setdefault(k, []).append(j)
    strata = {k: len(v) for k, v in key.items()}
    jobs = {}
    for k, v in key.items():
        pick = rng.choice(v, size=min(per, len(v)), replace=False)
        jobs[k] = [(reqs[j][2], reqs[j][3], None, reqs[j][4]) for j in sorted(int(i) for i in pick)]
    return _oracle_rate(jobs, strata)


def _precision_compare(items, mp):
    """The same instances (kind, potential, start, displaced start) as one
    batch run with MIXED precision and one with FP64 throughout: kernel time,
    iterations and converged count of each, by kind."""
    from minim_gb300 import abi, runtime
    out = {}
    for prec in ("mixed", "fp64"):
        m = abi.MinimiserParams.from_buffer_copy(mp)
        m.precision = {"mixed": abi.PREC_MIXED, "fp64": abi.PREC_FP64}[prec]
        b = runtime.Batch()
        for kind, p, x0, start in items:
            inst = runtime.Instance(p, x0)
            if start is not None:
                inst.coords = start
            b.add(inst, m)
        res = b.run()
        st = runtime.last_run_stats()
        kinds = {}
        for (kind, _, _, _), r in zip(items, res):
            k = kinds.setdefault(kind, {"converged": 0, "iterations": 0, "fp64_iterations": 0})
            k["converged"] += r.status == abi.RES_CONVERGED
            k["iterations"] += r.iter
            k["fp64_iterations"] += r.fp64_iters
        out[prec] = {"kernel_ms": st["kernel_ms"], "by_kind": kinds}
    out["mixed_over_fp64_time"] = out["mixed"]["kernel_ms"] / out["fp64"]["kernel_ms"]
    return out


def run_mixed(args):
    """One batch run of mixed phase-field and mesh instances (mixed_items),
    all kinds at once on their own streams; then the same instances with
    MIXED and with FP64 precision on their own (_precision_compare)."""
    from minim_gb300 import abi, runtime
    full = args.mixed_full
    n_grids = args.mixed_grids if args.mixed_grids >= 0 else (2 * args.mixed) // 3
    n_sheets = args.mixed_sheets if args.mixed_sheets >= 0 else args.mixed - (2 * args.mixed) // 3
    items = mixed_items(n_grids, n_sheets, full)
    mp = abi.minimiser("lbfgs", tol=1e-7, max_iter=args.mixed_max_iter)
    insts = []
    t_set = time.perf_counter()
    for kind, p, x0, start in items:
        inst = runtime.Instance(p, x0)
        if start is not None:
            inst.coords = start
        insts.append(inst)
    t_set = time.perf_counter() - t_set
    b = runtime.Batch()
    for inst in insts:
        b.add(inst, mp)
    res = b.run()
    st = runtime.last_run_stats()
    conv = sum(r.status == abi.RES_CONVERGED for r in res)
    kinds = {}
    for (kind, p, x0, _), r in zip(items, res):
        k = kinds.setdefault(kind, {"instances": 0, "converged": 0, "maxiter": 0, "dof": 0, "iterations": 0,
                                    "run_ms": []})
        k["instances"] += 1
        k["converged"] += r.status == abi.RES_CONVERGED
        k["maxiter"] += r.status == abi.RES_MAXITER
        k["dof"] += int(np.size(x0))
        k["iterations"] += r.iter
        k["run_ms"].append(r.run_ms)
    for k in kinds.values():
        # each instance's device time on its SM: the batch's makespan is at
        # least the longest of them
        t = np.array(k.pop("run_ms"))
        k["run_ms_p50_p99_max"] = [float(np.percentile(t, 50)), float(np.percentile(t, 99)), float(t.max())]
    prec = _precision_compare(items, mp) if not full else None
    cpu = None
    if args.cpu_sample > 0 and not args.no_cpu and not full:
        rate, cores, sample = _mixed_cpu(items, mp, max(1, args.cpu_sample // 32))
        cpu = {"value": rate, "unit": "converged minimisations/s", "cores": cores, "kind": "port",
               "sample": sample}
    desc = (f"{n_grids} 2-D ternary PhaseField grids (" + ("64^2-512^2" if full else "64^2/128^2") +
            f", fixed volume) + {n_sheets} BarAndHinge sheets (" + ("1k-100k" if full else "1k-4.2k") +
            " vertices), Lbfgs RMS<1e-7")
    return {"mixed_batch": {"value": conv / (st["kernel_ms"] / 1e3), "unit": "converged minimisations/s",
                            "instances": len(items), "converged": int(conv), "kernel_ms": st["kernel_ms"],
                            "tune_ms": st["tune_ms"], "setup_s": t_set, "by_kind": kinds,
                            "fp64_iteration_share": st["fp64_iterations"] / max(st["iterations"], 1),
                            "stated_sizes": bool(full), "workload": desc, "mixed_vs_fp64": prec,
                            "cpu_baseline": cpu}}


def run_rows(args):
    """The minimiser and potential beyond the headline path, each as one
    batch launch with the FP64 oracle timed on a sample of the same instances
    (one host thread, as the reference runs them):
      anneal: `args.anneal` Lennard-Jones clusters of 38 particles, Anneal
              (T0 0.3, displacement 0.02, rate 1) for 2000 iterations each,
              FP64 coordinates -- annealing iterations (one energy evaluation
              each) per second;
      pfu:    `args.pfu` PhaseFieldUnstructured 2-D three-fluid grids (64^2,
              DENSITY fixed: the last fluid from the others), Lbfgs to RMS
              < 1e-7 -- converged minimisations per second."""
    from minim_gb300 import abi, runtime
    from oracle.oracle import Oracle
    from tests.workloads import lj_cluster, pf_simplex
    rows = {}
    iters = 2000

    def anneal_mp(i):
        return abi.minimiser("anneal", temp_init=0.3, displacement=0.02, max_iter=iters - 1, seed=1 + i)

    if args.anneal > 0:
        b = runtime.Batch()
        xs = [lj_cluster(38, seed=9000 + i) for i in range(args.anneal)]
        insts = []
        for i, x in enumerate(xs):
            inst = runtime.Instance(abi.lj(), x)
            b.add(inst, anneal_mp(i))
            insts.append(inst)
        res = b.run()
        st = runtime.last_run_stats()
        gpu_it = sum(r.iter for r in res)
        gpu_rate = gpu_it / (st["kernel_ms"] / 1e3)
        t0, cpu_it, k = time.perf_counter(), 0, 0
        same = True
        while k < len(xs) and (k < 2 or time.perf_counter() - t0 < args.cpu_budget / 4):
            o = Oracle(abi.lj(), xs[k])
            ro = o.minimise(anneal_mp(k))
            cpu_it += ro.iter
            same &= (ro.iter == res[k].iter and abs(ro.energy - res[k].energy) <= 1e-12 * abs(ro.energy))
            k += 1
        cpu_rate = cpu_it / (time.perf_counter() - t0)
        rows["anneal"] = {"value": gpu_rate, "unit": "annealing iterations/s", "instances": len(xs),
                          "kernel_ms": st["kernel_ms"], "pairs_per_s": gpu_rate * 38 * 37 / 2,
                          "cpu_oracle": {"value": cpu_rate, "cores": 1, "sample": f"{k} clusters"},
                          "speedup_vs_cpu": gpu_rate / cpu_rate, "sample_runs_match_oracle": bool(same),
                          "workload": f"{len(xs)} LJ38 clusters, Anneal T0=0.3 d=0.02, {iters} iterations, FP64"}
    if args.pfu > 0:
        grid = (64, 64, 1)
        p = abi.phase_field_unstructured(grid, nfluid=3, density_constraint="fixed")
        mp = abi.minimiser("lbfgs", tol=1e-7, max_iter=20000)
        xs = [pf_simplex(grid, 3, seed=9500 + i) for i in range(args.pfu)]
        b = runtime.Batch()
        for x in xs:
            b.add(runtime.Instance(p, x), mp)
        res = b.run()
        st = runtime.last_run_stats()
        conv = sum(r.status == abi.RES_CONVERGED for r in res)
        gpu_rate = conv / (st["kernel_ms"] / 1e3)
        t0, k, cpu_conv = time.perf_counter(), 0, 0
        while k < len(xs) and (k < 1 or time.perf_counter() - t0 < args.cpu_budget / 4):
            ro = Oracle(p, xs[k]).minimise(mp)
            cpu_conv += ro.status == abi.RES_CONVERGED
            k += 1
        cpu_rate = cpu_conv / (time.perf_counter() - t0)
        rows["pfu"] = {"value": gpu_rate, "unit": "converged minimisations/s", "instances": len(xs),
                       "converged": int(conv), "kernel_ms": st["kernel_ms"],
                       "cpu_oracle": {"value": cpu_rate, "cores": 1, "sample": f"{k} grids"},
                       "speedup_vs_cpu": gpu_rate / cpu_rate if cpu_rate > 0 else None,
                       "workload": f"{len(xs)} PhaseFieldUnstructured 64^2 three-fluid grids, DENSITY fixed, "
                                   "Lbfgs RMS<1e-7"}
    return rows


def serving_requests(count, rate, full, seed=7):
    """A seeded Poisson stream of mixed requests: LjNd clusters (N
    log-uniform), 2-D / 3-D PhaseField grids (half of them with random solid
    spheres covering 20 % of the nodes) and BarAndHinge sheets.  full: the
    stated sizes -- N in [13, 5000], sides 64-128 per dimension, sheets of
    1k-50k vertices; otherwise capped so that the stream runs in seconds (N
    in [13, 400], sides 64-128 (2-D) or 24-48 (3-D), sheets of 32^2 .. 48^2
    vertices)."""
    from minim_gb300 import abi, runtime
    from tests.workloads import Rng, lj_cluster, pf_noise, sheet
    rng = Rng(seed)
    u = rng.uniform(6 * count).reshape(count, 6)
    t = np.cumsum(-np.log(1.0 - u[:, 0]) / rate)
    nmax = 5000 if full else 400
    reqs = []
    for i in range(count):
        kind = int(u[i, 1] * 3)
        if kind == 0:
            n = int(np.exp(np.log(13) + u[i, 2] * (np.log(nmax) - np.log(13))))
            reqs.append((t[i], "lj", abi.lj(), lj_cluster(n, seed=1000 + i), abi.minimiser("lbfgs", m=5, tol=1e-6)))
        elif kind == 1:
            if u[i, 3] < 0.5:
                side = 64 + int(u[i, 4] * 65)
                grid = (side, side, 1)
            else:
                side = (64 + int(u[i, 4] * 65)) if full else (24 + int(u[i, 4] * 25))
                grid = (side, side, side)
            x0 = pf_noise(grid, seed=3000 + i)
            p = abi.phase_field(grid, interface_size=1.0, surface_tension=1.0)
            if u[i, 5] < 0.5:
                # random spheres until about 20 % of the nodes are solid; a
                # layout with a node shape the reference cannot classify
                # (PhaseField::getType) is drawn again
                r2 = Rng(2000 + i)
                idx = np.indices(grid).reshape(3, -1).T
                on = np.array(grid) > 1
                for _ in range(20):
                    mask = np.zeros(int(np.prod(grid)), bool)
                    while mask.mean() < 0.2:
                        c = r2.uniform(3) * np.array(grid)
                        rad = 3 + r2.uniform() * grid[0] / 8
                        mask |= (((idx - c) ** 2) * on).sum(axis=1) < rad * rad
                    ps = abi.phase_field(grid, interface_size=1.0, surface_tension=1.0,
                                         solid=mask.astype(np.uint8))
                    try:
                        runtime.pf_setup(ps, x0)
                    except runtime.MinimGpuError:
                        continue
                    p = ps
                    break
            reqs.append((t[i], "pf", p, x0, abi.minimiser("lbfgs", m=5, tol=1e-7)))
        else:
            k = int(round(np.sqrt(1000 + u[i, 2] * 49000))) if full else 32 + int(u[i, 2] * 17)
            flat, tris, pert = sheet(k, seed=4000 + i)
            p0 = abi.bar_and_hinge(triangulation=tris, rigidity=(1, 0.01))
            _, bpar, _, hpar = runtime.bah_elements(p0, flat)
            p = abi.bar_and_hinge(triangulation=tris, rigidity=(1, 0.01), length0=bpar[:, 1].copy(),
                                  theta0=hpar[:, 1].copy())
            reqs.append((t[i], "bah", p, pert, abi.minimiser("lbfgs", m=5, tol=1e-7)))
    return reqs


def _serve_stream(reqs, slice_iters=0):
    """Submits each request when its arrival time has passed, steps the
    server while anything is resident or queued, and records completion
    times: (converged, wall s, latencies ms, statuses)."""
    from minim_gb300 import abi, runtime
    srv = runtime.Server(slice_iters=slice_iters)
    arrival, done_t, status = {}, {}, {}
    t0 = time.perf_counter()
    nxt = 0
    while len(done_t) < len(reqs):
        now = time.perf_counter() - t0
        while nxt < len(reqs) and reqs[nxt][0] <= now:
            _, _, p, x0, mp = reqs[nxt]
            rid = srv.submit(p, x0, mp)
            arrival[rid] = reqs[nxt][0]
            nxt += 1
        if srv.ndof:
            srv.step()
        elif nxt < len(reqs):
            time.sleep(max(0.0, reqs[nxt][0] - (time.perf_counter() - t0)))
        for rid, r in srv.poll():
            done_t[rid] = time.perf_counter() - t0
            status[rid] = r.status
            srv.take(rid)
    wall = time.perf_counter() - t0
    srv.close()
    lat = np.array([1e3 * (done_t[r] - arrival[r]) for r in done_t])
    conv = sum(1 for r in status.values() if r == abi.RES_CONVERGED)
    return conv, wall, lat, status


def run_serving(args):
    """Continuous batching under a Poisson arrival stream (serving_requests):
    requests are admitted as slots and memory free up, and latency is
    completion minus arrival.  Run at the stated offered load (2000
    requests/s, far above what the GPU completes, so latency there is mostly
    queueing) and again, with the same request mix, at half the throughput
    the first run measured (latency of requests the server can carry)."""
    from minim_gb300 import abi, runtime
    full = args.serve_full
    reqs = serving_requests(args.serve, args.serve_rate, full)
    # warm-up: a few requests of each kind
    _serve_stream([(0.0,) + r[1:] for r in reqs[:6]])
    conv, wall, lat, _ = _serve_stream(reqs)
    kinds = "LJ (N 13-5000), 2-D/3-D PhaseField (64-128 per side, half with 20% solid spheres), " \
            "BarAndHinge sheets (1k-50k vertices)" if full else \
            "LJ (N 13-400), 2-D/3-D PhaseField (half with 20% solid spheres), BarAndHinge sheets (1k-2.3k vertices)"
    out = {"value": conv / wall, "unit": "converged minimisations/s", "requests": len(reqs), "converged": conv,
           "wall_s": wall, "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
           "arrival_rate": args.serve_rate, "stated_sizes": bool(full),
           "workload": "Poisson stream of " + kinds + ", Lbfgs"}
    cap = conv / wall
    if args.cpu_sample > 0 and not args.no_cpu and not full:
        rate, cores, sample = _serving_cpu(reqs, max(1, args.cpu_sample // 32))
        out["cpu_baseline"] = {"value": rate, "unit": "converged minimisations/s", "cores": cores,
                               "kind": "port", "sample": sample + " (the request mix; arrivals ignored)"}
    if args.serve_carried and cap > 0:
        rate2 = 0.5 * cap
        reqs2 = serving_requests(args.serve_carried, rate2, full, seed=8)
        conv2, wall2, lat2, _ = _serve_stream(reqs2)
        out["carried_load"] = {"arrival_rate": rate2, "requests": len(reqs2), "converged": conv2,
                               "value": conv2 / wall2, "wall_s": wall2,
                               "p50_ms": float(np.percentile(lat2, 50)), "p99_ms": float(np.percentile(lat2, 99))}
    return {"serving": out}


def cpu_baseline(gpu_iters, budget_s=20.0):
    """CPU restatement (or the reference library where it was built) timed on
    all host threads over a bounded number of L-BFGS iterations of the same
    192^3 workload; the rate is extrapolated to a full minimisation with the
    GPU's iteration count (the same algorithm and stopping rule)."""
    from minim_gb300 import abi
    from oracle import oracle as O
    p, x0, mp = pf_setup()
    kind = "reference" if O.reference_available() else "port"
    cls = O.Reference if kind == "reference" else O.Oracle
    threads = os.cpu_count() or 1
    inst = cls(p, x0, threads=threads)
    # time one E+g to size the sample
    t = time.perf_counter()
    inst.energy_gradient()
    t_eval = time.perf_counter() - t
    iters = max(2, int(budget_s / max(t_eval * 5, 1e-3)))
    mps = abi.minimiser("lbfgs", m=10, tol=TOL, max_iter=iters - 1)
    inst = cls(p, x0, threads=threads)
    t = time.perf_counter()
    r = inst.minimise(mps)
    dt = time.perf_counter() - t
    per_iter = dt / (r.iter + 1 if r.status != 0 else r.iter + 1)
    rate = 1.0 / (per_iter * max(gpu_iters + 1, 1))
    return {"value": rate, "unit": "minimisations/s", "cores": threads, "kind": kind,
            "sample": f"{r.iter + 1} L-BFGS iterations of the 192^3 run ({dt:.1f} s), "
                      f"extrapolated to {gpu_iters + 1} iterations"}


def run_reference(args):
    """The reference arm: one complete minimisation of the 192^3 workload by
    the CPU restatement (or the reference library where it was built on this
    host) on all host threads, timed end to end (about a minute on the GPU
    host's 16 cores).  The line reports the one step actually run."""
    from minim_gb300 import abi
    from oracle import oracle as O
    p, x0, mp = pf_setup()
    kind = "reference" if O.reference_available() else "port"
    cls = O.Reference if kind == "reference" else O.Oracle
    threads = os.cpu_count() or 1
    inst = cls(p, x0, threads=threads)
    t = time.perf_counter()
    r = inst.minimise(abi.minimiser("lbfgs", m=10, tol=TOL))
    dt = time.perf_counter() - t
    rate = 1.0 / dt
    cb = {"value": rate, "unit": "minimisations/s", "cores": threads, "kind": kind,
          "sample": f"one complete minimisation of the 192^3 run: {r.iter + 1} L-BFGS iterations, "
                    f"status {abi.RES_NAMES.get(r.status, r.status)}, {dt:.1f} s"}
    return {"metric": METRIC, "value": rate, "unit": "minimisations/s", "n_gpus": args.gpus,
            "steps": 1, "steps_requested": args.steps, "warmup": 0, "ms_per_step": 1e3 * dt,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp64",
            "data": "synthetic (seeded noise field)", "impl": "reference",
            "config": {"workload": "PhaseField binary 192^3 periodic, Lbfgs m=10, RMS<1e-7"},
            "iterations": r.iter, "converged": r.status == abi.RES_CONVERGED, "energy": r.energy,
            "cpu_baseline": cb,
            "e2e": {"value": rate, "unit": "minimisations/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def run_profile_case(iters):
    """One short minimisation of the headline workload (a single launch of
    the fused minimiser kernel) for profiler captures."""
    from minim_gb300 import abi, runtime
    p, x0, _ = pf_setup()
    mp = abi.minimiser("lbfgs", m=10, tol=TOL, max_iter=iters - 1, precision="fp32")
    inst = runtime.Instance(p, x0)
    r = inst.minimise(mp)
    st = runtime.last_run_stats()
    print(json.dumps({"profile_case": "PhaseField 192^3 Lbfgs m=10", "iterations": iters,
                      "kernel_ms": st["kernel_ms"], "launches": st["launches"], "abytes": st["abytes"],
                      "abytes_per_launch": st["abytes"] / max(st["launches"], 1), "status": r.status}))


def run_profile_pf(iters, precision):
    """One batch launch of one 2-D 128^2 three-fluid PhaseField grid (hard
    density, fixed volumes), L-BFGS for `iters` iterations at `precision`:
    the instance kind that bounds the mixed PF/BAH batch (profiler capture)."""
    from minim_gb300 import abi, runtime
    from tests.workloads import pf_simplex
    g = (128, 128, 1)
    inst = runtime.Instance(abi.phase_field(g, nfluid=3, volume_fixed=True), pf_simplex(g, 3, seed=5001))
    b = runtime.Batch()
    b.add(inst, abi.minimiser("lbfgs", tol=1e-7, max_iter=iters, precision=precision))
    r = b.run()[0]
    st = runtime.last_run_stats()
    print(json.dumps({"iter": r.iter, "evals": r.evals, "kernel_ms": st["kernel_ms"], "precision": precision}))


def run_profile_lj(iters, precision="fp32"):
    """One batch launch of 304 Lennard-Jones clusters (N=300, Fire(0.1),
    `iters` iterations each; FP32 coordinates, or with "fp64" FP64
    coordinates and the double-float pair code of the FP64 stage) for
    profiler captures of the batched kernel."""
    from minim_gb300 import abi, runtime
    from tests.workloads import lj_cluster
    insts = [runtime.Instance(abi.lj(), lj_cluster(300, seed=i)) for i in range(304)]
    b = runtime.Batch()
    for a in insts:
        b.add(a, abi.minimiser("fire", dt_max=0.1, tol=1e-12, max_iter=iters, precision=precision))
    b.run(threads=256)
    st = runtime.last_run_stats()
    print(json.dumps({"profile_case": f"304 LJ clusters N=300 Fire(0.1) {precision}", "iterations": st["iterations"],
                      "pairs32": st["pairs32"], "pairs64": st["pairs64"],
                      "kernel_ms": st["kernel_ms"], "launches": st["launches"],
                      "phase_ms_summed_over_instances": st["phase_ms"]}))


def run_profile_cluster(iters):
    """One 512^2 three-fluid PhaseField grid (hard density, fixed volumes)
    on a thread-block cluster of 8 CTAs for `iters` L-BFGS iterations in FP32
    (profiler capture of the cluster batch kernel)."""
    from minim_gb300 import abi, runtime
    from tests.workloads import pf_simplex
    g = (512, 512, 1)
    inst = runtime.Instance(abi.phase_field(g, nfluid=3, volume_fixed=True), pf_simplex(g, 3, seed=5007))
    b = runtime.Batch()
    b.add(inst, abi.minimiser("lbfgs", tol=1e-7, max_iter=iters, precision="fp32"))
    r = b.run(threads=512, ctas=8)[0]
    st = runtime.last_run_stats()
    print(json.dumps({"profile_case": "PhaseField 512^2 three-fluid on a cluster of 8 CTAs", "iter": r.iter,
                      "kernel_ms": st["kernel_ms"], "abytes": st["abytes"]}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="minim_gb300")
    ap.add_argument("--batch", type=int, default=4096)
    ap.add_argument("--cpu-sample", type=int, default=64,
                    help="batched LJ instances run by the CPU oracle (stratified; 0 = skip)")
    ap.add_argument("--plain-sample", type=int, default=16)
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--serve", type=int, default=200, help="requests in the serving stream (0 = skip)")
    ap.add_argument("--serve-full", action="store_true", help="serving requests at the stated sizes")
    ap.add_argument("--serve-carried", type=int, default=100,
                    help="requests of the second stream, offered at half the measured throughput (0 = skip)")
    ap.add_argument("--mixed", type=int, default=96, help="instances in the mixed PF/BAH batch (0 = skip)")
    ap.add_argument("--mixed-grids", type=int, default=-1, help="PhaseField grids of the mixed batch")
    ap.add_argument("--mixed-sheets", type=int, default=-1, help="BarAndHinge sheets of the mixed batch")
    ap.add_argument("--mixed-full", action="store_true", help="mixed batch at the stated sizes")
    ap.add_argument("--mixed-max-iter", type=int, default=20000)
    ap.add_argument("--only", default="", help="comma list of sections to run without the headline "
                                                "(batched, mixed, serve, rows)")
    ap.add_argument("--serve-rate", type=float, default=2000.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--rows", type=int, default=1, help="1: also time Anneal and PhaseFieldUnstructured")
    ap.add_argument("--anneal", type=int, default=1024, help="LJ clusters in the Anneal batch")
    ap.add_argument("--pfu", type=int, default=64, help="grids in the PhaseFieldUnstructured batch")
    ap.add_argument("--cpu-budget", type=float, default=20.0)
    ap.add_argument("--profile", type=int, default=0,
                    help="run one short minimisation of N iterations (profiler capture) and exit")
    ap.add_argument("--profile-lj", type=int, default=0,
                    help="run one batch of 304 LJ clusters for N iterations (profiler capture) and exit")
    ap.add_argument("--profile-pf", type=int, default=0,
                    help="run one 128^2 three-fluid PhaseField grid for N iterations (profiler capture) and exit")
    ap.add_argument("--profile-prec", default="fp64", help="coordinate precision of --profile-pf")
    ap.add_argument("--profile-lj-prec", default="fp32", help="coordinate precision of --profile-lj")
    ap.add_argument("--profile-cluster", type=int, default=0,
                    help="run one 512^2 three-fluid grid on a cluster of 8 CTAs for N iterations and exit")
    args = ap.parse_args()
    if args.profile_pf:
        run_profile_pf(args.profile_pf, args.profile_prec)
        return
    if args.profile_cluster:
        run_profile_cluster(args.profile_cluster)
        return
    if args.profile:
        run_profile_case(args.profile)
        return
    if args.profile_lj:
        run_profile_lj(args.profile_lj, args.profile_lj_prec)
        return
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.only:
        # selected sections alone (no headline line): measurements at the
        # stated sizes that take longer than a default run should
        from minim_gb300 import runtime
        runtime.load()
        out = {"sections": args.only}
        for sec in args.only.split(","):
            if sec == "batched":
                out.update(run_batched(args))
            elif sec == "mixed":
                out.update(run_mixed(args))
            elif sec == "serve":
                out.update(run_serving(args))
            elif sec == "rows":
                out["rows"] = run_rows(args)
            else:
                raise SystemExit(f"unknown section {sec}")
        print(json.dumps(out))
        return
    if args.impl == "reference":
        if rank == 0:
            print(json.dumps(run_reference(args)))
        return
    if world > 1:
        # replicas: every rank runs its own copy of the workload on its GPU
        import torch
        import torch.distributed as dist
        dist.init_process_group("nccl")
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        args.no_cpu = rank != 0
        out = run_gpu(args)
        t = torch.tensor([out["ms_per_step"]], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        out["ms_per_step"] = float(t.item())
        out["value"] = world * 1e3 / out["ms_per_step"]
        out["n_gpus"] = world
        if rank == 0:
            print(json.dumps(out))
        dist.destroy_process_group()
        return
    print(json.dumps(run_gpu(args)))


if __name__ == "__main__":
    main()
