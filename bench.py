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
instances minimised one at a time with the whole GPU (a sample).

Also reported (key "rows"): Anneal on a batch of LJ clusters and
PhaseFieldUnstructured on a batch of three-fluid grids, each against the CPU
oracle on a sample.

--impl reference times the CPU restatement of the reference algorithm
(oracle/, or the reference library itself when it was built on this host)
on a bounded sample of the same workload.
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
# 24.20 GB against the kernels' own count of 21.52 GB
# (profiles/stepped_graph_pf1_192cubed.md).  Traffic per step = this ratio x
# the step's algorithmic bytes.
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
                   "oracle_rms_at_x": rms_chk},
        "e2e": {"value": e2e_value, "unit": "minimisations/s",
                "h2d_bytes_per_step": int(x0.size * 8), "d2h_bytes_per_step": int(x0.size * 8)},
        "gpu_launches": int(launches), "roofline": roofline, "clocks": clk,
        "wall_s_timed": t1 - t0,
    }
    if not args.no_batched:
        out.update(run_batched(args))
    if args.mixed > 0:
        out.update(run_mixed(args))
    if args.serve > 0:
        out.update(run_serving(args))
    if args.rows:
        out["rows"] = run_rows(args)
    if not args.no_cpu:
        out["cpu_baseline"] = cpu_baseline(results[-1].iter, budget_s=args.cpu_budget)
    return out


def run_batched(args):
    from minim_gb300 import abi, runtime
    p, items = lj_batch_setup(args.batch)
    insts = [runtime.Instance(p, x0) for x0, _ in items]
    b = runtime.Batch()
    for inst, (_, mp) in zip(insts, items):
        b.add(inst, mp)
    # warm-up: a short batch of both methods (module load, workspace pool)
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
    batched = len(items) / (st["kernel_ms"] / 1e3)
    # plain: the same instances one at a time on the whole GPU (sample)
    rng = np.random.default_rng(0)
    idx = rng.choice(len(items), size=min(args.plain_sample, len(items)), replace=False)
    plain_ms = 0.0
    for i in idx:
        inst = runtime.Instance(p, items[i][0])
        inst.minimise(items[i][1])
        plain_ms += runtime.last_run_stats()["kernel_ms"]
    plain = len(idx) / (plain_ms / 1e3)
    flops32 = st["pairs32"] * 20
    return {
        "batched": {"value": batched, "unit": "minimisations/s", "instances": len(items),
                    "converged": int(conv), "kernel_ms": st["kernel_ms"],
                    "fp32_tflops": flops32 / (st["kernel_ms"] / 1e3) / 1e12,
                    "workload": f"{len(items)} LJ clusters N~U{{13..400}}, half Fire(0.1) half Lbfgs(m=5), "
                                f"RMS<1e-6"},
        "plain": {"value": plain, "unit": "minimisations/s", "sample": int(len(idx))},
        "batched_vs_plain": batched / plain,
    }


def run_mixed(args):
    """One batch launch of mixed phase-field and mesh instances: 2-D
    three-fluid PhaseField grids (hard density constraint, fixed volumes,
    random simplex start) and BarAndHinge sheets (flat jittered rest shape,
    Gaussian out-of-plane start), all Lbfgs to RMS < 1e-7.  Sizes are capped
    (grids 64^2 / 128^2, sheets 32^2 .. 64^2 vertices) so that the launch runs
    in seconds."""
    from minim_gb300 import abi, runtime
    from tests.workloads import Rng, pf_simplex, sheet
    rng = Rng(11)
    npf, nbah = (2 * args.mixed) // 3, args.mixed - (2 * args.mixed) // 3
    u = rng.uniform(npf + nbah)
    insts, items = [], []
    for i in range(npf):
        side = 64 if u[i] < 0.5 else 128
        grid = (side, side, 1)
        p = abi.phase_field(grid, nfluid=3, volume_fixed=True)
        insts.append(runtime.Instance(p, pf_simplex(grid, 3, seed=5000 + i)))
        items.append(("pf", abi.minimiser("lbfgs", tol=1e-7, max_iter=20000)))
    for i in range(nbah):
        k = 32 + int(u[npf + i] * 33)
        flat, tris, pert = sheet(k, seed=6000 + i)
        inst = runtime.Instance(abi.bar_and_hinge(triangulation=tris, rigidity=(1, 0.01)), flat)
        inst.coords = pert
        insts.append(inst)
        items.append(("bah", abi.minimiser("lbfgs", tol=1e-7, max_iter=20000)))
    b = runtime.Batch()
    for inst, (_, mp) in zip(insts, items):
        b.add(inst, mp)
    res = b.run()
    st = runtime.last_run_stats()
    conv = sum(r.status == abi.RES_CONVERGED for r in res)
    return {"mixed_batch": {"value": conv / (st["kernel_ms"] / 1e3), "unit": "converged minimisations/s",
                            "instances": len(items), "converged": int(conv), "kernel_ms": st["kernel_ms"],
                            "workload": f"{npf} 2-D ternary PhaseField grids (64^2/128^2, fixed volume) + "
                                        f"{nbah} BarAndHinge sheets (1k-4.2k vertices), Lbfgs RMS<1e-7"}}


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


def serving_requests(count, rate, seed=7):
    """A seeded Poisson stream of mixed requests shaped like the serving
    workload (LjNd clusters, 2-D / 3-D PhaseField grids with and without solid
    spheres, BarAndHinge sheets), with sizes capped so that the whole stream
    runs in seconds: LJ N log-uniform in [13, 400], PF sides 64-128 (2-D) or
    24-48 (3-D), sheets of 32^2 .. 48^2 vertices."""
    from minim_gb300 import abi, runtime
    from tests.workloads import Rng, lj_cluster, pf_noise, sheet
    rng = Rng(seed)
    u = rng.uniform(6 * count).reshape(count, 6)
    t = np.cumsum(-np.log(1.0 - u[:, 0]) / rate)
    reqs = []
    for i in range(count):
        kind = int(u[i, 1] * 3)
        if kind == 0:
            n = int(np.exp(np.log(13) + u[i, 2] * (np.log(400) - np.log(13))))
            reqs.append((t[i], "lj", abi.lj(), lj_cluster(n, seed=1000 + i), abi.minimiser("lbfgs", m=5, tol=1e-6)))
        elif kind == 1:
            if u[i, 3] < 0.5:
                side = 64 + int(u[i, 4] * 65)
                grid = (side, side, 1)
            else:
                side = 24 + int(u[i, 4] * 25)
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
            k = 32 + int(u[i, 2] * 17)
            flat, tris, pert = sheet(k, seed=4000 + i)
            p0 = abi.bar_and_hinge(triangulation=tris, rigidity=(1, 0.01))
            _, bpar, _, hpar = runtime.bah_elements(p0, flat)
            p = abi.bar_and_hinge(triangulation=tris, rigidity=(1, 0.01), length0=bpar[:, 1].copy(),
                                  theta0=hpar[:, 1].copy())
            reqs.append((t[i], "bah", p, pert, abi.minimiser("lbfgs", m=5, tol=1e-7)))
    return reqs


def run_serving(args):
    """Continuous batching under a Poisson arrival stream: requests are
    submitted when their arrival time has passed, the server admits them as
    slots and memory free up, and latency is completion minus arrival."""
    from minim_gb300 import abi, runtime
    reqs = serving_requests(args.serve, args.serve_rate)
    srv = runtime.Server()
    # warm-up: a few requests of each kind
    for _, _, p, x0, mp in reqs[:6]:
        srv.submit(p, x0, mp)
    while srv.ndof:
        srv.step()
        for rid, _ in srv.poll():
            srv.take(rid)
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
    lat = np.array([1e3 * (done_t[r] - arrival[r]) for r in done_t])
    conv = sum(1 for r in status.values() if r == abi.RES_CONVERGED)
    srv.close()
    return {"serving": {"value": conv / wall, "unit": "converged minimisations/s", "requests": len(reqs),
                        "converged": conv, "wall_s": wall, "p50_ms": float(np.percentile(lat, 50)),
                        "p99_ms": float(np.percentile(lat, 99)), "arrival_rate": args.serve_rate,
                        "workload": "Poisson stream of LJ (N 13-400), 2-D/3-D PhaseField (half with 20% solid "
                                    "spheres) and BarAndHinge sheets (1k-2.3k vertices), Lbfgs"}}


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
    cb = cpu_baseline(args.ref_iters_hint, budget_s=args.cpu_budget)
    return {"metric": METRIC, "value": cb["value"], "unit": cb["unit"], "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 / cb["value"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp64",
            "data": "synthetic (seeded noise field)", "impl": "reference",
            "config": {"workload": "PhaseField binary 192^3 periodic, Lbfgs m=10, RMS<1e-7"},
            "cpu_baseline": cb,
            "e2e": {"value": cb["value"], "unit": cb["unit"], "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}


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


def run_profile_lj(iters):
    """One batch launch of 304 Lennard-Jones clusters (N=300, Fire(0.1), FP32
    coordinates, `iters` iterations each) for profiler captures of the batched
    kernel."""
    from minim_gb300 import abi, runtime
    from tests.workloads import lj_cluster
    insts = [runtime.Instance(abi.lj(), lj_cluster(300, seed=i)) for i in range(304)]
    b = runtime.Batch()
    for a in insts:
        b.add(a, abi.minimiser("fire", dt_max=0.1, tol=1e-12, max_iter=iters, precision="fp32"))
    b.run(threads=256)
    st = runtime.last_run_stats()
    print(json.dumps({"profile_case": "304 LJ clusters N=300 Fire(0.1) fp32", "iterations": st["iterations"],
                      "kernel_ms": st["kernel_ms"], "launches": st["launches"]}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="minim_gb300")
    ap.add_argument("--batch", type=int, default=1024)
    ap.add_argument("--plain-sample", type=int, default=16)
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--serve", type=int, default=200, help="requests in the serving stream (0 = skip)")
    ap.add_argument("--mixed", type=int, default=96, help="instances in the mixed PF/BAH batch (0 = skip)")
    ap.add_argument("--serve-rate", type=float, default=2000.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--rows", type=int, default=1, help="1: also time Anneal and PhaseFieldUnstructured")
    ap.add_argument("--anneal", type=int, default=1024, help="LJ clusters in the Anneal batch")
    ap.add_argument("--pfu", type=int, default=64, help="grids in the PhaseFieldUnstructured batch")
    ap.add_argument("--cpu-budget", type=float, default=20.0)
    ap.add_argument("--ref-iters-hint", type=int, default=985,
                    help="iterations of a full minimisation (the GPU run of the same algorithm needs 981-987)")
    ap.add_argument("--profile", type=int, default=0,
                    help="run one short minimisation of N iterations (profiler capture) and exit")
    ap.add_argument("--profile-lj", type=int, default=0,
                    help="run one batch of 304 LJ clusters for N iterations (profiler capture) and exit")
    ap.add_argument("--profile-pf", type=int, default=0,
                    help="run one 128^2 three-fluid PhaseField grid for N iterations (profiler capture) and exit")
    ap.add_argument("--profile-prec", default="fp64", help="coordinate precision of --profile-pf")
    args = ap.parse_args()
    if args.profile_pf:
        run_profile_pf(args.profile_pf, args.profile_prec)
        return
    if args.profile:
        run_profile_case(args.profile)
        return
    if args.profile_lj:
        run_profile_lj(args.profile_lj)
        return
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
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
