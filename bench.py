"""Benchmark: H54 energy+force evaluations per second on one GB300.

Workload (the metric's configuration): H54 as a bcc 3x3x3 lattice at rs 1.31
with N(0, 0.1 Bohr) displacements (seed 7, a new seed per step), gth-dzvp,
GGA-PBE, 81^3 grid (the reference's odd grid for the requested 80^3), Gamma
point; one step = SCF + adjoint forces + Ewald of one configuration through
the engine.  Inputs (positions) are resident in HBM before the timed region;
every step touches > 1 GB of grid data (AO values), more than the 129 MB L2,
so no flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--precision fp64|mixed]
  python bench.py --impl reference ...   (the CPU oracle, all host threads)

Prints one JSON line (rank 0).
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "H54 energy+force evals/s, mixed+batched vs FP64 plain @1e-6 Ha/atom"
UNIT = "evals/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="auto", choices=["auto", "fp64", "mixed"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    return ap.parse_args()


def workload(seed):
    from hqc_gb300.workloads import h54_bcc_pbe
    return h54_bcc_pbe(noise_seed=seed)


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait(timeout=5)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4)
                          if len(r) > 3 + k and r[3 + k].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.rows)}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d["hbm_gbs"], d["bf16_tflops"], "measured"
    return 6800.0, 1900.0, "fallback"


# algorithmic work of the dominant stages, per launch, for the roofline
def stage_work(stage, n, nao, N, precision):
    """(bound, algorithmic bytes or flops per launch) of a stage."""
    esize = 8 if precision == "fp64" else 4
    if stage == "density":
        # reads the AO grid once, writes rho (+ grad rho for GGA)
        return "hbm", nao * N * esize + 4 * N * 8
    if stage == "quadrature":
        return "hbm", 2 * nao * N * esize
    if stage == "fft":
        # 3 axis passes, complex read + write per pass
        return "hbm", 3 * 2 * 16 * N
    if stage in ("tc_density", "tc_quadrature"):
        return "tensor", 2.0 * N * nao * nao
    return None, None


def run_ours(args):
    import torch
    from hqc_gb300 import make_pes, _lib

    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    precision = "mixed" if args.precision == "auto" else args.precision
    w0 = workload(7)
    n, L, rs = w0["n"], w0["L"], w0["rs"]
    kw = dict(dft=True, xc=w0["xc"], grid_length=w0["grid_length"], tol=1e-7, max_cycle=100,
              precision=precision, forces=True)
    pes = make_pes(n, L, rs, w0["basis"], **kw)
    nao = pes.solver.plan.nao
    N = pes.solver.plan.ng ** 3
    # per-step configurations (different noise seeds), resident on the device
    total = args.warmup + args.steps
    xps = [torch.as_tensor(workload(1000 * rank + 7 + s)["xp"], device="cuda") for s in range(total)]
    iters = []

    def step(xp):
        E, g = pes.value_and_grad(xp)
        iters.append(pes.solver.iterations)
        return E, g

    for s in range(args.warmup):
        step(xps[s])
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    _lib.profile(1)
    _lib.load().hqcgb_launch_count(1)
    start = torch.cuda.Event(enable_timing=True)
    stop = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        start.record()
        for s in range(args.steps):
            E, g = step(xps[args.warmup + s])
        stop.record()
        torch.cuda.synchronize()
    ms = start.elapsed_time(stop)
    launches = int(_lib.load().hqcgb_launch_count(0))
    stats = _lib.stage_stats()
    _lib.profile(0)
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    value = world * args.steps / (ms / 1000.0)

    # roofline of the dominant stage
    hbm, bf16, src = peaks()
    dom = max((k for k in stats if stage_work(k, n, nao, N, precision)[0]), key=lambda k: stats[k][1])
    bound, work = stage_work(dom, n, nao, N, precision)
    cnt, tot_ms = stats[dom]
    avg_s = tot_ms / max(cnt, 1) / 1000.0
    if bound == "hbm":
        achieved = work / avg_s / 1e9
        roof = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                "frac": achieved / hbm, "traffic": None, "kernel": dom,
                "peak_source": f"{src} (MEASURED_PEAKS.json hbm_gbs)" if src == "measured" else src,
                "launches": cnt, "avg_ms": tot_ms / max(cnt, 1)}
    else:
        achieved = work / avg_s / 1e12
        roof = {"bound": "tensor", "achieved": achieved, "peak": bf16, "unit": "TFLOP/s",
                "frac": achieved / bf16, "traffic": None, "kernel": dom, "launches": cnt,
                "avg_ms": tot_ms / max(cnt, 1)}
    stage_ms = {k: round(v[1] / args.steps, 3) for k, v in stats.items() if v[0]}

    # end to end through the public API: host positions in, host E and forces out
    e2e = None
    if not args.no_e2e:
        xh = [np.ascontiguousarray(workload(1000 * rank + 500 + s)["xp"]) for s in range(args.steps)]
        pes.value_and_grad(xh[0])
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for s in range(args.steps):
            E, g = pes.value_and_grad(xh[s])
            _ = float(E), g.cpu().numpy()
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        e2e = {"value": args.steps / dt, "unit": UNIT, "h2d_bytes_per_step": n * 3 * 8,
               "d2h_bytes_per_step": 8 + n * 3 * 8}

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64" if precision == "fp64" else "tf32x3+f64",
            "data": "synthetic (bcc H54 + seeded N(0,0.1 Bohr) noise, new seed per step)",
            "config": {"workload": "H54 bcc rs=1.31 gth-dzvp PBE 81^3 Gamma, SCF tol 1e-7 Ry + forces",
                       "precision_path": precision, "batch": 1, "n_ao": nao, "grid": N,
                       "scf_iterations_mean": float(np.mean(iters[args.warmup:])),
                       "l2": "inputs > L2 (1.15 GB AO grid per step), no flush",
                       "parallelism": f"replicas x{world}"},
            "roofline": roof, "stage_ms_per_step": stage_ms, "e2e": e2e,
            "gpu_launches": launches, "clocks": clk.summary()}
    if rank == 0 and not args.no_cpu_baseline and world == 1:
        line["cpu_baseline"] = cpu_baseline(iters_per_eval=float(np.mean(iters)))
    if world > 1:
        torch.distributed.destroy_process_group()
    return line if rank == 0 else None


def cpu_baseline(iters_per_eval, budget_s=25.0):
    """The NumPy oracle on the host cores on a bounded sample of the workload:
    the AO grid (values and gradients) of one configuration plus Fock builds
    (density, gradient, Hartree FFT Poisson, PBE, quadrature) until the
    budget is used; one eval is extrapolated as the AO grid + (iterations + 3)
    Fock builds (the force pass costs about three builds)."""
    from oracle.gpw import Solver
    w = workload(7)
    xp = w.pop("xp") * w["rs"]
    s = Solver(w["n"], w["L"], w["rs"], w["basis"], dft=True, xc=w["xc"],
               grid_length=w["grid_length"], tol=1e-7)
    t0 = time.perf_counter()
    phi, grad, _ = s.st.ao_grid(xp, deriv=1)
    t1 = time.perf_counter()
    D = np.eye(s.st.nao) * (w["n"] / s.st.nao)
    nb = 0
    while nb < 1 or (nb < 3 and time.perf_counter() - t1 < budget_s):
        rho = s.density(D, phi)[0]
        s.hartree(rho, phi)
        s.xc_terms(D, phi, grad)
        nb += 1
    t2 = time.perf_counter()
    per_build = (t2 - t1) / nb
    t_eval = (t1 - t0) + per_build * (iters_per_eval + 3)
    cores = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()
    return {"value": 1.0 / t_eval, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"oracle AO grid {t1 - t0:.1f}s + {nb} Fock builds ({per_build:.2f}s each), "
                      f"extrapolated to {iters_per_eval:.0f} iterations + forces"}


def run_reference(args):
    rank, world, _ = dist_info()
    if rank != 0:
        return None
    from oracle.gpw import Solver  # noqa: F401  (the reference restatement; jax is absent)
    vals = []
    for _ in range(args.warmup + args.steps):
        cb = cpu_baseline(iters_per_eval=19.0, budget_s=20.0)
        vals.append(cb["value"])
    v = float(np.mean(vals[args.warmup:])) if args.steps else float(vals[-1])
    cb["value"] = v
    return {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": 0, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 / v, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "impl": "reference",
            "data": "synthetic", "config": {"workload": "H54 bcc rs=1.31 gth-dzvp PBE 81^3 Gamma"},
            "cpu_baseline": cb,
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "reference is JAX (not installable here, no network); timed its NumPy FP64 "
                    "restatement (oracle/) on the host cores"}


def main():
    args = parse()
    line = run_reference(args) if args.impl == "reference" else run_ours(args)
    if line is not None:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
