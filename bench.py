"""Benchmark: grid-point-steps/s of the 3D channel time step on GB300.

Workload: the single 128x128x65 channel (Re 180, dt 0.002, PI control to
U_bulk = 2/3, analytical perturbation amplitude 0.05, mode (2,1), 2/3 filter,
Crank-Nicolson), FP64 plain path.  A "step" is one pass of the reference's
time-loop body (DNS_pressure_BC_3D.f90:286-361 without IO).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

``value`` : device-timed throughput with the state resident in HBM (K graph
            replays bracketed by CUDA events on the library's stream).
``e2e``   : the same metric through the C-ABI with host-resident state: every
            step uploads u, v, w, p_total from pinned host memory, advances one
            step and downloads u, v, w, p_total and the diagnostics line.
With N > 1 (torchrun), every rank advances its own independent replica.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import signal
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

WORKLOAD = "channel_128x128x65_re180_pi"

# DRAM bytes of one launch of the dominant kernel (dram__bytes_read.sum +
# dram__bytes_write.sum), from one `ncu --set full --clock-control none`
# capture of that kernel on the same workload and build; --traffic overrides.
NCU_TRAFFIC = {
    ("channel_128x128x65_re180_pi", "viscous_helmholtz"): 154.447104e6 + 16.572160e6,
    ("channel_128x128x65_re180_pi", "viscous_helmholtz_tc"): 209.340416e6 + 17.577472e6,
}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
        return ws, rank, local, dist
    return 1, 0, local, None


def _barrier(dist):
    if dist is not None:
        import torch
        dist.barrier()
        torch.cuda.synchronize()


def _max_over_ranks(dist, x: float) -> float:
    """Slowest rank's value (NCCL groups reduce on the GPU, gloo on the CPU)."""
    if dist is None:
        return x
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(dist, world_size: int, points: int, steps: int, local_ms: float) -> tuple:
    """Whole-job point-steps/s of independent replicas: every rank advances its
    own run of `points` points for `steps` steps; the job takes as long as the
    slowest rank.  Returns (value, max_ms)."""
    ms = _max_over_ranks(dist, local_ms)
    return world_size * points * steps / (ms * 1e-3), ms


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int, log_dir: str | None = None):
        import tempfile
        self.index = index
        self.proc = None
        self.path = os.path.join(log_dir or tempfile.gettempdir(), f"dns3d_bench_clocks_rank{index}.csv")

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.fh, stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.send_signal(signal.SIGTERM)
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.fh.close()

    def summary(self) -> dict:
        try:
            rows = [r.split(",") for r in open(self.path).read().strip().splitlines() if r.strip()]
        except Exception:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
            except (ValueError, IndexError):
                continue
            for n, v in zip(names, r[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def algorithmic_flops(wl: dict) -> dict:
    """FP64 flops per step of the spectral-resident, parity-folded algorithm.

    Per complex mode column (Nm = (nx/2+1) ny columns per z-level) one nz x nz
    real operator costs, folded into its even/odd blocks (he = nz - nz/2,
    ho = nz/2): symmetric 4 (he^2 + ho^2) flops, antisymmetric 8 he ho flops.
    Per step: vorticity 2 antisymmetric (D.u, D.v); viscous 3 symmetric (the
    Helmholtz inverse of u, v, w; with Crank-Nicolson the explicit half is
    folded into the solve, see step.cu, so no D2 application remains);
    pressure 1 antisymmetric + 1 symmetric (D.w*, Poisson inverse);
    correction 1 antisymmetric (D.phi).
    Transforms: 9 real 2D FFTs per z-plane at 2.5 n log2 n flops (n = nx ny).
    """
    nx, ny, nz = wl["nx"], wl["ny"], wl["nz"]
    nm = (nx // 2 + 1) * ny
    ho = nz // 2
    he = nz - ho
    sym = 4.0 * (he * he + ho * ho) * nm
    anti = 8.0 * he * ho * nm
    n = nx * ny
    fft = 2.5 * n * math.log2(n) * nz
    out = {"vorticity": 2 * anti, "viscous_helmholtz": 3 * sym, "pressure_poisson": anti + sym,
           "pressure_correction": anti, "fft_total": 9 * fft}
    # the same solve with its FP64 products emulated on the tensor cores
    out["viscous_helmholtz_tc"] = out["viscous_helmholtz"]
    out["z_total"] = out["vorticity"] + out["viscous_helmholtz"] + out["pressure_poisson"] + out["pressure_correction"]
    out["total"] = out["z_total"] + out["fft_total"]
    return out


def cpu_sample(wl_name: str, steps: int, threads: int) -> dict:
    """Time the C/OpenMP restatement of the reference step (oracle/dns3d_cpu.c:
    physical-space transforms per plane, per-mode matrices rebuilt and
    LU-factored every call, as DNS_pressure_BC_3D.f90 does) on `steps` steps of
    the workload after one warm-up step, in a subprocess with `threads`
    OpenMP threads."""
    env = dict(os.environ, OMP_NUM_THREADS=str(threads))
    code = (
        "import json,sys,time; sys.path.insert(0, %r)\n"
        "from f90_dns_gb300.workloads import WORKLOADS\n"
        "from oracle import cpu_ref, dns3d_ref as ref\n"
        "wl = WORKLOADS[%r]\n"
        "names = set(ref.Config.__dataclass_fields__)\n"
        "cfg = ref.Config(**{k: v for k, v in wl.items() if k in names})\n"
        "c = cpu_ref.CpuChannel(cfg, threads=%d)\n"
        "c.step(1)\n"
        "t = time.perf_counter()\n"
        "c.step(%d)\n"
        "dt = time.perf_counter() - t\n"
        "print(json.dumps({'seconds': dt, 'threads': c.threads}))\n" % (ROOT, wl_name, threads, steps))
    res = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env, timeout=900)
    if res.returncode != 0:
        raise RuntimeError("cpu baseline failed: " + res.stderr[-2000:])
    out = json.loads(res.stdout.strip().splitlines()[-1])
    return {"seconds": out["seconds"], "steps": steps, "threads": out["threads"]}


CPU_SAMPLE_TEXT = ("C/OpenMP restatement of DNS_pressure_BC_3D.f90 (oracle/dns3d_cpu.c): per-plane r2c/c2r "
                   "round trips for every x/y derivative, per-mode Helmholtz and Poisson matrices rebuilt and "
                   "LU-factored with partial pivoting at every call as the reference's zgesv calls are; the Fortran "
                   "reference itself needs gfortran, FFTW3 and LAPACK, none of which exist on either machine")


def run_reference(args) -> None:
    """The reference arm: the C/OpenMP restatement of the reference algorithm
    timed on this host with one OpenMP thread per core (rank 0 only)."""
    if int(os.environ.get("RANK", "0")) != 0:
        return
    from f90_dns_gb300.workloads import WORKLOADS, point_count
    wl = WORKLOADS[args.workload]
    pts = point_count(wl)
    threads = os.cpu_count() or 1
    nsteps = max(3, int(round(args.ref_sample_frac * args.steps)))
    samp = cpu_sample(args.workload, nsteps, threads)
    threads = samp["threads"]
    value = pts * samp["steps"] / samp["seconds"]
    line = {
        "impl": "reference", "metric": "point-steps/s", "value": value, "unit": "point-steps/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * samp["seconds"] / samp["steps"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": args.workload, "grid": [wl["nx"], wl["ny"], wl["nz"]], "precision": "fp64"},
        "cpu_baseline": {"value": value, "unit": "point-steps/s", "cores": threads, "kind": "port",
                         "sample": f"{samp['steps']} steps of {args.workload} after 1 warm-up step, "
                                   f"{threads} threads: " + CPU_SAMPLE_TEXT},
        "e2e": {"value": value, "unit": "point-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def serving_leg(args, device: int) -> dict:
    """Serving stream: Poisson arrivals (mean `serve_rate` runs/s, seeded) of
    runs drawn as in the ensemble, 10% of them 256x256x97, each 200..2000
    steps, mixed precision, admitted by device footprint under 160 GiB."""
    import numpy as np
    from f90_dns_gb300 import Server, config_from
    from f90_dns_gb300.capi import PREC_MIXED
    from f90_dns_gb300.workloads import WORKLOADS, ensemble_draws, point_count
    rng = np.random.default_rng(args.seed + 1)
    draws = ensemble_draws(args.serve_requests, seed=args.seed + 2)
    big = WORKLOADS["channel_256x256x97_re180_dpdx"]
    reqs = []
    t = 0.0
    for d in draws:
        if rng.random() < 0.1:
            d = dict(big, re=d["re"], target_pressure_gradient=2.0 / d["re"],
                     perturbation_amplitude=d["perturbation_amplitude"],
                     analytical_mode_x=d["analytical_mode_x"], analytical_mode_y=d["analytical_mode_y"])
        t += float(rng.exponential(1.0 / args.serve_rate))
        reqs.append((t, d, int(rng.integers(200, 2001))))
    with Server(max_bytes=160 << 30, steps_per_round=args.serve_round, device=device) as srv:
        t0 = time.perf_counter()
        ids = []
        for at, d, n in reqs:
            dly = at - (time.perf_counter() - t0)
            if dly > 0:
                time.sleep(dly)
            ids.append(srv.submit(config_from(d, device=device, precision=PREC_MIXED), n))
        infos = [srv.wait(i, timeout=1800.0) for i in ids]
    lat = np.array([i.latency for i in infos])
    work = sum(point_count(d) * n for (_, d, n) in reqs)
    span = max(i.t_finish for i in infos) - min(i.t_submit for i in infos)
    return {"requests": len(reqs), "arrival_rate_per_s": args.serve_rate, "seed": args.seed + 1,
            "large_256x256x97": sum(1 for (_, d, _) in reqs if d["nx"] == 256),
            "completed": sum(1 for i in infos if i.status == 2),
            "p50_latency_s": float(np.percentile(lat, 50)), "p99_latency_s": float(np.percentile(lat, 99)),
            "aggregate_point_steps_per_s": work / span, "span_s": span,
            "precision": "mixed", "admission": "device footprint <= 160 GiB, FIFO",
            "steps_per_round": args.serve_round}


def run_ours(args) -> None:
    ws, rank, local, dist = _dist()
    from f90_dns_gb300 import ChannelDNS, build, config_from, footprint_bytes
    from f90_dns_gb300.capi import measure_fp64_tflops
    from f90_dns_gb300.workloads import WORKLOADS, point_count
    if not os.path.exists(os.path.join(ROOT, "f90_dns_gb300", "libdns3d_gpu.so")):
        build.build()
    wl = WORKLOADS[args.workload]
    pts = point_count(wl)
    if args.noise is not None:
        wl = dict(wl, noise_amplitude=args.noise)
    cfg = config_from(wl, device=local)
    d = ChannelDNS(cfg)
    d.step(args.warmup)
    d.synchronize()

    sampler = ClockSampler(local, args.clock_log)
    with sampler:
        _barrier(dist)
        ms = d.step_timed(args.steps)
        _barrier(dist)
    value, ms = replica_throughput(dist, ws, pts, args.steps, ms)
    clocks = sampler.summary()
    launches = d.launches_per_step() * args.steps

    # the mixed-precision form on the same workload, and its error against
    # FP64 after the same number of steps from the same initial condition
    mixed = None
    if args.mixed:
        from f90_dns_gb300.capi import PREC_MIXED
        dm = ChannelDNS(config_from(wl, device=local, precision=PREC_MIXED))
        dm.step(args.warmup)
        dm.synchronize()
        _barrier(dist)
        ms_m = dm.step_timed(args.steps)
        value_m, ms_m = replica_throughput(dist, ws, pts, args.steps, ms_m)
        prof_m = dm.profile_kernels(args.profile_steps)
        dm.close()
        # error: both forms from the initial condition for err_steps steps
        nerr = args.mixed_err_steps
        a = ChannelDNS(config_from(wl, device=local))
        b = ChannelDNS(config_from(wl, device=local, precision=PREC_MIXED))
        a.step(nerr)
        b.step(nerr)
        sa, sb = a.get_state(walls=False), b.get_state(walls=False)
        da, db = a.diagnostics(), b.diagnostics()
        a.close()
        b.close()
        import numpy as np
        scale = max(float(np.max(np.abs(sa[k]))) for k in ("u", "v", "w"))
        vel_err = max(float(np.max(np.abs(sa[k] - sb[k]))) for k in ("u", "v", "w")) / scale
        tot_m = sum(t for _, t in prof_m.values())
        mixed = {"value": value_m, "unit": "point-steps/s", "ms_per_step": ms_m / args.steps,
                 "speedup_vs_fp64": value_m / value, "dtype": "f32+f64",
                 "error_vs_fp64": {"steps": nerr, "max_rel_velocity": vel_err,
                                   "max_div_fp64": da.max_div, "max_div_mixed": db.max_div,
                                   "max_div_abs_diff": abs(da.max_div - db.max_div)},
                 "kernels": {k: {"launches": n, "avg_ms": t / n, "share": t / tot_m} for k, (n, t) in prof_m.items()}}

    # batched ensemble: seed-drawn runs of uneven grids, one ragged launch per stage
    ensemble = None
    if args.ensemble_runs > 0:
        from f90_dns_gb300 import Ensemble
        from f90_dns_gb300.capi import PREC_MIXED
        from f90_dns_gb300.workloads import ensemble_draws
        draws = ensemble_draws(args.ensemble_runs, seed=args.seed)
        res = {}
        for label, prec in (("mixed", PREC_MIXED), ("fp64", 0)):
            with Ensemble([config_from(d, device=local, precision=prec) for d in draws]) as ens:
                ens.step(args.warmup)
                _barrier(dist)
                ms_e = ens.step_timed(args.ensemble_steps)
                launches_e, ragged_e = ens.info()
                pts_e = sum(point_count(d) for d in draws)
                v_e, ms_e = replica_throughput(dist, ws, pts_e, args.ensemble_steps, ms_e)
                res[label] = {"value": v_e, "unit": "point-steps/s", "ms_per_step": ms_e / args.ensemble_steps,
                              "launches_per_step": launches_e, "ragged_runs": ragged_e}
        ensemble = {"runs": args.ensemble_runs, "seed": args.seed, "steps": args.ensemble_steps,
                    "points_per_step": sum(point_count(d) for d in draws),
                    "grids": sorted({f"{d['nx']}x{d['ny']}x{d['nz']}" for d in draws}),
                    "mixed": res["mixed"], "fp64": res["fp64"],
                    "mixed_speedup_vs_fp64": res["mixed"]["value"] / res["fp64"]["value"],
                    "launch": "one CUDA graph per step; each stage one ragged kernel launch over the runs of one "
                              "precision and kernel variant"}

    # serving: Poisson arrivals of seed-drawn runs, continuous batching
    serving = None
    if args.serve_requests > 0 and rank == 0:
        serving = serving_leg(args, local)

    # per-kernel device times (eager replay, events between launches)
    prof = d.profile_kernels(args.profile_steps)
    total_prof = sum(t for _, t in prof.values())
    flops = algorithmic_flops(wl)
    kernels = {k: {"launches": n, "avg_ms": t / n, "share": t / total_prof} for k, (n, t) in prof.items()}
    dom = max(kernels, key=lambda k: kernels[k]["avg_ms"] * kernels[k]["launches"])
    fp64_peak = measure_fp64_tflops(local)
    roofline = None
    if dom in flops:
        ach = flops[dom] / (kernels[dom]["avg_ms"] * 1e-3) / 1e12
        roofline = {"bound": "fp64", "kernel": dom, "achieved": ach, "peak": fp64_peak, "unit": "TFLOP/s",
                    "note": ("FP64-equivalent flops of the solve; its products run as exact FP16 digit-slice "
                             "MMAs on the tensor cores, so the kernel can exceed the FP64 pipe's rate")
                    if dom.endswith("_tc") else None,
                    "frac": ach / fp64_peak,
                    "traffic": args.traffic if args.traffic is not None else NCU_TRAFFIC.get((args.workload, dom)),
                    "traffic_source": "ncu capture of one launch (dram__bytes_read.sum + dram__bytes_write.sum)",
                    "peak_source": "FP64 FMA probe timed in this run (dns3d_measure_fp64_tflops); "
                                   "MEASURED_PEAKS.json has no FP64 figure",
                    "algorithmic_flops_per_launch": flops[dom]}
    step_roof = {"flops_per_step": flops["total"], "t_roof_ms": flops["total"] / (fp64_peak * 1e12) * 1e3,
                 "t_meas_ms": ms / args.steps,
                 "frac": (flops["total"] / (fp64_peak * 1e12) * 1e3) / (ms / args.steps),
                 "note": ("FP64-equivalent flops of the whole step against the FP64 FMA peak; the plane "
                          "transforms run in 64-bit fixed point on the integer pipes and the z-contractions as "
                          "exact digit-slice MMAs on the tensor cores, so the step can approach or pass 1")}

    # end-to-end through the C-ABI with host-resident state (pinned buffers)
    e2e = None
    if args.e2e_steps > 0:
        import numpy as np
        try:
            import torch
            pin = lambda: torch.empty(d.shape, dtype=torch.float64, pin_memory=True).numpy()
        except Exception:  # pragma: no cover
            pin = lambda: np.empty(d.shape)
        st = d.get_state(walls=False)
        bufs = {k: pin() for k in ("u", "v", "w", "p_total")}
        for k in bufs:
            bufs[k][...] = st[k]
        step0 = d.get_clock()[0]
        ndiv = 0
        _barrier(dist)
        t0 = time.perf_counter()
        for i in range(1, args.e2e_steps + 1):
            d.set_state(u=bufs["u"], v=bufs["v"], w=bufs["w"], p_total=bufs["p_total"])
            d.step(1)
            d.get_state_into(bufs["u"], bufs["v"], bufs["w"], bufs["p_total"])
            diag = d.output_diagnostics_3d()
            if (step0 + i) % 50 == 0:  # check_divergence_3d on the reference's schedule (3D:341-344)
                d.check_divergence_3d()
                ndiv += 1
        _barrier(dist)
        el = _max_over_ranks(dist, time.perf_counter() - t0)
        n = pts * 8
        e2e = {"value": ws * pts * args.e2e_steps / el, "unit": "point-steps/s",
               "h2d_bytes_per_step": 4 * n, "d2h_bytes_per_step": 4 * n + 8 * (16 + 6 * wl["nz"]),
               "steps": args.e2e_steps, "divergence_checks": ndiv,
               "path": "dns3d_set_state(u,v,w,p_total) from pinned host buffers + dns3d_step(1) + "
                       "dns3d_get_state into them + dns3d_output_diagnostics every step, dns3d_check_divergence "
                       "every 50th step (the reference loop with nwrt = 1, 3D:329-344)"}
        del diag

    cpu = None
    if rank == 0 and args.cpu_steps > 0:
        samp = cpu_sample(args.workload, args.cpu_steps, os.cpu_count() or 1)
        cpu = {"value": pts * samp["steps"] / samp["seconds"], "unit": "point-steps/s", "cores": samp["threads"],
               "kind": "port",
               "sample": f"{samp['steps']} steps of {args.workload} after 1 warm-up step, {samp['threads']} "
                         "threads: " + CPU_SAMPLE_TEXT}
    d.close()
    if rank == 0:
        line = {
            "metric": "point-steps/s", "value": value, "unit": "point-steps/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": args.workload, "grid": [wl["nx"], wl["ny"], wl["nz"]], "precision": "fp64",
                       "parallelism": "replicas" if ws > 1 else "single",
                       "l2": (f"device working set {footprint_bytes(cfg) / 1e9:.2f} GB (fields, per-mode inverses) "
                              + ("> 129 MB L2, re-read every step; no flush" if footprint_bytes(cfg) > 2 * 129e6
                                 else "fits in the 129 MB L2 (L2-resident timing; no flush)"))},
            "e2e": e2e, "gpu_launches": launches, "roofline": roofline, "step_roofline": step_roof,
            "kernels": kernels, "clocks": clocks, "cpu_baseline": cpu, "mixed": mixed, "ensemble": ensemble, "serving": serving,
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=WORKLOAD)
    ap.add_argument("--profile-steps", type=int, default=5)
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--cpu-steps", type=int, default=20)
    ap.add_argument("--ref-sample-frac", type=float, default=0.1,
                    help="reference arm: CPU steps timed per requested step (bounded sample, >= 3)")
    ap.add_argument("--no-mixed", dest="mixed", action="store_false",
                    help="skip the mixed-precision measurement")
    ap.add_argument("--mixed-err-steps", type=int, default=200)
    ap.add_argument("--ensemble-runs", type=int, default=64)
    ap.add_argument("--ensemble-steps", type=int, default=50)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--noise", type=float, default=None,
                    help="white-noise amplitude on the initial u, v, w (default: the workload's; the large "
                         "workload has 1e-3)")
    ap.add_argument("--serve-requests", type=int, default=32)
    ap.add_argument("--serve-rate", type=float, default=4.0)
    ap.add_argument("--serve-round", type=int, default=20)
    ap.add_argument("--clock-log", default=None,
                    help="directory for the nvidia-smi clock samples of the timed region (default: the temp dir)")
    ap.add_argument("--traffic", type=float, default=None,
                    help="ncu DRAM bytes per launch of the dominant kernel, if captured")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
