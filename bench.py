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
    ("channel_128x128x65_re180_pi", "viscous_helmholtz_tc"): 257.373952e6 + 18.197248e6,
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


def algorithmic_bytes(wl: dict) -> dict:
    """Compulsory DRAM bytes per launch of each profiled kernel of the FP64
    step (spectral-resident algorithm): every field the kernel must read and
    write once, plus the per-mode operators it applies.  One spectral field
    S = (nx/2+1) ny nz complex128 values, one physical field R = nx ny nz
    float64 values, one per-mode inverse set Inv = nq (he^2 + ho^2) float64
    values (nq = (ny/2+1)(nx/2+1) distinct k^2, folded even/odd blocks).
      vorticity: u, v, w -> omega (6 S);
      inverse y pass: 3 fields per launch, spectrum in and out (6 S);
      c2r x pass: 3 fields per launch (3 S + 3 R);
      products: 6 R in, 3 R out;  r2c x pass: 3 R in, 3 S out;
      forward y pass: the kx <= kx_max columns of 3 fields, in and out;
      viscous: u, v, w, su, sv, sw in, u*, v*, w* out (9 S) + Helmholtz Inv;
      pressure: u*, v*, w* in, phi out, phi in and out (6 S) + Poisson Inv;
      projection: phi, u*, v*, w*, p in, u, v, w, p out (9 S)."""
    nx, ny, nz = wl["nx"], wl["ny"], wl["nz"]
    nxhp = nx // 2 + 1
    S = nxhp * ny * nz * 16.0
    R = nx * ny * nz * 8.0
    ho = nz // 2
    he = nz - ho
    inv = (ny // 2 + 1) * nxhp * (he * he + ho * ho) * 8.0
    kxm = ((nx // 2) * 2) // 3 if wl.get("use_dealias_23_rule", True) else nxhp - 1
    fwd = 6 * S * min(kxm + 1, nxhp) / nxhp
    b = {"vorticity": 6 * S, "fft_y_inverse": 6 * S, "fft_x_c2r": 3 * S + 3 * R, "products": 9 * R,
         "fft_x_r2c": 3 * R + 3 * S, "fft_y_forward": fwd, "viscous_helmholtz": 9 * S + inv,
         "pressure_poisson": 6 * S + inv, "pressure_correction": 9 * S, "pi_update": nz * 16.0 + 64.0}
    for k in ("vorticity", "viscous_helmholtz", "pressure_poisson", "pressure_correction"):
        b[k + "_tc"] = b[k]
    return b


def measured_peaks() -> dict:
    """HBM copy bandwidth and bf16 tensor throughput measured on this machine's
    GB300s (MEASURED_PEAKS.json beside this file), else the published
    fallback of one earlier GB300 measurement."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return {"hbm_gbs": float(d["hbm_gbs"]), "bf16_tflops": float(d["bf16_tflops"]), "source": "measured"}
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "source": "fallback"}


def working_set_note(wl: dict) -> str:
    """L2 statement of the timed region, from the grid alone (the same text in
    both arms): the FP64 step re-reads its spectral state, work fields and
    per-mode inverses every step."""
    ab = algorithmic_bytes(wl)
    # the inverse passes run as two 3-field launches per step
    per_step = sum(v for k, v in ab.items() if not k.endswith("_tc")) + ab["fft_y_inverse"] + ab["fft_x_c2r"]
    return (f"each step moves >= {per_step / 1e6:.0f} MB of state, work fields and per-mode inverses "
            + ("> 129 MB L2, re-read every step; no flush" if per_step > 2 * 129e6
               else "(L2-resident timing; no flush)"))


def bench_config(wl_name: str, wl: dict, world_size: int) -> dict:
    return {"workload": wl_name, "grid": [wl["nx"], wl["ny"], wl["nz"]], "precision": "fp64",
            "parallelism": "replicas" if world_size > 1 else "single", "l2": working_set_note(wl)}


def cpu_sample(wl_name: str, steps: int, threads: int, warmup: int = 1) -> dict:
    """Time the C/OpenMP restatement of the reference step (oracle/dns3d_cpu.c:
    physical-space transforms per plane, per-mode matrices rebuilt and
    LU-factored every call, as DNS_pressure_BC_3D.f90 does) on `steps` steps of
    the workload after `warmup` untimed steps, in a subprocess with `threads`
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
        "c.step(%d)\n"
        "t = time.perf_counter()\n"
        "c.step(%d)\n"
        "dt = time.perf_counter() - t\n"
        "print(json.dumps({'seconds': dt, 'threads': c.threads}))\n" % (ROOT, wl_name, threads, warmup, steps))
    res = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env, timeout=900)
    if res.returncode != 0:
        raise RuntimeError("cpu baseline failed: " + res.stderr[-2000:])
    out = json.loads(res.stdout.strip().splitlines()[-1])
    return {"seconds": out["seconds"], "steps": steps, "warmup": warmup, "threads": out["threads"]}


CPU_SAMPLE_TEXT = ("C/OpenMP restatement of DNS_pressure_BC_3D.f90 (oracle/dns3d_cpu.c): per-plane r2c/c2r "
                   "round trips for every x/y derivative, per-mode Helmholtz and Poisson matrices rebuilt and "
                   "LU-factored with partial pivoting at every call as the reference's zgesv calls are; the Fortran "
                   "reference itself needs gfortran, FFTW3 and LAPACK, none of which exist on either machine")


def run_reference(args) -> None:
    """The reference arm: the C/OpenMP restatement of the reference algorithm
    timed on this host with one OpenMP thread per core (rank 0 only), on the
    same workload, metric and config as the GPU arm.  It times exactly the
    requested steps after the requested warm-up steps, unless that would take
    longer than --ref-budget seconds; then it times fewer and its line says how
    many it timed."""
    if int(os.environ.get("RANK", "0")) != 0:
        return
    from f90_dns_gb300.workloads import WORKLOADS, point_count
    wl = WORKLOADS[args.workload]
    pts = point_count(wl)
    threads = os.cpu_count() or 1
    probe = cpu_sample(args.workload, 1, threads, warmup=0)
    per_step = probe["seconds"]
    fit = max(1, int(args.ref_budget / max(per_step, 1e-9)))
    warm = min(args.warmup, max(0, fit // 4))
    nsteps = min(args.steps, max(1, fit - warm))
    samp = cpu_sample(args.workload, nsteps, threads, warmup=warm)
    threads = samp["threads"]
    value = pts * samp["steps"] / samp["seconds"]
    line = {
        "impl": "reference", "metric": "point-steps/s", "value": value, "unit": "point-steps/s",
        "n_gpus": args.gpus, "steps": samp["steps"], "warmup": samp["warmup"],
        "requested_steps": args.steps, "requested_warmup": args.warmup,
        "ms_per_step": 1e3 * samp["seconds"] / samp["steps"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": bench_config(args.workload, wl, int(os.environ.get("WORLD_SIZE", "1"))),
        "cpu_baseline": {"value": value, "unit": "point-steps/s", "cores": threads, "kind": "port",
                         "sample": f"{samp['steps']} steps of {args.workload} after {samp['warmup']} warm-up "
                                   f"steps, {threads} threads: " + CPU_SAMPLE_TEXT},
        "e2e": {"value": value, "unit": "point-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# per-launch DRAM traffic (ncu dram__bytes_read.sum + dram__bytes_write.sum)
# and tensor-pipe activity of the tensor-core kernels, from one capture each
NCU_TENSOR_PIPE = {
    ("channel_128x128x65_re180_pi", "viscous_helmholtz_tc"): 12.6,
}


def kernel_rooflines(wl, prof, step_ms, peaks, wl_name, traffic_override=None):
    """Per-kernel achieved HBM GB/s on algorithmic bytes (algorithmic_bytes)
    against the measured copy bandwidth; the dominant kernel's entry is the
    line's `roofline`; the whole step's algorithmic bytes against the same
    peak is `step_roofline`."""
    ab = algorithmic_bytes(wl)
    total = sum(t for _, t in prof.values())
    kernels = {}
    for k, (n, t) in prof.items():
        e = {"launches": n, "avg_ms": t / n, "share": t / total}
        if k in ab:
            gbs = ab[k] / (t / n * 1e-3) / 1e9
            e.update(algorithmic_bytes=ab[k], achieved_gbs=gbs, hbm_frac=gbs / peaks["hbm_gbs"])
        kernels[k] = e
    dom = max(kernels, key=lambda k: kernels[k]["avg_ms"] * kernels[k]["launches"])
    roofline = None
    if "achieved_gbs" in kernels[dom]:
        kd = kernels[dom]
        roofline = {"bound": "hbm", "kernel": dom, "achieved": kd["achieved_gbs"], "peak": peaks["hbm_gbs"],
                    "unit": "GB/s", "frac": kd["hbm_frac"],
                    "traffic": traffic_override if traffic_override is not None else NCU_TRAFFIC.get((wl_name, dom)),
                    "algorithmic_bytes_per_launch": kd["algorithmic_bytes"],
                    "peak_source": f"MEASURED_PEAKS.json hbm_gbs ({peaks['source']})",
                    "traffic_source": "ncu capture of one launch (dram__bytes_read.sum + dram__bytes_write.sum)",
                    "tensor_pipe_pct": NCU_TENSOR_PIPE.get((wl_name, dom))}
    per_step = sum(ab[k] * n / max(1, args_steps(prof)) for k, (n, _) in prof.items() if k in ab)
    t_roof = per_step / (peaks["hbm_gbs"] * 1e9) * 1e3
    step_roof = {"bound": "hbm", "bytes_per_step": per_step, "t_roof_ms": t_roof, "t_meas_ms": step_ms,
                 "frac": t_roof / step_ms, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                 "note": "algorithmic DRAM bytes of every kernel of one step against the measured copy bandwidth"}
    return kernels, roofline, step_roof


def args_steps(prof) -> int:
    """Profiled steps: launches of the once-per-step PI update (or of the
    viscous stage)."""
    for k in ("pi_update", "viscous_helmholtz_tc", "viscous_helmholtz", "viscous_mixed"):
        if k in prof:
            return prof[k][0]
    return 1


def large_leg(args, device: int, peaks: dict) -> dict:
    """The largest single run (512x384x129, Re 180, dt 0.001, PI control,
    amplitude 0.08, mode (2,2), white noise 1e-3): FP64 and mixed step
    throughput, per-kernel profile and the mixed form's error against FP64
    after the timed steps."""
    import numpy as np
    from f90_dns_gb300 import ChannelDNS, config_from
    from f90_dns_gb300.capi import PREC_MIXED
    from f90_dns_gb300.workloads import WORKLOADS, point_count
    name = "channel_512x384x129_re180_pi"
    wl = WORKLOADS[name]
    pts = point_count(wl)
    out = {"workload": name, "grid": [wl["nx"], wl["ny"], wl["nz"]], "steps": args.large_steps}
    states = {}
    for label, prec in (("fp64", 0), ("mixed", PREC_MIXED)):
        with ChannelDNS(config_from(wl, device=device, precision=prec)) as d:
            d.step(args.warmup)
            d.synchronize()
            ms = d.step_timed(args.large_steps)
            prof = d.profile_kernels(2)
            st = d.get_state(walls=False)
            states[label] = st
            e = {"value": pts * args.large_steps / (ms * 1e-3), "unit": "point-steps/s",
                 "ms_per_step": ms / args.large_steps}
            if prec == 0:
                kern, roof, sroof = kernel_rooflines(wl, prof, ms / args.large_steps, peaks, name)
                e.update(kernels=kern, roofline=roof, step_roofline=sroof)
            else:
                tot = sum(t for _, t in prof.values())
                e["kernels"] = {k: {"launches": n, "avg_ms": t / n, "share": t / tot} for k, (n, t) in prof.items()}
            out[label] = e
    a, b = states["fp64"], states["mixed"]
    scale = max(float(np.max(np.abs(a[k]))) for k in ("u", "v", "w"))
    out["mixed"]["speedup_vs_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
    out["mixed"]["error_vs_fp64"] = {"steps": args.warmup + args.large_steps + 2,
                                     "max_rel_velocity": max(float(np.max(np.abs(a[k] - b[k])))
                                                             for k in ("u", "v", "w")) / scale}
    return out


def serving_requests(args) -> list:
    """The seeded request stream: Poisson arrivals (mean `serve_rate` runs/s)
    of runs drawn as in the ensemble, 10% of them 256x256x97, each 200..2000
    steps."""
    import numpy as np
    from f90_dns_gb300.workloads import WORKLOADS, ensemble_draws
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
    return reqs


def serve(args, device: int, reqs: list, burst: bool) -> dict:
    """Submits `reqs` to a Server (at their arrival times, or all at once for
    a burst), mixed precision, admitted by device footprint under 160 GiB;
    latency percentiles and the aggregate point-steps/s over the span."""
    import numpy as np
    from f90_dns_gb300 import Server, config_from
    from f90_dns_gb300.capi import PREC_MIXED
    from f90_dns_gb300.workloads import point_count
    with Server(max_bytes=160 << 30, steps_per_round=args.serve_round, device=device) as srv:
        t0 = time.perf_counter()
        ids = []
        for at, d, n in reqs:
            dly = 0.0 if burst else at - (time.perf_counter() - t0)
            if dly > 0:
                time.sleep(dly)
            ids.append(srv.submit(config_from(d, device=device, precision=PREC_MIXED), n))
        infos = [srv.wait(i, timeout=1800.0) for i in ids]
    lat = np.array([i.latency for i in infos])
    work = sum(point_count(d) * n for (_, d, n) in reqs)
    span = max(i.t_finish for i in infos) - min(i.t_submit for i in infos)
    return {"completed": sum(1 for i in infos if i.status == 2),
            "p50_latency_s": float(np.percentile(lat, 50)), "p99_latency_s": float(np.percentile(lat, 99)),
            "aggregate_point_steps_per_s": work / span, "span_s": span}


def serving_leg(args, device: int) -> dict:
    """Serving: the seeded Poisson stream (latency under the stated arrival
    rate; its aggregate is bounded by the arrivals), then the same requests
    submitted at once (the server's capacity: continuous batching with every
    run resident)."""
    reqs = serving_requests(args)
    out = {"requests": len(reqs), "arrival_rate_per_s": args.serve_rate, "seed": args.seed + 1,
           "large_256x256x97": sum(1 for (_, d, _) in reqs if d["nx"] == 256),
           "precision": "mixed", "admission": "device footprint <= 160 GiB, FIFO",
           "steps_per_round": args.serve_round}
    out.update(serve(args, device, reqs, burst=False))
    out["burst"] = serve(args, device, reqs, burst=True)
    return out


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
        ra, rb = a.projection_residual(), b.projection_residual()
        a.close()
        b.close()
        import numpy as np
        scale = max(float(np.max(np.abs(sa[k]))) for k in ("u", "v", "w"))
        vel_err = max(float(np.max(np.abs(sa[k] - sb[k]))) for k in ("u", "v", "w")) / scale
        # the same mixed form with one refinement step of every Poisson solve
        dr = ChannelDNS(config_from(wl, device=local, precision=PREC_MIXED, poisson_refinement=1))
        dr.step(args.warmup)
        dr.synchronize()
        ms_r = dr.step_timed(args.steps)
        dr.close()
        c = ChannelDNS(config_from(wl, device=local, precision=PREC_MIXED, poisson_refinement=1))
        c.step(nerr)
        sc_ = c.get_state(walls=False)
        rc_ = c.projection_residual()
        c.close()
        refined = {"value": pts * args.steps / (ms_r * 1e-3), "ms_per_step": ms_r / args.steps,
                   "projection_residual": rc_,
                   "max_rel_velocity": max(float(np.max(np.abs(sa[k] - sc_[k]))) for k in ("u", "v", "w")) / scale}
        tot_m = sum(t for _, t in prof_m.values())
        mixed = {"value": value_m, "unit": "point-steps/s", "ms_per_step": ms_m / args.steps,
                 "speedup_vs_fp64": value_m / value, "dtype": "f32+f64",
                 "error_vs_fp64": {"steps": nerr, "max_rel_velocity": vel_err,
                                   "max_div_fp64": da.max_div, "max_div_mixed": db.max_div,
                                   "max_div_abs_diff": abs(da.max_div - db.max_div),
                                   "projection_residual_fp64": ra, "projection_residual_mixed": rb,
                                   "projection_residual_note": "max|b - P phi| / max|b| of the Galerkin Poisson "
                                   "system of the last pressure step (3D:1680-1714); mixed: the FP32 solve in the "
                                   "eigenbasis"},
                 "refined": refined,
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
    peaks = measured_peaks()
    kernels, roofline, step_roof = kernel_rooflines(wl, prof, ms / args.steps, peaks, args.workload, args.traffic)
    fp64_peak = measure_fp64_tflops(local)
    flops = algorithmic_flops(wl)
    if roofline is not None and roofline["kernel"] in flops:
        roofline["fp64_equivalent_tflops"] = flops[roofline["kernel"]] / (kernels[roofline["kernel"]]["avg_ms"] * 1e-3) / 1e12
        roofline["fp64_fma_peak_tflops"] = fp64_peak
    step_roof["fp64_equivalent_tflops"] = flops["total"] / (ms / args.steps * 1e-3) / 1e12
    step_roof["fp64_fma_peak_tflops"] = fp64_peak

    # the largest grid (512x384x129, white noise): FP64 and mixed, own roofline
    large = None
    if args.large_steps > 0 and rank == 0:
        large = large_leg(args, local, peaks)

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
            "config": bench_config(args.workload, wl, ws),
            "device_footprint_bytes": footprint_bytes(cfg),
            "e2e": e2e, "gpu_launches": launches, "roofline": roofline, "step_roofline": step_roof,
            "kernels": kernels, "clocks": clocks, "cpu_baseline": cpu, "mixed": mixed, "large": large,
            "ensemble": ensemble, "serving": serving,
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
    ap.add_argument("--ref-budget", type=float, default=120.0,
                    help="reference arm: seconds of CPU time allowed for warm-up plus timed steps")
    ap.add_argument("--no-mixed", dest="mixed", action="store_false",
                    help="skip the mixed-precision measurement")
    ap.add_argument("--mixed-err-steps", type=int, default=200)
    ap.add_argument("--ensemble-runs", type=int, default=64)
    ap.add_argument("--ensemble-steps", type=int, default=50)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--noise", type=float, default=None,
                    help="white-noise amplitude on the initial u, v, w (default: the workload's; the large "
                         "workload has 1e-3)")
    ap.add_argument("--large-steps", type=int, default=10,
                    help="timed steps of the 512x384x129 leg (0 skips it)")
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
