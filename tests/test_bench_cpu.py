"""CPU: bench.py's reference arm prints one JSON line with the keys of the
measurement contract, the serving stream it replays is seeded, and its
roofline entries follow from the algorithmic bytes and the kernel times."""
import json
import os
import subprocess
import sys
import types

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line():
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "3", "--warmup", "3"],
                       cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    for k in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["impl"] == "reference" and line["metric"] == "point-steps/s" and line["higher_is_better"]
    assert line["steps"] == 3 and line["warmup"] == 3 and line["value"] > 0
    assert line["config"]["workload"] == "channel_128x128x65_re180_pi"
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["value"] == line["value"]
    assert line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    assert line["e2e"]["value"] == line["value"]


def test_serving_stream_is_seeded():
    sys.path.insert(0, ROOT)
    import bench
    args = types.SimpleNamespace(serve_requests=32, serve_rate=4.0, seed=0)
    a = bench.serving_requests(args)
    b = bench.serving_requests(args)
    assert [(t, d["nx"], d["ny"], d["nz"], n) for t, d, n in a] == [(t, d["nx"], d["ny"], d["nz"], n) for t, d, n in b]
    assert len(a) == 32
    assert all(t1 < t2 for (t1, _, _), (t2, _, _) in zip(a, a[1:]))  # arrival times increase
    assert all(200 <= n <= 2000 for _, _, n in a)
    assert sum(1 for _, d, _ in a if d["nx"] == 256) == 4  # the large 256x256x97 runs of this seed


def test_roofline_arithmetic():
    """bench.py's roofline entries: algorithmic bytes per launch over the
    kernel's average launch time against the measured copy bandwidth; the
    dominant kernel by total time; its ncu traffic and tensor share from the
    committed captures; the step's bytes over the step time."""
    sys.path.insert(0, ROOT)
    import bench
    from f90_dns_gb300.workloads import WORKLOADS
    name = "channel_128x128x65_re180_pi"
    wl = WORKLOADS[name]
    ab = bench.algorithmic_bytes(wl)
    S = 65 * 128 * 65 * 16.0
    assert ab["viscous_helmholtz_tc"] == 9 * S + 4225 * (33 * 33 + 32 * 32) * 8.0 == 149294600.0
    assert ab["products"] == 9 * 128 * 128 * 65 * 8.0
    prof = {"pi_update": (5, 0.05), "viscous_helmholtz_tc": (5, 0.875), "products": (5, 0.09),
            "pressure_poisson_tc": (5, 0.57)}
    peaks = {"hbm_gbs": 6792.7, "source": "measured"}
    kernels, roof, step = bench.kernel_rooflines(wl, prof, 0.61, peaks, name)
    v = kernels["viscous_helmholtz_tc"]
    assert abs(v["avg_ms"] - 0.175) < 1e-12
    assert abs(v["achieved_gbs"] - 149294600.0 / 0.175e-3 / 1e9) < 1e-6
    assert abs(v["hbm_frac"] - v["achieved_gbs"] / 6792.7) < 1e-12
    assert abs(sum(k["share"] for k in kernels.values()) - 1.0) < 1e-12
    assert roof["kernel"] == "viscous_helmholtz_tc" and roof["unit"] == "GB/s" and roof["bound"] == "hbm"
    assert roof["frac"] == v["hbm_frac"] and roof["peak"] == 6792.7
    assert roof["traffic"] == bench.NCU_TRAFFIC[(name, "viscous_helmholtz_tc")]
    assert roof["tensor_pipe_pct"] == bench.NCU_TENSOR_PIPE[(name, "viscous_helmholtz_tc")]
    per_step = sum(ab[k] for k in prof)  # one launch of each per step (5 launches / 5 steps)
    assert abs(step["bytes_per_step"] - per_step) < 1e-3
    assert abs(step["frac"] - per_step / (6792.7e9) * 1e3 / 0.61) < 1e-12
    _, roof2, _ = bench.kernel_rooflines(wl, prof, 0.61, peaks, name, traffic_override=1.0)
    assert roof2["traffic"] == 1.0
