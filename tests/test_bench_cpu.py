"""CPU: bench.py's reference arm prints one JSON line with the keys of the
measurement contract, and the serving stream it replays is seeded."""
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
