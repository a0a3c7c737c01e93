"""bench.py's reference arm on the CPU: the JSON contract of `--impl reference` (one line, impl "reference", the same
metric and config as the GPU arm, a cpu_baseline describing the run, an e2e of the line's own value with no copies),
and under torchrun with two gloo ranks only rank 0 runs and prints."""
import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SMALL = ["--width", "64", "--height", "36", "--steps", "2", "--warmup", "3"]


def _json_lines(out):
    return [json.loads(l) for l in out.splitlines() if l.startswith("{")]


def _run(cmd, env=None):
    e = dict(os.environ)
    e.update(env or {})
    return subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600, env=e)


def test_reference_arm_contract():
    sys.path.insert(0, ROOT)
    import bench

    r = _run([sys.executable, "bench.py", "--impl", "reference", *SMALL])
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _json_lines(r.stdout)
    assert len(lines) == 1
    d = lines[0]
    assert d["impl"] == "reference" and d["metric"] == bench.METRIC
    assert d["unit"] == "frames/s" and d["higher_is_better"] is True and d["n_gpus"] == 1
    assert d["steps"] == 2 and d["warmup"] == 3 and d["value"] > 0
    assert abs(d["ms_per_step"] - 1e3 / d["value"]) < 1e-6 * d["ms_per_step"]
    assert d["config"]["width"] == 64 and d["config"]["height"] == 36 and d["config"]["mode"] == "full"
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_reference_arm_under_torchrun_prints_once():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    r = _run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
              "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference", "--gpus", "2", *SMALL],
             env={"OMP_NUM_THREADS": "2"})
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _json_lines(r.stdout)
    assert len(lines) == 1 and lines[0]["impl"] == "reference" and lines[0]["n_gpus"] == 2


def test_timed_window_holds_the_disocclusion():
    """Whatever --steps and --warmup the driver passes, the timed frames of the 60-frame sequence hold frame 30
    (where a plane appears) when they are fewer than the sequence, and the warm-up frames come just before them;
    the reference arm times the same frames."""
    sys.path.insert(0, ROOT)
    import bench

    for steps in (1, 2, 5, 20, 40, 59):
        for warmup in (0, 3, 5, 20):
            w0, t0 = bench.first_frames(steps, warmup, 60)
            assert t0 <= 30 <= t0 + steps - 1 and t0 + steps <= 60, (steps, warmup, t0)
            assert (w0 + warmup) % 60 == t0
    assert bench.first_frames(20, 5, 60) == (15, 20)
    w0, t0 = bench.first_frames(120, 5, 60)
    assert t0 == 5 and w0 == 0
    assert "20..39" in bench.window_text(20, 20, 60)
