"""bench.py's reference arm (the oracle on the host cores) prints one JSON line
with the fields the measurement contract asks for; it needs no GPU."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_line(tmp_path):
    env = dict(os.environ, MW3_CASES=str(tmp_path))
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload",
                          "j0_256x128x60", "--steps", "1", "--warmup", "3", "--cpu-seconds", "1"],
                         capture_output=True, text=True, env=env, cwd=ROOT, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference" and d["value"] > 0 and d["warmup"] >= 3
    assert d["cpu_baseline"]["kind"] in ("port", "reference") and d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["config"]["workload"] == "j0_256x128x60"


def test_timed_window_alignment():
    """The timed window starts on a multiple of 32 for whole ring cycles (with one
    captured graph block before it) and otherwise ends on the iteration that
    flushes the Cvj ring (31 mod 32)."""
    sys.path.insert(0, ROOT)
    import bench
    for warm in (3, 5, 40):
        for steps in (1, 7, 20, 31, 32, 64, 40):
            w = bench.warmup_count(1, warm, steps)
            assert w >= warm
            it0 = 1 + w                      # iteration count before the window
            if steps % 32 == 0:
                assert it0 % 32 == 0 and w >= warm + 32
            else:
                assert (it0 + steps) % 32 == 31
            # the window holds an iteration that is 31 mod 32
            assert any((it0 + j) % 32 == 31 for j in range(1, steps + 1))
