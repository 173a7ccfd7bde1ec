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


def test_end_to_end_leg_drives_every_context(monkeypatch):
    """run_e2e splits the waves over the contexts (every wave exactly once), each
    context's thread uploads psi_k, runs one iteration and downloads psi_k+1
    every step with the iteration counting on, and an error in a context's
    thread reaches the caller (a fake binding: no GPU)."""
    import threading
    import types

    import numpy as np
    import pytest

    sys.path.insert(0, ROOT)
    import bench
    import madwave3_gb300

    torch = pytest.importorskip("torch")
    monkeypatch.setattr(torch.Tensor, "pin_memory", lambda self: self)
    monkeypatch.setattr(torch.cuda, "synchronize", lambda: None)
    log, lock = [], threading.Lock()

    class FakeProp:
        fail_on = None

        def __init__(self, runs, precision):
            self.waves = [r.name for r in runs]
            self.n = sum(r.ntot for r in runs)
            self.it = 1

        def start(self):
            pass

        def run(self, n):
            if FakeProp.fail_on in self.waves and n == 1:      # inside the timed loop's thread
                raise RuntimeError("context of %s failed" % FakeProp.fail_on)
            self.it += n
            with lock:
                log.append(("run", tuple(self.waves), n))

        def state_all(self):
            return np.zeros(self.n), np.full(self.n, float(self.it)), self.it

        def upload_state_all(self, km1, k, it):
            assert km1 is None and k.shape == (self.n,) and it == self.it
            with lock:
                log.append(("up", tuple(self.waves), it))

        def state_k_all(self, out):
            out[:] = self.it

        def close(self):
            pass

    monkeypatch.setattr(madwave3_gb300, "Propagator", FakeProp)
    runs = [types.SimpleNamespace(name="J%d" % j, ntot=100 + 10 * j) for j in range(10)]
    ms, n = bench.run_e2e(runs, "mixed", 4, 3)
    assert n == 4 and ms > 0
    ups = [e for e in log if e[0] == "up"]
    groups = {e[1] for e in ups}
    assert sorted(w for g in groups for w in g) == sorted(r.name for r in runs)
    for g in groups:
        its = [e[2] for e in ups if e[1] == g]
        assert its == [its[0], its[0] + 1, its[0] + 2]
    FakeProp.fail_on = "J3"
    with pytest.raises(RuntimeError, match="J3"):
        bench.run_e2e(runs, "mixed", 4, 2)


def test_roofline_charges_the_executing_unit():
    """The dominant stage's roofline is taken against the unit that runs it."""
    sys.path.insert(0, ROOT)
    import bench
    peaks = (6677.8, 1908.8, "of measured")
    model = {"dst_R": ("flop", 6.0e11), "dst_r_pair": ("flop", 1.0e11), "angular": ("byte", 3.0e9),
             "angular_l2": ("flop", 1.0e10), "update": ("byte", 4.0e9)}
    fused = {"tc_dst": True, "tc_dst_fused": True, "tc_angular": True, "dst_f16": True}
    cuda_core = {"tc_dst": False, "tc_dst_fused": False, "tc_angular": False, "dst_f16": False}
    # 10 iterations; the fused DST dominates: tensor cores at the measured bf16 peak
    r = bench.dominant_roofline({"dst_R": 26.0, "angular": 20.0, "update": 14.0}, 10, model, fused, "mixed",
                                1e8, peaks)
    assert r["bound"] == "tensor" and r["kernel"] == "dst_R" and r["peak"] == 1908.8
    assert abs(r["achieved"] - 6.0e11 / 2.6e-3 / 1e12) < 1e-9 and r["traffic"] == 16.0 * 1e8
    # the factorised angular stage dominates: bytes against HBM
    r = bench.dominant_roofline({"dst_R": 10.0, "angular": 20.0}, 10, model, fused, "mixed", 1e8, peaks)
    assert r["bound"] == "hbm" and r["unit"] == "GB/s" and abs(r["achieved"] - 3.0e9 / 2e-3 / 1e9) < 1e-9
    # CUDA-core DSTs and explicit angular kernels: FP32 CUDA cores at the nominal rate
    for dom in ("dst_r_pair", "angular_l2"):
        st = {"dst_R": 1.0, "dst_r_pair": 2.0, "angular_l2": 2.0}
        st[dom] = 5.0
        r = bench.dominant_roofline(st, 10, model, cuda_core, "mixed", 1e8, peaks)
        assert r["bound"] == "fp32" and r["kernel"] == dom
        assert abs(r["peak"] - 152 * 128 * 2 * 2.07e9 / 1e12) < 1e-9 and r["traffic"] is None
    # FP64 path: the FP64 pipe at its nominal rate
    r = bench.dominant_roofline({"dst_r_pair": 5.0}, 10, model, cuda_core, "fp64", 1e8, peaks)
    assert r["bound"] == "fp64" and r["peak"] == bench.FP64_NOMINAL_TFLOPS


def test_cpu_baseline_sample(runs):
    """The bench's CPU-baseline leg (the oracle on every host core, a bounded
    sample) returns a well-formed entry."""
    sys.path.insert(0, ROOT)
    import bench
    out = bench.cpu_baseline(bench.sample_waves([runs["tiny_j0"]]), seconds=0.5)
    assert out["kind"] == "port" and out["unit"] == "grid-pt*iter/s" and out["value"] > 0
    assert out["cores"] >= 1 and "Chebyshev iterations" in out["sample"]
