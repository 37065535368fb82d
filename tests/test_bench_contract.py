"""The reference arm of bench.py (the C restatement of the reference algorithm on the host cores) runs
without a GPU: its one JSON line carries the keys of the bench contract."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line(monkeypatch, capsys):
    """The reference arm's line, on a small molecule in place of the 32-water cluster (same code path):
    the contract keys, and its K steps are exactly one full build (the hashed slices' counts add up to
    the unsampled build's)."""
    import argparse
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import bench
    import orc
    from unomol_gb300 import molecules
    from unomol_gb300.basis import Basis
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    small = Basis(text=molecules.patin_text(molecules.alkane(3), "6-31G"))
    monkeypatch.setattr(bench, "basis", lambda: small)
    assert bench.run_reference(argparse.Namespace(steps=4, warmup=1, gpus=1)) == 0
    lines = [l for l in capsys.readouterr().out.splitlines() if l.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e", "single_core"):
        assert k in d, k
    assert d["impl"] == "reference" and d["value"] > 0 and d["higher_is_better"] is True
    assert d["config"]["workload"].startswith("32-water cluster, 6-31G")
    assert d["config"]["extrapolated"] is False
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["cpu_baseline"]["value"] == d["value"]
    assert d["single_core"]["cores"] == 1 and d["single_core"]["value"] > 0
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert len(d["slice_s"]) == 4 and abs(d["ms_per_step"] * 4 / 1e3 - sum(d["slice_s"])) < 1e-2
    _, full = orc.fock(small, bench.synthetic_density(small))
    assert f"{int(full[0])} shell quartets, {int(full[1])} function quartets" in d["cpu_baseline"]["sample"]


FAKE_SMI = r'''#!{python}
import sys, time
period = float(sys.argv[sys.argv.index("-lms") + 1]) / 1e3
k = 0
while True:
    mhz = 1500 if k == 0 else 2070  # the first sample: before the load
    print(f"0, {{mhz}}, 2070, 900.5, 0x0000000000000004, Not Active, Not Active, Not Active, Active", flush=True)
    k += 1
    time.sleep(period)
'''


def test_clock_sampler_brackets_short_region(tmp_path, monkeypatch):
    """The sampler is live before the timed region opens and keeps a sample taken at or after its end,
    so a region shorter than the sampling period still has one; samples from before the region are not
    counted; throttle reasons reported Active are listed."""
    sys.path.insert(0, ROOT)
    import bench
    exe = tmp_path / "nvidia-smi"
    exe.write_text(FAKE_SMI.format(python=sys.executable))
    exe.chmod(0o755)
    monkeypatch.setenv("UNOMOL_CLOCKS_DIR", str(tmp_path))
    c = bench.Clocks(0, exe=str(exe))
    import time
    time.sleep(0.35)  # warm-up
    c.start()
    time.sleep(0.01)  # a region far shorter than the period
    clk = c.stop()
    assert clk["samples"] >= 1
    assert clk["sm_mhz"] == 2070.0 and clk["sm_max_mhz"] == 2070.0
    assert clk["reasons"] == ["sw_power_cap"]
    assert c.p.poll() is not None  # the sampler has ended


def test_clock_sampler_without_nvidia_smi(tmp_path, monkeypatch):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("UNOMOL_CLOCKS_DIR", str(tmp_path))
    c = bench.Clocks(0, exe=str(tmp_path / "absent"))
    c.start()
    assert c.stop() == {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}


def test_two_pipe_ceiling():
    """FP64-only work has the FP64 peak as ceiling; FP32-only the FP32 peak; mixed work is bounded by
    the longer pipe time (concurrent) and by the sum (one after the other)."""
    sys.path.insert(0, ROOT)
    import bench
    assert bench.two_pipe_ceiling(5.0, 0.0, 1.25, 78.5) == (1.25, 1.25)
    assert bench.two_pipe_ceiling(0.0, 7.0, 1.25, 78.5) == (78.5, 78.5)
    peak, serial = bench.two_pipe_ceiling(1.88, 30.48, 1.25, 78.5)
    t64, t32 = 1.88 / 1.25, 30.48 / 78.5
    assert abs(peak - (1.88 + 30.48) / t64) < 1e-12
    assert abs(serial - (1.88 + 30.48) / (t64 + t32)) < 1e-12
    assert serial < peak


def test_step_inputs_rebuild_every_eighth_build():
    """The measured sequence: the full density at builds 0, 8, 16, ... and the density change since
    the previous build otherwise, so that the incremental G sums back to G of the full density."""
    sys.path.insert(0, ROOT)
    import numpy as np
    import bench
    dens = [np.full(3, float(k * k)) for k in range(18)]
    steps = bench.step_inputs(dens)
    assert len(steps) == len(dens)
    for k, (full, x) in enumerate(steps):
        assert full == (k % bench.REBUILD == 0)
        base = k - k % bench.REBUILD
        acc = sum(steps[j][1] for j in range(base, k + 1))
        assert np.array_equal(acc, dens[k])
