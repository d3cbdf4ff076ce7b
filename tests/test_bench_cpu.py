"""bench.py's host-side pieces, without a GPU: the roofline's DRAM traffic comes from the
committed ncu summary of the same workload, the peak from the measured-peaks file (or the
stated fallback), and the command line offers every measurement mode the documentation
names."""
import json
import os

import bench


def test_traffic_is_read_from_the_committed_ncu_summary():
    for kernel in ("k_select", "k_step"):
        t = bench._traffic(kernel)
        assert t is not None and t > 0, kernel
    assert bench._traffic("k_no_such_kernel") is None


def test_traffic_lines_name_the_bench_workload():
    path = os.path.join(bench.ROOT, "profiles", "ncu_traffic.txt")
    work = f"{bench.N_JOBS}x{bench.N_MACH}_K{bench.K}_B{bench.BEAMS}"
    lines = [ln for ln in open(path) if ln.startswith("kernel=")]
    assert lines and all(f"workload={work}" in ln for ln in lines)


def test_peak_is_measured_or_the_stated_fallback():
    p = bench._peaks()
    path = os.path.join(bench.ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        assert p["source"] == "measured"
        assert p["hbm_gbs"] == float(json.load(open(path))["hbm_gbs"])
    else:
        assert p == {"hbm_gbs": 6800.0, "source": "fallback"}


def test_config_names_the_workload():
    c = bench._config(1)
    assert c["jobs"] == 50 and c["machines"] == 20 and c["beam_width"] == 4096
    assert c["beams_per_gpu"] == 8 and c["levels"] == 1000
    assert "workload" in c and "l2" in c


def test_command_line_modes(monkeypatch, capsys):
    import sys

    calls = {}
    for name in ("k_sweep", "chunk_sweep", "solve_times", "reference_arm", "gpu_arm"):
        monkeypatch.setattr(bench, name, lambda args, name=name: calls.setdefault(name, args) and 0)
    for argv, want in ((["--k-sweep"], "k_sweep"), (["--chunk-sweep"], "chunk_sweep"),
                       (["--solve-times"], "solve_times"), (["--impl", "reference"], "reference_arm"),
                       ([], "gpu_arm")):
        calls.clear()
        monkeypatch.setattr(sys, "argv", ["bench.py"] + argv)
        bench.main()
        assert list(calls) == [want]
        args = calls[want]
        assert args.warmup >= 3 and args.steps >= 1 and args.gpus == 1
