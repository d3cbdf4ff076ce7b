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


def test_command_line_modes(monkeypatch):
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


def test_reference_arm_line(monkeypatch, capsys):
    """The reference arm end to end on a small workload (10x5, K=64, 3 beams, whole
    50-level searches): one JSON line with the contract's keys, labelled as the BS-PMS
    semantics it runs, whose value is the oracle's scored children over the step time."""
    import sys

    from beamsearch_jssp_gpu_gb300.instance import synthetic_instance
    from oracle import oracle as O

    for k, v in (("N_JOBS", 10), ("N_MACH", 5), ("K", 64), ("BEAMS", 3), ("CPU_SAMPLE_LEVELS", 50)):
        monkeypatch.setattr(bench, k, v)
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference", "--steps", "1", "--warmup", "1"])
    assert bench.main() == 0
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "candidates/s" and line["higher_is_better"]
    assert line["metric"] == bench.METRIC and line["steps"] == 1 and line["warmup"] == 1
    assert line["config"]["mode"] == "pms" and "cpu/v1_pms" in line["config"]["workload"]
    assert line["e2e"] == {"value": line["value"], "unit": "candidates/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["value"] == line["value"] and 1 <= cb["cores"] <= 3
    mc, du = synthetic_instance(10, 5, bench.INSTANCE_SEED)
    expanded = sum(O.solve(mc, du, "pms", 64, s)["expanded"] for s in range(3))
    # one step: value = scored children of the 3 whole searches / the slowest beam's time
    assert abs(line["value"] * line["ms_per_step"] / 1000.0 - expanded) <= 1e-6 * expanded
