"""Instance format, path resolution and the synthetic generator (no GPU needed)."""
import os

import numpy as np
import pytest

from beamsearch_jssp_gpu_gb300.instance import (JSSPInstance, format_instance, parse_instance,
                                                resolve_instance_file, schedule_makespan,
                                                synthetic_instance, write_instance)
from oracle import oracle as O

needs_ref = pytest.mark.skipif(not O.ref_cpu_available(), reason="reference CPU build absent")


def test_synthetic_is_deterministic_and_well_formed():
    a = synthetic_instance(20, 15, 3)
    b = synthetic_instance(20, 15, 3)
    c = synthetic_instance(20, 15, 4)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert not np.array_equal(a[1], c[1])
    mc, du = a
    for j in range(20):
        assert sorted(mc[j].tolist()) == list(range(15))
    assert du.min() >= 1 and du.max() <= 99
    assert mc.dtype == np.int32 and du.dtype == np.int32


def test_roundtrip(tmp_path):
    mc, du = synthetic_instance(7, 3, 1)
    p = tmp_path / "x.txt"
    write_instance(str(p), mc, du)
    inst = parse_instance(str(p))
    assert inst.nbjob == 7 and inst.nbmachine == 3 and inst.nboperation == 23
    assert np.array_equal(inst.machine, mc) and np.array_equal(inst.duration, du)
    assert inst.operations[0].num_op == 0 and inst.operations[-1].num_op == 22
    assert inst.operations[1].num_mc == mc[0, 0] + 1
    assert format_instance(mc, du).startswith("7 3\n")


@needs_ref
def test_parser_matches_reference_parser(tmp_path):
    mc, du = synthetic_instance(9, 4, 2)
    p = tmp_path / "x.txt"
    write_instance(str(p), mc, du)
    # the reference parser also accepts tabs, trailing spaces and a truncated body
    (tmp_path / "tabs.txt").write_text("3\t2 \n0\t5\t1 7\n1 2 0 9\n 0 1 1 1 \n")
    (tmp_path / "trunc.txt").write_text("3 2\n0 5 1 7\n1 2\n")
    (tmp_path / "junk.txt").write_text("3 2\n0 5 x 7\n1 2 0 9\n0 1 1 1\n")
    for name in ("x.txt", "tabs.txt", "trunc.txt", "junk.txt"):
        path = str(tmp_path / name)
        ref = O.ref_parse(path)
        ours = parse_instance(path)
        assert ours.nbjob == ref["n"] and ours.nbmachine == ref["m"]
        assert ours.nboperation == ref["nboperation"]
        assert [o.num_mc for o in ours.operations] == ref["machine1"]
        assert [o.dure for o in ours.operations] == ref["duration"]
        assert [o.num_j for o in ours.operations] == ref["job"]
    assert parse_instance(str(tmp_path / "missing.txt")) is None
    assert O.ref_parse(str(tmp_path / "missing.txt")) is None
    (tmp_path / "empty.txt").write_text("")
    assert parse_instance(str(tmp_path / "empty.txt")) is None


@needs_ref
def test_reference_benchmark_files_parse_identically():
    """Lawrence / Taillard files are read by path only (never copied)."""
    root = O.reference_tree()
    paths = [os.path.join(root, "lawrence_instances", "la01.txt"),
             os.path.join(root, "taillard_instances", "ta01")]
    for p in paths:
        if not os.path.exists(p):
            pytest.skip("reference benchmark files absent")
        ref = O.ref_parse(p)
        ours = parse_instance(p)
        assert [o.num_mc for o in ours.operations] == ref["machine1"]
        assert [o.dure for o in ours.operations] == ref["duration"]


@needs_ref
def test_resolve_matches_reference(tmp_path, monkeypatch):
    (tmp_path / "lawrence_instances").mkdir()
    (tmp_path / "taillard_instances").mkdir()
    mc, du = synthetic_instance(3, 2, 0)
    write_instance(str(tmp_path / "lawrence_instances" / "la05.txt"), mc, du)
    write_instance(str(tmp_path / "taillard_instances" / "ta05"), mc, du)
    write_instance(str(tmp_path / "taillard_instances" / "ta77.txt"), mc, du)
    write_instance(str(tmp_path / "direct.txt"), mc, du)
    monkeypatch.chdir(tmp_path)
    for arg in ("05", "77", "direct.txt", "nothing"):
        assert resolve_instance_file(arg) == O.ref_resolve(arg), arg


def test_schedule_makespan_checks_precedence():
    mc, du = synthetic_instance(3, 2, 0)
    good = [1, 3, 5, 2, 4, 6]
    assert schedule_makespan(mc, du, good) > 0
    assert schedule_makespan(mc, du, [2, 1, 3, 4, 5, 6]) == -1
    assert schedule_makespan(mc, du, good[:-1]) == -1
    assert O.schedule_makespan(mc, du, np.array(good, dtype=np.int32)) == schedule_makespan(mc, du, good)


def test_from_arrays_matches_parse(tmp_path):
    mc, du = synthetic_instance(4, 3, 9)
    a = JSSPInstance.from_arrays(mc, du)
    write_instance(str(tmp_path / "y.txt"), mc, du)
    b = parse_instance(str(tmp_path / "y.txt"))
    assert a.operations == b.operations and a.nboperation == b.nboperation
