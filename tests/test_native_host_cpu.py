"""Host-side parts of libbsj.so and the command-line drivers, without a GPU.

- the C++ drop-in ``parse_instance`` / ``resolve_instance_file`` (include/bsj_solver.h)
  against the reference's own parser (cpu/common/instance_parser.cpp) and the Python
  mirror, on regular and malformed files;
- ``bsj_instance_read`` / ``bsj_instance_resolve`` (C ABI) likewise;
- ``bsj_schedule_decode`` against the oracle's schedule check;
- the drivers' argument errors, which return before any device is touched.
"""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

from beamsearch_jssp_gpu_gb300 import _native as nat
from beamsearch_jssp_gpu_gb300 import build as B
from beamsearch_jssp_gpu_gb300.instance import parse_instance, resolve_instance_file, synthetic_instance, write_instance
from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
needs_ref = pytest.mark.skipif(not O.ref_cpu_available(), reason="reference CPU build absent")

ODD_FILES = {
    "x.txt": None,  # synthetic, written below
    "tabs.txt": "3\t2 \n0\t5\t1 7\n1 2 0 9\n 0 1 1 1 \n",
    "trunc.txt": "3 2\n0 5 1 7\n1 2\n",
    "half.txt": "2 2\n0 5 1 7\n1\n",
    "junk.txt": "3 2\n0 5 x 7\n1 2 0 9\n0 1 1 1\n",
    "neg.txt": "2 2\n-1 5 1 7\n1 2 0 9\n",
    "zero.txt": "0 3\n",
}


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(nat.LIB_PATH) or not os.path.exists(B.CLI_BIN):
        B.build()
    return nat.load()


@pytest.fixture(scope="module")
def dump(lib, tmp_path_factory):
    """Build tests/native/parse_dump.cpp against libbsj.so."""
    out = str(tmp_path_factory.mktemp("native") / "parse_dump")
    cxx = shutil.which("g++") or "g++"
    subprocess.check_call([cxx, "-O1", "-std=c++17", os.path.join(ROOT, "tests", "native", "parse_dump.cpp"),
                           "-o", out, "-L" + B.OUT_DIR, "-lbsj", "-Wl,-rpath," + B.OUT_DIR])
    return out


def _files(tmp_path):
    mc, du = synthetic_instance(9, 4, 2)
    write_instance(str(tmp_path / "x.txt"), mc, du)
    for name, text in ODD_FILES.items():
        if text is not None:
            (tmp_path / name).write_text(text)
    return [str(tmp_path / n) for n in ODD_FILES]


def _run_dump(dump, arg, cwd=None):
    r = subprocess.run([dump, arg], capture_output=True, text=True, cwd=cwd)
    fields = {}
    for line in r.stdout.splitlines():
        k, _, v = line.partition(" ")
        fields[k] = v
    return r.returncode, fields


def test_cxx_parser_matches_python_mirror(dump, tmp_path):
    for path in _files(tmp_path):
        rc, f = _run_dump(dump, path)
        ours = parse_instance(path)
        assert rc == 0, path
        assert int(f["n"]) == ours.nbjob and int(f["m"]) == ours.nbmachine
        assert int(f["nboperation"]) == ours.nboperation
        assert [int(v) for v in f["machine1"].split()] == [o.num_mc for o in ours.operations], path
        assert [int(v) for v in f["duration"].split()] == [o.dure for o in ours.operations], path
        assert [int(v) for v in f["job"].split()] == [o.num_j for o in ours.operations], path
        assert [int(v) for v in f["id"].split()] == [o.num_op for o in ours.operations], path
    (tmp_path / "empty.txt").write_text("")
    assert _run_dump(dump, str(tmp_path / "empty.txt"))[0] == 4
    assert _run_dump(dump, str(tmp_path / "missing.txt"))[0] == 3


@needs_ref
def test_cxx_parser_matches_reference_parser(dump, tmp_path):
    for path in _files(tmp_path):
        ref = O.ref_parse(path)
        rc, f = _run_dump(dump, path)
        assert rc == 0
        assert (int(f["n"]), int(f["m"]), int(f["nboperation"])) == (ref["n"], ref["m"], ref["nboperation"])
        assert [int(v) for v in f["machine1"].split()] == ref["machine1"], path
        assert [int(v) for v in f["duration"].split()] == ref["duration"], path
        assert [int(v) for v in f["job"].split()] == ref["job"], path


@needs_ref
def test_cxx_resolve_matches_reference(dump, tmp_path, monkeypatch):
    (tmp_path / "lawrence_instances").mkdir()
    (tmp_path / "taillard_instances").mkdir()
    mc, du = synthetic_instance(3, 2, 0)
    write_instance(str(tmp_path / "lawrence_instances" / "la05.txt"), mc, du)
    write_instance(str(tmp_path / "taillard_instances" / "ta05"), mc, du)
    write_instance(str(tmp_path / "taillard_instances" / "ta06"), mc, du)
    write_instance(str(tmp_path / "taillard_instances" / "ta77.txt"), mc, du)
    write_instance(str(tmp_path / "direct.txt"), mc, du)
    monkeypatch.chdir(tmp_path)
    for arg in ("05", "06", "77", "direct.txt", "nothing"):
        rc, f = _run_dump(dump, arg, cwd=str(tmp_path))
        want = O.ref_resolve(arg)
        if want is None:
            assert rc == 3, arg
        else:
            assert f["path"] == want, arg
        assert resolve_instance_file(arg) == want


def test_c_abi_instance_read(lib, tmp_path):
    for path in _files(tmp_path):
        n, m = ctypes.c_int32(), ctypes.c_int32()
        st = lib.bsj_instance_read(path.encode(), ctypes.byref(n), ctypes.byref(m), None, None, 0)
        ours = parse_instance(path)
        if ours.nbjob < 1 or ours.nbmachine < 1:
            assert st == nat.BSJ_ERR_INVALID
            continue
        assert st == nat.BSJ_OK and (n.value, m.value) == (ours.nbjob, ours.nbmachine)
        N = n.value * m.value
        mc = np.zeros(N, dtype=np.int32)
        du = np.zeros(N, dtype=np.int32)
        p32 = ctypes.POINTER(ctypes.c_int32)
        assert lib.bsj_instance_read(path.encode(), ctypes.byref(n), ctypes.byref(m), mc.ctypes.data_as(p32),
                                     du.ctypes.data_as(p32), N - 1) == nat.BSJ_ERR_LIMIT
        assert lib.bsj_instance_read(path.encode(), ctypes.byref(n), ctypes.byref(m), mc.ctypes.data_as(p32),
                                     du.ctypes.data_as(p32), N) == nat.BSJ_OK
        assert mc.tolist() == [o.num_mc - 1 for o in ours.operations[1:N + 1]]
        assert du.tolist() == [o.dure for o in ours.operations[1:N + 1]]
    buf = ctypes.create_string_buffer(512)
    assert lib.bsj_instance_resolve(str(tmp_path / "x.txt").encode(), buf, 512) == nat.BSJ_OK
    assert buf.value.decode() == str(tmp_path / "x.txt")
    assert lib.bsj_instance_resolve(b"definitely-not-here", buf, 512) == nat.BSJ_ERR_INVALID


def _decode(lib, mc, du, seq):
    n, m = mc.shape
    inst = nat.Instance(n, m, mc.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                        du.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)))
    s = np.ascontiguousarray(seq, dtype=np.int32)
    start = np.full(n * m, -1, dtype=np.int32)
    cm = ctypes.c_int32()
    st = lib.bsj_schedule_decode(ctypes.byref(inst), s.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                 start.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), ctypes.byref(cm))
    return st, start, cm.value


def test_schedule_decode_matches_oracle(lib):
    for (n, m, iseed) in ((10, 5, 0), (20, 15, 3), (7, 1, 2)):
        mc, du = synthetic_instance(n, m, iseed)
        for mode, K, seed in (("v2", 64, 1), ("pms", 32, 7), ("ich", 16, 3)):
            r = O.solve(mc, du, mode, K, seed)
            if not r["found"]:
                continue
            st, start, cm = _decode(lib, mc, du, r["seq"])
            assert st == nat.BSJ_OK and cm == O.schedule_makespan(mc, du, r["seq"]) == r["makespan"]
            # semi-active: every op starts when both its machine and its job are free
            fin = start + du.ravel()
            for j in range(n):
                for k in range(1, m):
                    assert start[j * m + k] >= fin[j * m + k - 1]
            assert (start >= 0).all() and fin.max() == cm


def test_schedule_decode_rejects_infeasible_orders(lib):
    mc, du = synthetic_instance(3, 2, 0)
    good = np.array([1, 3, 5, 2, 4, 6], dtype=np.int32)
    assert _decode(lib, mc, du, good)[0] == nat.BSJ_OK
    for bad in ([2, 1, 3, 4, 5, 6], [1, 1, 3, 4, 5, 6], [0, 3, 5, 2, 4, 6], [1, 3, 5, 2, 4, 7]):
        assert _decode(lib, mc, du, bad)[0] == nat.BSJ_ERR_INVALID, bad


def _cli(name, *args, cwd=None):
    exe = os.path.join(B.OUT_DIR, name)
    return subprocess.run([exe, *args], capture_output=True, text=True, cwd=cwd, timeout=60)


def test_cli_names_and_argument_errors(lib, tmp_path):
    for name in B.CLI_NAMES:
        assert os.path.islink(os.path.join(B.OUT_DIR, name)), name
    r = subprocess.run([B.CLI_BIN], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stderr
    r = _cli("exec_gpu_v1", "no-such-instance", cwd=str(tmp_path))
    assert r.returncode == 1 and "Error: cannot locate instance file: no-such-instance" in r.stderr
    r = _cli("BS-PMS", "no-such-instance", cwd=str(tmp_path))
    assert r.returncode == 1 and "Error: cannot locate instance file for: no-such-instance" in r.stderr
    mc, du = synthetic_instance(4, 3, 0)
    write_instance(str(tmp_path / "i.txt"), mc, du)
    r = _cli("BS-ICH", str(tmp_path / "i.txt"), "0")
    assert r.returncode == 1 and "beam_width must be >= 1" in r.stderr
    r = _cli("exec_gpu_v2", str(tmp_path / "i.txt"), "--bogus")
    assert r.returncode == 1 and "unknown option" in r.stderr
    r = _cli("exec_gpu_v2", str(tmp_path / "i.txt"), "--ranks", "0")
    assert r.returncode == 1


def test_without_a_device_contexts_and_servers_fail_cleanly(lib):
    """No call exits or hangs when no GPU is usable: status codes come back."""
    count = ctypes.c_int32(-1)
    st = lib.bsj_device_count(ctypes.byref(count))
    if st == nat.BSJ_OK and count.value > 0:
        pytest.skip("a CUDA device is present")
    assert count.value == 0
    h = ctypes.c_void_p()
    assert lib.bsj_create(ctypes.byref(h), 0) != nat.BSJ_OK
    from beamsearch_jssp_gpu_gb300 import BsjError, Server

    with pytest.raises(BsjError):
        Server(0)
