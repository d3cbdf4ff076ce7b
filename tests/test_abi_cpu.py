"""The C-ABI library loads and exports every symbol include/*.h declares (no GPU needed;
no compute call is made)."""
import ctypes
import os
import re

import pytest

from beamsearch_jssp_gpu_gb300 import _native as nat

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared(header):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(bsj_[a-z_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(nat.LIB_PATH):
        from beamsearch_jssp_gpu_gb300 import build

        build.build()
    return ctypes.CDLL(nat.LIB_PATH)


def test_every_declared_c_symbol_is_exported(lib):
    names = _declared("bsj.h")
    assert len(names) >= 16
    for name in names:
        assert hasattr(lib, name), name
    assert set(names) == set(nat.EXPORTED)


def test_cxx_dropins_exported_with_reference_mangling(lib):
    # int run_gpu_beam_search_v1(const JSSPInstance&, int, int, int, int*)  (gpu/v1/solver.cuh:6)
    for sym in ("_Z22run_gpu_beam_search_v1RK12JSSPInstanceiiiPi",
                "_Z22run_gpu_beam_search_v2RK12JSSPInstanceiiiPi"):
        assert hasattr(lib, sym), sym


def test_pure_host_calls(lib):
    L = nat.load()
    assert L.bsj_version().decode().startswith("bsj-gb300")
    assert L.bsj_status_string(0).decode() == "ok"
    assert L.bsj_status_string(2).decode().startswith("size")


def test_struct_layouts_match_the_compiled_header(tmp_path):
    """Every public struct's size and member offsets, as a C compiler lays them out from
    include/bsj.h, equal the ctypes mirrors the Python binding passes to the library."""
    import shutil
    import subprocess

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    mirrors = {"bsj_instance": nat.Instance, "bsj_beam": nat.Beam, "bsj_result": nat.Result,
               "bsj_server_config": nat.ServerConfig, "bsj_request_times": nat.RequestTimes,
               "bsj_server_stats": nat.ServerStats}
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "bsj.h"', "int main(void) {"]
    for cname, py in mirrors.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for field, _ in py._fields_:
            lines.append(f'printf("{cname} {field} %zu\\n", offsetof({cname}, {field}));')
    lines += ["return 0; }"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    subprocess.run([cc, "-std=c99", "-I", inc, str(src), "-o", str(exe)], check=True)
    got = {}
    for line in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines():
        cname, field, value = line.split()
        got[(cname, field)] = int(value)
    for cname, py in mirrors.items():
        assert got[(cname, "size")] == ctypes.sizeof(py), cname
        for field, _ in py._fields_:
            assert got[(cname, field)] == getattr(py, field).offset, (cname, field)


def test_struct_layouts_match_header():
    # bsj_instance: 2 x int32 + 2 pointers; bsj_beam: 6 x 4 B; bsj_result as declared
    assert ctypes.sizeof(nat.Instance) == 8 + 2 * ctypes.sizeof(ctypes.c_void_p)
    assert ctypes.sizeof(nat.Beam) == 24
    assert nat.Result.sequence.offset == 8
    assert nat.Result.expanded.offset == 8 + ctypes.sizeof(ctypes.c_void_p)
