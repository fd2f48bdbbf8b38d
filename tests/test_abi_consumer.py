"""The C ABI from plain C: tests/abi_consumer.c compiles as strict C99 against
include/subsweep_gpu.h alone, links against the sweep library and runs.  Without a
device its handle creation must fail with SW_ERR_CUDA and a message (no fallback);
with one, the consumer steps a small column and reads the fields back."""
import ctypes
import pathlib
import shutil
import subprocess

import pytest

from subsweep_gb300 import _native

ROOT = pathlib.Path(__file__).resolve().parents[1]


def test_c99_consumer_links_and_runs(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lib = pathlib.Path(_native.load_gpu()._name)
    exe = tmp_path / "abi_consumer"
    build = subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I", str(ROOT / "include"),
                            str(ROOT / "tests" / "abi_consumer.c"), "-o", str(exe), str(lib),
                            f"-Wl,-rpath,{lib.parent}", "-lm"], capture_output=True, text=True)
    assert build.returncode == 0, build.stderr
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert run.returncode == 0, (run.returncode, run.stdout, run.stderr)
    first = run.stdout.splitlines()[0].split(" ", 2)
    assert first[0] == "create"
    status = int(first[1])
    if status == _native.SW_OK:
        x0, t0 = map(float, run.stdout.splitlines()[1].split()[1:])
        assert 0.0 < x0 <= 1.0 and t0 > 0.0
    else:
        assert status == _native.SW_ERR_CUDA and first[2].strip()


LAYOUTS = {
    "sw_params": _native.SwParams,
    "sw_grid_csr": _native.SwGridCsr,
    "sw_cell_init": _native.SwCellInit,
    "sw_time_series": _native.SwTimeSeries,
    "sw_stats": _native.SwStats,
}


def test_ctypes_mirrors_match_the_c_layouts(tmp_path):
    """Every struct of include/subsweep_gpu.h has the size, field names and field
    offsets of its ctypes mirror in subsweep_gb300/_native.py, as a C compiler lays it
    out: a field added on one side only would shift every later field."""
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "subsweep_gpu.h"', "int main(void) {"]
    for cname, mirror in LAYOUTS.items():
        lines.append(f'  printf("{cname} .sizeof %zu\\n", sizeof({cname}));')
        for field, _ in mirror._fields_:
            lines.append(f'  printf("{cname} {field} %zu\\n", offsetof({cname}, {field}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layouts.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layouts"
    build = subprocess.run([cc, "-std=c99", "-Wall", "-Werror", "-I", str(ROOT / "include"), str(src), "-o", str(exe)],
                           capture_output=True, text=True)
    assert build.returncode == 0, build.stderr
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60, check=True)
    got = {}
    for line in run.stdout.splitlines():
        cname, field, value = line.split()
        got[(cname, field)] = int(value)
    for cname, mirror in LAYOUTS.items():
        assert got[(cname, ".sizeof")] == ctypes.sizeof(mirror), cname
        for field, _ in mirror._fields_:
            assert got[(cname, field)] == getattr(mirror, field).offset, (cname, field)
