"""bench.py's CPU reference arm (the oracle timed on the host cores) and the workload
names it reports.  CPU only: `--impl reference` runs no GPU code."""
import json
import pathlib
import subprocess
import sys

import numpy as np
import pytest

from subsweep_gb300 import workloads

ROOT = pathlib.Path(__file__).resolve().parents[1]


@pytest.mark.parametrize("name,n", [("c1", 6), ("c2", 6), ("c4", 8)])
def test_label_is_the_constructors_name(name, n):
    make = {"c1": workloads.c1_small_periodic, "c2": workloads.c2_lognormal, "c4": workloads.c4_grf}[name]
    kw = {"num_sources": 4} if name == "c4" else {}
    assert make(n_per_side=n, nthreads=2, **kw).name == workloads.label(name, n)


def test_label_of_c3_boxes():
    box = workloads.c3_box(np.random.default_rng(0), 7, 512, 600, nthreads=2)
    assert workloads.c3_batched(boxes=[box] * 2).name == workloads.label("c3", 2)


def test_reference_arm_json_line():
    """One JSON line with the GPU arm's metric, unit and workload, the whole grid swept
    in bounded samples described in cpu_baseline, and an e2e block without device
    copies; the process maps the oracle's library and none of the package's."""
    import bench
    code = ("import sys, bench; sys.argv = ['bench.py', '--impl', 'reference', '--workload', 'c2', "
            "'--n-per-side', '8', '--steps', '3', '--warmup', '3']; bench.main(); "
            "maps = open('/proc/self/maps').read(); "
            "print('MAPPED', sorted({l.split()[-1].rsplit('/', 1)[-1] for l in maps.splitlines() "
            "if 'subsweep' in l or 'oracle' in l}))")
    out = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert (d["metric"], d["unit"], d["higher_is_better"]) == (bench.METRIC, bench.UNIT, True)
    assert (d["steps"], d["warmup"], d["n_gpus"]) == (3, 3, 1)
    assert d["value"] > 0 and d["chem_cells_per_s"] > 0
    assert d["config"]["workload"] == workloads.label("c2", 8)
    assert d["config"]["cells"] == 512
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert "full grid (512 cells)" in cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    mapped = [l for l in out.stdout.splitlines() if l.startswith("MAPPED")][0]
    assert "liboracle.so" in mapped and "libsubsweep" not in mapped, mapped


def test_write_back_split_reports_and_never_raises():
    """The e2e write-back split of the GPU arm, on stand-ins for a handle: the median
    times of fields() with and without the photon rate, and an error captured, not
    raised."""
    import time as _time

    import bench

    class Handle:
        num_cells = 4

        def __init__(self):
            self.calls = []

        def fields(self, out, photon_rate=True):
            self.calls.append(photon_rate)
            _time.sleep(0.004 if photon_rate else 0.001)
            return out

        def cell_state(self):
            return {"level": np.array([0, 3, 3, 1], np.uint8)}

    h = Handle()
    got = bench.write_back_split(h, reps=3)
    assert got["calls"] == 3 and h.calls == [True] * 4 + [False] * 3
    assert got["fields_ms"] > got["fields_without_photon_rate_ms"] > 0.5
    assert got["cells_per_level"] == [1, 1, 0, 2]

    class Broken(Handle):
        def fields(self, out, photon_rate=True):
            raise RuntimeError("no device")

    assert "no device" in bench.write_back_split(Broken())["error"]
