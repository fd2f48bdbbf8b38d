"""Register use and spills of the transport kernels as ptxas reports them for sm_103a,
on the CPU (nvcc cross-compiles): a change that makes the default shape or the fastest
candidate spill, or any shape spill heavily, fails here before it costs GPU time.

The lockstep kernel's shape k_sweep_pull_lockg<blocks per SM, lanes per task, prefetch,
streaming, words ahead> caps its registers through __launch_bounds__(256, blocks per SM);
the variant number of a shape is 100 * prefetch + 10 * lanes + blocks (lanes 16 as 6;
83 and 84 name 183 and 184), +1000 streaming, +2000 words ahead.
"""
import re
import shutil
import subprocess

import pytest

from subsweep_gb300 import build

MAX_SPILL_BYTES = 256


def ptxas_table(tmp_path):
    """{demangled kernel: (registers, spill store bytes)} of the mixed translation unit,
    compiled with the library's own flags plus -Xptxas -v."""
    nvcc = shutil.which(build.NVCC)
    if nvcc is None or shutil.which("c++filt") is None:
        pytest.skip("nvcc or c++filt not available")
    src = build.CSRC / "sweep_mixed.cu"
    cmd = [nvcc, *build.ARCH, "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
           "-fmad=true", "-Xptxas", "-v", "-c", str(src), "-o", str(tmp_path / "sweep_mixed.o")]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    table = {}
    for block in re.split(r"ptxas info\s*: Compiling entry function '", r.stdout + r.stderr)[1:]:
        name = block.split("'", 1)[0]
        spill = re.search(r"(\d+) bytes spill stores", block)
        regs = re.search(r"Used (\d+) registers", block)
        if spill and regs:
            table[name] = (int(regs.group(1)), int(spill.group(1)))
    names = subprocess.run(["c++filt"], input="\n".join(table), capture_output=True, text=True).stdout.split("\n")
    return {dem.split("(")[0].replace("void ", ""): v for dem, v in zip(names, table.values())}


def shape(variant: int) -> str:
    """Template arguments of a lockstep variant number."""
    streaming, words_ahead = variant >= 1000 and variant < 2000, variant >= 2000
    v = variant % 1000
    if v < 100:  # 83 and 84 name 183 and 184
        v += 100
    prefetch, lanes, blocks = v // 100, (v // 10) % 10, v % 10
    lanes = 16 if lanes == 6 else lanes
    return (f"swk::k_sweep_pull_lockg<{blocks}, {lanes}, {prefetch}, {str(streaming).lower()}, "
            f"{str(words_ahead).lower()}>")


def test_transport_kernels_do_not_spill(tmp_path):
    table = ptxas_table(tmp_path)
    lockg = {k: v for k, v in table.items() if "k_sweep_pull_lockg" in k}
    assert len(lockg) >= 16, sorted(table)
    # the default shape (143) and the 2-lane candidate (122) keep everything in registers
    for variant in (143, 122):
        regs, spill = lockg[shape(variant)]
        assert spill == 0, (variant, regs, spill)
    for name, (regs, spill) in lockg.items():
        assert regs <= 255 and spill <= MAX_SPILL_BYTES, (name, regs, spill)
    for name in ("swk::k_sweep_pull_geo<1>", "swk::k_sweep_pull_wave<2>", "swk::k_sweep_pull_staged"):
        assert table[name][1] == 0, (name, table[name])
