"""The Rust binding shown in INTEGRATION.md against the C header, on the CPU.

No Rust toolchain exists here, so the `extern "C"` block a maintainer would paste into
the reference (`src/sweep/gpu.rs`) is checked as text: it declares every entry point of
include/subsweep_gpu.h with the header's argument count and return kind, and each
`#[repr(C)]` struct lists the fields of its ctypes mirror (subsweep_gb300/_native.py,
itself held against the C layouts by tests/test_abi_consumer.py) in the same order and
with the same sizes.
"""
import ctypes
import pathlib
import re

from subsweep_gb300 import _native

ROOT = pathlib.Path(__file__).resolve().parents[1]

RUST_SIZES = {"i32": 4, "i64": 8, "u8": 1, "f64": 8, "usize": 8}
MIRRORS = {"SwParams": _native.SwParams, "SwGridCsr": _native.SwGridCsr, "SwCellInit": _native.SwCellInit,
           "SwTimeSeries": _native.SwTimeSeries, "SwStats": _native.SwStats}


def _rust_block() -> str:
    text = (ROOT / "INTEGRATION.md").read_text()
    blocks = re.findall(r"```rust\n(.*?)```", text, re.S)
    ffi = [b for b in blocks if 'extern "C"' in b]
    assert len(ffi) == 1
    return ffi[0]


def _rust_size(ty: str) -> int:
    ty = ty.strip()
    return 8 if ty.startswith("*") else RUST_SIZES[ty]


def _split_args(args: str):
    return [a for a in (x.strip() for x in args.replace("\n", " ").split(",")) if a]


def test_rust_structs_match_the_mirrors():
    block = _rust_block()
    structs = dict(re.findall(r"#\[repr\(C\)\] pub struct (\w+) \{(.*?)\n\}", block, re.S))
    assert set(structs) == set(MIRRORS)
    for name, body in structs.items():
        fields = re.findall(r"pub (\w+): ([^,\n]+)", body)
        mirror = MIRRORS[name]
        assert [f for f, _ in fields] == [f for f, _ in mirror._fields_], name
        for (field, ty), (_, cty) in zip(fields, mirror._fields_):
            assert _rust_size(ty) == ctypes.sizeof(cty), (name, field, ty)


def test_rust_functions_match_the_header():
    block = _rust_block()
    rust = {name: (_split_args(args), ret.strip())
            for name, args, ret in re.findall(r"pub fn (\w+)\((.*?)\)\s*(->[^;]*)?;", block, re.S)}
    header = (ROOT / "include" / "subsweep_gpu.h").read_text()
    header = re.sub(r"/\*.*?\*/", "", header, flags=re.S)
    protos = {name: (ret.strip(), _split_args(args))
              for ret, name, args in re.findall(r"^([\w ]+?\**)\s*(sw_\w+)\(([^;]*?)\);", header, re.S | re.M)}
    assert set(rust) == set(protos) == set(_native.ABI_SYMBOLS)
    for name, (args, ret) in rust.items():
        cret, cargs = protos[name]
        n_c = 0 if cargs == ["void"] else len(cargs)
        assert len(args) == n_c, name
        if cret == "sw_status":
            assert ret == "-> i32", name
        elif cret == "void":
            assert ret == "", name
        else:
            assert cret.startswith("const char") and ret.endswith("c_char"), name
