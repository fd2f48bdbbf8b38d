"""Generate direction_bins.inc from the reference's direction tables.

The sweep's direction sets for `directions: <num>` are fixed data tables in the
reference (src/sweep/direction/healpix.rs, selected by Directions::from_num in
src/sweep/direction/mod.rs:58-75).  Parity requires the identical vectors, so
this script copies the numeric literals verbatim (C and Rust both round decimal
literals to the nearest double) into a C include file.  Run it where the
reference checkout is available:

    python subsweep_gb300/csrc/gen_direction_bins.py /path/to/subsweep
"""
import pathlib
import re
import sys


def parse_tables(text):
    tables = {}
    for m in re.finditer(r"pub const DIRECTION_BINS_(\d+): \[\[f64; 3\]; (\d+)\] = \[(.*?)\];",
                         text, re.S):
        num = int(m.group(1))
        rows = re.findall(r"\[\s*([-0-9.eE+]+)\s*,\s*([-0-9.eE+]+)\s*,\s*([-0-9.eE+]+)\s*\]",
                          m.group(3))
        assert len(rows) == num == int(m.group(2)), (num, len(rows))
        tables[num] = rows
    return tables


def main():
    ref = pathlib.Path(sys.argv[1] if len(sys.argv) > 1 else ".")
    text = (ref / "src/sweep/direction/healpix.rs").read_text()
    tables = parse_tables(text)
    out = ["/* Generated by gen_direction_bins.py from the reference's direction tables",
           " * (src/sweep/direction/healpix.rs).  Do not edit. */"]
    for num in sorted(tables):
        out.append(f"static const double kDirectionBins{num}[{num}][3] = {{")
        for x, y, z in tables[num]:
            out.append(f"    {{{x}, {y}, {z}}},")
        out.append("};")
    dest = pathlib.Path(__file__).with_name("direction_bins.inc")
    dest.write_text("\n".join(out) + "\n")
    print(f"wrote {dest} with tables {sorted(tables)}")


if __name__ == "__main__":
    main()
