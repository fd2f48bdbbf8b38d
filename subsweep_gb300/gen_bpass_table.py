"""Generate bpass_table.py from the reference's BPASS table.

The ionizing photon output per solar mass of a simple stellar population, by age and
metallicity, is a fixed data table in the reference (src/arepo_postprocess/bpass.rs:58-886,
from the BPASS population synthesis models).  Source rates must match the reference's,
so this script copies the numeric literals verbatim into a Python module (Python and
Rust both round decimal literals to the nearest double).  Run it where the reference
checkout is available:

    python subsweep_gb300/gen_bpass_table.py /path/to/subsweep
"""
import pathlib
import re
import sys

NUMBER = r"[-0-9.eE+]+"


def parse(text):
    def const(name):
        m = re.search(rf"const {name}: [^=]+= \[(.*?)\];", text, re.S)
        assert m, name
        return m.group(1)

    ages = re.findall(NUMBER, const("BPASS_AGE_BINS"))
    metallicities = re.findall(NUMBER, const("BPASS_METALLICITY_BINS"))
    rows = [re.findall(NUMBER, r) for r in re.findall(r"\[(.*?)\]", const("BPASS_TABLE"), re.S)]
    n_ages = int(re.search(r"const NUM_BPASS_AGES: usize = (\d+);", text).group(1))
    n_met = int(re.search(r"const NUM_BPASS_METALLICITIES: usize = (\d+);", text).group(1))
    assert len(ages) == n_ages and len(metallicities) == n_met and len(rows) == n_ages
    assert all(len(r) == n_met for r in rows)
    return ages, metallicities, rows


def wrap(numbers, per_line=6, indent=4):
    return [" " * indent + ", ".join(numbers[i:i + per_line]) + ","
            for i in range(0, len(numbers), per_line)]


def main():
    ref = pathlib.Path(sys.argv[1] if len(sys.argv) > 1 else ".")
    ages, metallicities, rows = parse((ref / "src/arepo_postprocess/bpass.rs").read_text())
    out = ['"""BPASS ionizing photon output per solar mass (photons/s) of a simple stellar',
           "population by age (years) and metallicity, as src/arepo_postprocess/bpass.rs holds it.",
           "Generated by gen_bpass_table.py; do not edit.",
           '"""',
           "",
           "AGE_BINS = ("] + wrap(ages) + [")",
           "METALLICITY_BINS = ("] + wrap(metallicities) + [")",
           "TABLE = ("]
    for r in rows:
        out += ["    ("] + wrap(r, per_line=5, indent=8) + ["    ),"]
    out += [")", ""]
    dst = pathlib.Path(__file__).resolve().parent / "bpass_table.py"
    dst.write_text("\n".join(out))
    print(f"{dst}: {len(ages)} ages x {len(metallicities)} metallicities")


if __name__ == "__main__":
    main()
