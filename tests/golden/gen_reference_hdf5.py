"""Copy the reference's HDF5 input fixtures into tests/golden/hdf5/.

The reference's dataset-input tests (src/io/input/tests.rs:23-50) read two small files
written by its own output code (hdf5-rust, classic file format):

* tests/input/respect_scale_factor.hdf5: one `mass` value of 1 solar mass (1.988477e30 kg)
  with `scale_factor_si` 5, which must read as 5 solar masses;
* tests/input/panic_on_dimension_mismatch.hdf5: the same dataset with `scaling_length` 1,
  which must fail with "Mismatch in dimension while reading dataset mass."

The files are data, copied byte for byte; tests/test_hdf5.py holds the expectations.

Usage: python tests/golden/gen_reference_hdf5.py /path/to/subsweep
"""
import hashlib
import pathlib
import shutil
import sys

FILES = ("respect_scale_factor.hdf5", "panic_on_dimension_mismatch.hdf5")


def main():
    ref = pathlib.Path(sys.argv[1] if len(sys.argv) > 1 else ".")
    out = pathlib.Path(__file__).resolve().parent / "hdf5"
    out.mkdir(exist_ok=True)
    for name in FILES:
        shutil.copyfile(ref / "tests" / "input" / name, out / name)
        print(name, hashlib.sha256((out / name).read_bytes()).hexdigest())


if __name__ == "__main__":
    main()
