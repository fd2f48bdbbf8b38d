"""Extract the reference's known-answer tests for the sweep path into JSON fixtures.

Reads the reference's own test code (Rust source, parsed as text; nothing is run)
and writes tests/golden/reference_kats.json:

* timestep_level:  check_level(max_num_levels, secs_desired, result) cases of
                   src/sweep/timestep_level.rs (tests module)
* sweep_order:     the level sequences of iter_levels_in_sweep_order_advances_properly
                   and the lowest-allowed sequence of lowest_allowed
                   (src/sweep/timestep_state.rs tests)
* derivative_test: temperatures, step and tolerance of test_numerical_derivative
                   (src/chemistry/hydrogen_only/mod.rs tests)
* solver_extremes: inputs of fully_ionized_solver / fully_neutral_solver
* voronoi_kat:     points and expected geometry of right_volume_and_face_areas_three_d
                   (src/voronoi/mod.rs tests)
* direction_tables: SHA-256 of each direction table as little-endian doubles
* bpass:           the check_is_close cases and tolerance of the BPASS lookup test
                   (src/arepo_postprocess/bpass.rs tests)
* cosmology:       the parameters and bounds of time_difference_between_scalefactors and
                   get_scalefactor_from_scalefactor_and_time_difference (src/cosmology.rs tests)

Usage: python tests/golden/gen_reference_kats.py /path/to/subsweep
"""
import hashlib
import json
import pathlib
import re
import struct
import sys


def rust_float(s):
    return float(s.replace("_", ""))


def main():
    ref = pathlib.Path(sys.argv[1] if len(sys.argv) > 1 else ".")
    out = {}

    src = (ref / "src/sweep/timestep_level.rs").read_text()
    out["timestep_level"] = [
        {"max_num_levels": int(a), "max_timestep": 1.0, "desired": rust_float(b), "level": int(c)}
        for a, b, c in re.findall(r"check_level\((\d+),\s*([0-9.eE+-]+),\s*(\d+)\)", src)]

    src = (ref / "src/sweep/timestep_state.rs").read_text()
    m = re.search(r"TimestepState::new\(Time::megayears\(1\.0\), (\d+)\);\s*let mut get_next", src)
    n_levels = int(m.group(1))
    seqs = []
    for body in re.findall(r"get_next_levels_iter\(\),\s*&\[([0-9,\s]*)\]", src):
        seqs.append([int(v) for v in body.replace("\n", " ").split(",") if v.strip()])
    lowest = [int(v) for v in re.findall(r"current_lowest_allowed, TimestepLevel\((\d+)\)", src)]
    out["sweep_order"] = {"num_levels": n_levels, "orders_after_advances": seqs,
                          "lowest_allowed_after_advances": lowest}

    src = (ref / "src/chemistry/hydrogen_only/mod.rs").read_text()
    eps = rust_float(re.search(r"let epsilon = ([0-9.eE+-]+);", src).group(1))
    delta = rust_float(re.search(r"let delta = Temperature::kelvins\(([0-9.eE+-]+)\);", src).group(1))
    block = re.search(r"for temperature in \[(.*?)\]", src, re.S).group(1)
    temps = [rust_float(t) for t in re.findall(r"Temperature::kelvins\(([0-9.eE+-]+)\)", block)]
    pairs = re.findall(r"test_numerical_derivative\(\s*Solver::(\w+),\s*Solver::(\w+),?\s*\)", src)
    out["derivative_test"] = {"epsilon": eps, "delta": delta, "temperatures": temps,
                              "pairs": [list(p) for p in pairs]}
    extremes = {}
    for name in ("fully_ionized_solver", "fully_neutral_solver"):
        body = re.search(r"fn " + name + r"\(\) \{(.*?)\n    \}", src, re.S).group(1)
        extremes[name] = {
            "ionized_hydrogen_fraction": rust_float(re.search(r"ionized_hydrogen_fraction: ([0-9.eE+-]+)\.into\(\)", body).group(1)),
            "temperature_K": rust_float(re.search(r"Temperature::kelvins\(([0-9.eE+-]+)\)", body).group(1)),
            "density_g_per_cm3": rust_float(re.search(r"grams_per_cubic_centimeters\(\s*([0-9.eE+-]+),?\s*\)", body).group(1)),
            "volume_m3": rust_float(re.search(r"Volume::cubic_meters\(\s*([0-9.eE+-]+),?\s*\)", body).group(1)),
            "length_kpc": rust_float(re.search(r"Length::kiloparsec\(([0-9.eE+-]+)\)", body).group(1)),
            "rate_per_s": rust_float(re.search(r"photons_per_second\(([0-9.eE+-]+)\)", body).group(1)),
            "scale_factor": rust_float(re.search(r"scale_factor: ([0-9.eE+-]+)\.into\(\)", body).group(1)),
            "timestep_Myr": rust_float(re.search(r"perform_timestep\(Time::megayears\(([0-9.eE+-]+)\)", body).group(1)),
            "safety": rust_float(re.search(r", ([0-9.eE+-]+)\.into\(\)\);", body).group(1)),
        }
    out["solver_extremes"] = extremes

    src = (ref / "src/voronoi/mod.rs").read_text()
    body = re.search(r"fn right_volume_and_face_areas_three_d\(\) \{(.*?)\n    \}", src, re.S).group(1)
    pts = [[rust_float(a), rust_float(b), rust_float(c)] for a, b, c in
           re.findall(r"Point3d::new\(([0-9.eE+-]+), ([0-9.eE+-]+), ([0-9.eE+-]+)\)", body)]
    vol = rust_float(re.search(r"cell\.volume\(\), ([0-9.eE+-]+)\)", body).group(1))
    faces = []
    for nb, rest in re.findall(r"ParticleId::test\((\d+)\)\) \{(.*?)\}", body, re.S):
        area = rust_float(re.search(r"face\.area, ([0-9.eE+-]+)\)", rest).group(1))
        comps = re.findall(r"face\.normal\.([xyz]), (-?\(1\.0f64 / 3\.0\)\.sqrt\(\)|[0-9.eE+-]+)\)", rest)
        normal = []
        for _, v in comps:
            normal.append(-(1.0 / 3.0) ** 0.5 if "sqrt" in v else rust_float(v))
        faces.append({"neighbour": int(nb), "area": area, "normal": normal})
    out["voronoi_kat"] = {"points": pts, "cell": len(pts) - 1, "volume": vol, "faces": faces}

    src = (ref / "src/sweep/direction/healpix.rs").read_text()
    tables = {}
    for num, body in re.findall(r"DIRECTION_BINS_(\d+): \[\[f64; 3\]; \d+\] = \[(.*?)\];", src, re.S):
        vals = [float(v) for v in re.findall(r"-?[0-9.]+(?:[eE][-+]?\d+)?", body)]
        tables[num] = hashlib.sha256(struct.pack("<%dd" % len(vals), *vals)).hexdigest()
    tables["1"] = hashlib.sha256(struct.pack("<3d", 1.0, 0.0, 0.0)).hexdigest()
    out["direction_tables"] = tables

    src = (ref / "src/arepo_postprocess/bpass.rs").read_text()
    tests = src[src.index("#[cfg(test)]"):]
    tol = re.search(r"\(\(x - y\) / \(x\.abs\(\) \+ y\.abs\(\)\)\)\.abs\(\) < ([0-9.eE+-]+)", tests)
    out["bpass"] = {
        "relative_tolerance": rust_float(tol.group(1)),
        "cases": [{"age_years": rust_float(a), "metallicity": rust_float(m), "photons_per_s": rust_float(v)}
                  for a, m, v in re.findall(r"check_is_close\(([0-9.eE+-]+),\s*([0-9.eE+-]+),\s*([0-9.eE+-]+)\)",
                                            tests)]}
    assert len(out["bpass"]["cases"]) == 3

    src = (ref / "src/cosmology.rs").read_text()
    tests = src[src.index("#[cfg(test)]"):]
    ol = re.search(r"omega_lambda: ([0-9.]+)", tests).group(1)
    o0 = re.search(r"omega_0: ([0-9.]+)", tests).group(1)
    h = re.search(r"\(cosmology, ([0-9.]+)\.into\(\)\)", tests).group(1)
    diff = re.search(r"diff\(([0-9.]+), ([0-9.]+)\) - Time::gigayears\(([0-9.]+)\)\)\.abs\(\) < Time::years\(([0-9.]+)\)",
                     tests)
    grid = re.search(r"for a0 in \[([0-9., ]+)\]", tests).group(1)
    tol = re.search(r"assert!\(diff < ([0-9.eE+-]+)\)", tests).group(1)
    out["cosmology"] = {
        "omega_lambda": float(ol), "omega_0": float(o0), "h": float(h),
        "time_difference": {"a0": float(diff.group(1)), "a1": float(diff.group(2)),
                            "gigayears": float(diff.group(3)), "tolerance_years": float(diff.group(4))},
        "round_trip_scale_factors": [float(v) for v in grid.split(",")],
        "round_trip_tolerance": rust_float(tol)}

    dest = pathlib.Path(__file__).with_name("reference_kats.json")
    dest.write_text(json.dumps(out, indent=1) + "\n")
    print(f"wrote {dest}")


if __name__ == "__main__":
    main()
