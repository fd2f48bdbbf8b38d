"""CUDA sweep library vs the CPU FP64 oracle on the same seeded inputs.

Bars: dependency counts, level assignments and per-level cell counts bit-exact; the
FP64 drop-in within 1e-10 relative in x_HII and T and in the photon rates (absolute
floor 1e-12 of the largest rate: rates below it are exponential-tail values whose
threshold decisions may legitimately flip); the mixed path within max |dx_HII| <= 1e-4
and relative T error <= 1e-4.
"""
import numpy as np
import pytest

from oracle import binding
from subsweep_gb300 import _native, directions_from_num, grid as gridmod, workloads
from subsweep_gb300.sweep import MEGAYEAR, Sweep, SweepError, SweepParameters, mass_density_from_number_density

pytestmark = pytest.mark.gpu

X_RTOL = 1e-10
T_RTOL = 1e-10
RATE_RTOL = 1e-10


def oracle_dirs(params):
    if isinstance(params.directions, int):
        return directions_from_num(params.directions)
    v = np.asarray(params.directions, np.float64)
    inv = 1.0 / np.sqrt((v[:, 0] * v[:, 0] + v[:, 1] * v[:, 1]) + v[:, 2] * v[:, 2])
    return v * inv[:, None]


def make_pair(w, precision="fp64", mode=binding.PERIODIC_SNAPSHOT):
    args = (w.params, w.grid, w.density, w.ionized_hydrogen_fraction, w.temperature, w.source)
    gpu = Sweep(*args, precision=precision)
    orc = binding.OracleSweep(*args, oracle_dirs(w.params), periodic_mode=mode)
    return gpu, orc


def assert_rates_close(a, b, rtol):
    scale = max(np.abs(b).max(), 1e-300)
    np.testing.assert_allclose(a, b, rtol=rtol, atol=1e-12 * scale)


def compare_fp64(gpu, orc, rates=True):
    fg, fo = gpu.fields(), orc.fields()
    np.testing.assert_array_equal(gpu.cell_state()["level"], fo["level"])
    np.testing.assert_array_equal(gpu.level_counts(), orc.level_counts())
    np.testing.assert_allclose(fg["ionized_hydrogen_fraction"], fo["ionized_hydrogen_fraction"], rtol=X_RTOL)
    np.testing.assert_allclose(fg["temperature"], fo["temperature"], rtol=T_RTOL)
    np.testing.assert_allclose(fg["timestep"], fo["timestep"], rtol=1e-8)
    if rates:
        assert_rates_close(fg["photon_rate"], fo["photon_rate"], RATE_RTOL)
        rg, ro = gpu.rates(), orc.rates()
        for k in ("incoming", "outgoing", "periodic"):
            assert_rates_close(rg[k], ro[k], RATE_RTOL)


def run_and_compare(w, steps, check_counts=True):
    gpu, orc = make_pair(w)
    for step in range(steps):
        if check_counts:
            for level in range(w.params.num_timestep_levels):
                np.testing.assert_array_equal(gpu.dependency_counts(level), orc.dependency_counts(level),
                                              err_msg=f"step {step} level {level}")
        te_g, te_o = gpu.run_sweeps(), orc.run_sweeps()
        assert te_g == te_o
        compare_fp64(gpu, orc)
    tasks, chem = orc.work()
    st = gpu.stats()
    assert st["tasks"] == tasks and st["chem_cells"] == chem
    return gpu, orc


def test_c1_small_fp64_parity():
    w = workloads.c1_small_periodic(n_per_side=10, num_directions=84, nthreads=2)
    run_and_compare(w, steps=4)


@pytest.mark.parametrize("transport,records", [("levels", "1"), ("levels", "0"), ("queue", "0")])
def test_c2_small_lognormal_levels_fp64_parity(transport, records, monkeypatch):
    """Both transport kernels: the levelled schedule (over the precomputed downwind
    fractions, or computing the geometry on the fly) and the dependency-driven queue."""
    monkeypatch.setenv("SUBSWEEP_TRANSPORT", transport)
    monkeypatch.setenv("SUBSWEEP_FP64_RECORDS", records)
    w = workloads.c2_lognormal(n_per_side=12, num_directions=84, num_levels=4, nthreads=2, thick=True)
    gpu, orc = run_and_compare(w, steps=6)
    # the level hierarchy must actually be exercised
    assert len(np.unique(orc.fields()["level"])) > 1
    st = gpu.stats()
    assert (st["levelled_sweeps"] > 0) == (transport == "levels")
    assert st["schedule_levels"] > 0


def test_cartesian_column_analytic():
    w = workloads.cartesian_column(32, 1e3 * 3.0857e16, 5e-5, 1e50)
    run_and_compare(w, steps=3)


def test_walled_voronoi_boundary_faces():
    box = 3.0857e22 / 8
    pts = gridmod.poisson_points(700, box, 21)
    g = gridmod.voronoi(pts, box, periodic=False, nthreads=2)
    n = g.num_cells
    src = gridmod.place_sources(g, np.array([[box * 0.3, box * 0.6, box * 0.5]]), np.array([3e49]))
    params = SweepParameters(directions=32, num_timestep_levels=2, periodic=False, max_timestep=0.5 * MEGAYEAR,
                             significant_rate_threshold=1e-5)
    w = workloads.Workload("walled", params, g, np.full(n, float(mass_density_from_number_density(1e-3))),
                           np.full(n, 1e-10), np.full(n, 1e4), src, steps=3)
    run_and_compare(w, steps=3)


def test_explicit_directions_and_no_prevent_cooling():
    w = workloads.c1_small_periodic(n_per_side=7, num_directions=16, nthreads=2)
    w.params.directions = [[1.0, 0.2, 0.1], [-0.3, 1.0, 0.0], [0.0, -0.5, -2.0]]
    w.params.prevent_cooling = False
    run_and_compare(w, steps=3)


def test_zero_sources_and_threshold():
    w = workloads.c1_small_periodic(n_per_side=6, num_directions=16, nthreads=2)
    w.source[:] = 0.0
    run_and_compare(w, steps=2)


def test_poisson_periodic_fp64_parity():
    box = 3.0857e22 / 4
    pts = gridmod.poisson_points(900, box, 5)
    g = gridmod.voronoi(pts, box, periodic=True, nthreads=2)
    n = g.num_cells
    rng = np.random.default_rng(9)
    src = gridmod.place_sources(g, rng.uniform(0, box, (3, 3)), np.array([1e48, 5e48, 1e49]))
    params = SweepParameters(directions=32, num_timestep_levels=3, periodic=True, max_timestep=MEGAYEAR)
    w = workloads.Workload("poisson", params, g, np.full(n, float(mass_density_from_number_density(3e-4))),
                           np.full(n, 1e-10), np.full(n, 1e4), src, steps=4)
    run_and_compare(w, steps=4)


def test_dependency_cycle_reports_stalled_not_hang():
    """A cyclic dependency graph (which deadlocks the reference) ends the GPU sweep with
    SW_ERR_STALLED after the bounded wait for the never-filled queue slots."""
    from tests.test_abi import _cyclic_grid
    g = _cyclic_grid()
    n = g.num_cells
    p = SweepParameters(directions=[[0.0, 0.0, 1.0]], num_timestep_levels=1, periodic=False, max_timestep=1.0)
    s = Sweep(p, g, density=np.full(n, 1e-24), ionized_hydrogen_fraction=np.full(n, 1e-10),
              temperature=np.full(n, 1e4), source=np.zeros(n))
    assert s.stats()["schedule_levels"] == 0  # no levelled schedule for a cyclic graph
    with pytest.raises(SweepError) as e:
        s.run_sweeps()
    assert e.value.status == _native.SW_ERR_STALLED
    s.close()


def test_mixed_precision_error_bounds():
    """Pull-form FP32 transport + FP64 chemistry against the FP64 oracle."""
    w = workloads.c2_lognormal(n_per_side=12, num_directions=84, num_levels=4, nthreads=2)
    gpu, orc = make_pair(w, precision="mixed")
    for _ in range(6):
        assert gpu.run_sweeps() == orc.run_sweeps()
    fg, fo = gpu.fields(), orc.fields()
    dx = np.abs(fg["ionized_hydrogen_fraction"] - fo["ionized_hydrogen_fraction"]).max()
    dt = (np.abs(fg["temperature"] - fo["temperature"]) / fo["temperature"]).max()
    assert dx <= 1e-4, dx
    assert dt <= 1e-4, dt


def test_mixed_compaction_and_in_kernel_stamping_agree(monkeypatch):
    """Sweeps above level 0 either compact the active positions (stamping the inactive
    tasks' words in the compaction) or stamp them in the sweep kernel.  The two paths
    compute the same sums in the same order: fields and every rate agree bit for bit."""
    w = workloads.c2_lognormal(n_per_side=12, num_directions=32, num_levels=4, nthreads=2, thick=True)
    out = {}
    for mode in ("always", "never"):
        monkeypatch.setenv("SUBSWEEP_COMPACT", mode)
        gpu = Sweep(w.params, w.grid, w.density, w.ionized_hydrogen_fraction, w.temperature, w.source,
                    precision="mixed")
        for _ in range(6):
            gpu.run_sweeps()
        assert gpu.level_counts()[1:].min() > 0, "every level populated"
        out[mode] = (gpu.fields(), gpu.rates(), gpu.cell_state()["level"])
        gpu.close()
    (fa, ra, la), (fb, rb, lb) = out["always"], out["never"]
    np.testing.assert_array_equal(la, lb)
    for k in fa:
        np.testing.assert_array_equal(fa[k], fb[k], err_msg=k)
    for k in ra:
        np.testing.assert_array_equal(ra[k], rb[k], err_msg=k)


def test_mixed_precision_c1_rates_and_periodic():
    """Pull-form rates (incoming, outgoing, periodic, PhotonRate) against the oracle's
    push-form ones on a periodic box with an ionization front, within FP32 accuracy."""
    w = workloads.c1_small_periodic(n_per_side=10, num_directions=84, nthreads=2)
    gpu, orc = make_pair(w, precision="mixed")
    for _ in range(3):
        assert gpu.run_sweeps() == orc.run_sweeps()
    fg, fo = gpu.fields(), orc.fields()
    assert np.abs(fg["ionized_hydrogen_fraction"] - fo["ionized_hydrogen_fraction"]).max() <= 1e-4
    assert (np.abs(fg["temperature"] - fo["temperature"]) / fo["temperature"]).max() <= 1e-4
    # FP32 rates are stored in units of 2^-96 of the total source, so exponential-tail
    # rates below ~1e-20 of the total luminosity are not represented (flushed to zero)
    floor = 1e-20 * w.source.sum()
    np.testing.assert_allclose(fg["photon_rate"], fo["photon_rate"], rtol=1e-4, atol=floor)
    rg, ro = gpu.rates(), orc.rates()
    for k in ("incoming", "outgoing", "periodic"):
        np.testing.assert_allclose(rg[k], ro[k], rtol=1e-4, atol=floor, err_msg=k)


def test_mixed_precision_cycle_reports_stalled():
    from tests.test_abi import _cyclic_grid
    g = _cyclic_grid()
    n = g.num_cells
    p = SweepParameters(directions=[[0.0, 0.0, 1.0]], num_timestep_levels=1, periodic=False, max_timestep=1.0)
    s = Sweep(p, g, density=np.full(n, 1e-24), ionized_hydrogen_fraction=np.full(n, 1e-10),
              temperature=np.full(n, 1e4), source=np.zeros(n), precision="mixed")
    with pytest.raises(SweepError) as e:
        s.run_sweeps()
    assert e.value.status == _native.SW_ERR_STALLED
    s.close()


REFERENCE_SWEEP_CASES = [
    # src/sweep/tests.rs:89-114 (`simple_sweep`): 10^3 cartesian cells of 0.1 m, direction
    # (1, 1, 1), 1-2 timestep levels, walled or periodic
    (10, (1.0, 1.0, 1.0), 1, False, 0.0), (10, (1.0, 1.0, 1.0), 2, False, 0.0),
    (10, (1.0, 1.0, 1.0), 1, True, 0.0), (10, (1.0, 1.0, 1.0), 2, True, 0.0),
    # src/sweep/tests.rs:116-133: 5^3 cells swept along +x (faces parallel to the direction)
    (5, (1.0, 0.0, 0.0), 1, False, 0.0),
    # the same set-ups with a source in one cell, so that the transport is not trivial
    (10, (1.0, 1.0, 1.0), 2, True, 1e30), (5, (1.0, 0.0, 0.0), 1, False, 1e30),
]


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("n,direction,levels,periodic,source", REFERENCE_SWEEP_CASES)
def test_reference_sweep_setups(precision, n, direction, levels, periodic, source):
    """The reference's own sweep tests (ignored there; they assert only that the sweep
    neither deadlocks nor crashes): the same grids, parameters and initial conditions
    (`initialize_sweep_test_components_system`, src/sweep/mod.rs:783-797: 1e-10 kg/cm^3,
    x = 1e-10, T = 1000 K; safety factors 0, max timestep 1 ms, no cooling floor), run
    through the C ABI against the oracle."""
    g = gridmod.cartesian(n, n, n, 0.1, periodic)
    cells = g.num_cells
    p = SweepParameters(directions=[list(direction)], num_timestep_levels=levels, periodic=periodic,
                        max_timestep=1e-3, timestep_safety_factor=0.0, chemistry_timestep_safety_factor=0.0,
                        prevent_cooling=False, significant_rate_threshold=0.0)
    density = np.full(cells, 1e-10 / 1e-6)
    src = np.zeros(cells)
    src[0] = source
    args = (p, g, density, np.full(cells, 1e-10), np.full(cells, 1000.0), src)
    gpu = Sweep(*args, precision=precision)
    orc = binding.OracleSweep(*args, oracle_dirs(p))
    for _ in range(2):
        assert gpu.run_sweeps() == orc.run_sweeps()
    if precision == "fp64":
        compare_fp64(gpu, orc)
    else:
        fg, fo = gpu.fields(), orc.fields()
        np.testing.assert_array_equal(gpu.cell_state()["level"], fo["level"])
        assert np.abs(fg["ionized_hydrogen_fraction"] - fo["ionized_hydrogen_fraction"]).max() <= 1e-4
        assert (np.abs(fg["temperature"] - fo["temperature"]) / fo["temperature"]).max() <= 1e-4
    gpu.close()
