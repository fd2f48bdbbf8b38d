"""The GPU Voronoi producer (csrc/voronoi_gpu.cu) against the host producer.

Both clip a bounding polyhedron by bisector planes of nearby generators in distance
order; the GPU takes its candidates from bucket shells starting one shell closer, so
the clipping order, and the last bits of vertex positions, can differ.  Bars: the same
CSR topology (row pointers, neighbours, kinds) and normals bit for bit (they come from
generator differences), areas, volumes and sizes to 1e-10 relative.
"""
import time

import numpy as np
import pytest

from subsweep_gb300 import grid as gridmod

pytestmark = pytest.mark.gpu


def cases():
    rng = np.random.default_rng(4)
    yield "jittered periodic 8^3", gridmod.jittered_lattice(8, 1.0, 0.25, 3), 1.0, True
    yield "jittered periodic 13^3", gridmod.jittered_lattice(13, 2.0, 0.25, 5), 2.0, True
    yield "poisson walled 700", rng.random((700, 3)) * 3.0, 3.0, False
    yield "poisson periodic 900", rng.random((900, 3)) * 1.5, 1.5, True


@pytest.mark.parametrize("name,pts,box,periodic", list(cases()), ids=[c[0] for c in cases()])
def test_gpu_voronoi_matches_host(name, pts, box, periodic):
    h = gridmod.voronoi(pts, box, periodic=periodic, nthreads=2)
    g = gridmod.voronoi_gpu(pts, box, periodic=periodic)
    np.testing.assert_array_equal(g.row_ptr, h.row_ptr)
    np.testing.assert_array_equal(g.nbr, h.nbr)
    np.testing.assert_array_equal(g.kind, h.kind)
    np.testing.assert_array_equal(g.normal, h.normal)
    np.testing.assert_allclose(g.area, h.area, rtol=1e-10)
    np.testing.assert_allclose(g.volume, h.volume, rtol=1e-10)
    np.testing.assert_allclose(g.size, h.size, rtol=1e-10)
    assert np.isclose(g.volume.sum(), np.prod(np.broadcast_to(box, 3)), rtol=1e-9)


def test_gpu_voronoi_64_cubed_timing():
    """A C2-sized lattice (64^3): topology equal to the host producer's; prints both times."""
    pts = gridmod.jittered_lattice(64, 2.0, 0.25, 2)
    t0 = time.perf_counter()
    g = gridmod.voronoi_gpu(pts, 2.0, periodic=True)
    t_gpu = time.perf_counter() - t0
    t0 = time.perf_counter()
    h = gridmod.voronoi(pts, 2.0, periodic=True)
    t_host = time.perf_counter() - t0
    print(f"64^3 Voronoi: GPU {t_gpu:.2f} s, host {t_host:.2f} s")
    np.testing.assert_array_equal(g.row_ptr, h.row_ptr)
    np.testing.assert_array_equal(g.nbr, h.nbr)
    np.testing.assert_allclose(g.area, h.area, rtol=1e-10)
