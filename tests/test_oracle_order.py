"""The oracle's task order, threads and grid producer.

* The task heap is the oracle's restatement of the reference's queue, Rust's
  std::collections::BinaryHeap<Task> with Task ordered by direction only
  (src/sweep/mod.rs:104, task.rs:25-35).  It is held against a second, independent
  transcription of the standard library's published algorithm written here in Python
  (FromIterator -> rebuild by sift_down; push -> sift_up; pop -> swap the last element
  into the root, sift_down_to_bottom, sift_up), on operation sequences full of equal
  keys, where the algorithm alone decides the order.
* Threads split a level sweep's directions; in FIFO order results do not depend on
  their count.
* The oracle's Voronoi producer (voronoi_oracle.cpp) and the library's host producer
  are two implementations of one tessellation: same faces, same normals bit for bit,
  areas and volumes to rounding.
"""
import numpy as np
import pytest

from oracle import binding
from subsweep_gb300 import grid as gridmod
from subsweep_gb300 import workloads


class StdBinaryHeap:
    """Rust's BinaryHeap (library/alloc/src/collections/binary_heap/mod.rs) over
    (key, payload) pairs compared by key alone."""

    def __init__(self, items):
        self.data = list(items)
        n = len(self.data) // 2
        while n > 0:
            n -= 1
            self._sift_down_range(n, len(self.data))

    def push(self, item):
        self.data.append(item)
        self._sift_up(0, len(self.data) - 1)

    def pop(self):
        item = self.data.pop()
        if self.data:
            item, self.data[0] = self.data[0], item
            self._sift_down_to_bottom(0)
        return item

    def _sift_up(self, start, pos):
        elem = self.data[pos]
        while pos > start:
            parent = (pos - 1) // 2
            if elem[0] <= self.data[parent][0]:
                break
            self.data[pos] = self.data[parent]
            pos = parent
        self.data[pos] = elem

    def _sift_down_range(self, pos, end):
        elem = self.data[pos]
        child = 2 * pos + 1
        while child <= max(end - 2, 0) and child + 1 < end:
            if self.data[child][0] <= self.data[child + 1][0]:
                child += 1
            if elem[0] >= self.data[child][0]:
                self.data[pos] = elem
                return
            self.data[pos] = self.data[child]
            pos = child
            child = 2 * pos + 1
        if child == end - 1 and elem[0] < self.data[child][0]:
            self.data[pos] = self.data[child]
            pos = child
        self.data[pos] = elem

    def _sift_down_to_bottom(self, pos):
        end, start = len(self.data), pos
        elem = self.data[pos]
        child = 2 * pos + 1
        while child <= max(end - 2, 0) and child + 1 < end:
            if self.data[child][0] <= self.data[child + 1][0]:
                child += 1
            self.data[pos] = self.data[child]
            pos = child
            child = 2 * pos + 1
        if child == end - 1:
            self.data[pos] = self.data[child]
            pos = child
        self.data[pos] = elem
        self._sift_up(start, pos)


def replay_python(init, ops):
    heap = StdBinaryHeap([(d, i) for i, d in enumerate(init)])
    nxt, out = len(init), []
    for op in ops:
        if op >= 0:
            heap.push((op, nxt))
            nxt += 1
        else:
            out.append(heap.pop()[1])
    return out


def replay_oracle(init, ops):
    lib = binding.load()
    init = np.asarray(init, np.int64)
    ops = np.asarray(ops, np.int64)
    out = np.full(max(1, len(ops)), -7, np.int64)
    k = lib.orc_heap_replay(init.ctypes.data, len(init), ops.ctypes.data, len(ops), out.ctypes.data)
    assert k >= 0
    return list(out[:k])


def test_heap_small_known_order():
    # from([0, 1, 1]) heapifies to [t2, t1, t0]; pops take t2, then t1, then t0
    assert replay_oracle([0, 1, 1], [-1, -1, -1]) == [2, 1, 0]
    # equal keys: the pop order is the algorithm's, not insertion order
    assert replay_oracle([3, 3, 3, 3, 3], [-1] * 5) == replay_python([3] * 5, [-1] * 5)


@pytest.mark.parametrize("seed", range(6))
def test_heap_matches_independent_transcription(seed):
    rng = np.random.default_rng(seed)
    keys = int(rng.integers(1, 6))
    init = list(rng.integers(0, keys, size=int(rng.integers(0, 300))))
    ops, size = [], len(init)
    for _ in range(2000):
        if size and rng.random() < 0.55:
            ops.append(-1)
            size -= 1
        else:
            ops.append(int(rng.integers(0, keys)))
            size += 1
    ops += [-1] * size
    got = replay_oracle(init, ops)
    assert got == replay_python(init, ops)
    # every task comes out exactly once
    all_keys = list(init) + [o for o in ops if o >= 0]
    assert sorted(got) == list(range(len(all_keys)))
    # a max-heap by direction: the final drain pops keys in non-increasing order
    drain = [all_keys[i] for i in got[-size:]] if size else []
    assert drain == sorted(drain, reverse=True)


def _run(w, dirs, steps, **kw):
    o = binding.OracleSweep(w.params, w.grid, w.density, w.ionized_hydrogen_fraction, w.temperature, w.source,
                            dirs, **kw)
    for _ in range(steps):
        o.run_sweeps()
    return o


def test_threads_do_not_change_fifo_results():
    w = workloads.c2_lognormal(n_per_side=8, num_directions=16, num_levels=3, nthreads=2)
    dirs = binding.directions_from_num(16)
    a = _run(w, dirs, 3)
    b = _run(w, dirs, 3, num_threads=5)
    fa, fb = a.fields(), b.fields()
    for k in fa:
        np.testing.assert_array_equal(fa[k], fb[k])
    ra, rb = a.rates(), b.rates()
    for k in ra:
        np.testing.assert_array_equal(ra[k], rb[k])
    assert a.work() == b.work()


def test_heap_order_solves_every_task_and_matches_fifo_to_rounding():
    """Snapshot periodic semantics make a sweep's result independent of the task order
    up to the summation order of each cell's incoming corrections."""
    w = workloads.c2_lognormal(n_per_side=8, num_directions=16, num_levels=3, nthreads=2)
    dirs = binding.directions_from_num(16)
    fifo = _run(w, dirs, 3)
    heap = _run(w, dirs, 3, order=binding.ORDER_HEAP)
    assert fifo.work() == heap.work()
    ff, fh = fifo.fields(), heap.fields()
    np.testing.assert_array_equal(ff["level"], fh["level"])
    np.testing.assert_allclose(fh["ionized_hydrogen_fraction"], ff["ionized_hydrogen_fraction"], rtol=1e-12)
    np.testing.assert_allclose(fh["temperature"], ff["temperature"], rtol=1e-12)


def test_oracle_directions_are_the_reference_tables():
    from subsweep_gb300 import directions_from_num
    for num in (1, 16, 21, 32, 64, 84):
        np.testing.assert_array_equal(binding.directions_from_num(num), directions_from_num(num))
    with pytest.raises(ValueError):
        binding.directions_from_num(5)


@pytest.mark.parametrize("kind,scale", [("lattice", 1.0), ("lattice", workloads.C2_CELL), ("lattice", 1e-9),
                                        ("poisson", 1.0), ("poisson", workloads.C3_CELL)])
def test_oracle_voronoi_matches_host_producer(kind, scale):
    if kind == "lattice":
        box = 12.0 * scale
        pts = gridmod.jittered_lattice(12, box, 0.25, 9)
    else:
        box = 10.0 * scale
        pts = gridmod.poisson_points(1500, box, 4)
    o = binding.voronoi(pts, box, num_threads=3)
    h = gridmod.voronoi(pts, box, periodic=True, nthreads=3)
    assert o["failed_cells"] == 0 and o["dropped_faces"] == 0
    np.testing.assert_array_equal(o["row_ptr"], h.row_ptr)
    np.testing.assert_array_equal(o["nbr"], h.nbr)
    np.testing.assert_array_equal(o["kind"], h.kind)
    np.testing.assert_array_equal(o["normal"], h.normal)
    np.testing.assert_allclose(o["area"], h.area, rtol=1e-10, atol=1e-12 * h.area.max())
    np.testing.assert_allclose(o["volume"], h.volume, rtol=1e-10)
    assert abs(o["volume"].sum() / box ** 3 - 1.0) < 1e-12
