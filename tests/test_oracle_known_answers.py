"""Known-answer tests of the CPU oracle, restated from the reference's own tests.

src/tests/test_grid.cpp:403-458 (neighbour topology), :509-564 (every particle
distributed once), :908-977 (grid build and hashing); src/tests/test_kernel.cpp:
184-266 (kernel normalisation and derivatives).  They pin the grid hash, the
27-cell neighbour order and the kernel functions the CUDA path reproduces.
"""
import numpy as np
import pytest

from oracle import oracle as O

UNIT = {
    "spacing": 0.1, "grid_spacing_scale": 2.0, "target_density": 1000.0,
    "relative_kernel_radius": 2.0, "domain_min": (-1.0, -1.0, -1.0),
    "domain_max": (1.0, 1.0, 1.0), "colliders": [],
}


@pytest.fixture(scope="module", params=["f32", "f64"])
def grid10(request):
    sim = O.OracleSim(UNIT, np.zeros((1, 3)), variant=request.param)
    yield sim
    sim.close()


def test_uniform_grid3d(grid10):
    # test_grid.cpp:908-932: 10^3 cells of 0.2 over [-1, 1]^3
    dims, geo = grid10.grid_info()
    assert list(dims) == [10, 10, 10]
    assert np.all(np.abs(geo[3:6] - 0.2) < 1e-7)
    assert np.all(np.abs(geo[0:3] + 1.0) < 1e-7)
    assert np.all(geo[6:9] <= -1.0 + 1e-6) and np.all(geo[9:12] >= 1.0 - 1e-6)


def test_hash_quarter_points(grid10):
    # test_grid.cpp:934-977: points at 1/4 and 3/4 of a cell hash to that cell;
    # cell corners hash to the cell or a face neighbour
    exp_len, h_len, hh_len = 0.2, 0.1, 0.05
    pts, want = [], []
    for ci in range(10):
        for cj in range(10):
            for ck in range(10):
                c = np.array([-1 + ci * exp_len + h_len, -1 + cj * exp_len + h_len,
                              -1 + ck * exp_len + h_len])
                for d in ([-hh_len, -hh_len, -hh_len], [-hh_len, hh_len, -hh_len],
                          [hh_len, -hh_len, -hh_len], [hh_len, hh_len, -hh_len],
                          [0, 0, -hh_len]):
                    pts.append(c + d)
                    want.append(ci + 10 * cj + 100 * ck)
    ids, uc = grid10.hash_points(np.array(pts))
    assert np.array_equal(ids, np.array(want, np.uint32))
    corners = []
    for ci in range(10):
        c = np.array([-1 + ci * exp_len + h_len] * 3)
        corners += [c + [-h_len, -h_len, -hh_len], c + [h_len, h_len, -hh_len]]
    _, uc2 = grid10.hash_points(np.array(corners))
    assert np.all(uc2 < 10)


def test_neighbor_query_grid3d(grid10):
    # test_grid.cpp:403-458: 8 / 27 / 12 or 18 neighbours; all within one cell
    for cell in range(1000):
        cols, rows, depth = cell % 10, (cell // 10) % 10, cell // 100
        nb = grid10.cell_neighbors(cell)
        edge = [v in (0, 9) for v in (cols, rows, depth)]
        if all(edge):
            assert len(nb) == 8
        elif not any(edge):
            assert len(nb) == 27
        else:
            assert len(nb) in (12, 18)
        u = np.stack([nb % 10, (nb // 10) % 10, nb // 100], axis=1)
        assert np.all(np.abs(u - [cols, rows, depth]) < 2)


def test_neighbor_list_order(grid10):
    # GetNeighborListFor loops y, then x, then z (grid.h:568-591)
    nb = grid10.cell_neighbors(5 + 5 * 10 + 5 * 100)
    order = [(i, j, k) for j in (4, 5, 6) for i in (4, 5, 6) for k in (4, 5, 6)]
    assert list(nb) == [i + 10 * j + 100 * k for i, j, k in order]


@pytest.mark.parametrize("variant", ["f32", "f64"])
def test_distribute_every_particle_once(variant):
    # test_grid.cpp:509-564: random particles, each in exactly one chain, chain order
    # after DistributeByParticle = particle index order (stable)
    rng = np.random.default_rng(3)
    pos = rng.uniform(-0.99, 0.99, size=(5000, 3))
    sim = O.OracleSim(UNIT, pos, variant=variant)
    cell_of, counts, chains = sim.cells()
    assert counts.sum() == len(pos)
    assert np.array_equal(np.sort(chains), np.arange(len(pos)))
    stable = np.lexsort((np.arange(len(pos)), cell_of))
    assert np.array_equal(chains, stable.astype(np.uint32))
    # one update later the cell contents are the same sets
    sim.update_grid_distribution()
    cell_of2, counts2, chains2 = sim.cells()
    assert np.array_equal(counts, counts2)
    start = np.concatenate([[0], np.cumsum(counts2.astype(np.int64))]).astype(int)
    for c in np.nonzero(counts2)[0][:200]:
        c = int(c)
        assert set(chains2[start[c]:start[c + 1]]) == set(np.nonzero(cell_of2 == c)[0])
    sim.close()


def _radial_integral(fn, h, n=200001):
    r = np.linspace(0.0, h, n)
    vals = np.array([fn(x) for x in r])
    return np.trapezoid(vals * 4 * np.pi * r * r, r)


@pytest.mark.parametrize("variant", ["f64"])
def test_kernel_normalisation(variant):
    # test_kernel.cpp:184-203: both kernels integrate to 1 over the ball (0.05 there)
    h = 1.0
    std = _radial_integral(lambda r: O.kernel_eval(0, h, r, variant), h, 20001)
    spiky = _radial_integral(lambda r: O.kernel_eval(1, h, r, variant), h, 20001)
    assert abs(std - 1.0) < 1e-3
    assert abs(spiky - 1.0) < 1e-3


def test_kernel_derivatives():
    # test_kernel.cpp:210-262: finite differences at radius 10, step 0.01
    h, e = 10.0, 0.01
    rng = np.random.default_rng(7)
    for d in rng.uniform(0.05, h - 2 * e, size=256):
        w = lambda r: O.kernel_eval(1, h, r, "f64")
        fd1 = (w(d + e) - w(d - e)) / (2 * e)
        fd2 = (w(d + e) - 2 * w(d) + w(d - e)) / (e * e)
        assert abs(fd1 - O.kernel_eval(2, h, d, "f64")) < 1e-3
        assert abs(fd2 - O.kernel_eval(3, h, d, "f64")) < 1e-3


def test_within_tests_match_definitions():
    # IsWithinStd / IsWithinSpiky (kernel.cpp:224-233): strict, with a 1e-8 dead band
    h = 0.04
    assert O.kernel_eval(4, h, 0.0399, "f64") == 1
    assert O.kernel_eval(4, h, 0.04, "f64") == 0
    assert O.kernel_eval(5, h, 0.04 - 2e-8, "f64") == 1
    assert O.kernel_eval(5, h, 0.04 - 5e-9, "f64") == 0
