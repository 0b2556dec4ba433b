"""Synthetic mesh generator: sizes of the benchmark configurations,
orientation and boundary groups."""
import numpy as np

from arcanefem_gb300 import meshgen


def test_square_counts_and_orientation():
    m = meshgen.unit_square_tri(256, jitter=0.2, seed=0)      # 2D Poisson configuration
    assert m.nb_cell == 131072 and m.nb_node == 66049
    assert meshgen.signed_measures(m).min() > 0
    assert meshgen.nnz_formula(m) == 460289
    assert m.groups["boundary"].size == 4 * 256


def test_cube_counts_and_orientation():
    m = meshgen.unit_cube_tet(8, jitter=0.15, seed=0)
    assert m.nb_cell == 6 * 512 and m.nb_node == 729
    assert meshgen.signed_measures(m).min() > 0
    # nnz = N + 2 E with E = edges of the Kuhn split (7 per hex + boundary)
    n = 8
    edges = 3 * n * (n + 1) ** 2 + 3 * n * n * (n + 1) + n ** 3
    assert meshgen.nnz_formula(m) == m.nb_node + 2 * edges


def test_config_sizes_closed_form():
    # 128^3 (3D Poisson) and 96^3 (elasticity) configurations, without building them
    for n, nodes, nnz in ((128, 2146689, 31802497), (96, 912673, 13465441)):
        edges = 3 * n * (n + 1) ** 2 + 3 * n * n * (n + 1) + n ** 3
        assert (n + 1) ** 3 == nodes and nodes + 2 * edges == nnz


def test_jitter_is_seeded_and_bounded():
    a = meshgen.unit_cube_tet(4, seed=7)
    b = meshgen.unit_cube_tet(4, seed=7)
    c = meshgen.unit_cube_tet(4, seed=8)
    assert np.array_equal(a.coords, b.coords) and not np.array_equal(a.coords, c.coords)
    base = meshgen.unit_cube_tet(4, jitter=0.0).coords
    assert np.abs(a.coords - base).max() <= 0.15 / 4 + 1e-15
    assert np.array_equal(a.coords[a.groups["boundary"]], base[a.groups["boundary"]])
