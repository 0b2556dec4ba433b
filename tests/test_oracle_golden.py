"""Pin the CPU oracle against the reference's own golden vectors.

Each case reruns, with the oracle, what the reference test does: node-wise
assembly, source term, penalty Dirichlet (1e30 / 1e31), transformation and
CG, then compares the nodal solution with the reference's check file
(tolerance of the reference test: 1e-4 Poisson/testlab, 1e-3 elasticity).
"""
import numpy as np
import pytest

import golden_cases as G
from oracle import oracle as O


def oracle_solve(name):
    spec = G.CASES[name]
    d = G.load(name)
    coords, cells = d["coords"], d["cells"]
    n = coords.shape[0]
    dim = 2 if cells.shape[1] == 3 else 3
    ptr, nc, _ = O.node_cell(n, cells)
    rp, cols = O.sparsity(n, cells)
    if spec["kind"] == "elasticity":
        E, nu = spec["E"], spec["nu"]
        mu = E / (2 * (1 + nu))
        lam = E * nu / ((1 + nu) * (1 - 2 * nu))
        vals = O.assemble(O.ELASTICITY_TET4, coords, cells, ptr, nc, rp, cols, lam=lam, mu=mu)
        srp, scols = G.scalar_csr_from_block(rp, cols, 3)
        rhs = O.rhs_body_force_tet4(coords, cells, spec["body_force"])
        nd = 3 * n
        fi, fv = np.zeros(nd, np.uint8), np.zeros(nd)
        for g, v3 in spec["dirichlet3"]:
            for comp, v in enumerate(v3):
                if v is not None:
                    O.dirichlet_penalty(d["group__" + g], 3, comp, v, spec["penalty"], fi, fv, rhs)
        rp, cols = srp, scols
    else:
        if spec["kind"] == "testlab":
            kind = O.TESTLAB_TRI3 if dim == 2 else O.TESTLAB_TET4
        else:
            kind = O.POISSON_TRI3 if dim == 2 else O.POISSON_TET4
        vals = O.assemble(kind, coords, cells, ptr, nc, rp, cols)
        rhs = O.rhs_constant_source(dim, coords, cells, ptr, nc, spec["f"])
        nd = n
        fi, fv = np.zeros(nd, np.uint8), np.zeros(nd)
        for g, v in spec["dirichlet"]:
            O.dirichlet_penalty(d["group__" + g], 1, 0, v, spec["penalty"], fi, fv, rhs)
    ei, ev = np.zeros(nd, np.uint8), np.zeros(nd)
    O.apply_transformations(rp, cols, vals, rhs, fi, fv, ei, ev)
    x, it, rr = O.pcg_jacobi(rp, cols, vals, rhs, rtol=1e-13, max_iter=20000, norm_skip=fi)
    return x, d


@pytest.mark.parametrize("name", list(G.CASES))
def test_oracle_matches_reference_check_file(name):
    x, d = oracle_solve(name)
    err = G.compare(name, x, d)
    assert err < G.CASES[name]["eps"], f"{name}: max rel err {err:.3e}"


def test_golden_fixtures_are_consistent():
    for name in G.CASES:
        d = G.load(name)
        n = d["coords"].shape[0]
        assert d["cells"].min() >= 0 and d["cells"].max() < n
        assert set(d["check_uid"].tolist()) <= set(d["node_tags"].tolist())
