"""Basis tables: pinned against the reference's own generator, plus the properties the
reference's test/test_Basis.cpp checks for Gauss_legendre."""
import json
import os

import numpy as np
import pytest

from hexed_gb300.basis import Basis, load_tables

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "gauss_legendre_ref.json")
ROW_SIZES = range(2, 9)


@pytest.fixture(scope="module")
def golden():
    with open(GOLDEN) as fh:
        return json.load(fh)


def colmajor(m):
    return np.asarray(m).T.ravel()


@pytest.mark.parametrize("rs", ROW_SIZES)
def test_tables_match_reference_generator(golden, rs):
    ref = golden[str(rs)]
    mine = load_tables()[rs]
    # the generator emits 20 significant digits; every table rounds to the same double
    np.testing.assert_array_equal(np.array(ref["node"]), mine["node"])
    np.testing.assert_array_equal(np.array(ref["weight"]), mine["weight"])
    # the centre entry of odd row sizes is 0 up to the 50-digit working precision
    np.testing.assert_allclose(np.array(ref["diff_mat"]), colmajor(mine["diff_mat"]), rtol=0, atol=1e-40)
    np.testing.assert_array_equal(np.array(ref["boundary"]), np.ravel(mine["boundary"]))
    np.testing.assert_array_equal(np.array(ref["orthogonal"]), np.ravel(mine["orthogonal"]))
    np.testing.assert_array_equal(np.array(ref["filter"]), colmajor(mine["filter"]))
    np.testing.assert_array_equal(np.array(ref["prolong"]),
                                  np.concatenate([colmajor(mine["prolong"][h]) for h in (0, 1)]))
    np.testing.assert_array_equal(np.array(ref["restrict"]),
                                  np.concatenate([colmajor(mine["restrict"][h]) for h in (0, 1)]))
    # eigenvalues come out of a float64 eigensolver in both generators
    np.testing.assert_allclose(mine["eigenvals"], ref["eigenvals"], rtol=1e-13)


@pytest.mark.parametrize("rs", ROW_SIZES)
def test_diff_mat(rs):  # test/test_Basis.cpp:8-46
    b = Basis(rs)
    assert np.abs(b.diff_mat.sum(axis=1)).max() < 1e-13
    x = b.nodes
    np.testing.assert_allclose(b.diff_mat @ (-2.14 + 9.07 * x), 9.07, rtol=1e-5)
    if rs > 2:
        np.testing.assert_allclose(b.diff_mat @ (0.07 - 0.38 * x - 4.43 * x * x), -0.38 - 2 * 4.43 * x, rtol=1e-5,
                                   atol=1e-9)


@pytest.mark.parametrize("rs", ROW_SIZES)
def test_quadrature_boundary_orthogonal(rs):  # test/test_Basis.cpp:48-86
    b = Basis(rs)
    assert b.node_weights.sum() == pytest.approx(1.)
    if rs >= 3:
        assert (b.node_weights * b.nodes ** 2).sum() == pytest.approx(1. / 3.)
    vals = b.boundary @ (0.15 * b.nodes + 0.37)
    assert vals[0] == pytest.approx(0.37) and vals[1] == pytest.approx(0.52)
    for i in range(rs):
        for j in range(rs):
            dot = (b.orthogonal(i) * b.node_weights) @ b.orthogonal(j)
            assert dot == pytest.approx(1. if i == j else 0., abs=1e-10)


@pytest.mark.parametrize("rs", ROW_SIZES)
def test_transform(rs):  # test/test_Basis.cpp:88-112
    b = Basis(rs)
    ident = sum(b.restrict[h] @ b.prolong[h] for h in (0, 1))
    assert np.linalg.norm(np.eye(rs) - ident) < 1e-10
    prolong = np.vstack(b.prolong)
    restrict = np.hstack(b.restrict)
    mono = np.array([[((b.nodes[i] + h) / 2.) ** d for d in range(rs)] for h in (0, 1) for i in range(rs)])
    assert np.linalg.norm(prolong @ restrict @ mono - mono) < 1e-10


def test_time_step_constants():
    """max_cfl = -2*0.9/min_eig_convection, step_ratio = 0.5/0.9 (src/Basis.cpp:6-14)."""
    for rs in ROW_SIZES:
        t = load_tables()[rs]
        assert t["max_cfl"] == -2 * 0.9 / t["eigenvals"][0]
        assert t["step_ratio"] == 0.5 / 0.9
        assert t["eigenvals"][0] < 0 and t["eigenvals"][1] < 0
