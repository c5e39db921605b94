"""Solver::fix_admissibility restated in the oracle (src/Solver.cpp:961-1095): the
pde::Fix_therm_admis diffusion (include/pde.hpp:437-493) restores positive density and
energy, conserves every conserved quantity (its boundary conditions pass no flux), leaves an
admissible state alone, and runs inside Solver::update after every stage."""
import numpy as np
import pytest

from hexed_gb300 import abi, problems
import oracle
from helpers import planted_inadmissible as planted


def quadrature_weights(ar):
    """Gauss-Legendre weight of each quadrature point of an element, on [0, 1]^nd."""
    _, w = np.polynomial.legendre.leggauss(ar.row_size)
    w = w/2
    q = np.arange(ar.nq)
    out = np.ones(ar.nq)
    for d in range(ar.n_dim):
        out *= w[(q // ar.row_size**(ar.n_dim - 1 - d)) % ar.row_size]
    return out


def integrals(ar):
    """Integral of each conserved variable over the mesh."""
    w = quadrature_weights(ar)
    vol = ar.nom_size**ar.n_dim
    det = np.ones((ar.n_elem, ar.nq))
    if ar.n_def:
        nd = ar.n_dim
        det[ar.n_car:] = ar.jac[:, nd*nd]
    return np.einsum("evq,q,e,eq->v", ar.elem[:, :ar.nv], w, vol, det)


def admissible(ar):
    nd = ar.n_dim
    return bool((ar.elem[:, nd] > 0).all() and (ar.elem[:, nd + 1] > 0).all())


@pytest.mark.parametrize("kind", ["cartesian", "deformed", "tree"])
def test_fix_restores_admissibility(kind):
    ar = planted(kind)
    assert not admissible(ar)
    before = integrals(ar)
    o = oracle.Oracle(ar)
    p = abi.update_params(max_safety=0.5)
    iters = o.fix_admissibility(p, 0.7)
    assert iters > 0
    assert admissible(ar)
    if kind == "cartesian":
        # On a uniform Cartesian mesh the local time step is the same at every point, and the
        # boundary conditions pass no flux: the diffusion conserves every conserved quantity.
        # (With the varying local time step of a deformed mesh it does not, in the reference
        # as here.)
        np.testing.assert_allclose(integrals(ar), before, rtol=1e-12, atol=1e-12*np.abs(before).max())


def test_fix_leaves_admissible_state_alone():
    ar = problems.vortex_2d(n_per_side=4, row_size=4)
    oracle.Oracle(ar).write_face()
    ref = ar.copy()
    assert oracle.Oracle(ar).fix_admissibility(abi.update_params(max_safety=0.5), 0.7) == 0
    np.testing.assert_array_equal(ar.elem, ref.elem)
    np.testing.assert_array_equal(ar.face, ref.face)


def test_update_with_fix_admis():
    """Solver::update with set_fix_admissibility(true): the fix runs after each stage and, on
    an admissible state, changes nothing (src/Solver.cpp:866-868)."""
    ar = planted("cartesian")
    p0 = abi.update_params(max_safety=0.5)
    oracle.Oracle(ar).fix_admissibility(p0, 0.7)
    with_fix, without = ar.copy(), ar.copy()
    dt_a = oracle.Oracle(with_fix).update(abi.update_params(max_safety=0.5, fix_admis=True))
    dt_b = oracle.Oracle(without).update(p0)
    assert dt_a == dt_b
    assert admissible(with_fix)
    np.testing.assert_array_equal(with_fix.elem[:, :ar.nv], without.elem[:, :ar.nv])
