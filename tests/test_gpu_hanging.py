"""FP64 parity on meshes with hanging faces (Prolong_refined / Restrict_refined and the
fine-mortar connections of Refined_connection)."""
import numpy as np
import pytest

import oracle
from hexed_gb300 import abi, problems
from hexed_gb300.mesh import bc_spec
from hexed_gb300.solver import Context
from hexed_gb300.tree import tree_mesh
from helpers import FP64_TOL, air_transport, compare_arenas, smooth_state
from test_oracle_reference import exp_face, refined_arena
from hexed_gb300.basis import Basis

pytestmark = pytest.mark.gpu


def run_pair(ar, op_oracle, op_gpu):
    a, b = ar.copy(), ar.copy()
    op_oracle(oracle.Oracle(a))
    with Context(b) as ctx:
        op_gpu(ctx)
        ctx.download_all()
    return a, b


def small_tree(nd, rs, kind=abi.BC_RIEMANN):
    fs = problems.freestream_state(nd, 0.3, 7., 1.2, 1e5)
    spec = bc_spec(kind, freestream=fs)
    ar = tree_mesh(nd, rs, 2, 2, problems.sphere_refinement(2, 0.3),
                   {(d, s): spec for d in range(nd) for s in range(2)})
    assert len(ar.ref_face) > 0
    return smooth_state(ar, 3)


@pytest.mark.parametrize("stretch", [(False, False), (True, False), (False, True)])
@pytest.mark.parametrize("scale", [False, True])
@pytest.mark.parametrize("offset", [False, True])
def test_prolong_restrict_kernels(stretch, scale, offset):
    b = Basis(6)
    ar = refined_arena(6, stretch)
    ar.face[0, int(offset)] = exp_face(b)
    for k in range(4):
        ar.face[6 + k, int(offset)] = exp_face(b, k // 2, .5, k % 2, .5)
    a, g = run_pair(ar, lambda o: o.prolong(scale, offset), lambda c: c.prolong(scale, offset))
    errs, bad = compare_arenas(a, g)
    assert not bad, errs
    a, g = run_pair(ar, lambda o: o.restrict(scale, offset), lambda c: c.restrict(scale, offset))
    errs, bad = compare_arenas(a, g)
    assert not bad, errs


@pytest.mark.parametrize("nd,rs", [(2, 4), (2, 6), (3, 3), (3, 4)])
def test_tree_euler_update(nd, rs):
    ar = small_tree(nd, rs)
    oracle.Oracle(ar).write_face()
    oracle.Oracle(ar).prolong()
    p = abi.update_params(max_safety=0.5)
    res = {}

    def o_op(o):
        res["o"] = [o.update(p) for _ in range(3)]

    def g_op(c):
        res["g"] = [c.update(p) for _ in range(3)]
    a, g = run_pair(ar, o_op, g_op)
    errs, bad = compare_arenas(a, g)
    assert not bad, errs
    np.testing.assert_allclose(res["g"], res["o"], rtol=FP64_TOL)


@pytest.mark.parametrize("nd,rs", [(2, 4), (3, 3)])
def test_tree_navier_stokes(nd, rs):
    ar = small_tree(nd, rs, abi.BC_NONPENETRATION)
    oracle.Oracle(ar).write_face()
    oracle.Oracle(ar).prolong()
    visc, cond = air_transport()

    def o_op(o):
        o.apply_state_bcs()
        o.compute_navier_stokes(1e-6, 0, visc, cond)

    def g_op(c):
        c.apply_state_bcs()
        c.compute_navier_stokes(1e-6, 0, visc, cond)
    a, g = run_pair(ar, o_op, g_op)
    errs, bad = compare_arenas(a, g)
    assert not bad, errs


@pytest.mark.parametrize("n", [3, 5])
def test_art_visc_admis(n):
    """Solver::set_art_visc_admis: indicator, vertex max, interpolation; then an AV update."""
    ar = problems.mach2_jump_3d(n_per_side=n, row_size=4)
    oracle.Oracle(ar).write_face()
    cs = ar.av_char_speed
    a, g = run_pair(ar, lambda o: o.set_art_visc_admis(cs), lambda c: c.set_art_visc_admis(cs))
    assert a.elem[:, a.nv + 2].max() > 0
    errs, bad = compare_arenas(a, g)
    assert not bad, errs
    np.testing.assert_allclose(g.elem[:, g.nv + 2], a.elem[:, a.nv + 2], rtol=1e-12, atol=1e-12 * a.elem[:, a.nv + 2].max())
    p = abi.update_params(max_safety=0.5, av_admis_char_speed=cs)
    res = {}

    def o_op(o):
        res["o"] = [o.update(p) for _ in range(2)]

    def g_op(c):
        res["g"] = [c.update(p) for _ in range(2)]
    a, g = run_pair(ar, o_op, g_op)
    errs, bad = compare_arenas(a, g, what=("elem",))
    assert not bad, errs
    np.testing.assert_allclose(res["g"], res["o"], rtol=FP64_TOL)
