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


def ramp_arena(row_size=4, n=4):
    """The Mach-2 arena with each element's specific volume carrying the highest Legendre mode
    along the first reference dimension, amplitudes log-spaced over the elements, so that the
    smoothness indicator (src/stabilizing_art_visc.cpp:47-55) falls below its ramp, inside it
    and above it. Returns the arena and each element's log10 non-smoothness, restated here."""
    ar = problems.mach2_jump_3d(n_per_side=n, row_size=row_size)
    b = Basis(row_size)
    rs, nq, nd = row_size, ar.nq, ar.n_dim
    mode = b.orthogonal(rs - 1)
    node0 = (np.arange(nq) // rs ** (nd - 1)) % rs      # node index along the first dimension
    amps = np.logspace(-3.5, 0., ar.n_elem)
    vel = ar.freestream[0] / ar.freestream[nd]
    log_ns = np.empty(ar.n_elem)
    w = b.node_weights
    qw = np.prod([w[(np.arange(nq) // rs ** (nd - 1 - d)) % rs] for d in range(nd)], axis=0)
    for e in range(ar.n_elem):
        iv = (1. + 0.5 * amps[e] * mode[node0]) / 1.2
        rho = 1. / iv
        ar.elem[e, 0] = rho * vel
        ar.elem[e, 1:nd] = 0.
        ar.elem[e, nd] = rho
        ar.elem[e, nd + 1] = 1e5 / (problems.HEAT_RAT - 1) + 0.5 * rho * vel * vel
        # rows along the first dimension carry the mode; the other rows project to zero
        rows = iv.reshape(rs, -1)
        fw = np.prod([w[(np.arange(nq // rs) // rs ** (nd - 2 - d)) % rs] for d in range(nd - 1)], axis=0)
        dots = (mode * w) @ rows
        log_ns[e] = np.log10(np.sum(dots ** 2 * fw) / (np.sum(iv * iv * qw) * nd))
    return ar, log_ns


@pytest.mark.parametrize("precision", [abi.FP64, abi.MIXED])
def test_art_visc_ramp_regimes(precision):
    """Elements below, inside and above the indicator's ramp: the device classifies the outer
    two by thresholds on the ratio and evaluates the ramp as the reference does; the AV row
    must match the oracle's in every regime (FP64 to 1e-12; the mixed form's float sums to
    1e-5 of the largest coefficient)."""
    rs = 4
    ar, log_ns = ramp_arena(rs)
    center = -4.25 * np.log10(rs - 1)
    assert (log_ns < center - 0.5).sum() >= 3
    assert ((log_ns > center - 0.5) & (log_ns < center + 0.5)).sum() >= 3
    assert (log_ns > center + 0.5).sum() >= 3
    oracle.Oracle(ar).write_face()
    cs = ar.av_char_speed
    a = ar.copy()
    oracle.Oracle(a).set_art_visc_admis(cs)
    g = ar.copy()
    with Context(g, precision) as ctx:
        ctx.set_art_visc_admis(cs)
        ctx.download_all()
    ref = a.elem[:, a.nv + 2]
    assert ref.max() > 0 and ref.min() == 0
    if precision == abi.FP64:
        np.testing.assert_allclose(g.elem[:, g.nv + 2], ref, rtol=1e-12, atol=1e-12 * ref.max())
    else:
        np.testing.assert_allclose(g.elem[:, g.nv + 2], ref, rtol=0, atol=1e-5 * ref.max())
