"""Smoothness-based artificial viscosity on the GPU (hexed_gpu_update_art_visc_smoothness)
against the oracle's restatement of Solver::update_art_visc_smoothness (src/Solver.cpp:457-582)
with Solver::diffuse_art_visc (src/Solver.cpp:428-455), on the meshes the oracle's own tests
use: the reference test's strip (Cartesian, and deformed with an identity mapping), every wall
kind, a 3D strip, curved deformed meshes and tree meshes with hanging faces, with Chebyshev
sub-steps, and two calls in a row (the advection state carries over between calls).

Compared after each run: the bulk AV coefficient, art_visc_residual, the forcing rows and the
advection state of the storage, the time-step-scale row (the last pseudo-time step), the flow
state put back and its re-extrapolated face traces.

Bars: 1e-12 relative (max norm of each variable or storage row against its own largest
magnitude; momentum components against the momentum's) for the flow state, the time-step
scale and the advection state. 1e-10 for the forcing rows, the coefficient and the residual:
these come from the highest Legendre mode of advected scalars that are 1 plus a small
variation, proj = sum_i a_i w_i o_i with sum_i w_i o_i = 0, so the cancellation amplifies the
roundoff of the a_i (FMA contraction on the GPU, none in the oracle) by |a|/|proj|, and the
result is then squared and smeared by the diffusion iterations.

Setting HEXED_PARITY_REPORT to a file path appends one JSON line of measured errors per case.
"""
import json
import os

import numpy as np
import pytest

import oracle
from hexed_gb300 import abi, problems
from hexed_gb300.mesh import bc_spec, structured_mesh
from hexed_gb300.solver import Context
from helpers import FP64_TOL, group_rel, per_variable_rel
from test_oracle_smooth_av import strip, tanh_state

pytestmark = pytest.mark.gpu

DERIVED_TOL = 1e-10


def perturbed(ar, seed=0):
    """Flow along x with a tanh front and a smooth seeded perturbation in every variable, so
    that the coefficient is not zero anywhere and every code path sees data."""
    nd = ar.n_dim
    rng = np.random.default_rng(seed)
    k = rng.uniform(1, 3, size=(3, nd))
    ph = rng.uniform(0, 2 * np.pi, size=3)

    def st(pos):
        pert = sum(np.sin(sum(k[i, d] * pos[d] for d in range(nd)) + ph[i]) for i in range(3)) / 3
        x = pos[0]
        out = [1. - .1 * np.tanh((x - .5) / .1) + .02 * pert]
        out += [.02 * np.roll(pert, d + 1) for d in range(nd - 1)]
        out += [1. + .03 * pert, 1.5 + .02 * pert]
        return np.stack(out)
    ar.set_state(st)
    return ar


def run_pair(ar, length, calls, precision, **kw):
    a = ar.copy()
    st = oracle.SavStorage(a)
    po = oracle.sav_params(length, ar.row_size, 1., 1.5, **kw)
    res_o = [oracle.Oracle(a).update_art_visc_smoothness(st, po) for _ in range(calls)]
    b = ar.copy()
    pg = abi.sav_params(length, ar.row_size, 1., 1.5, **kw)
    with Context(b, precision) as c:
        c.write_face()
        c.prolong()
        res_g = [c.update_art_visc_smoothness(pg) for _ in range(calls)]
        elem = c.download(abi.ARRAY_ELEM)
        aux, _ = c.sav_storage()
        face = c.download(abi.ARRAY_FACE) if precision == abi.FP64 else None
    return a, st, res_o, elem, aux, face, res_g


def check(ar, length, calls=1, precision=abi.FP64, name=None, **kw):
    a, st, res_o, elem, aux, face, res_g = run_pair(ar, length, calls, precision, **kw)
    nv, rs = ar.nv, ar.row_size
    assert a.elem[:, nv + 1].max() > 0, "the case must produce a coefficient"
    errs = {
        "state": max(per_variable_rel(elem[:, :nv], a.elem[:, :nv], nv=nv)),
        "tss": per_variable_rel(elem[:, nv:nv + 1], a.elem[:, nv:nv + 1])[0],
        "advection": max(per_variable_rel(aux[:, 4:4 + rs], st.aux[:, 4:4 + rs])),
        "forcing": max(per_variable_rel(aux[:, :4], st.aux[:, :4])),
        "coefficient": per_variable_rel(elem[:, nv + 1:nv + 2], a.elem[:, nv + 1:nv + 2])[0],
        "residual": max(abs(g - o) / abs(o) for g, o in zip(res_g, res_o)),
    }
    if face is not None:
        errs["flow_traces"] = group_rel(face[:, 0], a.face[:, 0], nv, 1)
    path = os.environ.get("HEXED_PARITY_REPORT")
    if path and name:
        with open(path, "a") as fh:
            fh.write(json.dumps({"case": name, **errs}) + "\n")
    bars = {"state": FP64_TOL, "tss": FP64_TOL, "advection": FP64_TOL, "flow_traces": FP64_TOL,
            "forcing": DERIVED_TOL, "coefficient": DERIVED_TOL, "residual": DERIVED_TOL}
    bad = {k: v for k, v in errs.items() if not v <= bars[k]}
    assert not bad, (bad, errs)
    return errs


@pytest.mark.parametrize("deformed", [False, True])
def test_strip(deformed):
    ar = strip(4, (10, 2), deformed=deformed)
    tanh_state(ar, 0.1)
    check(ar, 0.1, name=f"sav_strip_{'deformed' if deformed else 'cartesian'}", advect_iters=100, diff_iters=50)


@pytest.mark.parametrize("wall", [abi.BC_NO_SLIP, abi.BC_COPY, abi.BC_OUTFLOW, abi.BC_RIEMANN])
def test_wall_kinds(wall):
    ar = strip(4, (10, 2), wall=wall)
    tanh_state(ar, 0.1)
    check(ar, 0.1, advect_iters=60, diff_iters=30)


def test_strip_3d():
    ar = strip(4, (10, 2, 2))
    tanh_state(ar, 0.1)
    check(ar, 0.1, name="sav_strip_3d", advect_iters=60, diff_iters=30)


@pytest.mark.parametrize("nd,rs", [(2, 4), (2, 6), (3, 3), (3, 5), (3, 6)])
def test_curved_mesh(nd, rs):
    spec = bc_spec(abi.BC_FREESTREAM, freestream=[1.1] + [0.] * (nd - 1) + [1., 1.5])
    ar = structured_mesh(nd, rs, 3, 0., 1., deformed=True,
                         displacement=problems.sinusoid_displacement(1. / 3, 0.1, 0, n_dim=nd),
                         bcs={(d, s): spec for d in range(nd) for s in range(2)})
    perturbed(ar)
    check(ar, 0.2, name=f"sav_curved_{nd}d_rs{rs}", advect_iters=40, diff_iters=20)


@pytest.mark.parametrize("nd", [2, 3])
def test_tree_hanging_faces(nd):
    from hexed_gb300.tree import tree_mesh
    spec = bc_spec(abi.BC_FREESTREAM, freestream=[1.1] + [0.] * (nd - 1) + [1., 1.5])
    ar = tree_mesh(nd, 4, 2, 2, problems.sphere_refinement(nd, 0.3), {(d, s): spec for d in range(nd) for s in range(2)})
    assert len(ar.ref_face) > 0
    perturbed(ar, 1)
    check(ar, 0.2, name=f"sav_tree_{nd}d", advect_iters=40, diff_iters=20)


def test_chebyshev_substeps_and_av_row_size():
    ar = strip(6, (8, 2))
    tanh_state(ar, 0.1)
    check(ar, 0.1, advect_iters=50, diff_iters=20, n_cheby=3, av_row_size=4)


def test_two_calls_carry_the_advection_state():
    ar = strip(4, (10, 2))
    tanh_state(ar, 0.1)
    check(ar, 0.1, calls=2, advect_iters=40, diff_iters=20)


def test_mixed_context_same_coefficient():
    """The smoothness AV runs in FP64 in both precision forms: a mixed-form context gives the
    FP64 coefficient (its flow traces are float offsets and are not compared)."""
    ar = strip(4, (10, 2))
    tanh_state(ar, 0.1)
    check(ar, 0.1, precision=abi.MIXED, advect_iters=60, diff_iters=30)


def test_invalid_parameters():
    ar = strip(4, (4, 2))
    tanh_state(ar, 0.1)
    with Context(ar) as c:
        for bad in (abi.sav_params(0.1, 4, 1., 1.5, av_row_size=5), abi.sav_params(0.1, 4, 1., 1.5, av_row_size=1),
                    abi.sav_params(0., 4, 1., 1.5), abi.sav_params(0.1, 4, 1., 1.5, n_cheby=0)):
            with pytest.raises(abi.HexedError):
                c.update_art_visc_smoothness(bad)


def test_graph_replay_matches_eager_launches():
    """From the second pseudo-time iteration on, each iteration replays a captured CUDA graph;
    with the per-kernel profiler on, every launch is eager. Both give the same bits."""
    ar = strip(4, (10, 2))
    tanh_state(ar, 0.1)
    pg = abi.sav_params(0.1, ar.row_size, 1., 1.5, advect_iters=30, diff_iters=12, n_cheby=2)
    out = []
    for profile in (False, True):
        b = ar.copy()
        with Context(b) as c:
            c.write_face()
            c.prolong()
            if profile:
                c.profile_enable(True)
            res = [c.update_art_visc_smoothness(pg) for _ in range(2)]
            if profile:
                assert c.profile_read()["sav_local_advection"][0] == 2 * 2 * 30
            out.append((res, c.download(abi.ARRAY_ELEM), c.sav_storage()[0]))
    assert out[0][0] == out[1][0]
    assert np.array_equal(out[0][1], out[1][1]) and np.array_equal(out[0][2], out[1][2])


def test_reference_convergence():
    """The reference's "artificial viscosity convergence" test (test/test_Solver.cpp:829-877)
    on the GPU with its settings: row size 8, 100 x 2 elements, 6000 advection and 3000
    diffusion iterations, diffusion ratio 1e-6, unscaled maximum 1000, one solver throughout
    (the advection state carries over between calls). Doubling the advection length
    multiplies the coefficient by more than 2^(row_size - 1); halving the flow's length scale,
    by more than 2^(row_size - 2)."""
    import math
    rs = 8
    ar = strip(rs, (100, 2))
    tanh_state(ar, 0.04)
    kw = dict(advect_iters=6000, diff_iters=3000, diff_ratio=1e-6, unscaled_max=1000.)
    with Context(ar.copy()) as c:
        c.write_face()
        c.prolong()

        def coef(length):
            resid = c.update_art_visc_smoothness(abi.sav_params(length, rs, 1., 1.5, **kw))
            assert resid > 0 and np.isfinite(resid)
            return c.download(abi.ARRAY_ELEM)[:, ar.nv + 1].max()
        init_max = coef(0.01)
        assert init_max > 0
        assert math.log2(coef(0.02) / init_max) > rs - 1.
        tanh_state(ar, 0.02)
        c.write_state(ar.elem[:, :ar.nv])
        assert math.log2(coef(0.01) / init_max) > rs - 2.
