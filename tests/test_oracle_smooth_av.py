"""The oracle's smoothness-based artificial viscosity (Solver::update_art_visc_smoothness,
src/Solver.cpp:457-582), pinned by the reference's own test "artificial viscosity convergence"
(test/test_Solver.cpp:829-877) and cross-checked between its code paths: deformed elements
with an identity mapping against Cartesian ones, 3D against 2D on data that does not vary
across the extra dimension, boundary conditions that must agree, and a uniform flow."""
import math

import numpy as np
import pytest

import oracle
from hexed_gb300 import abi
from hexed_gb300.mesh import bc_spec, structured_mesh


def strip(row_size, counts, wall=abi.BC_NONPENETRATION, deformed=False):
    """The reference test's mesh: elements of size 1/counts[0] in a row along x, walls on the
    other faces, freestream (1.1, 0, 1, 1.5) at x = 0 and (0.9, 0, 1, 1.5) at x = 1."""
    nd = len(counts)
    fs0 = [1.1] + [0.] * (nd - 1) + [1., 1.5]
    fs1 = [0.9] + [0.] * (nd - 1) + [1., 1.5]
    bcs = {(d, s): bc_spec(wall) for d in range(1, nd) for s in range(2)}
    bcs[(0, 0)] = bc_spec(abi.BC_FREESTREAM, freestream=fs0)
    bcs[(0, 1)] = bc_spec(abi.BC_FREESTREAM, freestream=fs1)
    return structured_mesh(nd, row_size, counts, 0., 1., deformed=deformed, bcs=bcs)


def tanh_state(ar, width):
    """Tanh (test/test_Solver.cpp:172-187): x-momentum 1 - 0.1 tanh((x - 0.5)/width), density 1,
    energy 1.5."""
    nd = ar.n_dim

    def st(pos):
        x = pos[0]
        out = [1. - .1 * np.tanh((x - .5) / width)] + [0 * x] * (nd - 1) + [1. + 0 * x, 1.5 + 0 * x]
        return np.stack(out)
    ar.set_state(st)


def run(ar, storage, length, **kw):
    p = oracle.sav_params(length, ar.row_size, 1., 1.5, **kw)
    resid = oracle.Oracle(ar).update_art_visc_smoothness(storage, p)
    return ar.elem[:, ar.nv + 1].copy(), resid


def test_reference_convergence():
    """test/test_Solver.cpp:829-877 with its settings (row size 8, 100 x 2 elements, 6000
    advection and 3000 diffusion iterations, diffusion ratio 1e-6, unscaled maximum 1000):
    doubling the advection length multiplies the coefficient by more than 2^(row_size - 1);
    halving the flow's length scale, by more than 2^(row_size - 2)."""
    rs = 8
    ar = strip(rs, (100, 2))
    tanh_state(ar, 0.04)
    st = oracle.SavStorage(ar)
    kw = dict(advect_iters=6000, diff_iters=3000, diff_ratio=1e-6, unscaled_max=1000.)
    av0, resid = run(ar, st, 0.01, **kw)
    assert resid > 0 and np.isfinite(resid)
    init_max = av0.max()
    assert init_max > 0
    av1, _ = run(ar, st, 0.02, **kw)
    assert math.log2(av1.max() / init_max) > rs - 1.
    tanh_state(ar, 0.02)
    av2, _ = run(ar, st, 0.01, **kw)
    assert math.log2(av2.max() / init_max) > rs - 2.


def test_uniform_flow():
    """A uniform flow keeps the advected scalars at 1, so the highest-mode projection and the
    coefficient vanish to roundoff; the momentum comes back to its last bits or one ulp."""
    ar = strip(4, (6, 2))
    ar.set_state(lambda pos: np.stack([0.3 + 0 * pos[0], 0 * pos[0], 1. + 0 * pos[0], 1.5 + 0 * pos[0]]))
    mom = ar.elem[:, 0].copy()
    st = oracle.SavStorage(ar)
    av, _ = run(ar, st, 0.2, advect_iters=50, diff_iters=20)
    np.testing.assert_allclose(st.advection, 1., rtol=0, atol=1e-13)
    assert np.abs(av).max() < 1e-20
    np.testing.assert_allclose(ar.elem[:, 0], mom, rtol=2.3e-16, atol=0)


def test_deformed_identity_matches_cartesian():
    """Deformed elements with an identity mapping (no displacement) take the deformed
    branches (reference-level normals, determinants, face normals, signed connections) and
    must give the Cartesian result to roundoff."""
    results = []
    for deformed in (False, True):
        ar = strip(4, (10, 2), deformed=deformed)
        tanh_state(ar, 0.1)
        st = oracle.SavStorage(ar)
        av, resid = run(ar, st, 0.1, advect_iters=100, diff_iters=50)
        results.append((av, st.forcing.copy(), resid))
    (a, fa, ra), (b, fb, rb) = results
    assert a.max() > 0
    np.testing.assert_allclose(b, a, rtol=1e-11, atol=1e-11 * a.max())
    np.testing.assert_allclose(fb, fa, rtol=1e-11, atol=1e-11 * np.abs(fa).max())
    assert rb == pytest.approx(ra, rel=1e-10)


def test_3d_matches_2d():
    """Data that does not vary along z: the 3D kernels must reproduce the 2D result in every
    z-layer. Cartesian vertex time-step scales are h/n_dim (src/Element.cpp:17), so the 2D
    mesh is given the 3D value to take the same pseudo-time steps (the converged states agree
    whatever the step; the iterates only with equal steps)."""
    ar2 = strip(4, (10, 2))
    ar2.vert_tss[:] *= 2. / 3.
    tanh_state(ar2, 0.1)
    st2 = oracle.SavStorage(ar2)
    av2, _ = run(ar2, st2, 0.1, advect_iters=100, diff_iters=50)
    ar3 = strip(4, (10, 2, 2))
    tanh_state(ar3, 0.1)
    st3 = oracle.SavStorage(ar3)
    av3, _ = run(ar3, st3, 0.1, advect_iters=100, diff_iters=50)
    rs = 4
    # element (i, j, k) of the 3D mesh against (i, j) of the 2D one; qpoint (a, b, c) against (a, b)
    av3 = av3.reshape(10, 2, 2, rs, rs, rs)
    av2 = av2.reshape(10, 2, rs, rs)
    assert av2.max() > 0
    for kz in range(2):
        for c in range(rs):
            np.testing.assert_allclose(av3[:, :, kz, :, :, c], av2, rtol=1e-10, atol=1e-10 * av2.max())


@pytest.mark.parametrize("wall", [abi.BC_NO_SLIP, abi.BC_COPY])
def test_wall_kinds_agree(wall):
    """With no velocity across the walls, Nonpenetration (velocity reflected), No_slip
    (velocity negated) and Copy (traces copied) give the wall faces the same advection flux,
    so the coefficient must agree; a default boundary (advected scalars mirrored about 1)
    must not, which shows the walls are exercised."""
    out = {}
    for kind in (abi.BC_NONPENETRATION, wall, abi.BC_OUTFLOW):
        ar = strip(4, (10, 2), wall=kind)
        tanh_state(ar, 0.1)
        out[kind], _ = run(ar, oracle.SavStorage(ar), 0.1, advect_iters=100, diff_iters=50)
    ref = out[abi.BC_NONPENETRATION]
    np.testing.assert_allclose(out[wall], ref, rtol=1e-13, atol=1e-13 * ref.max())
    assert np.abs(out[abi.BC_OUTFLOW] - ref).max() > 1e-6 * ref.max()


def test_invalid_arguments():
    ar = strip(4, (4, 2))
    tanh_state(ar, 0.1)
    st = oracle.SavStorage(ar)
    o = oracle.Oracle(ar)
    for bad in (oracle.sav_params(0.1, 4, 1., 1.5, av_row_size=5), oracle.sav_params(0.1, 4, 1., 1.5, av_row_size=1),
                oracle.sav_params(0., 4, 1., 1.5)):
        with pytest.raises(RuntimeError):
            o.update_art_visc_smoothness(st, bad)
    with pytest.raises(ValueError):
        st.aux = np.asfortranarray(st.aux)
        o.update_art_visc_smoothness(st, oracle.sav_params(0.1, 4, 1., 1.5))


@pytest.mark.parametrize("nd", [2, 3])
def test_hanging_faces_uniform_flow(nd):
    """On a tree mesh with hanging faces, a uniform flow keeps the advected scalars at 1 and
    the coefficient at zero: prolongation is exact for constants and the coarse face's flux is
    the restriction of the fine fluxes (Spatial.hpp:138-285)."""
    from hexed_gb300 import problems
    from hexed_gb300.tree import tree_mesh
    fs = problems.freestream_state(nd, 0.3, 20., 1.2, 1e5)
    spec = bc_spec(abi.BC_FREESTREAM, freestream=fs)
    ar = tree_mesh(nd, 4, 2, 2, problems.sphere_refinement(nd, 0.3), {(d, s): spec for d in range(nd) for s in range(2)})
    assert len(ar.ref_face) > 0
    ar.set_state(lambda pos: np.stack([fs[v] + 0 * pos[0] for v in range(nd + 2)]))
    st = oracle.SavStorage(ar)
    p = oracle.sav_params(0.2, 4, fs[nd], fs[nd + 1], advect_iters=40, diff_iters=20)
    resid = oracle.Oracle(ar).update_art_visc_smoothness(st, p)
    assert np.isfinite(resid)
    np.testing.assert_allclose(st.advection, 1., rtol=0, atol=1e-12)
    assert np.abs(ar.elem[:, ar.nv + 1]).max() < 1e-12


@pytest.mark.parametrize("nd", [2, 3])
def test_curved_mesh_uniform_flow(nd):
    """Deformed elements with a smooth non-affine mapping (reference-level normals and
    determinants that vary over the element): a uniform flow keeps the advected scalars at 1
    and the coefficient at roundoff, i.e. the advection operator preserves a uniform state
    through the metric terms."""
    from hexed_gb300 import problems
    fs = problems.freestream_state(nd, 0.3, 20., 1.2, 1e5)
    spec = bc_spec(abi.BC_FREESTREAM, freestream=fs)
    ar = structured_mesh(nd, 4, 4, 0., 1., deformed=True,
                         displacement=problems.sinusoid_displacement(1. / 4, 0.1, 0, n_dim=nd),
                         bcs={(d, s): spec for d in range(nd) for s in range(2)})
    ar.set_state(lambda pos: np.stack([fs[v] + 0 * pos[0] for v in range(nd + 2)]))
    st = oracle.SavStorage(ar)
    p = oracle.sav_params(0.2, 4, fs[nd], fs[nd + 1], advect_iters=40, diff_iters=20)
    oracle.Oracle(ar).update_art_visc_smoothness(st, p)
    np.testing.assert_allclose(st.advection, 1., rtol=0, atol=1e-12)
    assert np.abs(ar.elem[:, ar.nv + 1]).max() < 1e-10


def test_chebyshev_substeps_same_steady_state():
    """n_cheby_av > 1 splits each diffusion iteration into Chebyshev sub-steps
    (src/Solver.cpp:447-454); the pseudo-time steady state does not depend on the split, so
    converged coefficients agree."""
    out = []
    for n_cheby, iters in ((1, 2400), (3, 800)):
        ar = strip(4, (10, 2))
        tanh_state(ar, 0.1)
        av, _ = run(ar, oracle.SavStorage(ar), 0.1, advect_iters=2000, diff_iters=iters, n_cheby=n_cheby)
        out.append(av)
    assert out[0].max() > 0
    np.testing.assert_allclose(out[1], out[0], rtol=0, atol=1e-10 * out[0].max())
