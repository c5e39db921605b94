"""The reference's own hot-path tests, restated against the CPU oracle.

These pin the oracle (and through the parity tests, the CUDA library) to the reference's
behaviour: test/test_Derivative.cpp, test/test_Max_dt.cpp, test/test_Prolong_refined.cpp,
test/test_Restrict_refined.cpp, test/test_Face_permutation.cpp, test/test_Characteristics.cpp,
test/test_Boundary_condition.cpp and test/test_Solver.cpp (marching, conservation).
Catch's default Approx is 1.2e-5 relative; the bounds here are as tight or tighter.
"""
import itertools
import math

import numpy as np
import pytest

import oracle
from hexed_gb300 import abi, mesh, problems
from hexed_gb300.basis import Basis
from hexed_gb300.mesh import Arena, bc_spec, general_mesh, oriented_neighbor, pack_dir, structured_mesh

MAX_RS = 8


# ---------------------------------------------------------------- helpers
def single_elements(n_dim, rs, n_elem, nom_size=1.):
    ar = Arena(n_dim, rs, n_elem, 0)
    ar.nom_size[:] = nom_size
    ar.vert_tss[:] = nom_size / n_dim
    return ar.finalize()


def face_arena(n_dim, rs, spec, i_dim, ifs, normal):
    """One Cartesian element with one boundary connection on face (i_dim, ifs)."""
    ar = Arena(n_dim, rs, 1, 0)
    ar.nom_size[:] = 1.
    ar.bc_specs = [spec]
    ar.bc_con = np.array([[ar.slot_of(0, 2 * i_dim + ifs), 2 * n_dim, i_dim | (ifs << 2), 0]], np.int32)
    ar.bc_nrml = np.array(normal, float).reshape(1, n_dim, ar.nfq)
    ar.n_slot = 2 * n_dim + 1
    return ar.finalize()


def inside(ar, ldg=False):
    return ar.face[ar.bc_con[0, 0], int(ldg)]


def ghost(ar, ldg=False):
    return ar.face[ar.bc_con[0, 1], int(ldg)]


# ---------------------------------------------------------------- Derivative
def test_derivative():  # test/test_Derivative.cpp:11-46
    rs = MAX_RS
    b = Basis(rs)
    x = b.nodes
    poly = [0.1 * x * x - i * x - 3. for i in range(3)]
    bvals = [np.array([0.1 * s * s - i * s - 3. for s in (0., 1.)]) for i in range(3)]
    bvals[2] = np.array([0.2, 0.5])
    for i in range(2):
        np.testing.assert_allclose(oracle.derivative(rs, poly[i], bvals[i]), 0.2 * x - i, atol=1e-11)
    res = oracle.derivative(rs, poly[2], bvals[2])
    assert (res * b.node_weights).sum() == pytest.approx(0.5 - 0.2, abs=1e-12)


# ---------------------------------------------------------------- Max_dt
def test_max_dt_cartesian_2d():  # test/test_Max_dt.cpp:40-58
    ar = single_elements(2, 2, 1)
    for q in range(4):
        ar.elem[0, :4, q] = [2.25, 24.5, 1.225, 101235 / 0.4 + 0.5 * 1.225 * 500]
    o = oracle.Oracle(ar)
    o.max_dt(1., 1., local_time=True)
    max_cfl = Basis(2).max_cfl
    np.testing.assert_allclose(ar.tss[0], max_cfl / 360. / 2., rtol=0.01)


def test_max_dt_deformed():  # test/test_Max_dt.cpp:60-105
    rs, nd, h = 4, 3, 0.3
    basis = Basis(rs)
    bits = np.array(list(itertools.product(range(2), repeat=3)), float)
    verts = np.stack([bits * h] * 3)
    sound = [100., 1000., 100.]

    def build(verts):
        ar = Arena(nd, rs, 0, 3)
        ar.nom_size[:] = h
        jac, fn, vtss, qpos = mesh.deformed_metrics(verts, ar.nom_size, basis, nd)
        ar.jac[:] = jac
        ar.face_nrml[:] = fn
        ar.vert_tss[:] = vtss
        ar.finalize()
        for e in range(3):
            ar.elem[e, :3] = 0.
            ar.elem[e, 3] = 1.4
            ar.elem[e, 4] = (1e6 if e == 1 else 1e4) / 0.4
        return ar
    ar = build(verts)
    oracle.Oracle(ar).max_dt(1., 1., local_time=True)
    for e in range(3):
        np.testing.assert_allclose(ar.tss[e], basis.max_cfl / (sound[e] / h) / 3., rtol=1e-12)
    verts = verts.copy()
    verts[1, :, 0] *= .5
    verts[1, :, 1] *= .5
    ar = build(verts)
    dt = oracle.Oracle(ar).max_dt(1., 1., local_time=False)
    assert dt == pytest.approx(basis.max_cfl / (1e3 * (1. + 2 * 2.) / 3. / h) / 3., rel=1e-12)


# ---------------------------------------------------------------- Prolong / Restrict
def refined_arena(rs, stretch):
    ar = Arena(3, rs, 1, 0)
    ar.nom_size[:] = 1.
    ar.ref_face = np.array([[0, 6, 7, 8, 9, int(stretch[0]), int(stretch[1])]], np.int32)
    ar.n_slot = 10
    return ar.finalize()


def exp_face(b, i_off=0., i_scale=1., j_off=0., j_scale=1.):
    x = b.nodes
    xi = (x[:, None] + i_off) * i_scale
    xj = (x[None, :] + j_off) * j_scale
    return np.stack([np.exp(xi + 0.5 * xj) + v for v in range(5)]).reshape(5, -1)


@pytest.mark.parametrize("stretch", [(False, False), (True, False), (False, True)])
def test_prolong_refined(stretch):  # test/test_Prolong_refined.cpp:6-84
    rs = MAX_RS
    b = Basis(rs)
    ar = refined_arena(rs, stretch)
    ar.face[0, 0] = exp_face(b)
    oracle.Oracle(ar).prolong()
    for k in range(4 // (1 + stretch[0]) // (1 + stretch[1])):
        if stretch == (False, False):
            ih, jh = k // 2, k % 2
            want = exp_face(b, ih, .5, jh, .5)
        elif stretch[0]:
            want = exp_face(b, 0., 1., k, .5)
        else:
            want = exp_face(b, k, .5, 0., 1.)
        np.testing.assert_allclose(ar.face[6 + k, 0], want, atol=1e-4)


@pytest.mark.parametrize("stretch", [(False, False), (True, False), (False, True)])
def test_restrict_refined(stretch):  # test/test_Restrict_refined.cpp:6-88
    rs = MAX_RS
    b = Basis(rs)
    ar = refined_arena(rs, stretch)
    for k in range(4 // (1 + stretch[0]) // (1 + stretch[1])):
        if stretch == (False, False):
            ar.face[6 + k, 0] = exp_face(b, k // 2, .5, k % 2, .5)
        elif stretch[0]:
            ar.face[6 + k, 0] = exp_face(b, 0., 1., k, .5)
        else:
            ar.face[6 + k, 0] = exp_face(b, k, .5, 0., 1.)
    oracle.Oracle(ar).restrict()
    factor = 1. if stretch == (False, False) else .5
    np.testing.assert_allclose(ar.face[0, 0], factor * exp_face(b), atol=1e-4)


# ---------------------------------------------------------------- Face_permutation
def face_positions(ar, e, i_face):
    """Physical position of face qpoints (Element::face_position, src/Element.cpp:74-97)."""
    nd, rs = ar.n_dim, ar.row_size
    b = Basis(rs)
    pos = ar.qpoint_pos[e].reshape((nd,) + (rs,) * nd)
    d, s = i_face // 2, i_face % 2
    f = np.moveaxis(pos, 1 + d, -1) @ b.boundary[s]
    return f.reshape(nd, -1)


def all_directions(nd):
    for i0, i1 in itertools.product(range(nd), repeat=2):
        for s0, s1 in itertools.product(range(2), repeat=2):
            if i0 == i1 and s0 == s1:
                continue   # forbidden (src/Accessible_mesh.cpp:181-185)
            yield pack_dir(i0, i1, s0, s1)


@pytest.mark.parametrize("nd", [2, 3])
def test_face_permutation(nd):  # test/test_Face_permutation.cpp:8-74
    rs = 4
    for d in all_directions(nd):
        p0, p1 = oriented_neighbor(nd, d)
        i0, i1, s0, s1 = d & 3, (d >> 2) & 3, (d >> 4) & 1, (d >> 5) & 1
        ar = general_mesh(nd, rs, np.stack([p0, p1]), [1., 1.], [True, True],
                          [(0, 1, i0, i1, s0, s1)], [], [])
        f0 = face_positions(ar, 0, 2 * i0 + s0)
        f1 = face_positions(ar, 1, 2 * i1 + s1)
        perm = [oracle.perm_index(nd, rs, d, q) for q in range(ar.nfq)]
        np.testing.assert_allclose(f1[:, perm], f0, atol=1e-12, err_msg=f"direction {d}")
        # python restatement used by the mesh builder agrees with the oracle
        assert perm == [mesh.face_perm_index(nd, rs, d, q) for q in range(ar.nfq)]


# ---------------------------------------------------------------- Characteristics
def flux_1d(state, normal):
    nd = len(normal)
    m = state[nd]
    kin = 0.5 * sum(state[i] ** 2 for i in range(nd)) / m
    p = 0.4 * (state[nd + 1] - kin)
    mom_n = sum(state[i] * normal[i] for i in range(nd))
    f = np.empty(nd + 2)
    f[nd] = mom_n
    f[nd + 1] = (state[nd + 1] + p) * mom_n / m
    for i in range(nd):
        f[i] = state[i] * mom_n / m + p * normal[i]
    return f


def test_characteristics():  # test/test_Characteristics.cpp:4-43
    mass = 1.225
    veloc = np.array([10., 4., 12.])
    pres = 101325.
    state = np.concatenate([mass * veloc, [mass, pres / .4 + .5 * mass * veloc @ veloc]])
    normal = np.array([1., 1., 1.])
    state1 = np.array([1., 2., 3., 1.3, 2e5])
    eig, dec = oracle.characteristics(3, state, normal, state1)
    assert np.linalg.norm((dec.sum(axis=1) - state1) / state1) < 1e-12
    diff = 1e-6
    for i in range(3):
        vec = dec[:, i]
        pert = (flux_1d(state + diff * vec, normal) - flux_1d(state, normal)) / np.linalg.norm(normal)
        assert np.linalg.norm(pert / (diff * eig[i] * vec) - 1.) < 1e-4


# ---------------------------------------------------------------- boundary conditions
def test_freestream_and_copy():  # test/test_Boundary_condition.cpp:50-76, 276-302
    rs = MAX_RS
    fs = [10., 30., -20., 1.3, 1.2e5]
    for kind, want in ((abi.BC_FREESTREAM, fs), (abi.BC_COPY, [20., -10., 50., 0.9, 1e4])):
        ar = face_arena(3, rs, bc_spec(kind, freestream=fs), 1, 0, np.zeros((3, rs * rs)))
        inside(ar)[:] = np.array([20., -10., 50., 0.9, 1e4])[:, None]
        oracle.Oracle(ar).apply_state_bcs()
        np.testing.assert_allclose(ghost(ar), np.array(want)[:, None] * np.ones(rs * rs))


def test_riemann_invariants_supersonic_inflow():  # test/test_Boundary_condition.cpp:78-123
    rs = MAX_RS
    nfq = rs * rs
    fs = np.array([10., 30., -20., 1.3, 4e5])
    nrml = np.zeros((3, nfq))
    nrml[1] = 1.
    ar = face_arena(3, rs, bc_spec(abi.BC_RIEMANN, freestream=fs), 1, 0, nrml)
    ins = np.array([1 / 1.2, -600 / 1.2, 1 / 1.2, 1.2, 101325 / .4 + .5 * 1.2 * 360002])
    for q in range(nfq):
        st = ins.copy()
        if q:
            st[1] *= -1
        inside(ar)[:, q] = st
    o = oracle.Oracle(ar)
    o.apply_state_bcs()
    for q in range(nfq):
        np.testing.assert_allclose(ghost(ar)[:, q], fs if q else ins, rtol=1e-10)
    inside(ar, True)[:] = 1.
    o.apply_flux_bcs()
    for q in range(nfq):
        np.testing.assert_allclose(ghost(ar, True)[:, q], 1. if q else 0., atol=1e-9)


def test_nonpenetration():  # test/test_Boundary_condition.cpp:150-193
    rs = MAX_RS
    nrml = np.array([[-4.] * rs, [3.] * rs])
    ar = face_arena(2, rs, bc_spec(abi.BC_NONPENETRATION), 0, 1, nrml)
    state = np.array([1., 1., 1.2, 1e5 / 0.4 + 0.5 * 1.2 * 2.])
    for ldg in (False, True):
        inside(ar, ldg)[:] = state[:, None]
    o = oracle.Oracle(ar)
    o.apply_state_bcs()
    g = ghost(ar)
    np.testing.assert_allclose(3 * g[0] + 4 * g[1], 7.)
    np.testing.assert_allclose(-4 * g[0] + 3 * g[1], 1.)
    o.apply_flux_bcs()
    g = ghost(ar, True)
    np.testing.assert_allclose(3 * g[0] + 4 * g[1], -7.)
    np.testing.assert_allclose(-4 * g[0] + 3 * g[1], -1.)
    np.testing.assert_allclose(g[2:], -inside(ar, True)[2:])


@pytest.mark.parametrize("thermal", ["isothermal", "flux", "emissivity"])
def test_no_slip(thermal):  # test/test_Boundary_condition.cpp:195-274
    rs = MAX_RS
    nrml = np.full((2, rs), .7 / math.sqrt(2.))
    state = np.array([1., 1., 1.2, 1e5 / 0.4 + 0.5 * 1.2 * 2.])
    flux = np.array([10., -20., 1.3, 10.])
    if thermal == "isothermal":
        spec = bc_spec(abi.BC_NO_SLIP, thermal_kind=abi.THERMAL_ENERGY, thermal_value=1e6)
    elif thermal == "flux":
        spec = bc_spec(abi.BC_NO_SLIP, thermal_kind=abi.THERMAL_HEAT_FLUX, thermal_value=3.)
    else:
        spec = bc_spec(abi.BC_NO_SLIP, thermal_kind=abi.THERMAL_EQUILIBRIUM, emissivity=.8)
        state[3] = 1e5 / .4
    ar = face_arena(2, rs, spec, 0, 0, nrml)
    inside(ar)[:] = state[:, None]
    o = oracle.Oracle(ar)
    o.apply_state_bcs()
    g = ghost(ar)
    if thermal == "isothermal":
        np.testing.assert_allclose(g[:2], -1.)
        np.testing.assert_allclose(g[2], 1.2)
        np.testing.assert_allclose(np.sqrt(g[3] * inside(ar)[3]), 1e6 * 1.2)
    elif thermal == "flux":
        np.testing.assert_allclose(g[:2], -1.)
        np.testing.assert_allclose(g[2:], state[2:, None] * np.ones(rs))
    inside(ar, True)[:] = flux[:, None]
    if thermal == "emissivity":
        inside(ar)[:] = 0.
    o.apply_flux_bcs()
    g = ghost(ar, True)
    want = flux.copy()
    want[2] *= -1
    if thermal == "isothermal":
        np.testing.assert_allclose(g, want[:, None] * np.ones(rs))
    elif thermal == "flux":
        np.testing.assert_allclose(g[:3], want[:3, None] * np.ones(rs))
        np.testing.assert_allclose((g[3] + inside(ar, True)[3]) / 2, -3. * .7)
    else:
        sb = 2 * math.pi ** 5 * 1.380649e-23 ** 4 / (15 * 299792458. ** 2 * 6.62607015e-34 ** 3)
        temp = 1e5 / 1.2 / 287.05287
        np.testing.assert_allclose((g[3] + inside(ar, True)[3]) / 2, -.8 * sb * temp ** 4 * .7, rtol=1e-12)


# ---------------------------------------------------------------- Solver
VELOCS = np.array([0.3, -0.7, 0.8])
WAVE = np.array([-0.1, 0.3, 0.2])


def nonuniform_mass(pos):  # test/test_Solver.cpp:103-124
    nd = pos.shape[0]
    sp = sum(WAVE[d] * pos[d] for d in range(nd))
    vsq = float((VELOCS[:nd] ** 2).sum())
    mass = 1. + 0.1 * np.sin(sp)
    return np.stack([mass * VELOCS[d] for d in range(nd)] + [mass, 1e5 / 0.4 + mass * 0.5 * vsq])


def nonuniform_residual(pos):  # test/test_Solver.cpp:149-168
    nd = pos.shape[0]
    sp = sum(WAVE[d] * pos[d] for d in range(nd))
    vsq = float((VELOCS[:nd] ** 2).sum())
    d_mass = -0.1 * float(VELOCS[:nd] @ WAVE[:nd]) * np.cos(sp)
    return np.stack([d_mass * VELOCS[d] for d in range(nd)] + [d_mass, d_mass * 0.5 * vsq])


@pytest.mark.parametrize("case", ["cartesian_3d", "deformed_2d", "tree_2d", "tree_3d"])
def test_marching(case):  # test/test_Solver.cpp:555-586
    ar = marching_mesh(case)
    ar.set_state(nonuniform_mass)
    o = oracle.Oracle(ar)
    o.write_face()
    o.prolong()
    state0 = ar.state.copy()
    p = abi.update_params(max_safety=1e-3)
    dt = o.update(p)
    assert dt > 0
    o.compute_residual(p)
    update = ar.rcache / ar.tss[:, None, :]
    correct = nonuniform_residual(ar.qpoint_pos.transpose(1, 0, 2)).transpose(1, 0, 2)
    assert np.all(np.abs(update - correct) <= 1e-3 * np.abs(ar.state)), np.abs(update - correct).max()
    assert np.abs(ar.state - state0).max() > 0


def sinusoid_veloc0(pos):  # test/test_Solver.cpp:57-75
    """Constant density and pressure, divergence-free sinusoidal velocity."""
    nd = pos.shape[0]
    cos_part = np.cos(sum(pos[d] for d in range(nd)))
    mom = [1.2 * cos_part for _ in range(nd)]
    mom[0] = mom[0] * (1 - nd)
    energy = 1e5 / 0.4 + .5 * 1.2 * (nd - 1 + (1 - nd) * (1 - nd)) * cos_part * cos_part
    return np.stack(mom + [1.2 + 0 * cos_part, energy])


def marching_mesh(case, rs=6):
    """The meshes of the restated marching tests, with Copy boundaries: Cartesian 3D, deformed
    2D, and tree meshes with hanging faces (2D, 3D) standing in for the reference's extruded
    hanging-node meshes."""
    copy = bc_spec(abi.BC_COPY)
    if case.startswith("tree"):
        from hexed_gb300.tree import tree_mesh
        nd = int(case[-2])
        ar = tree_mesh(nd, rs, 2, 2, problems.sphere_refinement(2, 0.3), {(d, s): copy for d in range(nd) for s in range(2)})
        assert len(ar.ref_face) > 0
        return ar
    if case == "cartesian_3d":
        return structured_mesh(3, rs, 2, 0., 2., bcs={(d, s): copy for d in range(3) for s in range(2)})
    return structured_mesh(2, rs, 3, 0., 3., deformed=True, displacement=problems.sinusoid_displacement(1., .1, 3, 2),
                           bcs={(d, s): copy for d in range(2) for s in range(2)})


def viscous_rate_check(ar, rcache, tss, state):
    """test/test_Solver.cpp:588-615: with constant viscosity 3 the momentum rate is
    -n_dim 3 u (u = momentum / 1.2), to an absolute margin of 1.2 x 1e-3 when the row size is
    above 6 and 1.2 otherwise (the reference runs the test at its build's maximum row size and
    takes the margin from that)."""
    nd = ar.n_dim
    rate = rcache[:, :nd] / tss[:, None, :]
    want = -nd * 3. * state[:, :nd] / 1.2
    err = np.abs(rate - want).max()
    assert err <= 1.2 * (1e-3 if ar.row_size > 6 else 1.), err
    return err


VISCOSITY_CASES = [("cartesian_3d", 8), ("deformed_2d", 8), ("tree_2d", 8), ("tree_3d", 8), ("cartesian_3d", 6),
                   ("deformed_2d", 6)]


@pytest.mark.parametrize("case,rs", VISCOSITY_CASES)
def test_viscosity(case, rs):  # test/test_Solver.cpp:588-615
    ar = marching_mesh(case, rs)
    ar.set_state(sinusoid_veloc0)
    o = oracle.Oracle(ar)
    o.write_face()
    o.prolong()
    visc = abi.transport_constant(3.)
    p = abi.update_params(max_safety=1e-4, visc=visc, cond=abi.transport_inviscid())
    dt = o.update(p)
    assert dt > 0
    o.compute_residual(p)
    viscous_rate_check(ar, ar.rcache, ar.tss, ar.state)


@pytest.mark.parametrize("nd,deformed", [(2, False), (3, False), (2, True), (3, True)])
def test_conservation(nd, deformed):  # test/test_Solver.cpp:617-639
    rng = np.random.default_rng(406)
    nonpen = bc_spec(abi.BC_NONPENETRATION)
    n = 3
    disp = problems.sinusoid_displacement(1. / n, .1, 5, nd) if deformed else None
    ar = structured_mesh(nd, 4, n, 0., 1., deformed=deformed, displacement=disp,
                         bcs={(d, s): nonpen for d in range(nd) for s in range(2)})

    def random_perturbation(pos):
        shape = pos.shape[1:]
        rp = lambda: 1. + 0.1 * rng.integers(0, 1000, size=shape) / 1000  # noqa: E731
        return np.stack([1.05 * VELOCS[d] * rp() for d in range(nd)] + [1.05 * rp(), 1e5 / 0.4 * rp()])
    ar.set_state(random_perturbation)
    ar.elem[:, ar.nv + 1] = 30.   # Solver::set_art_visc_constant (src/Solver.cpp:415-425)
    o = oracle.Oracle(ar)
    o.write_face()
    visc = abi.transport_inviscid()
    p = abi.update_params(max_safety=.01, visc=visc, cond=visc, use_ldg=True)
    o.update(p)
    o.compute_residual(p)
    b = Basis(4)
    w = np.prod(np.stack(np.meshgrid(*([b.node_weights] * nd), indexing="ij")), axis=0).ravel()
    det = ar.jac[:, nd * nd] if deformed else np.ones((ar.n_elem, ar.nq))
    vol = ar.nom_size[:, None] ** nd * w[None] * det
    for v in (nd, nd + 1):
        resid = (ar.rcache[:, v] / ar.tss * vol).sum()
        total = (ar.state[:, v] * vol).sum()
        assert abs(resid) <= 1e-9 * abs(total), (v, resid, total)


def test_invalid_row_size_rejected():
    """kernel_factory throws for out-of-range (n_dim, row_size) (include/kernel_factory.hpp:111-119)."""
    ar = single_elements(2, 2, 1)
    d = ar.desc()
    d.row_size = 9
    import ctypes
    lib = oracle.load()
    assert lib.oracle_write_face(ctypes.byref(d)) != 0
