"""Deformed-element metrics against the reference's own "jacobian calculation" test
(test/test_Deformed_element.cpp:84-137), restated for the Gauss-Legendre basis.

The reference checks Deformed_element::set_jacobian on two elements of nominal size 0.2 with
one vertex moved to 0.8 x 0.2 in every coordinate: a 2D quad (vertex 3) and a 3D hex
(vertex 7). Its expected values are the multilinear map's Jacobian at equidistant nodes, the
determinant, and the vertex time-step scales h/n_dim and h/2 (0.8^2 - 0.2^2)/sqrt(0.8^2 + 0.2^2).
The map is multilinear, so its Jacobian, cofactor normals and determinant are polynomials
that every row size here represents exactly, and the analytic values hold at any node set:

* `analytic_jacobian` reproduces the reference's listed values at its equidistant nodes
  (the known answers are checked first);
* the host set-up (hexed_gb300.mesh.deformed_metrics) matches the analytic cofactor normals,
  determinant, face normals and vertex time-step scales at the Gauss-Legendre nodes;
* on the GPU, hexed_gpu_compute_jacobian recomputes the same arrays from the vertex
  positions and matches them too.
"""
import itertools

import numpy as np
import pytest

from hexed_gb300 import abi
from hexed_gb300.basis import Basis
from hexed_gb300.mesh import bc_spec, deformed_metrics, general_mesh

H = 0.2
TOL = 1e-13


def element_vertices(nd):
    """Vertices of the reference test's element: the unit hypercube scaled by h, with the
    last vertex (all bits set) moved to 0.8 h in every coordinate. Vertex bit d <-> dim d,
    dim 0 most significant."""
    verts = np.array([[(v >> (nd - 1 - d)) & 1 for d in range(nd)] for v in range(2 ** nd)], float) * H
    verts[-1] = 0.8 * H
    return verts


def analytic_jacobian(verts, xi):
    """d x_i / d xi_j / h of the multilinear map of `verts` at reference points xi [n][nd]."""
    nd = verts.shape[1]
    bits = np.array([[(v >> (nd - 1 - d)) & 1 for d in range(nd)] for v in range(2 ** nd)])
    jac = np.zeros((len(xi), nd, nd))
    for v, b in enumerate(bits):
        shape = np.where(b, xi, 1 - xi)                       # [n][nd]
        for j in range(nd):
            dshape = np.prod(np.delete(shape, j, axis=1), axis=1) * (1 if b[j] else -1)
            jac[:, :, j] += dshape[:, None] * verts[v][None, :]
    return jac / H


def cofactor(jac):
    """nrml[i][j] = det(J with column i replaced by e_j) and det(J)."""
    nd = jac.shape[-1]
    nrml = np.empty_like(jac)
    for i, j in itertools.product(range(nd), repeat=2):
        m = jac.copy()
        m[..., :, i] = 0.
        m[..., j, i] = 1.
        nrml[..., i, j] = np.linalg.det(m)
    return nrml, np.linalg.det(jac)


def grid(nodes, nd):
    """Reference coordinates of the qpoints (dim 0 slowest, include/Row_index.hpp)."""
    return np.array(list(itertools.product(nodes, repeat=nd)))


def test_analytic_map_reproduces_reference_values():
    """The known answers of test/test_Deformed_element.cpp:98-137 (equidistant row size 3)."""
    eq = np.array([0., .5, 1.])
    j2 = analytic_jacobian(element_vertices(2), grid(eq, 2))
    assert np.allclose(j2[0], [[1, 0], [0, 1]])
    assert np.allclose(j2[6], [[1, -.2], [0, .8]])
    assert np.allclose(j2[8], [[.8, -.2], [-.2, .8]])
    assert np.isclose(np.linalg.det(j2[6]), .8)
    j3 = analytic_jacobian(element_vertices(3), grid(eq, 3))
    assert np.array_equal(j3[0], np.eye(3))
    assert np.allclose([j3[26][0, 0], j3[26][0, 1], j3[26][0, 2], j3[26][2, 1], j3[26][2, 2]],
                       [.8, -.2, -.2, -.2, .8])


def expected_vertex_tss(nd):
    """Vertex time-step scale h det / sum_i |n_i| at the vertices (the reference lists vertex
    0, h/n_dim, and the moved vertex of the 2D element)."""
    verts = element_vertices(nd)
    corners = np.array([[(v >> (nd - 1 - d)) & 1 for d in range(nd)] for v in range(2 ** nd)], float)
    nrml, det = cofactor(analytic_jacobian(verts, corners))
    return H * det / np.sqrt((nrml ** 2).sum(axis=2)).sum(axis=1)


def test_vertex_tss_formula_matches_reference_values():
    v2 = expected_vertex_tss(2)
    assert v2[0] == pytest.approx(.2 / 2, rel=1e-15)
    assert v2[3] == pytest.approx(.2 / 2 * (.8 * .8 - .2 * .2) / np.sqrt(.8 * .8 + .2 * .2), rel=1e-14)


def check_metrics(nd, rs, jac_dat, face_nrml, vtss):
    b = Basis(rs)
    verts = element_vertices(nd)
    nrml, det = cofactor(analytic_jacobian(verts, grid(b.nodes, nd)))
    want = np.concatenate([np.moveaxis(nrml, 0, 2).reshape(nd * nd, -1), det[None]])
    assert np.abs(jac_dat - want).max() <= TOL
    for i_dim, sign in itertools.product(range(nd), range(2)):
        face_pts = grid(b.nodes, nd - 1)
        xi = np.insert(face_pts, i_dim, float(sign), axis=1)
        fn, _ = cofactor(analytic_jacobian(verts, xi))
        assert np.abs(face_nrml[2 * i_dim + sign] - fn[:, i_dim, :].T).max() <= TOL, (i_dim, sign)
    assert np.abs(vtss - expected_vertex_tss(nd)).max() <= TOL


@pytest.mark.parametrize("nd,rs", [(2, 2), (2, 3), (2, 6), (3, 3), (3, 4), (3, 6)])
def test_host_setup_matches_reference_element(nd, rs):
    jac_dat, face_nrml, vtss, _ = deformed_metrics(element_vertices(nd)[None], np.array([H]), Basis(rs), nd)
    check_metrics(nd, rs, jac_dat[0], face_nrml[0], vtss[0])


def single_element(nd, rs):
    spec = bc_spec(abi.BC_NONPENETRATION)
    bounds = [(0, d, s, 0) for d in range(nd) for s in range(2)]
    return general_mesh(nd, rs, element_vertices(nd)[None], [H], [True], [], bounds, [spec])


@pytest.mark.gpu
@pytest.mark.parametrize("nd,rs", [(2, 3), (2, 6), (3, 3), (3, 6)])
def test_device_setup_matches_reference_element(nd, rs):
    from hexed_gb300.solver import Context
    ar = single_element(nd, rs)
    with Context(ar.copy()) as c:
        for which, host in ((abi.ARRAY_JAC, ar.jac), (abi.ARRAY_FACE_NRML, ar.face_nrml),
                            (abi.ARRAY_VERT_TSS, ar.vert_tss)):
            c.write_range(which, 0, np.zeros(host.size))
        c.compute_jacobian(ar.vert_pos[ar.n_car:])
        jac = c.read_range(abi.ARRAY_JAC, 0, ar.jac.size).reshape(ar.jac.shape)
        fn = c.read_range(abi.ARRAY_FACE_NRML, 0, ar.face_nrml.size).reshape(ar.face_nrml.shape)
        vt = c.read_range(abi.ARRAY_VERT_TSS, 0, ar.vert_tss.size).reshape(ar.vert_tss.shape)
    check_metrics(nd, rs, jac[0], fn[0], vt[0])
