"""Artificial viscosity (Stab_art_visc + Solver::set_art_visc_admis) on the CPU oracle:
smooth states get no viscosity, a discontinuity does, and the vertex-maximum sharing makes
the coefficient continuous across elements."""
import numpy as np

import oracle
from hexed_gb300 import abi, problems


def test_av_zero_for_smooth_and_positive_at_jump():
    n = 5   # odd: the jump plane x = pi cuts the middle layer of elements
    ar = problems.mach2_jump_3d(n_per_side=n, row_size=4)
    o = oracle.Oracle(ar)
    o.set_art_visc_admis(ar.av_char_speed)
    lap = ar.elem[:, ar.nv + 2]
    x_centre = ar.qpoint_pos[:, 0].mean(axis=1)
    h = 2 * np.pi / n
    near = np.abs(x_centre - np.pi) < h / 2
    assert lap[near].min() > 0
    # elements whose vertices are not shared with the cut layer see none
    far = np.abs(x_centre - np.pi) > 2 * h
    assert np.all(lap[far] == 0)
    assert np.all(lap >= 0)


def test_av_vertex_continuity():
    """Coefficients of neighbouring elements agree at shared vertices (C^0)."""
    ar = problems.mach2_jump_3d(n_per_side=3, row_size=3)
    oracle.Oracle(ar).set_art_visc_admis(ar.av_char_speed)
    # corner qpoints are not at vertices (Gauss nodes); compare the multilinear vertex values
    # recovered from two elements sharing a face through their qpoint fits instead: simplest,
    # the element-wise vertex values must match the shared maximum table.
    vals = {}
    lap = ar.elem[:, ar.nv + 2]
    for e in range(ar.n_elem):
        # recover the 8 vertex values from the trilinear field by least squares
        from hexed_gb300.basis import Basis
        b = Basis(3)
        x = b.nodes
        rows = []
        for q in range(27):
            c = [x[(q // 3 ** (2 - d)) % 3] for d in range(3)]
            rows.append([np.prod([c[d] if (v >> (2 - d)) & 1 else 1 - c[d] for d in range(3)]) for v in range(8)])
        vv = np.linalg.lstsq(np.array(rows), lap[e], rcond=None)[0]
        for v in range(8):
            vid = ar.vert_ids[e, v]
            if vid in vals:
                assert abs(vals[vid] - vv[v]) <= 1e-9 * max(1., abs(vv[v]))
            vals[vid] = vv[v]


def test_av_update_runs_and_conserves():
    ar = problems.mach2_jump_3d(n_per_side=3, row_size=3)
    o = oracle.Oracle(ar)
    o.write_face()
    p = abi.update_params(max_safety=0.5, av_admis_char_speed=ar.av_char_speed)
    assert p.use_ldg == 1
    for _ in range(3):
        o.update(p)
    assert np.isfinite(ar.elem).all()
