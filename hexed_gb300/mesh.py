"""Mesh arena construction (set-up time, host side, numpy).

Builds the flat arena of include/hexed_gpu.h for structured meshes of Cartesian or
deformed (multilinear) quad/hex elements and for tree-refined meshes with hanging faces.
Mesh generation is not on the hot path; this module restates only what the kernels need
from the reference's set-up:

* element storage and vertex time-step scale (src/Element.cpp:7-52),
* Deformed_element::set_jacobian: qpoint positions by multilinear vertex interpolation,
  Jacobian by the differentiation matrix, reference-level normals as determinants with
  one column replaced by a unit vector, face normals, vertex time-step scale
  (src/Deformed_element.cpp:15-135),
* Solver::calc_jacobian: shared face normals of deformed connections and boundary faces,
  vertex-minimum sharing of the vertex time-step scale (src/Solver.cpp:273-381),
* element / boundary connections and their directions (include/connection.hpp:20-36,
  321-382).
"""
from __future__ import annotations

import ctypes
import itertools

import numpy as np

from . import abi
from .basis import Basis


def _ptr(a, ctype=ctypes.c_double):
    if a is None:
        return ctypes.POINTER(ctype)()
    return a.ctypes.data_as(ctypes.POINTER(ctype))


def bc_spec(kind, freestream=None, pressure=0., coercion=2., thermal_kind=abi.THERMAL_HEAT_FLUX,
            thermal_value=0., emissivity=0., heat_transfer_coef=0., temperature=0.):
    fs = list(freestream) if freestream is not None else []
    fs = fs + [0.] * (5 - len(fs))
    return abi.BcSpec(kind, thermal_kind, (ctypes.c_double * 5)(*fs), pressure, coercion, thermal_value,
                      emissivity, heat_transfer_coef, temperature)


class Arena:
    """Host mirror of the device arena (see include/hexed_gpu.h for the layout)."""

    def __init__(self, n_dim, row_size, n_car, n_def):
        self.n_dim, self.row_size = n_dim, row_size
        self.nq = row_size ** n_dim
        self.nfq = row_size ** (n_dim - 1)
        self.nv = n_dim + 2
        self.nvert = 2 ** n_dim
        self.n_car, self.n_def = n_car, n_def
        self.n_elem = n_car + n_def
        E, nv, nq, nfq, nd = self.n_elem, self.nv, self.nq, self.nfq, n_dim
        self.elem = np.zeros((E, nv + 3, nq))
        self.elem[:, nv, :] = 1.  # time-step scale initialised to 1 (src/Element.cpp:22)
        self.rcache = np.zeros((E, nv, nq))
        self.nom_size = np.zeros(E)
        self.vert_tss = np.zeros((E, self.nvert))
        self.jac = np.zeros((n_def, nd * nd + 1, nq))
        self.face_nrml = np.zeros((n_def, 2 * nd, nd, nfq))
        self.car_con = np.zeros((0, 3), np.int32)
        self.def_con = np.zeros((0, 3), np.int32)
        self.def_con_nrml = np.zeros((0, nd, nfq))
        self.bc_con = np.zeros((0, 4), np.int32)
        self.bc_nrml = np.zeros((0, nd, nfq))
        self.ref_face = np.zeros((0, 7), np.int32)
        self.bc_specs = []
        self.n_slot = E * 2 * nd
        self.face = None
        self.bc_cache = None
        # set-up only data (not part of the device arena)
        self.qpoint_pos = None        # [E][nd][nq] physical qpoint positions
        self.vert_ids = None          # [E][nvert] global vertex ids
        self.vert_pos = None          # [E][nvert][nd] element vertex positions

    def finalize(self):
        nv, nfq = self.nv, self.nfq
        self.face = np.zeros((self.n_slot, 2, nv, nfq))
        self.bc_cache = np.zeros((len(self.bc_con), 2, nv, nfq))
        for name in ("car_con", "def_con", "bc_con", "ref_face"):
            setattr(self, name, np.ascontiguousarray(getattr(self, name), dtype=np.int32))
        for name in ("elem", "rcache", "nom_size", "vert_tss", "jac", "face_nrml", "def_con_nrml", "bc_nrml"):
            setattr(self, name, np.ascontiguousarray(getattr(self, name), dtype=np.float64))
        return self

    def desc(self):
        """hexed_mesh_desc pointing at this arena's arrays (kept alive by self)."""
        specs = (abi.BcSpec * max(1, len(self.bc_specs)))(*self.bc_specs)
        self._specs_keepalive = specs
        d = abi.MeshDesc()
        d.n_dim, d.row_size = self.n_dim, self.row_size
        d.n_car_elem, d.n_def_elem = self.n_car, self.n_def
        d.n_slot = self.n_slot
        d.n_car_con, d.n_def_con = len(self.car_con), len(self.def_con)
        d.n_bc_con, d.n_ref_face, d.n_bc_spec = len(self.bc_con), len(self.ref_face), len(self.bc_specs)
        d.elem, d.rcache, d.face = _ptr(self.elem), _ptr(self.rcache), _ptr(self.face)
        d.nom_size, d.vert_tss = _ptr(self.nom_size), _ptr(self.vert_tss)
        d.jac, d.face_nrml = _ptr(self.jac), _ptr(self.face_nrml)
        d.car_con = _ptr(self.car_con, ctypes.c_int)
        d.def_con = _ptr(self.def_con, ctypes.c_int)
        d.def_con_nrml = _ptr(self.def_con_nrml)
        d.bc_con = _ptr(self.bc_con, ctypes.c_int)
        d.bc_nrml, d.bc_cache = _ptr(self.bc_nrml), _ptr(self.bc_cache)
        d.ref_face = _ptr(self.ref_face, ctypes.c_int)
        d.bc_spec = ctypes.cast(specs, ctypes.POINTER(abi.BcSpec))
        if self.vert_ids is not None:
            ids = np.ascontiguousarray(self.vert_ids, dtype=np.int32)
            self._vid_keepalive = ids
            d.n_vert = int(ids.max()) + 1
            d.vert_id = _ptr(ids, ctypes.c_int)
        return d

    def copy(self):
        other = Arena.__new__(Arena)
        for k, v in self.__dict__.items():
            if isinstance(v, np.ndarray):
                v = v.copy()
            elif isinstance(v, list):
                v = list(v)
            setattr(other, k, v)
        return other

    @property
    def state(self):
        return self.elem[:, :self.nv, :]

    @property
    def tss(self):
        return self.elem[:, self.nv, :]

    def slot_of(self, e, i_face):
        return e * 2 * self.n_dim + i_face

    def n_dof(self):
        return self.n_elem * self.nv * self.nq

    # ------------------------------------------------------------- set-up helpers
    def set_state(self, fn):
        """Sample an initial condition fn(pos[nd][...]) -> state[nv][...] at the qpoints
        (Solver::initialize, src/Solver.cpp:383-397)."""
        st = fn(self.qpoint_pos.transpose(1, 0, 2))  # [nd][E][nq] -> [nv][E][nq]
        self.elem[:, :self.nv, :] = np.asarray(st).transpose(1, 0, 2)


def _node_coords(basis, n_dim):
    """coords[d][q] = node of qpoint q along dim d (include/Row_index.hpp)."""
    rs = basis.row_size
    q = np.arange(rs ** n_dim)
    return np.stack([basis.nodes[(q // rs ** (n_dim - 1 - d)) % rs] for d in range(n_dim)])


def _contract_axis(arr, mat, axis):
    """Apply mat[a][k] along `axis` of arr (elements leading)."""
    arr = np.moveaxis(arr, axis, -1)
    out = arr @ mat.T
    return np.moveaxis(out, -1, axis)


def _qpoint_positions(vert_pos, basis, n_dim):
    """Multilinear interpolation of the vertex positions to the qpoints, contracting the
    last reference dimension first (Deformed_element::position, src/Deformed_element.cpp:15-58).
    vert_pos [E][nvert][nd] -> [E][nd][rs, ...]"""
    rs = basis.row_size
    lin = np.stack([1. - basis.nodes, basis.nodes], axis=1)  # [rs][2]
    E = vert_pos.shape[0]
    out = []
    for i in range(n_dim):
        v = vert_pos[:, :, i].reshape((E,) + (2,) * n_dim)
        for j in reversed(range(n_dim)):
            v = _contract_axis(v, lin, 1 + j)
        out.append(v)
    return np.stack(out, axis=1)  # [E][nd][rs]*nd


def _cofactor_normals(jac):
    """jac[..., i, j] = d x_i / d xi_j. Returns nrml[..., i, j] = det(J with column i
    replaced by unit vector e_j) (src/Deformed_element.cpp:75-86) and det(J)."""
    nd = jac.shape[-1]
    det = np.linalg.det(jac)
    nrml = np.empty_like(jac)
    for i in range(nd):
        for j in range(nd):
            m = jac.copy()
            m[..., :, i] = 0.
            m[..., j, i] = 1.
            nrml[..., i, j] = np.linalg.det(m)
    return nrml, det


def deformed_metrics(vert_pos, nom_size, basis, n_dim):
    """Deformed_element::set_jacobian for all elements at once.

    Returns jac_dat [E][nd*nd+1][nq], face normals [E][2nd][nd][nfq], vertex
    time-step scale [E][nvert] and qpoint positions [E][nd][nq]."""
    rs = basis.row_size
    E = vert_pos.shape[0]
    nq, nfq = rs ** n_dim, rs ** (n_dim - 1)
    pos = _qpoint_positions(vert_pos, basis, n_dim)             # [E][nd][rs..]
    D = basis.diff_mat
    # jac[E][i][j][rs..] = d pos_i / d ref_j / nom_size
    jac = np.empty((E, n_dim, n_dim) + (rs,) * n_dim)
    for i in range(n_dim):
        for j in range(n_dim):
            jac[:, i, j] = _contract_axis(pos[:, i], D, 1 + j) / nom_size.reshape((E,) + (1,) * n_dim)
    jq = np.moveaxis(jac.reshape(E, n_dim, n_dim, nq), 3, 1)     # [E][nq][i][j]
    nrml, det = _cofactor_normals(jq)
    jac_dat = np.empty((E, n_dim * n_dim + 1, nq))
    jac_dat[:, :n_dim * n_dim] = np.moveaxis(nrml, 1, 3).reshape(E, n_dim * n_dim, nq)
    jac_dat[:, n_dim * n_dim] = det
    # face normals (src/Deformed_element.cpp:88-116)
    face_nrml = np.empty((E, 2 * n_dim, n_dim, nfq))
    for i_dim in range(n_dim):
        for sign in range(2):
            b = basis.boundary[sign:sign + 1]                     # [1][rs]
            fj = _contract_axis(jac, b, 3 + i_dim)                # [E][nd][nd][..1..]
            fj = fj.reshape(E, n_dim, n_dim, nfq)
            fj = np.moveaxis(fj, 3, 1)                            # [E][nfq][i][j]
            for j in range(n_dim):
                m = fj.copy()
                m[..., :, i_dim] = 0.
                m[..., j, i_dim] = 1.
                face_nrml[:, 2 * i_dim + sign, j] = np.linalg.det(m)
    # vertex time-step scale (src/Deformed_element.cpp:117-134)
    B = basis.boundary

    def to_vertices(field):  # field [E][rs..] -> [E][nvert]
        v = field
        for d in range(n_dim):
            v = _contract_axis(v, B, 1 + d)
        return v.reshape(E, 2 ** n_dim)

    vnrml = np.stack([to_vertices(jac_dat[:, k].reshape((E,) + (rs,) * n_dim)) for k in range(n_dim * n_dim)],
                     axis=2)                                      # [E][nvert][nd*nd]
    vdet = to_vertices(det.reshape((E,) + (rs,) * n_dim))
    norm_sum = np.zeros_like(vdet)
    for i in range(n_dim):
        norm_sum += np.sqrt((vnrml[:, :, i * n_dim:(i + 1) * n_dim] ** 2).sum(axis=2))
    vtss = nom_size[:, None] * vdet / norm_sum
    return jac_dat, face_nrml, vtss, pos.reshape(E, n_dim, nq)


def cartesian_positions(origin, nom_size, basis, n_dim):
    """Element::position (src/Element.cpp:63-72): (node + nominal position)*size + origin.
    `origin` [E][nd] is the element's lower corner."""
    coords = _node_coords(basis, n_dim)                           # [nd][nq]
    return origin[:, :, None] + coords[None] * nom_size[:, None, None]


def share_vertex_min(values, vert_ids):
    """Solver::share_vertex_data with Vertex::vector_min (src/Solver.cpp:35-54, 380)."""
    n = int(vert_ids.max()) + 1
    m = np.full(n, np.inf)
    np.minimum.at(m, vert_ids.ravel(), values.ravel())
    return m[vert_ids]


def share_vertex_max(values, vert_ids):
    n = int(vert_ids.max()) + 1
    m = np.full(n, -np.inf)
    np.maximum.at(m, vert_ids.ravel(), values.ravel())
    return m[vert_ids]


def structured_mesh(n_dim, row_size, n_per_dim, lo, hi, deformed=False, displacement=None, bcs=None):
    """Uniform structured mesh of n_per_dim^n_dim elements on [lo, hi]^n_dim.

    n_per_dim may also be a sequence of per-dimension counts: the elements keep the size
    (hi - lo)/n_per_dim[0], so dimension d spans lo + [0, n_per_dim[d]*size].

    deformed: make every element a Deformed_element (connections are deformed
      connections with direction {{d,d},{1,0}}, include/connection.hpp:35).
    displacement: fn(vertex positions [N][nd], on_boundary [N][nd] bool) -> displacement [N][nd]
      applied to the vertices (deformed only).
    bcs: dict {(i_dim, face_sign): BcSpec} for the 2*n_dim domain boundaries.
    """
    basis = Basis(row_size)
    counts = tuple(int(c) for c in n_per_dim) if np.ndim(n_per_dim) else (int(n_per_dim),) * n_dim
    E = int(np.prod(counts))
    h = (hi - lo) / counts[0]
    ar = Arena(n_dim, row_size, 0 if deformed else E, E if deformed else 0)
    idx = np.array(list(itertools.product(*[range(c) for c in counts])))   # [E][nd], dim 0 outermost
    ar.nom_size[:] = h
    # global vertex grid
    vbits = np.array(list(itertools.product(range(2), repeat=n_dim)))  # [nvert][nd], dim 0 most significant
    vidx = idx[:, None, :] + vbits[None]                               # [E][nvert][nd]
    vert_ids = np.zeros(vidx.shape[:2], dtype=np.int64)
    for d in range(n_dim):
        vert_ids = vert_ids * (counts[d] + 1) + vidx[:, :, d]
    ar.vert_ids = vert_ids
    gv = np.array(list(itertools.product(*[range(c + 1) for c in counts])))   # global vertices, same ordering
    gpos = lo + gv * h
    if deformed and displacement is not None:
        on_b = (gv == 0) | (gv == np.array(counts))
        gpos = gpos + displacement(gpos.copy(), on_b)
    vert_pos = gpos[vert_ids]                                           # [E][nvert][nd]
    ar.vert_pos = vert_pos
    if deformed:
        jac_dat, fn, vtss, qpos = deformed_metrics(vert_pos, ar.nom_size, basis, n_dim)
        ar.jac[:] = jac_dat
        ar.qpoint_pos = qpos
        elem_face_nrml = fn
    else:
        vtss = np.full((E, 2 ** n_dim), h / n_dim)   # src/Element.cpp:17
        ar.qpoint_pos = cartesian_positions(lo + idx * h, ar.nom_size, basis, n_dim)
        elem_face_nrml = None
    ar.vert_tss[:] = share_vertex_min(vtss, vert_ids)
    nd, nfq = n_dim, ar.nfq
    strides = np.array([int(np.prod(counts[d + 1:])) for d in range(n_dim)])
    cons, con_nrml, bcons, bnrml = [], [], [], []
    face_nrml = np.zeros((E if deformed else 0, 2 * nd, nd, nfq))
    bcs = bcs or {}
    spec_index = {}
    for key in sorted(bcs):
        spec_index[key] = len(ar.bc_specs)
        ar.bc_specs.append(bcs[key])
    next_slot = E * 2 * nd
    for e in range(E):
        for d in range(nd):
            if idx[e, d] + 1 < counts[d]:
                b = e + strides[d]
                s0, s1 = ar.slot_of(e, 2 * d + 1), ar.slot_of(b, 2 * d)
                if deformed:
                    # Solver::calc_jacobian normal averaging (src/Solver.cpp:327-352); both
                    # signs are +1 for direction {{d,d},{1,0}} and no permutation applies
                    nn = 0.5 * elem_face_nrml[e, 2 * d + 1] + 0.5 * elem_face_nrml[b, 2 * d]
                    cons.append((s0, s1, d | (d << 2) | (1 << 4)))
                    con_nrml.append(nn)
                    face_nrml[e, 2 * d + 1] = nn
                    face_nrml[b, 2 * d] = nn
                else:
                    cons.append((s0, s1, d))
            for sign in range(2):
                at_b = (idx[e, d] == 0) if sign == 0 else (idx[e, d] == counts[d] - 1)
                if not at_b:
                    continue
                if (d, sign) not in spec_index:
                    raise ValueError(f"no boundary condition for face ({d}, {sign})")
                bcons.append((ar.slot_of(e, 2 * d + sign), next_slot, d | (sign << 2), spec_index[(d, sign)]))
                next_slot += 1
                if deformed:
                    nrm = elem_face_nrml[e, 2 * d + sign]
                    face_nrml[e, 2 * d + sign] = nrm
                else:
                    nrm = np.zeros((nd, nfq))
                    nrm[d] = 1.
                bnrml.append(nrm)
    ar.n_slot = next_slot
    if deformed:
        ar.def_con = np.array(cons, np.int32).reshape(-1, 3)
        ar.def_con_nrml = np.array(con_nrml).reshape(-1, nd, nfq)
        ar.face_nrml = face_nrml
    else:
        ar.car_con = np.array(cons, np.int32).reshape(-1, 3)
    ar.bc_con = np.array(bcons, np.int32).reshape(-1, 4)
    ar.bc_nrml = np.array(bnrml).reshape(-1, nd, nfq)
    return ar.finalize()


# ------------------------------------------------------------------ general meshes
def face_perm_index(n_dim, row_size, dir_packed, q):
    """Face-1 qpoint that lands on face-0 qpoint q after Face_permutation::match_faces
    (include/Spatial.hpp:85-129, include/Kernel_connection.hpp:55-85)."""
    rs = row_size
    i0, i1 = dir_packed & 3, (dir_packed >> 2) & 3
    s0, s1 = (dir_packed >> 4) & 1, (dir_packed >> 5) & 1
    flip_n0, flip_n1 = (s0 == 0), (s1 == 1)
    flip_tan = (i0 != i1) and (flip_n0 == flip_n1)
    transpose = (i0, i1) in ((0, 2), (2, 0))
    if n_dim == 3:
        r, c = q % rs, q // rs
        if flip_tan:
            colwise = (i0 > 3 - i0 - i1) != transpose
            if colwise:
                r = rs - 1 - r
            else:
                c = rs - 1 - c
        idx = r + c * rs
        if transpose:
            idx = (idx % rs) * rs + idx // rs
        return idx
    return rs - 1 - q if flip_tan else q


def pack_dir(i_dim0, i_dim1, sign0, sign1):
    return i_dim0 | (i_dim1 << 2) | (int(sign0) << 4) | (int(sign1) << 5)


def general_mesh(n_dim, row_size, vert_pos, nom_size, is_deformed, connections, boundaries, bc_specs,
                 vert_ids=None, refined=()):
    """Arena for an arbitrary conforming (or hanging-node) mesh.

    vert_pos [E][nvert][nd]: element vertex positions (vertex bit d <-> reference dim d,
      dim 0 most significant), Cartesian elements first (is_deformed False) then deformed.
    connections: list of (e0, e1, i_dim0, i_dim1, face_sign0, face_sign1). A connection of
      two Cartesian elements must be {{d,d},{1,0}}; any connection involving a deformed
      element of the other kind is also treated as Cartesian (Accessible_mesh::connect_cartesian),
      otherwise it is a deformed connection.
    boundaries: list of (e, i_dim, face_sign, bc_index).
    refined: list of (coarse_e, coarse_i_face, [(fine_e, fine_i_face), ...], stretch) hanging
      faces between Cartesian elements whose fine faces are listed in row-major order.
    """
    basis = Basis(row_size)
    nd, rs = n_dim, row_size
    is_deformed = np.asarray(is_deformed, bool)
    n_def = int(is_deformed.sum())
    n_car = len(is_deformed) - n_def
    assert not is_deformed[:n_car].any(), "Cartesian elements must come first"
    E = n_car + n_def
    ar = Arena(nd, rs, n_car, n_def)
    nfq = ar.nfq
    ar.nom_size[:] = nom_size
    vert_pos = np.asarray(vert_pos, dtype=np.float64)
    ar.vert_pos = vert_pos
    if n_def:
        jac_dat, fn, vtss_def, qpos_def = deformed_metrics(vert_pos[n_car:], ar.nom_size[n_car:], basis, nd)
        ar.jac[:] = jac_dat
    qpos = np.zeros((E, nd, ar.nq))
    vtss = np.zeros((E, ar.nvert))
    if n_car:
        qpos[:n_car] = cartesian_positions(vert_pos[:n_car, 0], ar.nom_size[:n_car], basis, nd)
        vtss[:n_car] = (ar.nom_size[:n_car] / nd)[:, None]
    if n_def:
        qpos[n_car:] = qpos_def
        vtss[n_car:] = vtss_def
    ar.qpoint_pos = qpos
    if vert_ids is not None:
        ar.vert_ids = np.asarray(vert_ids)
        ar.vert_tss[:] = share_vertex_min(vtss, ar.vert_ids)
    else:
        ar.vert_tss[:] = vtss
    ar.bc_specs = list(bc_specs)
    face_nrml = np.zeros((n_def, 2 * nd, nd, nfq))
    if n_def:
        # identity rows for faces that end up in Cartesian connections (include/Spatial.hpp:331-339)
        for i_face in range(2 * nd):
            face_nrml[:, i_face, i_face // 2, :] = 1.
    car, dcon, dnrml = [], [], []
    for (e0, e1, i0, i1, s0, s1) in connections:
        slot0, slot1 = ar.slot_of(e0, 2 * i0 + s0), ar.slot_of(e1, 2 * i1 + s1)
        if not (is_deformed[e0] and is_deformed[e1]):
            assert i0 == i1 and s0 == 1 and s1 == 0, "Cartesian connections are {{d,d},{1,0}}"
            car.append((slot0, slot1, i0))
            continue
        d = pack_dir(i0, i1, s0, s1)
        sign = [1 - 2 * (s0 == 0), 1 - 2 * (s1 == 1)]
        n0 = fn[e0 - n_car, 2 * i0 + s0]
        n1 = fn[e1 - n_car, 2 * i1 + s1]
        perm = np.array([face_perm_index(nd, rs, d, q) for q in range(nfq)])
        # Solver::calc_jacobian (src/Solver.cpp:327-352)
        n = 0.5 * sign[0] * n0 + 0.5 * sign[1] * n1[:, perm]
        side0 = sign[0] * n
        side1 = np.empty_like(n)
        side1[:, perm] = sign[1] * n
        face_nrml[e0 - n_car, 2 * i0 + s0] = side0
        face_nrml[e1 - n_car, 2 * i1 + s1] = side1
        dcon.append((slot0, slot1, d))
        dnrml.append(side0)
    next_slot = E * 2 * nd
    bcon, bnrml = [], []
    for (e, i_dim, sign, bc) in boundaries:
        bcon.append((ar.slot_of(e, 2 * i_dim + sign), next_slot, i_dim | (sign << 2), bc))
        next_slot += 1
        if is_deformed[e]:
            nrm = fn[e - n_car, 2 * i_dim + sign]
            face_nrml[e - n_car, 2 * i_dim + sign] = nrm
        else:
            nrm = np.zeros((nd, nfq))
            nrm[i_dim] = 1.
        bnrml.append(nrm)
    refs = []
    for (ce, cf, fines, stretch) in refined:
        assert not is_deformed[ce], "hanging faces are built between Cartesian elements"
        i_dim = cf // 2
        row = [ar.slot_of(ce, cf)]
        for (fe, ff) in fines:
            assert not is_deformed[fe] and ff // 2 == i_dim and ff % 2 != cf % 2
            # Fine_connection: fine element face <-> mortar face (src: include/connection.hpp:173-190)
            mortar = next_slot
            next_slot += 1
            if cf % 2 == 1:   # coarse on the low side: connection direction {{d,d},{1,0}}, mortar is side 0
                car.append((mortar, ar.slot_of(fe, ff), i_dim))
            else:
                car.append((ar.slot_of(fe, ff), mortar, i_dim))
            row.append(mortar)
        row += [-1] * (5 - len(row))
        row += [int(stretch[0]), int(stretch[1])]
        refs.append(row)
    ar.n_slot = next_slot
    ar.car_con = np.array(car, np.int32).reshape(-1, 3)
    ar.def_con = np.array(dcon, np.int32).reshape(-1, 3)
    ar.def_con_nrml = np.array(dnrml).reshape(-1, nd, nfq)
    ar.bc_con = np.array(bcon, np.int32).reshape(-1, 4)
    ar.bc_nrml = np.array(bnrml).reshape(-1, nd, nfq)
    ar.ref_face = np.array(refs, np.int32).reshape(-1, 7)
    ar.face_nrml = face_nrml
    return ar.finalize()


def _vertex_bits(n_dim):
    return np.array(list(itertools.product(range(2), repeat=n_dim)))


def oriented_neighbor(n_dim, dir_packed, origin0=None):
    """Vertex positions of two unit elements joined through a connection with the given
    direction: element 0 is the unit cube at origin0, element 1 is the rotated unit cube on
    the other side of face (i_dim0, face_sign0) whose face (i_dim1, face_sign1) coincides
    with it in the vertex correspondence the reference assumes for that direction
    (vertex_inds, src/connection.cpp:29-50)."""
    nd = n_dim
    i0, i1 = dir_packed & 3, (dir_packed >> 2) & 3
    s0, s1 = (dir_packed >> 4) & 1, (dir_packed >> 5) & 1
    bits = _vertex_bits(nd)
    origin0 = np.zeros(nd) if origin0 is None else np.asarray(origin0, float)
    p0 = origin0 + bits.astype(float)
    inds0, inds1 = vertex_inds(nd, i0, i1, s0, s1)
    for perm in itertools.permutations(range(nd)):
        for flips in itertools.product((1, -1), repeat=nd):
            A = np.zeros((nd, nd))
            for r in range(nd):
                A[r, perm[r]] = flips[r]
            if np.linalg.det(A) < 0.5:
                continue
            local = bits.astype(float) @ A.T
            b = p0[inds0[0]] - local[inds1[0]]
            p1 = local + b
            if not all(np.allclose(p1[inds1[k]], p0[inds0[k]]) for k in range(len(inds0))):
                continue
            c0, c1 = p0.mean(axis=0), p1.mean(axis=0)
            if (c1 - c0)[i0] * (1 if s0 else -1) <= 0:
                continue
            return p0, p1
    raise ValueError(f"no rotation realises direction {dir_packed}")


def vertex_inds(n_dim, i0, i1, s0, s1):
    """src/connection.cpp:6-50 (face_vertex_inds + vertex_inds)."""
    n_vert = 2 ** (n_dim - 1)
    flip_n0, flip_n1 = (s0 == 0), (s1 == 1)
    flip_tan = (i0 != i1) and (flip_n0 == flip_n1)
    transpose = (i0, i1) in ((0, 2), (2, 0))
    perm = list(range(n_vert))
    if flip_tan:
        stride = 1
        if n_dim == 3:
            unused = 3 - i0 - i1
            if unused > i0:
                stride = 2
        perm = [i + stride * (1 - 2 * ((i // stride) % 2)) for i in perm]
    if transpose:
        perm[1], perm[2] = perm[2], perm[1]
    inds = []
    for side, (idim, sgn) in enumerate(((i0, s0), (i1, s1))):
        stride = 2 ** (n_dim - idim - 1)
        inds.append([v for v in range(2 * n_vert) if (v // stride) % 2 == sgn])
    inds[1] = [inds[1][perm[k]] for k in range(n_vert)]
    return inds
