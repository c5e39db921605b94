"""Tree-refined Cartesian meshes with 2:1 hanging faces (set-up time, host side).

Restates what the kernels need from the reference's tree meshing (src/Tree.cpp,
src/Accessible_mesh.cpp:743-812): a base grid, cells split into 2^n_dim children where a
predicate asks for it, 2:1 balance across faces, conforming connections between cells of
equal level and `Refined_connection`s (include/connection.hpp:168-286) where a coarse face
meets 2^(n_dim-1) fine faces. The vertex time-step scale is min-shared over coincident
vertices and then set on hanging vertices by the bilinear interpolation of
Hanging_vertex_matcher::match (src/Hanging_vertex_matcher.cpp:13-40).
"""
from __future__ import annotations

import itertools

import numpy as np

from .mesh import general_mesh


def _children(n_dim, level, c):
    return [(level + 1, tuple(2 * c[d] + b[d] for d in range(n_dim)))
            for b in itertools.product(range(2), repeat=n_dim)]


def build_leaves(n_dim, n_base, max_level, refine):
    """refine(level, idx) -> bool. Returns (leaves, internal) sets of (level, idx)."""
    leaves = {(0, c) for c in itertools.product(range(n_base), repeat=n_dim)}
    internal = set()
    for level in range(max_level):
        for cell in sorted(c for c in leaves if c[0] == level):
            if refine(*cell):
                leaves.remove(cell)
                internal.add(cell)
                leaves.update(_children(n_dim, *cell))
    # 2:1 balance across faces
    changed = True
    while changed:
        changed = False
        for cell in sorted(leaves):
            level, c = cell
            n_side = n_base * 2 ** level
            bad = False
            for d in range(n_dim):
                for s in (-1, 1):
                    nb = list(c)
                    nb[d] += s
                    if not 0 <= nb[d] < n_side:
                        continue
                    nbc = (level, tuple(nb))
                    if nbc not in internal:
                        continue
                    # children of the neighbour adjacent to this cell's face
                    for ch in _children(n_dim, *nbc):
                        if ch[1][d] % 2 == (1 if s == -1 else 0) and ch in internal:
                            bad = True
            if bad:
                leaves.remove(cell)
                internal.add(cell)
                leaves.update(_children(n_dim, *cell))
                changed = True
    return leaves, internal


def tree_mesh(n_dim, row_size, n_base, max_level, refine, bcs, lo=0., hi=1.):
    """Arena of a Cartesian tree mesh on [lo, hi]^n_dim. bcs: {(i_dim, sign): BcSpec}."""
    leaves, internal = build_leaves(n_dim, n_base, max_level, refine)
    order = sorted(leaves)
    index = {cell: i for i, cell in enumerate(order)}
    E = len(order)
    size = np.array([(hi - lo) / (n_base * 2 ** lev) for lev, _ in order])
    bits = np.array(list(itertools.product(range(2), repeat=n_dim)))
    origin = np.array([[lo + c[d] * size[i] for d in range(n_dim)] for i, (lev, c) in enumerate(order)])
    vert_pos = origin[:, None, :] + bits[None, :, :] * size[:, None, None]
    finest = n_base * 2 ** max_level
    # integer vertex coordinates at the finest level identify coincident vertices
    vkey = np.rint((vert_pos - lo) / (hi - lo) * finest).astype(np.int64)
    flat = np.zeros(vkey.shape[:2], dtype=np.int64)
    for d in range(n_dim):
        flat = flat * (finest + 1) + vkey[:, :, d]
    _, vert_ids = np.unique(flat, return_inverse=True)
    vert_ids = vert_ids.reshape(E, -1)
    spec_keys = sorted(bcs)
    spec_index = {k: i for i, k in enumerate(spec_keys)}
    connections, boundaries, refined = [], [], []
    for i, (level, c) in enumerate(order):
        n_side = n_base * 2 ** level
        for d in range(n_dim):
            for s in (0, 1):
                nb = list(c)
                nb[d] += 1 if s else -1
                if not 0 <= nb[d] < n_side:
                    boundaries.append((i, d, s, spec_index[(d, s)]))
                    continue
                nbc = (level, tuple(nb))
                if nbc in leaves:
                    if s == 1:
                        connections.append((i, index[nbc], d, d, 1, 0))
                    continue
                if nbc in internal:
                    fines = [ch for ch in _children(n_dim, *nbc) if ch[1][d] % 2 == (0 if s == 1 else 1)]
                    # natural row-major order over the two face dimensions
                    fines.sort(key=lambda ch: tuple(ch[1][k] for k in range(n_dim) if k != d))
                    refined.append((i, 2 * d + s, [(index[ch], 2 * d + (1 - s)) for ch in fines], (False, False)))
    ar = general_mesh(n_dim, row_size, vert_pos, size, [False] * E, connections, boundaries,
                      [bcs[k] for k in spec_keys], vert_ids=vert_ids, refined=refined)
    _match_hanging_vertices(ar, refined, vert_pos, n_dim)
    ar.levels = np.array([lev for lev, _ in order])
    return ar


def _match_hanging_vertices(ar, refined, vert_pos, n_dim):
    """Hanging_vertex_matcher::match: fine-face vertex values = bilinear interpolation of the
    coarse face's corner values (applied after the vertex-minimum sharing)."""
    for (ce, cf, fines, _) in refined:
        d, s = cf // 2, cf % 2
        stride = 2 ** (n_dim - 1 - d)
        face_verts = [v for v in range(2 ** n_dim) if (v // stride) % 2 == s]
        corners = vert_pos[ce, face_verts]           # coarse face corners
        lo = corners.min(axis=0)
        hi = corners.max(axis=0)
        other = [k for k in range(n_dim) if k != d]
        cval = {}
        for v in face_verts:
            key = tuple(int(round((vert_pos[ce, v, k] - lo[k]) / (hi[k] - lo[k]))) for k in other)
            cval[key] = ar.vert_tss[ce, v]
        for (fe, ff) in fines:
            fd, fs = ff // 2, ff % 2
            fstride = 2 ** (n_dim - 1 - fd)
            for v in range(2 ** n_dim):
                if (v // fstride) % 2 != fs:
                    continue
                coord = [(vert_pos[fe, v, k] - lo[k]) / (hi[k] - lo[k]) for k in other]
                val = 0.
                for key, cv in cval.items():
                    w = 1.
                    for a, x in zip(key, coord):
                        w *= x if a else (1. - x)
                    val += w * cv
                ar.vert_tss[fe, v] = val
