"""Shared set-ups and comparison helpers for the parity tests."""
import numpy as np

from hexed_gb300 import abi, problems
from hexed_gb300.mesh import bc_spec, structured_mesh

# FP64 parity bar: GPU vs CPU oracle, max-norm relative error per variable.
FP64_TOL = 1e-12


def smooth_state(ar, seed=0, mach=0.3, amp=0.05, density=1.2, pressure=1e5):
    """Freestream plus a seeded smooth perturbation (5 Fourier modes) in every variable."""
    nd = ar.n_dim
    rng = np.random.default_rng(seed)
    fs = problems.freestream_state(nd, mach, 7., density, pressure)
    pos = ar.qpoint_pos.transpose(1, 0, 2)
    base = np.stack([np.full(pos.shape[1:], v) for v in fs])
    pert = np.zeros_like(pos[0])
    for _ in range(5):
        k = rng.uniform(0.5, 2.5, size=nd)
        ph = rng.uniform(0, 2 * np.pi)
        pert = pert + np.sin(sum(k[d] * pos[d] for d in range(nd)) + ph)
    pert /= 5
    st = base.copy()
    rho = density * (1 + amp * pert)
    vel = [fs[d] / fs[nd] * (1 + amp * np.roll(pert, d)) for d in range(nd)]
    p = pressure * (1 + amp * 0.5 * pert)
    for d in range(nd):
        st[d] = rho * vel[d]
    st[nd] = rho
    st[nd + 1] = p / 0.4 + 0.5 * rho * sum(v * v for v in vel)
    ar.elem[:, :ar.nv, :] = st.transpose(1, 0, 2)
    ar.freestream = fs
    return ar


def cartesian_case(nd=2, rs=4, n=5, kind=abi.BC_RIEMANN, seed=0):
    fs = problems.freestream_state(nd, 0.3, 7., 1.2, 1e5)
    spec = bc_spec(kind, freestream=fs, pressure=0.9e5)
    ar = structured_mesh(nd, rs, n, 0., 1., bcs={(d, s): spec for d in range(nd) for s in range(2)})
    return smooth_state(ar, seed)


def deformed_case(nd=3, rs=3, n=3, kind=abi.BC_NONPENETRATION, seed=0, amp=0.1):
    fs = problems.freestream_state(nd, 0.3, 7., 1.2, 1e5)
    spec = bc_spec(kind, freestream=fs, pressure=0.9e5)
    h = 1. / n
    ar = structured_mesh(nd, rs, n, 0., 1., deformed=True,
                         displacement=problems.sinusoid_displacement(h, amp, seed, nd),
                         bcs={(d, s): spec for d in range(nd) for s in range(2)})
    return smooth_state(ar, seed)


def air_transport():
    visc = abi.transport_sutherland(1.716e-5 * 100, 273., 111.)
    cond = abi.transport_sutherland(0.0241 * 100, 273., 194.)
    return visc, cond


def group_rel(x, y, nv, axis):
    """Max-norm relative error per conserved quantity: the momentum vector (variables
    0..nv-3 together), density and energy. `axis` is the variable axis."""
    x = np.moveaxis(np.asarray(x), axis, 0)
    y = np.moveaxis(np.asarray(y), axis, 0)
    out = 0.
    for sl in (slice(0, nv - 2), slice(nv - 2, nv - 1), slice(nv - 1, nv)):
        scale = np.abs(y[sl]).max()
        diff = np.abs(x[sl] - y[sl]).max()
        out = max(out, diff / scale if scale > 0 else diff)
    return float(out)


def _quantity_scales(y, nv, norm):
    """Scale of each variable's conserved quantity (rows of y, variable axis first): for a
    momentum component the norm of the momentum vector (all its components together), for
    density and energy their own norm, for rows beyond nv (time-step scale, AV) their own."""
    own = [norm(yv) for yv in y]
    mom = norm(y[:nv - 2]) if nv else 0.
    return [mom if v < nv - 2 else own[v] for v in range(len(y))], own


def per_variable_rel(x, y, axis=1, nv=None):
    """Max-norm error of each variable on its own (every momentum component separately):
    max |x_v - y_v| over S_v. With nv given, S_v is the scale of the variable's conserved
    quantity (_quantity_scales: a momentum component against the momentum vector's largest
    magnitude); without, S_v = max |y_v|. A variable whose scale is zero reports its absolute
    error."""
    x = np.moveaxis(np.asarray(x), axis, 0)
    y = np.moveaxis(np.asarray(y), axis, 0)
    scales, _ = _quantity_scales(y, nv, lambda a: float(np.abs(a).max())) if nv else \
        ([float(np.abs(yv).max()) for yv in y], None)
    out = []
    for xv, yv, sc in zip(x, y, scales):
        diff = float(np.abs(xv - yv).max())
        out.append(diff / sc if sc > 0 else diff)
    return out


def l2_per_variable(x, y, axis=1, nv=None):
    """L2 error of each variable on its own, relative to the L2 norm of its scale (as in
    per_variable_rel: the momentum vector's for a momentum component when nv is given, else
    the variable's own)."""
    x = np.moveaxis(np.asarray(x), axis, 0)
    y = np.moveaxis(np.asarray(y), axis, 0)
    scales, _ = _quantity_scales(y, nv, lambda a: float(np.linalg.norm(a))) if nv else \
        ([float(np.linalg.norm(yv)) for yv in y], None)
    return [float(np.linalg.norm(xv - yv) / sc) if sc > 0 else float(np.linalg.norm(xv - yv))
            for xv, yv, sc in zip(x, y, scales)]


def compare_arenas(a, b, tol=FP64_TOL, what=("elem", "rcache", "face", "bc_cache")):
    """Relative errors of GPU arena `b` against oracle arena `a` (see group_rel)."""
    errs = {}
    nv = a.nv
    if "elem" in what:
        errs["state"] = group_rel(b.elem[:, :nv], a.elem[:, :nv], nv, 1)
        errs["tss"] = _rel(b.elem[:, nv], a.elem[:, nv], None)
    if "rcache" in what:
        errs["rcache"] = group_rel(b.rcache, a.rcache, nv, 1)
    if "face" in what:
        for part, name in ((0, "face"), (1, "face_ldg")):
            errs[name] = group_rel(b.face[:, part], a.face[:, part], nv, 1)
    if "bc_cache" in what and a.bc_cache.size:
        for part in (0, 1):
            ref_scale = a.face[:, part]
            x, y = b.bc_cache[:, part], a.bc_cache[:, part]
            err = 0.
            for sl in (slice(0, nv - 2), slice(nv - 2, nv - 1), slice(nv - 1, nv)):
                scale = max(np.abs(ref_scale[:, sl]).max(), np.abs(y[:, sl]).max())
                d = np.abs(x[:, sl] - y[:, sl]).max()
                err = max(err, d / scale if scale > 0 else d)
            errs[f"bc_cache{part}"] = float(err)
    bad = {k: v for k, v in errs.items() if not (v <= tol)}
    return errs, bad


def _rel(x, y, axis):
    from conftest import rel_err
    return rel_err(x, y, axis)


def all_directions(nd):
    """Every Connection_direction a deformed connection can have (faces of equal sign along
    the same dimension are forbidden, src/Accessible_mesh.cpp:181-185)."""
    import itertools
    from hexed_gb300.mesh import pack_dir
    for i0, i1 in itertools.product(range(nd), repeat=2):
        for s0, s1 in itertools.product(range(2), repeat=2):
            if i0 == i1 and s0 == s1:
                continue
            yield pack_dir(i0, i1, s0, s1)


def rotated_pair_case(nd, rs, direction, kind=abi.BC_RIEMANN, seed=0):
    """Two deformed elements joined through a connection of the given direction (so the
    second element's face data must be permuted), smoothly warped, all other faces on
    boundary conditions."""
    from hexed_gb300.mesh import general_mesh, oriented_neighbor
    p0, p1 = oriented_neighbor(nd, direction)
    verts = np.stack([p0, p1])
    warp = 0.08 * np.sin(1.3 * verts[..., ::-1] + 0.4)
    verts = verts + warp
    i0, i1, s0, s1 = direction & 3, (direction >> 2) & 3, (direction >> 4) & 1, (direction >> 5) & 1
    bounds = [(0, d, s, 0) for d in range(nd) for s in range(2) if (d, s) != (i0, s0)]
    bounds += [(1, d, s, 0) for d in range(nd) for s in range(2) if (d, s) != (i1, s1)]
    fs = problems.freestream_state(nd, 0.3, 7., 1.2, 1e5)
    spec = bc_spec(kind, freestream=fs, pressure=0.9e5)
    ar = general_mesh(nd, rs, verts, [1., 1.], [True, True], [(0, 1, i0, i1, s0, s1)], bounds, [spec])
    return smooth_state(ar, seed)


def planted_inadmissible(kind):
    """An admissible flow with a dip of negative energy at a few points of one element, its
    face traces (and hanging-face mortars) written: "cartesian" (2D vortex, Riemann
    boundaries), "deformed" (3D Taylor-Green, walls) or "tree" (3D pulse on a tree mesh with
    hanging faces)."""
    import oracle
    from hexed_gb300 import problems
    if kind == "cartesian":
        ar = problems.vortex_2d(n_per_side=6, row_size=4)
        e = 14
    elif kind == "tree":
        ar = problems.pulse_tree_3d(n_base=2, row_size=3, levels=1)
        e = 5
    else:
        ar = problems.taylor_green_3d(n_per_side=3, row_size=3)
        e = 13
    energy = ar.elem[e, ar.nv - 1]
    energy[:3] = -0.05*np.abs(energy).mean()
    o = oracle.Oracle(ar)
    o.write_face()
    o.prolong()
    return ar
