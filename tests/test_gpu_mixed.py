"""Mixed precision (FP32 fluxes, derivatives and traces; FP64 state, update, metrics, time
step): error of the mixed state against the FP64 GPU state on every mesh kind.

The bar is 1e-6 on the L2 error of every conserved variable on its own (each momentum
component separately), relative to the L2 norm of its conserved quantity in the FP64 state:
the momentum vector's for a momentum component, its own for density and energy.

Why not each momentum component against its own norm: a component that starts at zero
(z-momentum in the Taylor-Green vortex and in the deformed test states, whose velocity lies in
the x-y plane) is made only by the rates, and FP32 rates carry the relative roundoff of an
FP32 line derivative of a smooth field, about |D| eps_32 ~ 20 x 6e-8 ~ 1e-6 at row size 6
(|D| the largest row sum of the derivative operator's entries times the in-element variation
over the derivative). After 200 Taylor-Green updates z-momentum is 1/150 of x-momentum; its L2
error is 1.3e-6 of its own norm and 9e-9 of the momentum's. The report (below) carries both.

Setting HEXED_PARITY_REPORT to a file path appends one JSON line of measured errors per case."""
import json
import os

import numpy as np
import pytest

from hexed_gb300 import abi, problems
from hexed_gb300.solver import Context
from helpers import all_directions, cartesian_case, deformed_case, l2_per_variable, rotated_pair_case

pytestmark = pytest.mark.gpu

MIXED_TOL = 1e-6


def run(ar, params, steps, precision, prolong=False):
    ar = ar.copy()
    with Context(ar, precision) as c:
        c.write_face()
        if prolong:
            c.prolong()
        for _ in range(steps):
            c.update(params)
        return c.download(abi.ARRAY_ELEM)[:, :ar.nv]


def check(ar, params, steps, tol=MIXED_TOL, prolong=False, name=None):
    s64 = run(ar, params, steps, abi.FP64, prolong)
    s32 = run(ar, params, steps, abi.MIXED, prolong)
    assert np.isfinite(s32).all()
    err = l2_per_variable(s32, s64, nv=ar.nv)
    path = os.environ.get("HEXED_PARITY_REPORT")
    if path and name:
        with open(path, "a") as fh:
            fh.write(json.dumps({"case": name, "mixed_l2_per_variable": err,
                                 "mixed_l2_per_variable_own": l2_per_variable(s32, s64), "steps": steps}) + "\n")
    assert max(err) <= tol, err
    # the update really moved the state (the comparison is not vacuous)
    assert np.abs(s64 - ar.elem[:, :ar.nv]).max() > 0
    return err


def test_mixed_vortex_2d():
    ar = problems.vortex_2d(n_per_side=32, row_size=6)
    check(ar, abi.update_params(max_safety=0.5), 100, name="mixed_vortex_2d_32sq_rs6")


def test_mixed_taylor_green():
    ar = problems.taylor_green_3d(n_per_side=4, row_size=4)
    check(ar, abi.update_params(max_safety=0.5, visc=ar.visc, cond=ar.cond), 50)


def test_mixed_taylor_green_32cube_rs6_200_updates():
    """The Taylor-Green workload at its benchmark size."""
    ar = problems.taylor_green_3d(n_per_side=32, row_size=6)
    check(ar, abi.update_params(max_safety=0.5, visc=ar.visc, cond=ar.cond), 200,
          name="mixed_taylor_green_3d_ns_32cube_deformed_rs6")


@pytest.mark.parametrize("deformed", [False, True])
def test_mixed_euler_and_bcs(deformed):
    for kind in (abi.BC_RIEMANN, abi.BC_NONPENETRATION, abi.BC_FREESTREAM, abi.BC_PRESSURE_OUTFLOW):
        ar = deformed_case(3, 4, 3, kind) if deformed else cartesian_case(2, 4, 5, kind)
        check(ar, abi.update_params(max_safety=0.5), 20)


@pytest.mark.parametrize("nd,rs", [(2, 2), (2, 5), (2, 8), (3, 2), (3, 3), (3, 5), (3, 7), (3, 8)])
def test_mixed_row_sizes(nd, rs):
    """Every row size's float kernels (odd point counts take the unaligned-copy paths) on a
    deformed mesh, viscous: the state after 5 updates against FP64."""
    from helpers import air_transport
    ar = deformed_case(nd, rs, 2 if nd == 3 else 3, abi.BC_NONPENETRATION)
    rng = np.random.default_rng(rs)
    ar.elem[:, ar.nv + 2] = rng.uniform(0, 1e-3, size=ar.elem[:, 0].shape)   # Laplacian AV
    visc, cond = air_transport()
    check(ar, abi.update_params(max_safety=0.5, visc=visc, cond=cond), 5)


def test_mixed_rotated_connections():
    for d in list(all_directions(3))[::5]:
        ar = rotated_pair_case(3, 3, d)
        check(ar, abi.update_params(max_safety=0.5), 10)


def test_mixed_hanging_faces():
    ar = problems.pulse_tree_3d(n_base=2, row_size=4, levels=1)
    check(ar, abi.update_params(max_safety=0.5), 20, prolong=True, name="mixed_pulse_tree_2base_1level_rs4")


def test_mixed_artificial_viscosity():
    ar = problems.mach2_jump_3d(n_per_side=3, row_size=4)
    check(ar, abi.update_params(max_safety=0.5, av_admis_char_speed=ar.av_char_speed), 10,
          name="mixed_mach2_jump_3cube_rs4")


def test_mixed_artificial_viscosity_32cube_rs6():
    ar = problems.mach2_jump_3d(n_per_side=32, row_size=6)
    check(ar, abi.update_params(max_safety=0.5, av_admis_char_speed=ar.av_char_speed), 20,
          name="mixed_mach2_jump_32cube_rs6")


@pytest.mark.parametrize("rs", [4, 6])
def test_mixed_pulse_tree_16base_2levels(rs):
    ar = problems.pulse_tree_3d(n_base=16, row_size=rs, levels=2)
    check(ar, abi.update_params(max_safety=0.5), 50, prolong=True, name=f"mixed_pulse_tree_16base_2levels_rs{rs}")


def test_integer_conversions_match_hardware():
    """The mixed form converts between double and float with integer operations; they must
    give the bits of the hardware conversions."""
    import ctypes
    rng = np.random.default_rng(3)
    vals = [rng.standard_normal(200_000) * 10.0 ** rng.integers(-30, 30, 200_000),
            rng.uniform(-3, 3, 200_000),
            np.array([0., -0., 1., -1., 1.5, 3.4028234663852886e38, 3.4028235677973366e38, 1e39, -1e39,
                      np.inf, -np.inf, np.nan, 1.1754943508222875e-38, 1e-45, 5e-324, 2.0 ** -149,
                      1 + 2.0 ** -24, 1 + 3 * 2.0 ** -24, 1 + 2.0 ** -24 + 2.0 ** -40, 0.1, 1 / 3])]
    # values exactly half-way between two floats (ties to even)
    f = rng.standard_normal(10_000).astype(np.float32).astype(np.float64)
    vals.append(f + np.spacing(f.astype(np.float32)).astype(np.float64) / 2)
    x = np.ascontiguousarray(np.concatenate(vals))
    lib = abi.load_library()
    bad = ctypes.c_long()
    abi.check(lib.hexed_gpu_check_conversions(x.ctypes.data_as(abi.P_double), x.size, ctypes.byref(bad)))
    assert bad.value == 0


@pytest.mark.parametrize("viscous", [False, True])
def test_mixed_max_dt_follows_vertex_scales(viscous):
    """The mixed form's Max_dt reads a float copy of the vertex time-step scales. Uploading new
    scales (whole array, then a range) refreshes it: after each, the mixed step matches the FP64
    step to float precision, and the steps really changed. (Recomputing the metrics on the
    device refreshes it too: test_gpu_metrics' mixed case updates after hexed_gpu_compute_jacobian
    has rewritten the scales from zero.)"""
    from helpers import air_transport
    ar = deformed_case(3, 4, 3, abi.BC_RIEMANN)
    visc, cond = air_transport()
    n = ar.vert_tss.size
    dts = {}
    for prec in (abi.FP64, abi.MIXED):
        with Context(ar.copy(), prec) as c:
            out = [c.max_dt(0.7, 0.5, False, viscous, visc, cond)]
            c.upload(abi.ARRAY_VERT_TSS, 0.5 * ar.vert_tss)
            out.append(c.max_dt(0.7, 0.5, False, viscous, visc, cond))
            c.write_range(abi.ARRAY_VERT_TSS, n // 2, 0.25 * ar.vert_tss.reshape(-1)[n // 2:])
            out.append(c.max_dt(0.7, 0.5, False, viscous, visc, cond))
            dts[prec] = out
    d64, d32 = np.array(dts[abi.FP64]), np.array(dts[abi.MIXED])
    assert np.all(np.abs(np.diff(d64)) > 1e-3 * d64[0])
    assert np.max(np.abs(d32 - d64) / d64) < 1e-6, (d32, d64)
