"""FP64 parity at the benchmark sizes: the CUDA path against the CPU oracle on the full mesh
of every configuration, compared per variable (each momentum component on its own).

* isentropic vortex, 32 x 32 Cartesian quads, row size 6: 100 updates with the global step;
* Navier-Stokes Taylor-Green vortex, 32^3 deformed hexes, row size 6: 200 updates;
* Mach 2 density jump on the same deformed 32^3 mesh with stabilising artificial
  viscosity (inviscid, LDG chain for the AV): 10 updates;
* Gaussian pressure pulse on the 16^3 base tree refined twice inside a sphere (27,224 hexes,
  hanging faces), row sizes 4 and 6: 10 updates.

Each update's time step, the final value of every conserved variable, the time-step scale and
artificial-viscosity rows, and the residual norms after the last update must agree with the
oracle to 1e-12 relative. Every variable is compared on its own (each momentum component
separately, max norm); its error is measured against the scale of its conserved quantity:
a momentum component against the largest momentum magnitude; density, energy, time-step scale
and AV rows against their own largest magnitude. The sequence is Solver::update's
(src/Solver.cpp:834-886) after Solver::initialize (src/Solver.cpp:398-407), with
compute_residual (src/Solver.cpp:899-913) at the end.

Why a momentum component is not measured against its own magnitude: the GPU contracts a*b + c
into FMAs and the oracle does not, so the two differ by roundoff of the largest flux terms,
which scale with the momentum and the pressure. A component that starts at zero (z-momentum of
the Taylor-Green vortex, the transverse momentum of the Mach 2 jump and of the pulse) is made
only by those rates: after 200 Taylor-Green updates z-momentum is 1/150 of x-momentum, and its
difference from the oracle is 1.4e-12 of its own magnitude but 1e-14 of the momentum's. The
report (below) carries both figures: `state_per_variable` (gated) and
`state_per_variable_own`.

Setting HEXED_PARITY_REPORT to a file path appends one JSON line of measured errors per case.
"""
import json
import os

import numpy as np
import pytest

import oracle
from hexed_gb300 import abi, problems
from hexed_gb300.solver import Context
from helpers import FP64_TOL, per_variable_rel

pytestmark = pytest.mark.gpu


def _report(name, errs):
    path = os.environ.get("HEXED_PARITY_REPORT")
    if path:
        with open(path, "a") as fh:
            fh.write(json.dumps({"case": name, **errs}) + "\n")


def run_both(ar, params, steps):
    """The same initialize + `steps` updates + compute_residual on the oracle and on the GPU."""
    a = ar.copy()
    o = oracle.Oracle(a)
    o.write_face()
    o.prolong()
    dt_o = [o.update(params) for _ in range(steps)]
    elem_o = a.elem.copy()
    o.compute_residual(params)
    norms_o = o.residual_norm()
    b = ar.copy()
    with Context(b) as c:
        c.write_face()
        c.prolong()
        dt_g = [c.update(params) for _ in range(steps)]
        elem_g = c.download(abi.ARRAY_ELEM)
        c.compute_residual(params)
        norms_g = c.residual_norm()
        assert c.device_flags() == 0
    nv = ar.nv
    errs = {
        "steps": steps,
        "n_elem": ar.n_elem,
        "state_per_variable": per_variable_rel(elem_g[:, :nv], elem_o[:, :nv], nv=nv),
        "state_per_variable_own": per_variable_rel(elem_g[:, :nv], elem_o[:, :nv]),
        "tss": per_variable_rel(elem_g[:, nv:nv + 1], elem_o[:, nv:nv + 1])[0],
        "av_rows": per_variable_rel(elem_g[:, nv + 1:nv + 3], elem_o[:, nv + 1:nv + 3]),
        "dt": float(np.max(np.abs(np.array(dt_g) - dt_o) / np.abs(dt_o))),
        "residual_norms": [float(abs(g - r) / abs(r)) if r else float(abs(g)) for g, r in zip(norms_g, norms_o)],
    }
    # the updates really moved every variable (the comparison is not vacuous)
    moved = per_variable_rel(elem_o[:, :nv], ar.elem[:, :nv], nv=nv)
    return errs, moved


def check(name, errs, tol=FP64_TOL, norm_tol=FP64_TOL):
    _report(name, errs)
    bad = {k: v for k, v in errs.items()
           if k in ("state_per_variable", "tss", "av_rows", "dt") and np.max(v) > tol}
    if np.max(errs["residual_norms"]) > norm_tol:
        bad["residual_norms"] = errs["residual_norms"]
    assert not bad, f"{name}: above the bar: {bad} (all: {errs})"


def test_vortex_32sq_rs6_100_updates():
    ar = problems.vortex_2d(n_per_side=32, row_size=6)
    p = abi.update_params(max_safety=0.5)
    errs, moved = run_both(ar, p, 100)
    assert min(moved) > 0
    check("isentropic_vortex_2d_32sq_rs6", errs)


def test_taylor_green_32cube_rs6_200_updates():
    ar = problems.taylor_green_3d(n_per_side=32, row_size=6)
    p = abi.update_params(max_safety=0.5, visc=ar.visc, cond=ar.cond)
    errs, moved = run_both(ar, p, 200)
    assert min(moved) > 0 and np.abs(ar.elem[:, 2]).max() == 0   # w starts at zero
    check("taylor_green_3d_ns_32cube_deformed_rs6", errs)


def test_mach2_jump_32cube_rs6_av_10_updates():
    ar = problems.mach2_jump_3d(n_per_side=32, row_size=6)
    p = abi.update_params(max_safety=0.5, av_admis_char_speed=ar.av_char_speed)
    errs, moved = run_both(ar, p, 10)
    check("mach2_density_jump_3d_euler_av_32cube_deformed_rs6", errs)


@pytest.mark.parametrize("rs", [4, 6])
def test_pulse_tree_16base_2levels_10_updates(rs):
    ar = problems.pulse_tree_3d(n_base=16, row_size=rs, levels=2)
    assert ar.n_elem == 27224 and len(ar.ref_face) > 0
    p = abi.update_params(max_safety=0.5)
    errs, moved = run_both(ar, p, 10)
    check(f"pulse_tree_3d_16base_2levels_rs{rs}", errs)
