"""Solver::is_admissible on the device (hexed_gpu_is_admissible): positivity of density and
energy over states, face traces and mortar faces, per-element records, and the non-finite
state error; Solver::fix_admissibility on the device (hexed_gpu_fix_admissibility) against
the oracle. The inadmissible states are planted on the host; nothing faults."""
import numpy as np
import pytest

from hexed_gb300 import abi, problems
from hexed_gb300.solver import Context
import oracle
from helpers import FP64_TOL, compare_arenas, planted_inadmissible

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [abi.FP64, abi.MIXED])
def test_admissible_and_records(precision):
    ar = problems.vortex_2d(n_per_side=8, row_size=4)
    with Context(ar.copy(), precision) as c:
        c.write_face()
        ok, rec = c.is_admissible(records=True)
        assert ok and not rec.any()
        c.update(abi.update_params(max_safety=0.5))
        assert c.is_admissible()
    bad = ar.copy()
    bad.elem[5, 2, 3] = -0.1          # negative density at one point of element 5
    bad.elem[11, 3, :] = -1.          # negative energy everywhere in element 11
    with Context(bad, precision) as c:
        c.write_face()
        ok, rec = c.is_admissible(records=True)
        assert not ok
        assert set(np.flatnonzero(rec)) <= {5, 11} and rec[11] == 1


@pytest.mark.parametrize("precision", [abi.FP64, abi.MIXED])
def test_non_finite_state_is_an_error(precision):
    ar = problems.vortex_2d(n_per_side=4, row_size=4)
    ar.elem[2, 0, 1] = np.nan
    with Context(ar, precision) as c:
        c.write_face()
        with pytest.raises(abi.HexedError, match="not finite") as exc:
            c.is_admissible()
        assert exc.value.status == -3


def test_hanging_face_mortars_checked():
    ar = problems.pulse_tree_3d(n_base=2, row_size=3, levels=1)
    with Context(ar, abi.FP64) as c:
        c.write_face()
        c.prolong()
        assert c.is_admissible()


@pytest.mark.parametrize("kind", ["cartesian", "deformed", "tree"])
def test_fix_admissibility_matches_oracle(kind):
    """The Fix_therm_admis diffusion loop: same iteration count as the oracle and the same
    state (and artificial-viscosity rows, which the loop rewrites) to the FP64 bar."""
    ar = planted_inadmissible(kind)
    ref = ar.copy()
    p = abi.update_params(max_safety=0.5)
    it_o = oracle.Oracle(ref).fix_admissibility(p, 0.7)
    with Context(ar, abi.FP64) as c:
        it_g = c.fix_admissibility(p, 0.7)
        assert c.is_admissible()
        c.download_all()
    assert it_g == it_o > 0
    errs, bad = compare_arenas(ref, ar, FP64_TOL, what=("elem",))
    assert not bad, errs


def test_update_with_fix_admis_matches_oracle():
    """Solver::update with the fix after every stage (viscous Taylor-Green, deformed), from
    the state the fix repaired: the same steps and states as the oracle. (An update cannot
    start from the planted state itself: its negative energy has no sound speed.)"""
    ar = planted_inadmissible("deformed")
    ref = ar.copy()
    p0 = abi.update_params(max_safety=0.5)
    p = abi.update_params(max_safety=0.5, visc=ar.visc, cond=ar.cond, fix_admis=True)
    o = oracle.Oracle(ref)
    o.fix_admissibility(p0, 0.7)
    dts_o = [o.update(p) for _ in range(2)]
    with Context(ar, abi.FP64) as c:
        c.fix_admissibility(p0, 0.7)
        dts_g = [c.update(p) for _ in range(2)]
        c.download_all()
    np.testing.assert_allclose(dts_g, dts_o, rtol=FP64_TOL)
    errs, bad = compare_arenas(ref, ar, FP64_TOL, what=("elem",))
    assert not bad, errs


@pytest.mark.parametrize("kind", ["cartesian", "deformed"])
def test_fix_admissibility_mixed(kind):
    """The mixed form restores admissibility too, in a comparable number of iterations; an
    update_n of a context with the fix runs eagerly (the fix reads back to the host)."""
    ar = planted_inadmissible(kind)
    p = abi.update_params(max_safety=0.5)
    it_o = oracle.Oracle(ar.copy()).fix_admissibility(p, 0.7)
    with Context(ar.copy(), abi.MIXED) as c:
        it = c.fix_admissibility(p, 0.7)
        assert c.is_admissible()
    assert abs(it - it_o) <= 2
    with Context(ar.copy(), abi.MIXED) as c:
        c.fix_admissibility(p, 0.7)
        c.update_n(abi.update_params(max_safety=0.5, fix_admis=True), 3, use_graph=True)
        assert c.is_admissible()
