"""Solver::is_admissible on the device (hexed_gpu_is_admissible): positivity of density and
energy over states, face traces and mortar faces, per-element records, and the non-finite
state error. The inadmissible states are planted on the host; nothing faults."""
import numpy as np
import pytest

from hexed_gb300 import abi, problems
from hexed_gb300.solver import Context

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
