"""State checkpoints: Solver.write_state / read_state (Solver::write_state / read_state,
src/Solver.cpp:232-271) store every element's numeric storage, [n_elem][n_var_numeric]
[n_qpoint] doubles in the rows of Element's storage, as the reference's `.state.h5` does
(in NumPy's container: HDF5 is not available here). A solver restored from the file and
one that kept running from the same point then agree bit for bit."""
import numpy as np
import pytest

from hexed_gb300 import abi, problems
from hexed_gb300.solver import Solver

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [abi.FP64, abi.MIXED])
def test_restart_from_checkpoint_is_bit_identical(tmp_path, precision):
    ar = problems.taylor_green_3d(n_per_side=3, row_size=4)
    p = abi.update_params(max_safety=0.5, visc=ar.visc, cond=ar.cond)
    a = Solver(ar.copy(), p, precision)
    a.initialize()
    for _ in range(3):
        a.update()
    # populate the smoothness-AV rows too (forcing, advection state)
    a.ctx.update_art_visc_smoothness(abi.sav_params(0.3, ar.row_size, 1., 1.5, advect_iters=4, diff_iters=2))
    a.initialize()
    path = str(tmp_path / "tgv")
    a.write_state(path)
    saved = a.numeric_storage()
    with np.load(path + ".state.npz") as f:
        st = f["state"]
    nv, rs = ar.nv, ar.row_size
    assert st.shape == (ar.n_elem, nv + 3 + 4 + rs + max(nv, rs), ar.nq)
    assert np.array_equal(st, saved)
    assert np.array_equal(st[:, :nv], a.state())
    assert np.abs(st[:, nv + 3:nv + 7]).max() > 0   # the forcing rows were written

    b = Solver(ar.copy(), p, precision)   # same initial state, hence the same mixed references
    b.read_state(path)
    assert np.array_equal(b.numeric_storage(), saved)
    b.initialize()
    for _ in range(3):
        a.update()
        b.update()
    assert np.array_equal(a.numeric_storage(), b.numeric_storage())
    a.close()
    b.close()


def test_read_state_rejects_another_mesh(tmp_path):
    ar = problems.taylor_green_3d(n_per_side=3, row_size=4)
    a = Solver(ar.copy())
    path = str(tmp_path / "small")
    a.write_state(path)
    other = Solver(problems.taylor_green_3d(n_per_side=2, row_size=4))
    with pytest.raises(ValueError):
        other.read_state(path)
    a.close()
    other.close()
