"""Metric set-up on the device (hexed_gpu_compute_jacobian) against the host restatement of
Deformed_element::set_jacobian and Solver::calc_jacobian (hexed_gb300.mesh.deformed_metrics
and the connection/boundary normal logic of structured_mesh and general_mesh): the device
metrics are wiped, recomputed from the vertex positions and compared."""
import numpy as np
import pytest

from hexed_gb300 import abi, problems
from hexed_gb300.solver import Context
from helpers import all_directions, deformed_case, rotated_pair_case

pytestmark = pytest.mark.gpu

TOL = 1e-12


def metric_arrays(ar):
    return {abi.ARRAY_JAC: ar.jac, abi.ARRAY_FACE_NRML: ar.face_nrml, abi.ARRAY_DEF_CON_NRML: ar.def_con_nrml,
            abi.ARRAY_BC_NRML: ar.bc_nrml, abi.ARRAY_VERT_TSS: ar.vert_tss}


def check_device_metrics(ar, precision=abi.FP64):
    with Context(ar.copy(), precision) as c:
        for which, host in metric_arrays(ar).items():
            if host.size:
                c.write_range(which, 0, np.zeros(host.size))
        c.compute_jacobian(ar.vert_pos[ar.n_car:])
        for which, host in metric_arrays(ar).items():
            if not host.size:
                continue
            got = c.read_range(which, 0, host.size).reshape(host.shape)
            scale = np.abs(host).max()
            assert np.abs(got - host).max() <= TOL * scale, (which, np.abs(got - host).max() / scale)
        # an update on the device metrics gives the state of an update on the host metrics (the
        # cases use wall boundaries: the Riemann-invariant BC switches characteristics on the sign
        # of the normal velocity, so a last-bit change of a normal can move a ghost state by O(1)
        # where that velocity is zero)
        p = abi.update_params(max_safety=0.5)
        c.write_face()
        c.update(p)
        got = c.download(abi.ARRAY_ELEM)[:, :ar.nv]
    with Context(ar.copy(), precision) as c:
        c.write_face()
        c.update(p)
        ref = c.download(abi.ARRAY_ELEM)[:, :ar.nv]
    tol = TOL if precision == abi.FP64 else 1e-6
    assert np.abs(got - ref).max() <= tol * np.abs(ref).max()


@pytest.mark.parametrize("nd,rs", [(2, 4), (2, 6), (3, 3), (3, 5)])
def test_structured_deformed(nd, rs):
    check_device_metrics(deformed_case(nd, rs, 3, abi.BC_NONPENETRATION))


@pytest.mark.parametrize("nd", [2, 3])
def test_every_connection_orientation(nd):
    for d in all_directions(nd):
        check_device_metrics(rotated_pair_case(nd, 3, d, abi.BC_NONPENETRATION))


def test_taylor_green_mesh_mixed():
    check_device_metrics(problems.taylor_green_3d(n_per_side=3, row_size=4), abi.MIXED)
