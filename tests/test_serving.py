"""Host logic of the serving loop: request streams, the vectorised case builder against the
structured-mesh builder, and the range allocator."""
import numpy as np

from hexed_gb300 import abi, serving
from hexed_gb300.mesh import structured_mesh


def test_request_stream_is_seeded_and_in_range():
    a = serving.request_stream(64, 200., seed=3)
    b = serving.request_stream(64, 200., seed=3)
    assert [(r.side, r.row_size, r.mach, r.angle_deg, r.arrival) for r in a] == \
           [(r.side, r.row_size, r.mach, r.angle_deg, r.arrival) for r in b]
    assert all(8 <= r.side <= 96 and r.row_size in (4, 6) and 0.2 <= r.mach <= 0.8 and -10 <= r.angle_deg <= 10
               for r in a)
    t = np.array([r.arrival for r in a])
    assert t[0] == 0 and np.all(np.diff(t) >= 0)
    # mean gap of a Poisson stream at 200/s
    assert 0.002 < np.diff(t).mean() < 0.009


def _rowset(rows):
    return sorted(map(tuple, np.asarray(rows).tolist()))


def test_case_builder_matches_structured_mesh():
    for side, rs in ((3, 4), (5, 6), (8, 4)):
        req = serving.Request(0, side, rs, 0.5, 5., seed=11)
        case = serving.build_case(req)
        spec = case.spec
        ar = structured_mesh(2, rs, side, 0., 1., bcs={(d, s): spec for d in range(2) for s in range(2)})
        assert case.n_elem == ar.n_elem
        assert _rowset(case.con) == _rowset(ar.car_con)
        # boundary rows: same inside slots and directions (ghost numbering and spec index differ)
        assert _rowset(case.bc[:, [0, 2]]) == _rowset(ar.bc_con[:, [0, 2]])
        assert np.allclose(case.nom_size, ar.nom_size) and np.allclose(case.vert_tss, ar.vert_tss)
        # qpoint positions: the builder's state is the perturbation sampled at the same points
        pos = ar.qpoint_pos  # [E][nd][nq]
        ref = serving.perturbed_state(pos[:, 0], pos[:, 1], req).transpose(1, 0, 2)
        assert np.abs(case.elem[:, :4] - ref).max() < 1e-13
        order = np.argsort(case.bc[:, 0])
        ref_order = np.argsort(ar.bc_con[:, 0])
        assert np.array_equal(case.bc_nrml[order], ar.bc_nrml[ref_order])


def test_perturbation_amplitude():
    req = serving.Request(0, 16, 4, 0.4, -7., seed=5)
    case = serving.build_case(req)
    rho = case.elem[:, 2]
    assert np.abs(rho - 1).max() <= 0.02 + 1e-12 and np.abs(rho - 1).max() > 0.002
    fs = serving.freestream(0.4, -7.)
    assert np.allclose(fs[:2], 0.4 * np.array([np.cos(np.radians(-7.)), np.sin(np.radians(-7.))]))


def test_range_allocator_first_fit_and_coalescing():
    a = serving.RangeAllocator(100)
    assert a.alloc(30) == 0 and a.alloc(30) == 30 and a.alloc(30) == 60
    assert a.alloc(20) is None and a.used_end() == 90
    a.release(30, 30)
    assert a.alloc(40) is None
    assert a.alloc(10) == 30
    a.release(60, 30)
    assert a.used_end() == 40 and a.free == [(40, 100)]
    a.release(0, 30)
    a.release(30, 10)
    assert a.free == [(0, 100)] and a.used_end() == 0 and a.n_free() == 100


def test_pool_memory_estimate_orders():
    b64 = serving.pool_bytes_per_element(6, abi.FP64)
    b32 = serving.pool_bytes_per_element(6, abi.MIXED)
    assert 4000 < b64 < 6000 and b32 < b64
