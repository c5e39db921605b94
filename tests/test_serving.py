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


class FakePool:
    """Pool stand-in for the scheduler: a solve 'converges' after a fixed number of updates
    (its side, in batches); `fail` solve ids report non-finite residuals."""

    def __init__(self, rs, cap=400, k=10, fail=()):
        self.rs, self.cap, self.k, self.fail = rs, cap, k, set(fail)
        self.slots = []
        self.used = 0
        self.admitted, self.retired = [], []

    def admit(self, req, case=None, now=0.):
        n = req.side * req.side
        if self.used + n > self.cap:
            return None
        self.used += n
        slot = serving.Slot(req, 0, n, 0, None, None, None, admitted_at=now)
        self.slots.append(slot)
        self.admitted.append(req.rid)
        return slot

    def enqueue_batch(self):
        for s in self.slots:
            s.updates += self.k

    def residuals(self):
        out = []
        for s in self.slots:
            if s.req.rid in self.fail:
                out.append([np.nan] * 3)
            else:
                out.append([10.0 ** (-s.updates / (self.k * s.req.side))] * 3)
        return np.array(out)

    def retire(self, slot, diverged=False):
        self.slots.remove(slot)
        self.used -= slot.n_elem
        self.retired.append((slot.req.rid, diverged))


def _reqs(specs):
    return [serving.Request(i, side, rs, 0.5, 0., seed=i, arrival=t) for i, (side, rs, t) in enumerate(specs)]


def test_scheduler_admits_in_arrival_order_within_capacity():
    pools = {4: FakePool(4, cap=300), 6: FakePool(6, cap=300)}
    srv = serving.Server(pools=pools, tol=1e-3)
    reqs = _reqs([(10, 4, 0.), (10, 4, 0.), (10, 4, 0.), (10, 4, 0.), (12, 6, 0.)])
    st = srv.run(reqs, sleep=lambda s: None)
    res = {r.rid: r for r in st.results}
    assert all(res[i].status == "converged" for i in range(5))
    # three 10x10 solves fit in 300 elements; the fourth waits for a retirement
    assert pools[4].admitted[:3] == [0, 1, 2] and pools[4].admitted[3] == 3
    assert res[3].admitted > 0 or res[3].updates == res[0].updates
    # every solve needs 3*side batches after its first (the normalizing one) to reach 1e-3 here,
    # whatever else shares the pool
    for r in st.results:
        assert r.updates == (reqs[r.rid].side * 3 + 1) * pools[reqs[r.rid].row_size].k


def test_scheduler_rejects_cancels_and_retires_diverged():
    pools = {4: FakePool(4, cap=200, fail={2})}
    srv = serving.Server(pools=pools, tol=1e-3, max_live=1)
    reqs = _reqs([(8, 4, 0.), (20, 4, 0.), (8, 4, 0.), (8, 6, 0.), (8, 4, 0.)])
    srv.cancel(4)
    st = srv.run(reqs, sleep=lambda s: None)
    status = {r.rid: r.status for r in st.results}
    assert status == {0: "converged", 1: "rejected", 2: "diverged", 3: "rejected", 4: "cancelled"}
    assert (2, True) in pools[4].retired and (0, False) in pools[4].retired
    summ = st.summary()
    assert summ["solves"] == 2 and summ["rejected"] == 2 and summ["cancelled"] == 1


def test_scheduler_max_updates():
    pools = {4: FakePool(4, cap=500)}
    srv = serving.Server(pools=pools, tol=1e-30, max_updates=50)
    st = srv.run(_reqs([(5, 4, 0.)]), sleep=lambda s: None)
    assert st.results[0].status == "max_updates" and st.results[0].updates == 50
