"""Serving pool on the GPU: one solve in the pool against the same solve through the plain
context and the oracle, and every solve's result alone against in a mix with other solves
admitted and retired around it."""
import numpy as np
import pytest

import oracle
from hexed_gb300 import abi, serving
from hexed_gb300.mesh import structured_mesh
from hexed_gb300.solver import Context

pytestmark = pytest.mark.gpu

PARAMS = abi.update_params(max_safety=0.5, local_time=True)


def plain_arena(req):
    case = serving.build_case(req)
    ar = structured_mesh(2, req.row_size, req.side, 0., 1., bcs={(d, s): case.spec for d in range(2) for s in range(2)})
    ar.elem[:] = case.elem
    return ar


@pytest.mark.parametrize("precision", [abi.FP64, abi.MIXED])
def test_pool_solve_matches_plain_context_and_oracle(precision):
    req = serving.Request(0, 6, 4, 0.6, 8., seed=21)
    pool = serving.Pool(4, precision, capacity=512, max_cases=8, params=PARAMS, updates_per_batch=5)
    try:
        # a neighbour in the pool before it, so the solve sits at a non-zero offset
        pool.admit(serving.Request(1, 5, 4, 0.3, -4., seed=3))
        slot = pool.admit(req)
        assert slot.elem_begin == 25
        for _ in range(2):
            pool.enqueue_batch()
        got = pool.state(slot)
    finally:
        pool.close()
    ar = plain_arena(req)
    with Context(ar.copy(), precision) as c:
        # the pool's mixed form uses the solve's freestream as its elements' reference state
        c.set_reference_state(serving.freestream(req.mach, req.angle_deg))
        c.write_face()
        for _ in range(10):
            c.update(PARAMS)
        ref = c.download(abi.ARRAY_ELEM)[:, :4]
    assert np.array_equal(got, ref)
    if precision == abi.FP64:
        o = oracle.Oracle(ar.copy())
        o.write_face()
        for _ in range(10):
            o.update(PARAMS)
        orc = o.arena.elem[:, :4]
        assert np.abs(got - orc).max() <= 1e-12 * np.abs(orc).max()


@pytest.mark.parametrize("precision", [abi.FP64, abi.MIXED])
def test_alone_equals_in_mix(precision):
    """Each solve's converged state and update count are the same served alone and in a
    stream where other solves arrive, share the pools and retire around it."""
    reqs = serving.request_stream(10, 400., seed=5, sides=(4, 10))
    tol = 1e-3
    captured = {}

    def grab(pool, slot):
        captured[slot.req.rid] = (pool.state(slot).copy(), slot.updates, slot.elem_begin)

    with serving.Server(precision, capacity=2048, tol=tol, updates_per_batch={4: 10, 6: 10}, params=PARAMS,
                        tune=False) as srv:
        stats = srv.run(reqs, on_retire=grab)
    assert len(stats.results) == len(reqs) and all(r.converged for r in stats.results)
    # elements were reused by later solves somewhere in the stream
    assert len({v[2] for v in captured.values()}) < len(reqs) or stats.batches > 1
    for req in reqs[:4]:
        alone = {}

        def grab1(pool, slot):
            alone[slot.req.rid] = (pool.state(slot).copy(), slot.updates)

        r = serving.Request(req.rid, req.side, req.row_size, req.mach, req.angle_deg, req.seed, 0.)
        with serving.Server(precision, row_sizes=(req.row_size,), capacity=256, tol=tol,
                            updates_per_batch={4: 10, 6: 10}, params=PARAMS, tune=False) as srv:
            srv.run([r], on_retire=grab1)
        s_mix, n_mix, _ = captured[req.rid]
        s_alone, n_alone = alone[req.rid]
        assert n_mix == n_alone
        assert np.array_equal(s_mix, s_alone)


def test_one_at_a_time_and_batched_reach_tolerance():
    reqs = serving.request_stream(4, 0., seed=9, sides=(4, 6))
    with serving.Server(abi.FP64, capacity=1024, tol=1e-4, max_live=1, params=PARAMS, tune=False) as srv:
        one = srv.run(reqs).summary()
    with serving.Server(abi.FP64, capacity=1024, tol=1e-4, params=PARAMS) as srv:
        assert set(srv.tuning) == {4, 6} and all(len(t) == len(serving.LAUNCH_SHAPES) for t in srv.tuning.values())
        many = srv.run(reqs).summary()
    assert one["converged"] == many["converged"] == 4
    assert one["updates"] == many["updates"]


@pytest.mark.parametrize("rs", [4, 6])
def test_launch_shapes_give_identical_results(rs):
    """Every launch shape the autotuner may pick computes the same bits."""
    req = serving.Request(0, 7, rs, 0.45, 3., seed=8)
    states = {}
    for shape in serving.LAUNCH_SHAPES:
        pool = serving.Pool(rs, abi.FP64, capacity=256, max_cases=4, params=PARAMS, updates_per_batch=4)
        try:
            pool.ctx.set_launch_shape(*shape)
            slot = pool.admit(req)
            pool.enqueue_batch()
            pool.enqueue_batch()
            states[shape] = pool.state(slot)
            epc, ft = pool.ctx.launch_shape()
            assert ft == shape[1] and epc >= 1
        finally:
            pool.close()
    ref = states[(0, 256)]
    for shape, st in states.items():
        assert np.array_equal(st, ref), shape


def test_mixed_solve_reaches_fp64_tolerance():
    """The mixed form forms fluxes as offsets from each solve's freestream, so its residual
    keeps falling with the FP64 one instead of stalling at float roundoff of the full fluxes:
    a steady solve reaches a 1e-8 residual drop in about the same number of updates."""
    reqs = [serving.Request(0, 6, 4, 0.5, 4., seed=2), serving.Request(1, 6, 6, 0.3, -6., seed=3)]
    counts = {}
    for prec in (abi.FP64, abi.MIXED):
        with serving.Server(prec, capacity=512, tol=1e-8, max_updates=80_000, params=PARAMS, tune=False,
                            updates_per_batch={4: 50, 6: 50}) as srv:
            st = srv.run(reqs)
        assert all(r.converged for r in st.results), [(r.rid, r.updates, r.residual) for r in st.results]
        counts[prec] = {r.rid: r.updates for r in st.results}
    for rid in (0, 1):
        assert counts[abi.MIXED][rid] <= 1.2 * counts[abi.FP64][rid] + 100


def test_diverged_solve_is_retired_without_touching_the_others():
    """A request whose initial state is not finite (planted on the host) is retired as
    diverged; the solves sharing its pool finish bit-identical to a run without it."""
    reqs = [serving.Request(0, 6, 4, 0.5, 2., seed=1), serving.Request(1, 5, 4, 0.4, -3., seed=2),
            serving.Request(2, 7, 4, 0.6, 5., seed=3)]
    bad = serving.build_case(reqs[1])
    bad.elem[3, 2, 5] = np.nan
    runs = {}
    for with_bad in (True, False):
        got = {}

        def grab(pool, slot):
            got[slot.req.rid] = pool.state(slot).copy()

        with serving.Server(abi.FP64, row_sizes=(4,), capacity=512, tol=1e-3, params=PARAMS, tune=False,
                            updates_per_batch={4: 10}) as srv:
            st = srv.run(reqs if with_bad else [reqs[0], reqs[2]], on_retire=grab,
                         cases={1: bad} if with_bad else None)
        runs[with_bad] = (got, {r.rid: r.status for r in st.results})
    got_bad, status_bad = runs[True]
    got_ok, status_ok = runs[False]
    assert status_bad == {0: "converged", 1: "diverged", 2: "converged"}
    for rid in (0, 2):
        assert np.array_equal(got_bad[rid], got_ok[rid])


@pytest.mark.parametrize("static_scratch", [False, True])
def test_segment_norms_match_oracle(static_scratch):
    """The segmented residual norms that retire solves, through both entry points (the one
    that grows its buffers and the one with a fixed array), against the oracle: each solve's
    segment equals the oracle's residual_norm of that solve alone. On the same pool, one
    segment over every live element equals hexed_gpu_residual_norm, and the squared segment
    norms sum to the squared whole-pool norm."""
    reqs = [serving.Request(0, 6, 4, 0.6, 8., seed=21), serving.Request(1, 5, 4, 0.3, -4., seed=3),
            serving.Request(2, 7, 4, 0.75, 2., seed=9)]
    pool = serving.Pool(4, abi.FP64, capacity=512, max_cases=8, params=PARAMS, updates_per_batch=5)
    try:
        slots = [pool.admit(r) for r in reqs]
        for _ in range(2):
            pool.enqueue_batch()
        c = pool.ctx
        c.compute_residual(PARAMS)
        begin = np.array([s.elem_begin for s in slots], np.int32)
        count = np.array([s.n_elem for s in slots], np.int32)
        seg = c.segment_residual_norms(begin, count, static_scratch=static_scratch)
        end = int((begin + count).max())
        whole = c.segment_residual_norms(np.array([0], np.int32), np.array([end], np.int32),
                                         static_scratch=static_scratch)[0]
        total = np.array(c.residual_norm())
    finally:
        pool.close()
    # the pool's active prefix holds only these solves: the whole-pool norms are theirs
    np.testing.assert_allclose(whole, total, rtol=1e-12)
    np.testing.assert_allclose((seg ** 2).sum(axis=0), total ** 2, rtol=1e-12)
    for req, got in zip(reqs, seg):
        ar = plain_arena(req)
        o = oracle.Oracle(ar)
        o.write_face()
        for _ in range(10):
            o.update(PARAMS)
        o.compute_residual(PARAMS)
        np.testing.assert_allclose(got, o.residual_norm(), rtol=1e-11)
