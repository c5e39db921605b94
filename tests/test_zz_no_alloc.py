"""The segment residual norms entry point that allocates no device memory
(hexed_gpu_segment_residual_norms_static) against the allocating one, called through the C ABI.
Collected last so that it also runs after every other GPU test in the same process."""
import numpy as np
import pytest

from hexed_gb300 import abi, problems
from hexed_gb300.solver import Context

pytestmark = pytest.mark.gpu

TOL = 1e-12   # relative, per segment and quantity (same kernel, same order: equal in practice)


def segments(n_elem, rng):
    cuts = np.sort(rng.choice(np.arange(1, n_elem), size=6, replace=False))
    edges = np.concatenate([[0], cuts, [n_elem]])
    return edges[:-1].astype(np.int32), np.diff(edges).astype(np.int32)


@pytest.mark.parametrize("precision", [abi.FP64, abi.MIXED])
def test_static_scratch_matches_allocating_entry(precision):
    ar = problems.vortex_2d(n_per_side=12, row_size=6)
    params = abi.update_params(max_safety=0.5)
    rng = np.random.default_rng(7)
    begin, count = segments(ar.n_elem, rng)
    with Context(ar, precision) as c:
        c.write_face()
        for _ in range(3):
            c.update(params)
        c.compute_residual(params)
        for _ in range(2):   # two calls in a row on each entry point
            ref = c.segment_residual_norms(begin, count)
            got = c.segment_residual_norms(begin, count, static_scratch=True)
            assert np.all(np.isfinite(got)) and np.all(ref > 0)
            assert np.abs(got - ref).max() <= TOL * np.abs(ref).max(), (got, ref)
        # a different segment table next: the shared array keeps nothing the call depends on
        got = c.segment_residual_norms(begin[:3], count[:3], static_scratch=True)
        ref = c.segment_residual_norms(begin[:3], count[:3])
        assert np.abs(got - ref).max() <= TOL * np.abs(ref).max()


def test_static_scratch_rejects_oversized_table():
    ar = problems.vortex_2d(n_per_side=4, row_size=4)
    with Context(ar, abi.FP64) as c:
        n = 4097
        with pytest.raises(abi.HexedError, match="exceed the fixed scratch"):
            c.segment_residual_norms(np.zeros(n), np.ones(n), static_scratch=True)
