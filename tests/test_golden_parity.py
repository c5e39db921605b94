"""Stored oracle records of one Solver::update on reduced versions of every benchmark
configuration (tests/golden/parity_*.npz, written by tests/golden/make_parity_golden.py).

* CPU: the workload generators still give the stored initial states, and the oracle still
  gives the stored state, time step and residual norms. The bar is 1e-13 relative per
  variable rather than bit equality: the records were made on x86 and are checked on Arm too,
  where libm's exp/log/sin may round differently in the last place, and the residual norm is
  an OpenMP sum whose order follows the thread count.
* GPU: the CUDA path, started from the stored initial state, gives the stored record to the
  FP64 bar (1e-12 per variable; residual norms 1e-11, as their parity test holds them).

Each variable is compared on its own, its error measured against the scale of its conserved
quantity (a momentum component against the largest momentum magnitude; see
helpers.per_variable_rel): the transverse momentum of the Mach 2 case is roundoff-level noise
whose own magnitude means nothing.
"""
import numpy as np
import pytest

from hexed_gb300 import abi
from helpers import FP64_TOL, per_variable_rel
from golden.make_parity_golden import cases, oracle_record, path

CASES = {name: (make, params) for name, make, params in cases()}
HOST_TOL = 1e-13


def load(name):
    with np.load(path(name)) as f:
        return {k: f[k] for k in f.files}


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - b) / np.abs(b)))


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_reproduces_record(name):
    make, params = CASES[name]
    rec = load(name)
    ar = make()
    nv = ar.nv
    assert max(per_variable_rel(ar.elem[:, :nv], rec["state_in"], nv=nv)) <= HOST_TOL
    ar.elem[:, :nv] = rec["state_in"]
    out = oracle_record(ar, params(ar))
    assert max(per_variable_rel(out["elem_out"], rec["elem_out"], nv=nv)) <= HOST_TOL
    assert rel(out["dt"], rec["dt"]) <= HOST_TOL
    assert rel(out["norms"], rec["norms"]) <= HOST_TOL


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(CASES))
def test_gpu_reproduces_record(name):
    from hexed_gb300.solver import Context
    make, params = CASES[name]
    rec = load(name)
    ar = make()
    nv = ar.nv
    ar.elem[:, :nv] = rec["state_in"]
    p = params(ar)
    with Context(ar.copy()) as c:
        c.write_face()
        c.prolong()
        dt = c.update(p)
        elem = c.download(abi.ARRAY_ELEM)[:, :nv + 3]
        c.compute_residual(p)
        norms = c.residual_norm()
    errs = per_variable_rel(elem, rec["elem_out"], nv=nv)
    assert max(errs) <= FP64_TOL, errs
    assert rel([dt], rec["dt"]) <= FP64_TOL
    assert rel(norms, rec["norms"]) <= 1e-11
