"""Generate tests/golden/parity_<case>.npz: oracle outputs of one Solver::update on reduced
versions of the benchmark configurations.

Each file holds the case's initial conserved state (`state_in`, [n_elem][nv][nq], as the
workload generators of hexed_gb300.problems sample it), the element rows after one
initialize + update (`elem_out`: state, time-step scale, bulk and Laplacian AV rows), the
update's time step (`dt`) and the residual norms of compute_residual after it (`norms`).

These fixtures anchor the CPU oracle and the CUDA path to a fixed record: an edit of the
oracle that moves its arithmetic, or of a workload generator that moves its inputs, shows up
as a mismatch against the stored values instead of moving both sides of the parity tests
together. They are oracle outputs (the reference itself cannot be built without Eigen), so
they pin the restatement to itself over time, not to the reference's own arithmetic.

    python tests/golden/make_parity_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from hexed_gb300 import abi, problems  # noqa: E402


def cases():
    """(name, arena factory, update-parameter factory) of each reduced configuration."""
    return [
        ("vortex_2d_8sq_rs6", lambda: problems.vortex_2d(n_per_side=8, row_size=6),
         lambda ar: abi.update_params(max_safety=0.5)),
        ("taylor_green_3d_ns_2cube_deformed_rs6", lambda: problems.taylor_green_3d(n_per_side=2, row_size=6),
         lambda ar: abi.update_params(max_safety=0.5, visc=ar.visc, cond=ar.cond)),
        ("mach2_jump_3d_av_2cube_deformed_rs6", lambda: problems.mach2_jump_3d(n_per_side=2, row_size=6),
         lambda ar: abi.update_params(max_safety=0.5, av_admis_char_speed=ar.av_char_speed)),
        ("pulse_tree_3d_2base_1level_rs4", lambda: problems.pulse_tree_3d(n_base=2, row_size=4, levels=1),
         lambda ar: abi.update_params(max_safety=0.5)),
    ]


def path(name):
    return os.path.join(HERE, f"parity_{name}.npz")


def oracle_record(ar, params):
    """initialize + one update + compute_residual on the oracle, in place on `ar`."""
    import oracle
    o = oracle.Oracle(ar)
    o.write_face()
    o.prolong()
    dt = o.update(params)
    elem = ar.elem[:, :ar.nv + 3].copy()
    o.compute_residual(params)
    return {"elem_out": elem, "dt": np.array([dt]), "norms": np.array(o.residual_norm())}


def main():
    for name, make, params in cases():
        ar = make()
        state_in = ar.elem[:, :ar.nv].copy()
        rec = oracle_record(ar, params(ar))
        np.savez_compressed(path(name), state_in=state_in, **rec)
        print("wrote", path(name), ar.n_elem, "elements")


if __name__ == "__main__":
    main()
