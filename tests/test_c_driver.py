"""A compiled C program drives Solver::update through the kernel-layer entry points of
include/hexed_gpu.h (tests/c_driver/kernel_layer_update.c): initialize, then per update Max_dt
and, per stage, the state BCs and compute_navier_stokes / compute_euler, exactly as
src/Solver.cpp:834-886 calls them. This is the sequence a reference-side shim runs when
Solver::update keeps its own body and only the free functions of include/kernels.hpp and the
Solver members that touch the flow storage go to the GPU.

* CPU: the program compiles against the header and links against libhexed_gpu.so.
* GPU: its result equals hexed_gpu_update's on a second context, and the oracle's
  Solver::update, per variable to the FP64 bar (1e-12; momentum components against the
  momentum's magnitude, see helpers.per_variable_rel), with the same time step each update, on
  a Cartesian Euler mesh, a deformed viscous mesh, a tree mesh with hanging faces and a
  deformed mesh with artificial viscosity.
"""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from hexed_gb300 import abi, problems
from helpers import FP64_TOL, per_variable_rel

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "c_driver", "kernel_layer_update.c")
MAGIC = 0x48584431


def build_driver(out_dir):
    from hexed_gb300 import build
    lib = build.build()
    exe = os.path.join(str(out_dir), "kernel_layer_update")
    lib_dir = os.path.dirname(lib)
    cuda_lib = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "lib64")
    subprocess.run(["gcc", "-std=c99", "-O2", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
                    SRC, "-o", exe, "-L", lib_dir, "-lhexed_gpu", f"-Wl,-rpath,{lib_dir}",
                    f"-Wl,-rpath-link,{cuda_lib}", "-lm"], check=True)
    return exe


def write_arena(path, ar, params, n_updates):
    """The arena file the driver reads (format in its header comment)."""
    d = ar.desc()
    header = np.array([MAGIC, d.n_dim, d.row_size, d.n_car_elem, d.n_def_elem, d.n_slot, d.n_car_con,
                       d.n_def_con, d.n_bc_con, d.n_ref_face, d.n_bc_spec, d.n_vert, n_updates, 0, 0, 0], np.int32)
    with open(path, "wb") as fh:
        fh.write(header.tobytes())
        fh.write(bytes(params))
        for a in (ar.elem, ar.rcache, ar.face, ar.nom_size, ar.vert_tss, ar.jac, ar.face_nrml):
            fh.write(np.ascontiguousarray(a, np.float64).tobytes())
        fh.write(np.ascontiguousarray(ar.car_con, np.int32).tobytes())
        fh.write(np.ascontiguousarray(ar.def_con, np.int32).tobytes())
        fh.write(np.ascontiguousarray(ar.def_con_nrml, np.float64).tobytes())
        fh.write(np.ascontiguousarray(ar.bc_con, np.int32).tobytes())
        fh.write(np.ascontiguousarray(ar.bc_nrml, np.float64).tobytes())
        fh.write(np.ascontiguousarray(ar.bc_cache, np.float64).tobytes())
        fh.write(np.ascontiguousarray(ar.ref_face, np.int32).tobytes())
        fh.write(ctypes.string_at(d.bc_spec, ctypes.sizeof(abi.BcSpec) * d.n_bc_spec))
        if d.n_vert > 0:
            fh.write(np.ascontiguousarray(ar.vert_ids, np.int32).tobytes())


def read_output(path, ar, n_updates):
    raw = np.fromfile(path, np.float64)
    dt_layer, dt_update = raw[:n_updates], raw[n_updates:2 * n_updates]
    elems = raw[2 * n_updates:].reshape(2, *ar.elem.shape)
    return dt_layer, dt_update, elems[0], elems[1]


def test_driver_compiles_against_header(tmp_path):
    exe = build_driver(tmp_path)
    assert os.access(exe, os.X_OK)


CASES = {
    "vortex_cartesian_euler": (lambda: problems.vortex_2d(n_per_side=8, row_size=6),
                               lambda ar: abi.update_params(max_safety=0.5), 10),
    "taylor_green_deformed_viscous": (lambda: problems.taylor_green_3d(n_per_side=3, row_size=4),
                                      lambda ar: abi.update_params(max_safety=0.5, visc=ar.visc, cond=ar.cond), 5),
    "pulse_tree_hanging_faces": (lambda: problems.pulse_tree_3d(n_base=2, row_size=4, levels=1),
                                 lambda ar: abi.update_params(max_safety=0.5), 5),
    "mach2_deformed_art_visc": (lambda: problems.mach2_jump_3d(n_per_side=3, row_size=4),
                                lambda ar: abi.update_params(max_safety=0.5, av_admis_char_speed=ar.av_char_speed), 5),
}


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(CASES))
def test_kernel_layer_sequence_from_c(tmp_path, name):
    import oracle
    make, params, n_updates = CASES[name]
    ar = make()
    p = params(ar)
    exe = build_driver(tmp_path)
    arena_file, out_file = str(tmp_path / "arena.bin"), str(tmp_path / "out.bin")
    write_arena(arena_file, ar, p, n_updates)
    run = subprocess.run([exe, arena_file, out_file], capture_output=True, text=True)
    assert run.returncode == 0, run.stderr
    dt_layer, dt_update, elem_layer, elem_update = read_output(out_file, ar, n_updates)
    ref = ar.copy()
    o = oracle.Oracle(ref)
    o.write_face()
    o.prolong()
    dt_oracle = np.array([o.update(p) for _ in range(n_updates)])
    nv = ar.nv
    # state (momentum components against the momentum magnitude), step scale, AV rows
    assert max(per_variable_rel(elem_layer, elem_update, nv=nv)) <= FP64_TOL
    assert max(per_variable_rel(elem_layer, ref.elem, nv=nv)) <= FP64_TOL
    np.testing.assert_allclose(dt_layer, dt_update, rtol=FP64_TOL)
    np.testing.assert_allclose(dt_layer, dt_oracle, rtol=FP64_TOL)
    assert np.abs(elem_layer[:, :nv] - ar.elem[:, :nv]).max() > 0
