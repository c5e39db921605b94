"""The C-ABI library: it loads, exports every entry point include/hexed_gpu.h declares,
its structures have the layout the ctypes mirror assumes, and invalid arenas are rejected
on the host before any device work (no GPU needed)."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from hexed_gb300 import abi
from hexed_gb300.mesh import Arena, bc_spec, structured_mesh

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "hexed_gpu.h")


def declared_functions():
    with open(HEADER) as fh:
        text = fh.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(hexed_gpu_\w+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from hexed_gb300 import build
    build.build()
    return abi.load_library()


def test_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) >= 20
    out = subprocess.run(["nm", "-D", "--defined-only", abi.LIB_PATH], capture_output=True, text=True, check=True)
    exported = set(re.findall(r" T (\w+)", out.stdout))
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    for n in names:
        getattr(lib, n)


def test_struct_layout_matches_header(tmp_path):
    src = tmp_path / "sizes.c"
    src.write_text(f'#include "{HEADER}"\n#include <stdio.h>\n#include <stddef.h>\n'
                   'int main(void) { printf("%zu %zu %zu %zu %zu %zu %zu\\n", sizeof(hexed_mesh_desc), '
                   'sizeof(hexed_bc_spec), sizeof(hexed_transport), sizeof(hexed_update_params), '
                   'sizeof(hexed_kernel_time), offsetof(hexed_mesh_desc, bc_spec), '
                   'offsetof(hexed_update_params, cond)); return 0; }\n')
    exe = tmp_path / "sizes"
    subprocess.run(["gcc", "-std=c99", str(src), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    want = [ctypes.sizeof(abi.MeshDesc), ctypes.sizeof(abi.BcSpec), ctypes.sizeof(abi.Transport),
            ctypes.sizeof(abi.UpdateParams), ctypes.sizeof(abi.KernelTime), abi.MeshDesc.bc_spec.offset,
            abi.UpdateParams.cond.offset]
    assert got == want


def create_status(lib, ar):
    d = ar.desc()
    h = ctypes.c_void_p()
    st = lib.hexed_gpu_create(ctypes.byref(d), abi.FP64, ctypes.byref(h))
    return st, h, lib.hexed_gpu_last_error().decode()


def small_arena():
    spec = bc_spec(abi.BC_COPY)
    return structured_mesh(2, 3, 2, 0., 1., bcs={(d, s): spec for d in range(2) for s in range(2)})


def test_invalid_row_size_rejected(lib):
    ar = small_arena()
    ar.row_size = 9
    st, h, msg = create_status(lib, ar)
    assert st == -1 and "invalid kernel" in msg and not h.value


def test_out_of_range_slot_rejected(lib):
    ar = small_arena()
    ar.car_con = ar.car_con.copy()
    ar.car_con[0, 1] = ar.n_slot + 5
    st, h, msg = create_status(lib, ar)
    assert st == -1 and "out of range" in msg


def test_bad_bc_spec_rejected(lib):
    ar = small_arena()
    ar.bc_con = ar.bc_con.copy()
    ar.bc_con[0, 3] = 7
    st, _, msg = create_status(lib, ar)
    assert st == -1 and "boundary connection" in msg


def test_null_arguments(lib):
    assert lib.hexed_gpu_create(None, 0, None) == -1
    assert lib.hexed_gpu_update(None, None, None) == -1
    assert lib.hexed_gpu_destroy(None) == 0
    assert "sm_103a" in lib.hexed_gpu_version().decode()
