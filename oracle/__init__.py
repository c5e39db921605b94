"""TEST INFRASTRUCTURE: ctypes wrapper of the CPU oracle (oracle/hexed_oracle.cpp).

Only the tests, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use this
package; the product (hexed_gb300) never imports it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "hexed_oracle.cpp")
LIB = os.path.join(HERE, "_build", "libhexed_oracle.so")

_lib = None


def build(force=False):
    """g++ -O3 -fopenmp -ffp-contract=off (no FMA contraction: identical results on x86 and Arm)."""
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(
            os.path.getmtime(SRC), os.path.getmtime(os.path.join(HERE, "..", "include", "hexed_gpu.h"))):
        return LIB
    cmd = ["g++", "-std=c++17", "-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
           "-o", LIB + ".tmp", SRC]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


def load():
    global _lib
    if _lib is None:
        from hexed_gb300 import abi
        build()
        lib = ctypes.CDLL(LIB)
        D = ctypes.POINTER(abi.MeshDesc)
        T = ctypes.POINTER(abi.Transport)
        U = ctypes.POINTER(abi.UpdateParams)
        c_int, c_double = ctypes.c_int, ctypes.c_double
        P = ctypes.POINTER(c_double)
        sig = {
            "oracle_write_face": [D],
            "oracle_prolong": [D, c_int, c_int],
            "oracle_restrict": [D, c_int, c_int],
            "oracle_apply_state_bcs": [D],
            "oracle_apply_flux_bcs": [D],
            "oracle_neighbor": [D, c_int],
            "oracle_compute_euler": [D, c_double, c_int, c_int, c_int],
            "oracle_compute_navier_stokes": [D, c_double, c_int, c_int, c_int, T, T],
            "oracle_max_dt": [D, c_double, c_double, c_int, c_int, T, T, P],
            "oracle_residual_norm": [D, P],
            "oracle_set_art_visc_admis": [D, c_double],
            "oracle_update": [D, U, P],
            "oracle_fix_admissibility": [D, U, c_double, ctypes.POINTER(c_int)],
            "oracle_compute_residual": [D, U],
            "oracle_derivative": [c_int, P, P, P],
            "oracle_perm_index": [c_int, c_int, c_int, c_int],
            "oracle_characteristics": [c_int, P, P, P, P, P],
            "oracle_sav_slot_dof": [c_int, c_int],
            "oracle_update_art_visc_smoothness": [D, P, P, ctypes.POINTER(SavParams), P],
            "oracle_set_threads": [c_int],
        }
        for name, args in sig.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = c_int
        _lib = lib
    return _lib


class SavParams(ctypes.Structure):
    """oracle_sav_params: Solver::update_art_visc_smoothness's settings, the reference's
    defaults (src/Solver.cpp:154-163) unless given."""
    _fields_ = [("advect_length", ctypes.c_double), ("advect_iters", ctypes.c_int),
                ("diff_iters", ctypes.c_int), ("n_cheby", ctypes.c_int), ("av_row_size", ctypes.c_int),
                ("advect_safety", ctypes.c_double), ("diff_safety", ctypes.c_double),
                ("diff_ratio", ctypes.c_double), ("visc_mult", ctypes.c_double),
                ("unscaled_max", ctypes.c_double), ("freestream_mass", ctypes.c_double),
                ("freestream_energy", ctypes.c_double)]


def sav_params(advect_length, row_size, freestream_mass, freestream_energy, advect_iters=1, diff_iters=1,
               n_cheby=1, av_row_size=None, advect_safety=0.7, diff_safety=0.7, diff_ratio=0.3,
               visc_mult=1e2, unscaled_max=5.):
    return SavParams(advect_length, advect_iters, diff_iters, n_cheby, av_row_size or row_size, advect_safety,
                     diff_safety, diff_ratio, visc_mult, unscaled_max, freestream_mass, freestream_energy)


class SavStorage:
    """Storage of the smoothness-based AV beside an arena: `aux` [n_elem][4 + 2*row_size][nq]
    (forcing rows at 0, the advection state at 1 as Solver's constructor sets it
    (src/Solver.cpp:201-211), its residual cache) and the face slots [n_slot][slot_dof]."""

    def __init__(self, arena):
        rs, nq = arena.row_size, arena.nq
        self.aux = np.zeros((arena.n_elem, 4 + 2 * rs, nq))
        self.aux[:, 4:4 + rs] = 1.
        slot_dof = load().oracle_sav_slot_dof(arena.n_dim, rs)
        self.face = np.zeros((arena.n_slot, slot_dof))

    @property
    def forcing(self):
        return self.aux[:, :4]

    @property
    def advection(self):
        n = (self.aux.shape[1] - 4) // 2
        return self.aux[:, 4:4 + n]


def _inplace(a):
    """Pointer to an array the oracle updates in place (no copy is made)."""
    if a.dtype != np.float64 or not a.flags.c_contiguous:
        raise ValueError("in-place oracle storage must be C-contiguous float64")
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _dp(a):
    import numpy as np
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def derivative(row_size, f, fb):
    """Derivative::operator() on one row: diff.f + lift.(fb - B.f)."""
    import numpy as np
    lib = load()
    f, pf = _dp(f)
    fb, pb = _dp(fb)
    out = np.zeros(row_size)
    _, po = _dp(out)
    po = out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    assert lib.oracle_derivative(row_size, pf, pb, po) == 0
    return out


def set_threads(n=0):
    """OpenMP threads of the oracle (n <= 0: unchanged); returns the count in effect."""
    return load().oracle_set_threads(int(n))


def perm_index(n_dim, row_size, direction, q):
    return load().oracle_perm_index(n_dim, row_size, direction, q)


def characteristics(n_dim, state, normal, state1):
    """(eigenvalues[3], decomposition[nv][3]) of Navier_stokes::Pde::Characteristics."""
    import numpy as np
    lib = load()
    s, ps = _dp(state)
    n, pn = _dp(normal)
    s1, ps1 = _dp(state1)
    ev = np.zeros(3)
    dec = np.zeros((n_dim + 2) * 3)
    assert lib.oracle_characteristics(n_dim, ps, pn, ps1, ev.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                      dec.ctypes.data_as(ctypes.POINTER(ctypes.c_double))) == 0
    return ev, dec.reshape(n_dim + 2, 3)


class Oracle:
    """Runs the oracle in place on a hexed_gb300.mesh.Arena."""

    def __init__(self, arena):
        self.arena = arena
        self.desc = arena.desc()
        self.lib = load()

    def _chk(self, st):
        if st != 0:
            raise RuntimeError(f"oracle call failed with status {st}")

    def write_face(self):
        self._chk(self.lib.oracle_write_face(ctypes.byref(self.desc)))

    def prolong(self, scale=False, offset=False):
        self._chk(self.lib.oracle_prolong(ctypes.byref(self.desc), int(scale), int(offset)))

    def restrict(self, scale=True, offset=False):
        self._chk(self.lib.oracle_restrict(ctypes.byref(self.desc), int(scale), int(offset)))

    def apply_state_bcs(self):
        self._chk(self.lib.oracle_apply_state_bcs(ctypes.byref(self.desc)))

    def apply_flux_bcs(self):
        self._chk(self.lib.oracle_apply_flux_bcs(ctypes.byref(self.desc)))

    def compute_euler(self, dt, i_stage, compute_residual=False, use_filter=False):
        self._chk(self.lib.oracle_compute_euler(ctypes.byref(self.desc), dt, i_stage, int(compute_residual),
                                                int(use_filter)))

    def compute_navier_stokes(self, dt, i_stage, visc, cond, compute_residual=False, use_filter=False):
        self._chk(self.lib.oracle_compute_navier_stokes(ctypes.byref(self.desc), dt, i_stage, int(compute_residual),
                                                        int(use_filter), ctypes.byref(visc), ctypes.byref(cond)))

    def max_dt(self, msc, msd, local_time=False, viscous=False, visc=None, cond=None):
        from hexed_gb300 import abi
        visc = visc or abi.transport_inviscid()
        cond = cond or abi.transport_inviscid()
        out = ctypes.c_double()
        self._chk(self.lib.oracle_max_dt(ctypes.byref(self.desc), msc, msd, int(local_time), int(viscous),
                                         ctypes.byref(visc), ctypes.byref(cond), ctypes.byref(out)))
        return out.value

    def update(self, params):
        out = ctypes.c_double()
        self._chk(self.lib.oracle_update(ctypes.byref(self.desc), ctypes.byref(params), ctypes.byref(out)))
        return out.value

    def compute_residual(self, params):
        self._chk(self.lib.oracle_compute_residual(ctypes.byref(self.desc), ctypes.byref(params)))

    def fix_admissibility(self, params, stability_ratio=0.7):
        """Solver::fix_admissibility (src/Solver.cpp:961-1095): the iteration count."""
        out = ctypes.c_int()
        self._chk(self.lib.oracle_fix_admissibility(ctypes.byref(self.desc), ctypes.byref(params), stability_ratio,
                                                    ctypes.byref(out)))
        return out.value

    def set_art_visc_admis(self, char_speed):
        self._chk(self.lib.oracle_set_art_visc_admis(ctypes.byref(self.desc), char_speed))

    def update_art_visc_smoothness(self, storage, params):
        """Solver::update_art_visc_smoothness (src/Solver.cpp:457-582):
        writes the bulk AV row of the arena; returns art_visc_residual."""
        out = ctypes.c_double()
        self._chk(self.lib.oracle_update_art_visc_smoothness(ctypes.byref(self.desc), _inplace(storage.aux),
                                                             _inplace(storage.face), ctypes.byref(params),
                                                             ctypes.byref(out)))
        return out.value

    def residual_norm(self):
        out = (ctypes.c_double * 3)()
        self._chk(self.lib.oracle_residual_norm(ctypes.byref(self.desc), out))
        return list(out)
