"""Python host mirror of hexed's Solver / kernel layer over the C ABI of libhexed_gpu.so.

``Context`` exposes one method per entry point of include/hexed_gpu.h (the free
functions of the reference's include/kernels.hpp:22-42). ``Solver`` mirrors the
reference's Solver methods used on the hot path (include/Solver.hpp:107-236):
``update``, ``max_dt``, ``compute_residual``, ``initialize`` and the residual norms that
Case.hil's ``compute_residuals`` reports. There is no CPU fallback: constructing a
Context without the built library or without a GPU raises.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import abi


class Context:
    def __init__(self, arena, precision=abi.FP64):
        self.lib = abi.load_library()
        self.arena = arena
        self.precision = precision
        self._desc = arena.desc()
        handle = ctypes.c_void_p()
        abi.check(self.lib.hexed_gpu_create(ctypes.byref(self._desc), precision, ctypes.byref(handle)))
        self.handle = handle

    # -------------------------------------------------------------- lifetime / data
    def close(self):
        if getattr(self, "handle", None):
            self.lib.hexed_gpu_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _array(self, which):
        a = self.arena
        return {abi.ARRAY_ELEM: a.elem, abi.ARRAY_RCACHE: a.rcache, abi.ARRAY_FACE: a.face,
                abi.ARRAY_BC_CACHE: a.bc_cache}[which]

    def upload(self, which, host=None):
        host = self._array(which) if host is None else host
        host = np.ascontiguousarray(host, dtype=np.float64)
        abi.check(self.lib.hexed_gpu_upload(self.handle, which, host.ctypes.data_as(abi.P_double)))

    def download(self, which, out=None):
        ref = self._array(which)
        out = np.empty_like(ref) if out is None else out
        abi.check(self.lib.hexed_gpu_download(self.handle, which, out.ctypes.data_as(abi.P_double)))
        return out

    def upload_all(self):
        for w in (abi.ARRAY_ELEM, abi.ARRAY_RCACHE, abi.ARRAY_FACE, abi.ARRAY_BC_CACHE):
            self.upload(w)

    def download_all(self):
        """Copy the device arena back into the host arena (in place)."""
        for w in (abi.ARRAY_ELEM, abi.ARRAY_RCACHE, abi.ARRAY_FACE, abi.ARRAY_BC_CACHE):
            self.download(w, self._array(w))

    def write_state(self, state):
        """Conserved state [n_elem][nv][nq] into the device arena (hexed_gpu_write_state)."""
        st = np.ascontiguousarray(state, dtype=np.float64)
        abi.check(self.lib.hexed_gpu_write_state(self.handle, st.ctypes.data_as(abi.P_double)))

    def read_state(self, out=None):
        """Conserved state [n_elem][nv][nq] from the device arena (hexed_gpu_read_state)."""
        a = self.arena
        out = np.empty((a.n_elem, a.nv, a.nq)) if out is None else out
        abi.check(self.lib.hexed_gpu_read_state(self.handle, out.ctypes.data_as(abi.P_double)))
        return out

    def synchronize(self):
        abi.check(self.lib.hexed_gpu_synchronize(self.handle))

    # -------------------------------------------------------------- kernel layer
    def compute_euler(self, dt, i_stage, compute_residual=False, use_filter=False):
        abi.check(self.lib.hexed_gpu_compute_euler(self.handle, dt, i_stage, int(compute_residual), int(use_filter)))

    def compute_navier_stokes(self, dt, i_stage, visc, cond, compute_residual=False, use_filter=False):
        abi.check(self.lib.hexed_gpu_compute_navier_stokes(self.handle, dt, i_stage, int(compute_residual),
                                                           int(use_filter), ctypes.byref(visc), ctypes.byref(cond)))

    def max_dt(self, msc, msd, local_time=False, viscous=False, visc=None, cond=None, use_filter=False):
        visc = visc or abi.transport_inviscid()
        cond = cond or abi.transport_inviscid()
        out = ctypes.c_double()
        abi.check(self.lib.hexed_gpu_max_dt(self.handle, msc, msd, int(local_time), int(use_filter), int(viscous),
                                            ctypes.byref(visc), ctypes.byref(cond), ctypes.byref(out)))
        return out.value

    def prolong(self, scale=False, offset=False):
        abi.check(self.lib.hexed_gpu_compute_prolong(self.handle, int(scale), int(offset)))

    def restrict(self, scale=True, offset=False):
        abi.check(self.lib.hexed_gpu_compute_restrict(self.handle, int(scale), int(offset)))

    def write_face(self):
        abi.check(self.lib.hexed_gpu_compute_write_face(self.handle))

    def apply_state_bcs(self):
        abi.check(self.lib.hexed_gpu_apply_state_bcs(self.handle))

    def set_art_visc_admis(self, char_speed):
        abi.check(self.lib.hexed_gpu_set_art_visc_admis(self.handle, char_speed))

    def update_art_visc_smoothness(self, params):
        """Solver::update_art_visc_smoothness: writes the bulk AV row; returns art_visc_residual."""
        out = ctypes.c_double()
        abi.check(self.lib.hexed_gpu_update_art_visc_smoothness(self.handle, ctypes.byref(params), ctypes.byref(out)))
        return out.value

    def sav_storage(self):
        """The smoothness-AV storage: aux [n_elem][4 + 2 rs][nq] (forcing rows, advection state,
        its residual cache) and the face slots [n_slot][max(2 nv, nd + rs) nfq]."""
        a = self.arena
        slot_dof = max(2 * a.nv, a.n_dim + a.row_size) * a.nfq
        aux = self.read_range(abi.ARRAY_SAV_AUX, 0, a.n_elem * (4 + 2 * a.row_size) * a.nq)
        face = self.read_range(abi.ARRAY_SAV_FACE, 0, a.n_slot * slot_dof)
        return aux.reshape(a.n_elem, 4 + 2 * a.row_size, a.nq), face.reshape(a.n_slot, slot_dof)

    def apply_flux_bcs(self):
        abi.check(self.lib.hexed_gpu_apply_flux_bcs(self.handle))

    def fix_admissibility(self, params, stability_ratio=0.7):
        """Solver::fix_admissibility: diffuse until admissible (and as long again); returns the
        iteration count the reference returns (0: the state was admissible)."""
        out = ctypes.c_int()
        abi.check(self.lib.hexed_gpu_fix_admissibility(self.handle, ctypes.byref(params), stability_ratio,
                                                       ctypes.byref(out)))
        return out.value

    def is_admissible(self, records=False):
        """Solver::is_admissible: True if density and energy are positive everywhere
        (raises HexedError HEXED_ERR_NUMERICAL for a non-finite state); with records=True
        also the per-element flags."""
        ok = ctypes.c_int()
        rec = np.zeros(self.arena.n_elem, dtype=np.int32) if records else None
        abi.check(self.lib.hexed_gpu_is_admissible(self.handle, ctypes.byref(ok),
                                                   rec.ctypes.data_as(abi.P_int) if records else None))
        return (bool(ok.value), rec) if records else bool(ok.value)

    def compute_jacobian(self, vert_pos_def):
        """Metric set-up of the deformed elements on the device from their vertex positions
        [n_def][nvert][nd] (hexed_gpu_compute_jacobian)."""
        vp = np.ascontiguousarray(vert_pos_def, dtype=np.float64)
        abi.check(self.lib.hexed_gpu_compute_jacobian(self.handle, vp.ctypes.data_as(abi.P_double)))

    def device_flags(self):
        """Flags raised by the kernels (hexed_gpu_device_flags); 0 when none."""
        f = ctypes.c_int()
        abi.check(self.lib.hexed_gpu_device_flags(self.handle, ctypes.byref(f)))
        return f.value

    # -------------------------------------------------------------- solver layer
    def update(self, params, read_dt=True):
        out = ctypes.c_double()
        abi.check(self.lib.hexed_gpu_update(self.handle, ctypes.byref(params),
                                            ctypes.byref(out) if read_dt else None))
        return out.value if read_dt else None

    def compute_residual(self, params):
        abi.check(self.lib.hexed_gpu_compute_residual(self.handle, ctypes.byref(params)))

    def residual_norm(self):
        out = (ctypes.c_double * 3)()
        abi.check(self.lib.hexed_gpu_residual_norm(self.handle, out))
        return list(out)

    # -------------------------------------------------------------- pool (continuous batching)
    def set_launch_shape(self, local_variant=0, face_threads=256):
        abi.check(self.lib.hexed_gpu_set_launch_shape(self.handle, local_variant, face_threads))

    def launch_shape(self):
        """(elements per volume-kernel CTA, face-kernel threads per CTA)."""
        e, f = ctypes.c_int(), ctypes.c_int()
        abi.check(self.lib.hexed_gpu_launch_shape(self.handle, ctypes.byref(e), ctypes.byref(f)))
        return e.value, f.value

    def set_reference_state(self, state):
        """Reference state of every element (mixed form; ignored by the FP64 form)."""
        st = np.ascontiguousarray(state, dtype=np.float64)
        abi.check(self.lib.hexed_gpu_set_reference_state(self.handle, st.ctypes.data_as(abi.P_double)))

    def write_face_range(self, elem_begin, elem_count):
        abi.check(self.lib.hexed_gpu_write_face_range(self.handle, elem_begin, elem_count))

    def write_range(self, which, offset, values):
        v = np.ascontiguousarray(values, dtype=np.float64).ravel()
        abi.check(self.lib.hexed_gpu_write_range(self.handle, which, offset, v.size, v.ctypes.data_as(abi.P_double)))

    def read_range(self, which, offset, count):
        out = np.empty(count, dtype=np.float64)
        abi.check(self.lib.hexed_gpu_read_range(self.handle, which, offset, count, out.ctypes.data_as(abi.P_double)))
        return out

    def write_int_range(self, which, offset_rows, rows):
        r = np.ascontiguousarray(rows, dtype=np.int32)
        abi.check(self.lib.hexed_gpu_write_int_range(self.handle, which, offset_rows, r.shape[0],
                                                     r.ctypes.data_as(ctypes.POINTER(ctypes.c_int))))

    def write_bc_spec(self, index, spec):
        abi.check(self.lib.hexed_gpu_write_bc_spec(self.handle, index, ctypes.byref(spec)))

    def set_active(self, n_car_elem, n_car_con, n_bc_con):
        abi.check(self.lib.hexed_gpu_set_active(self.handle, n_car_elem, n_car_con, n_bc_con))

    def segment_residual_norms(self, elem_begin, elem_count, static_scratch=False):
        """Residual norms (momentum, density, energy) of each element segment: [n_seg, 3].
        static_scratch selects the entry point that allocates no device memory."""
        b = np.ascontiguousarray(elem_begin, dtype=np.int32)
        n = np.ascontiguousarray(elem_count, dtype=np.int32)
        out = np.empty((b.size, 3), dtype=np.float64)
        ip = ctypes.POINTER(ctypes.c_int)
        fn = (self.lib.hexed_gpu_segment_residual_norms_static if static_scratch
              else self.lib.hexed_gpu_segment_residual_norms)
        abi.check(fn(self.handle, b.size, b.ctypes.data_as(ip), n.ctypes.data_as(ip),
                     out.ctypes.data_as(abi.P_double)))
        return out

    def update_n(self, params, n, use_graph=True):
        """Enqueue n updates (as one CUDA graph when use_graph); returns without synchronising."""
        abi.check(self.lib.hexed_gpu_update_n(self.handle, ctypes.byref(params), n, int(use_graph)))

    # -------------------------------------------------------------- instrumentation
    @property
    def stream_ptr(self):
        """cudaStream_t (as int) the context's kernels run on."""
        return self.lib.hexed_gpu_stream(self.handle)

    def profile_enable(self, enable=True):
        abi.check(self.lib.hexed_gpu_profile_enable(self.handle, int(enable)))

    def profile_read(self):
        """{kernel name: (launches, total device ms)} since profile_enable."""
        buf = (abi.KernelTime * 64)()
        n = ctypes.c_int()
        abi.check(self.lib.hexed_gpu_profile_read(self.handle, buf, 64, ctypes.byref(n)))
        return {buf[i].name.decode(): (buf[i].launches, buf[i].total_ms) for i in range(n.value)}


class Solver:
    """Solver-shaped driver (src/Solver.cpp:834-913) on one GPU context."""

    def __init__(self, arena, params=None, precision=abi.FP64):
        self.arena = arena
        self.params = params or abi.update_params()
        self.ctx = Context(arena, precision)
        self.iteration = 0
        self.flow_time = 0.
        self.init_residual = None

    def initialize(self):
        """Solver::initialize after the state has been sampled (src/Solver.cpp:398-407):
        extrapolate to the faces and prolong to hanging-face mortars."""
        self.ctx.write_face()
        self.ctx.prolong()

    def update(self):
        dt = self.ctx.update(self.params)
        self.iteration += 1
        self.flow_time += dt * self.params.flow_iters * self.params.n_cheby_flow
        return dt

    def max_dt(self):
        p = self.params
        from .solver import chebyshev_step  # noqa: F401  (documented helper)
        return self.ctx.max_dt(p.max_safety / chebyshev_step(p.n_cheby_flow, p.n_cheby_flow - 1), p.max_safety,
                               p.local_time, p.use_ldg, p.visc, p.cond)

    def compute_residuals(self):
        """Case.hil compute_residuals: residual norms (momentum, density, energy)."""
        self.ctx.compute_residual(self.params)
        return self.ctx.residual_norm()

    def normalized_residual(self):
        """Mean of the three residual ratios to the first iteration's (include/Case.hil:23)."""
        r = self.compute_residuals()
        if self.init_residual is None:
            self.init_residual = r
        return sum(a / b for a, b in zip(r, self.init_residual)) / 3.

    def state(self):
        return self.ctx.download(abi.ARRAY_ELEM)[:, :self.arena.nv]

    def n_var_numeric(self):
        """Storage_params::n_var_numeric (src/Storage_params.cpp:32-35) for two stages: the
        numeric rows of an element's storage."""
        a = self.arena
        return a.nv + 3 + 4 + a.row_size + max(a.nv, a.row_size)

    def numeric_storage(self):
        """Every element's numeric storage [n_elem][n_var_numeric][nq], rows in the order of
        Element's storage (src/Element.cpp:114-188): the state, time-step scale, bulk and
        Laplacian AV coefficients, the four art_visc_forcing rows, the row_size advection
        rows, then the residual cache (the flow's nv rows; rows beyond them zero). The
        reference lets the flow's residual cache and the advection's share those last rows,
        and each is written before it is read, so their content between calls does not
        matter; here they are separate arrays and the flow's is the one stored."""
        a = self.arena
        nv, rs = a.nv, a.row_size
        out = np.zeros((a.n_elem, self.n_var_numeric(), a.nq))
        out[:, :nv + 3] = self.ctx.download(abi.ARRAY_ELEM)
        aux, _ = self.ctx.sav_storage()
        out[:, nv + 3:nv + 7 + rs] = aux[:, :4 + rs]
        out[:, nv + 7 + rs:nv + 7 + rs + nv] = self.ctx.download(abi.ARRAY_RCACHE)
        return out

    def set_numeric_storage(self, storage):
        """Inverse of numeric_storage: the device arena and smoothness-AV storage from it."""
        a = self.arena
        nv, rs = a.nv, a.row_size
        storage = np.asarray(storage, dtype=np.float64)
        want = (a.n_elem, self.n_var_numeric(), a.nq)
        if storage.shape != want:
            raise ValueError(f"numeric storage of shape {storage.shape}, this mesh needs {want}")
        self.ctx.upload(abi.ARRAY_ELEM, storage[:, :nv + 3])
        aux, _ = self.ctx.sav_storage()
        aux[:, :4 + rs] = storage[:, nv + 3:nv + 7 + rs]
        self.ctx.write_range(abi.ARRAY_SAV_AUX, 0, aux.reshape(-1))
        self.ctx.upload(abi.ARRAY_RCACHE, storage[:, nv + 7 + rs:nv + 7 + rs + nv])

    def write_state(self, file_name):
        """Solver::write_state (src/Solver.cpp:253-271): one dataset `state`, [n_elem]
        [n_var_numeric][n_qpoint] doubles (numeric_storage), in `file_name + ".state.npz"`.
        The reference writes the same dataset to `.state.h5`; HDF5 is not available to this
        package, so the container is NumPy's (h5py can copy the array into HDF5 as is)."""
        np.savez(file_name + ".state.npz", state=self.numeric_storage())

    def read_state(self, file_name):
        """Solver::read_state (src/Solver.cpp:232-251) from write_state's file. Like the
        reference, it restores the element storage only; call initialize() (Write_face and
        prolongation of the restored state) before the next update."""
        with np.load(file_name + ".state.npz") as f:
            self.set_numeric_storage(f["state"])

    def close(self):
        self.ctx.close()


def fp64_peak_tflops():
    """Measured FP64 FMA throughput of the current device (TFLOP/s)."""
    lib = abi.load_library()
    out = ctypes.c_double()
    abi.check(lib.hexed_gpu_fp64_peak(ctypes.byref(out)))
    return out.value


def chebyshev_step(n_steps, i_step):
    """math::chebyshev_step (src/math.cpp:104-107)."""
    import math
    return 1 / (1 - math.cos((n_steps - i_step - 0.5) * math.pi / n_steps))
