"""Continuous-batching serving loop for streams of small steady 2D Euler solves.

The reference runs one case per process: ``Case.hil`` builds one mesh, calls
``Solver::update`` until ``normalized_residual`` drops below its tolerance
(include/Case.hil:23, 282-300) and exits. Here many such solves share the GPU:

* One device arena ("pool", :class:`Pool`) per row size, sized from free device memory,
  holds the state, face traces and connection lists of every admitted solve. A solve
  occupies a contiguous element range (first-fit over free ranges); its Cartesian and
  boundary connections occupy a contiguous run of the pool's compact connection lists,
  which are re-packed on the host when a solve retires.
* Requests are admitted between batches of updates, as soon as their arrival time has
  passed and their pool has room; each batch of ``k`` updates of every live solve of a
  pool is one CUDA graph replay (``hexed_gpu_update_n``), and the pools of different row
  sizes run on their own streams, so their batches overlap on the device.
* After each batch the pool computes every live solve's residual norms with one CTA per
  solve (``hexed_gpu_segment_residual_norms``) and retires the solves whose normalized
  residual has reached the tolerance.

Every kernel of the update touches only an element's own data and its own connections,
and local time stepping makes the time step of an element its own (the global step is 1),
so a solve's result does not depend on which other solves share the pool: the same solve
alone and in a mix gives the same state after the same number of updates.

Elements of retired solves stay in the active prefix until a new solve reuses them (or
the prefix shrinks). Their connections are gone and their vertex time-step scale is zero,
so their local time step is zero and their state does not change.
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass, field

import numpy as np

from . import abi
from .basis import Basis
from .mesh import bc_spec
from .problems import HEAT_RAT
from .solver import Context

N_DIM = 2
NV = N_DIM + 2


# ------------------------------------------------------------------ requests and cases
@dataclass
class Request:
    """One steady solve: a side x side Cartesian mesh of [0, 1]^2 at row size row_size,
    freestream Mach `mach` at `angle_deg`, initial state freestream plus a seeded smooth
    perturbation."""
    rid: int
    side: int
    row_size: int
    mach: float
    angle_deg: float
    seed: int
    arrival: float = 0.


def request_stream(n, rate, seed=0, sides=(8, 96), row_sizes=(4, 6), mach=(0.2, 0.8), angle=(-10., 10.)):
    """n requests with Poisson arrivals at `rate` per second (all at t = 0 if rate <= 0)
    and parameters drawn uniformly from the given ranges (sides inclusive)."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1. / rate, n) if rate > 0 else np.zeros(n)
    arrival = np.cumsum(gaps) - gaps[0]
    out = []
    for i in range(n):
        out.append(Request(rid=i, side=int(rng.integers(sides[0], sides[1] + 1)),
                           row_size=int(rng.choice(row_sizes)), mach=float(rng.uniform(*mach)),
                           angle_deg=float(rng.uniform(*angle)), seed=int(rng.integers(1 << 30)),
                           arrival=float(arrival[i])))
    return out


def freestream(mach, angle_deg):
    """Nondimensional conserved freestream: density 1, pressure 1/gamma (sound speed 1)."""
    a = math.radians(angle_deg)
    vel = mach * np.array([math.cos(a), math.sin(a)])
    p = 1. / HEAT_RAT
    return np.array([vel[0], vel[1], 1., p / (HEAT_RAT - 1) + 0.5 * mach * mach])


def perturbed_state(x, y, req, n_modes=5, amplitude=0.02):
    """Freestream plus, in each primitive variable (density, both velocity components,
    pressure), a sum of n_modes Fourier modes with seeded integer wave numbers 1..3 and
    phases, scaled so that the sum is at most `amplitude` relative to the freestream
    (velocity: relative to the freestream speed)."""
    rng = np.random.default_rng(req.seed)
    fields = []
    for _ in range(4):
        k = rng.integers(1, 4, size=(n_modes, 2))
        ph = rng.uniform(0, 2 * math.pi, n_modes)
        w = rng.uniform(-1, 1, n_modes)
        w *= amplitude / np.abs(w).sum()
        g = sum(w[m] * np.sin(2 * math.pi * (k[m, 0] * x + k[m, 1] * y) + ph[m]) for m in range(n_modes))
        fields.append(g)
    a = math.radians(req.angle_deg)
    rho = 1. + fields[0]
    u = req.mach * (math.cos(a) + fields[1])
    v = req.mach * (math.sin(a) + fields[2])
    p = (1. + fields[3]) / HEAT_RAT
    return np.stack([rho * u, rho * v, rho, p / (HEAT_RAT - 1) + 0.5 * rho * (u * u + v * v)])


@dataclass
class CaseData:
    """Host arrays of one solve in its own numbering (elements from 0, slots e*4 + face,
    ghost slots numbered from 0 in boundary-connection order)."""
    n_elem: int
    elem: np.ndarray        # [n][nv + 3][nq]
    nom_size: np.ndarray    # [n]
    vert_tss: np.ndarray    # [n][4]
    con: np.ndarray         # [m][3] slot0, slot1, i_dim
    bc: np.ndarray          # [b][4] inside slot, ghost index, i_dim | sign << 2, 0
    bc_nrml: np.ndarray     # [b][nd][nfq]
    spec: abi.BcSpec


def build_case(req):
    """Arrays of a side x side Cartesian mesh of [0, 1]^2 with Riemann-invariant freestream
    BCs on all four sides, built with array operations. The numbering matches
    ``mesh.structured_mesh`` (element e = i*side + j, dim 0 outermost; connection
    direction {{d,d},{1,0}}; vertex time-step scale h/n_dim, src/Element.cpp:17)."""
    n, rs = req.side, req.row_size
    nq, nfq = rs * rs, rs
    h = 1. / n
    nodes = Basis(rs).nodes
    E = n * n
    i = np.repeat(np.arange(n), n)
    j = np.tile(np.arange(n), n)
    # qpoint q = a*rs + b: x from node a, y from node b
    x = (i[:, None] + np.repeat(nodes, rs)[None, :]) * h
    y = (j[:, None] + np.tile(nodes, rs)[None, :]) * h
    elem = np.zeros((E, NV + 3, nq))
    elem[:, :NV, :] = perturbed_state(x, y, req).transpose(1, 0, 2)
    elem[:, NV, :] = 1.
    e = np.arange(E)
    con0 = np.stack([e * 4 + 1, (e + n) * 4 + 0, np.zeros(E, int)], 1)[i < n - 1]
    con1 = np.stack([e * 4 + 3, (e + 1) * 4 + 2, np.ones(E, int)], 1)[j < n - 1]
    bcs = []
    for d, coord in ((0, i), (1, j)):
        for sign in (0, 1):
            sel = e[coord == (0 if sign == 0 else n - 1)]
            bcs.append(np.stack([sel * 4 + 2 * d + sign, np.zeros_like(sel), np.full_like(sel, d | (sign << 2)),
                                 np.zeros_like(sel)], 1))
    bc = np.concatenate(bcs)
    bc[:, 1] = np.arange(len(bc))
    bc_nrml = np.zeros((len(bc), N_DIM, nfq))
    bc_nrml[np.arange(len(bc)), bc[:, 2] & 3, :] = 1.
    spec = bc_spec(abi.BC_RIEMANN, freestream(req.mach, req.angle_deg))
    return CaseData(E, elem, np.full(E, h), np.full((E, 4), h / N_DIM),
                    np.concatenate([con0, con1]).astype(np.int32), bc.astype(np.int32), bc_nrml, spec)


def quiescent_state(nq):
    """State of unused pool elements: density 1 at rest, pressure 1/gamma."""
    s = np.zeros((NV + 3, nq))
    s[N_DIM] = 1.
    s[N_DIM + 1] = 1. / (HEAT_RAT * (HEAT_RAT - 1))
    s[NV] = 1.
    return s


class PoolArena:
    """Descriptor of an empty pool arena: no host state (the device arrays of states, traces
    and caches start at zero), quiet elements (vertex time-step scale 0), connection lists of
    the pool's capacity with none active, and one boundary-condition record per solve."""

    def __init__(self, row_size, capacity, cap_con, cap_bc, max_cases):
        self.row_size, self.capacity, self.n_slot = row_size, capacity, capacity * 4 + cap_bc
        self.nom_size = np.ones(capacity)
        self.vert_tss = np.zeros((capacity, 4))
        self.car_con = np.zeros((cap_con, 3), np.int32)
        self.bc_con = np.zeros((cap_bc, 4), np.int32)
        self.bc_nrml = np.zeros((cap_bc, N_DIM, row_size))
        self.specs = (abi.BcSpec * max_cases)(*([bc_spec(abi.BC_RIEMANN, quiescent_state(1)[:NV, 0])] * max_cases))

    def desc(self):
        d = abi.MeshDesc()
        d.n_dim, d.row_size = N_DIM, self.row_size
        d.n_car_elem, d.n_def_elem, d.n_slot = self.capacity, 0, self.n_slot
        d.n_car_con, d.n_def_con, d.n_bc_con = len(self.car_con), 0, len(self.bc_con)
        d.n_ref_face, d.n_bc_spec = 0, len(self.specs)
        d.nom_size = self.nom_size.ctypes.data_as(abi.P_double)
        d.vert_tss = self.vert_tss.ctypes.data_as(abi.P_double)
        d.car_con = self.car_con.ctypes.data_as(abi.P_int)
        d.bc_con = self.bc_con.ctypes.data_as(abi.P_int)
        d.bc_nrml = self.bc_nrml.ctypes.data_as(abi.P_double)
        d.bc_spec = self.specs
        return d


# ------------------------------------------------------------------ range allocator
class RangeAllocator:
    """First-fit allocator of contiguous ranges of [0, capacity)."""

    def __init__(self, capacity):
        self.capacity = capacity
        self.free = [(0, capacity)]     # sorted, coalesced (begin, end)

    def alloc(self, n):
        for k, (b, e) in enumerate(self.free):
            if e - b >= n:
                if e - b == n:
                    del self.free[k]
                else:
                    self.free[k] = (b + n, e)
                return b
        return None

    def release(self, b, n):
        e = b + n
        k = 0
        while k < len(self.free) and self.free[k][0] < b:
            k += 1
        self.free.insert(k, (b, e))
        merged = []
        for r in self.free:
            if merged and merged[-1][1] == r[0]:
                merged[-1] = (merged[-1][0], r[1])
            else:
                merged.append(r)
        self.free = merged

    def used_end(self):
        """End of the highest allocated range (0 if nothing is allocated)."""
        if self.free and self.free[-1][1] == self.capacity:
            return self.free[-1][0]
        return self.capacity

    def n_free(self):
        return sum(e - b for b, e in self.free)


# ------------------------------------------------------------------ pool
@dataclass
class Slot:
    req: Request
    elem_begin: int
    n_elem: int
    spec_index: int
    con: np.ndarray         # [m][3] in pool slot numbers
    bc: np.ndarray          # [b][4] with pool inside slot and spec index; ghost filled at packing
    bc_nrml: np.ndarray
    updates: int = 0
    r0: np.ndarray | None = None
    residual: float = 1.
    admitted_at: float = 0.


def pool_bytes_per_element(row_size, precision):
    """Device bytes per pool element: state and time-step rows, residual cache, four face
    slots plus half a ghost slot (each 2 x nv x nfq), nominal size and vertex time-step scales,
    and its share of the connection lists (two Cartesian rows, half a boundary row with its
    normal)."""
    nq, nfq = row_size ** 2, row_size
    w = 8 if precision == abi.FP64 else 4
    slot = 2 * NV * nfq * w
    return 8 * (NV + 3) * nq + w * NV * nq + 4.5 * slot + 8 * 5 + 2 * 12 + 0.5 * (16 + 8 * N_DIM * nfq)


class Pool:
    """Device arena of many solves of one row size (see the module docstring)."""

    def __init__(self, row_size, precision=abi.FP64, capacity=200_000, max_cases=1024, params=None,
                 updates_per_batch=20, use_graph=True):
        self.rs, self.precision = row_size, precision
        self.nq, self.nfq = row_size ** 2, row_size
        self.cap = capacity
        self.cap_con = 2 * capacity
        self.cap_bc = capacity // 2 + 64
        self.max_cases = max_cases
        self.k = updates_per_batch
        self.use_graph = use_graph
        self.params = params or abi.update_params(max_safety=0.5, local_time=True)
        if not self.params.local_time:
            raise ValueError("the pool needs local time stepping: a global time step would couple the solves")
        self.ctx = Context(PoolArena(row_size, capacity, self.cap_con, self.cap_bc, max_cases), precision)
        self.ctx.set_reference_state(quiescent_state(1)[:NV, 0])
        self.ctx.set_active(0, 0, 0)
        self.elements = RangeAllocator(capacity)
        self.free_specs = list(range(max_cases - 1, -1, -1))
        self.slots: list[Slot] = []      # in connection-list order
        self.n_con = 0
        self.n_bc = 0

    def close(self):
        self.ctx.close()

    # -------------------------------------------------------------- admission
    def fits(self, req):
        n = req.side * req.side
        return (bool(self.free_specs) and self.n_con + 2 * n <= self.cap_con and self.n_bc + 4 * req.side <= self.cap_bc
                and any(e - b >= n for b, e in self.elements.free))

    def admit(self, req, case=None, now=0.):
        """Place one solve in the pool; returns its Slot, or None if it does not fit."""
        if not self.fits(req):
            return None
        case = case or build_case(req)
        e0 = self.elements.alloc(case.n_elem)
        spec = self.free_specs.pop()
        shift = 4 * e0
        con = case.con.copy()
        con[:, :2] += shift
        bc = case.bc.copy()
        bc[:, 0] += shift
        bc[:, 3] = spec
        slot = Slot(req, e0, case.n_elem, spec, con, bc, case.bc_nrml, admitted_at=now)
        c, nq = self.ctx, self.nq
        c.write_range(abi.ARRAY_ELEM, e0 * (NV + 3) * nq, case.elem)
        c.write_range(abi.ARRAY_NOM_SIZE, e0, case.nom_size)
        c.write_range(abi.ARRAY_VERT_TSS, e0 * 4, case.vert_tss)
        if self.precision == abi.MIXED:
            # the solve's freestream is the reference state of its elements
            c.write_range(abi.ARRAY_REF_STATE, e0 * NV, np.tile(np.array(case.spec.freestream[:NV]), case.n_elem))
        c.write_bc_spec(spec, case.spec)
        self.slots.append(slot)
        self._write_connections(len(self.slots) - 1)
        c.write_face_range(e0, case.n_elem)
        self._set_active()
        return slot

    def retire(self, slot, diverged=False):
        """Remove a solve: its connections leave the lists, its elements go quiet."""
        k = self.slots.index(slot)
        del self.slots[k]
        c = self.ctx
        c.write_range(abi.ARRAY_VERT_TSS, slot.elem_begin * 4, np.zeros(slot.n_elem * 4))
        if diverged:
            q = np.broadcast_to(quiescent_state(self.nq), (slot.n_elem, NV + 3, self.nq))
            c.write_range(abi.ARRAY_ELEM, slot.elem_begin * (NV + 3) * self.nq, q)
        self.elements.release(slot.elem_begin, slot.n_elem)
        self.free_specs.append(slot.spec_index)
        self._write_connections(k)
        self._set_active()

    def state(self, slot):
        """Conserved state of one solve [n][nv][nq]."""
        per = (NV + 3) * self.nq
        raw = self.ctx.read_range(abi.ARRAY_ELEM, slot.elem_begin * per, slot.n_elem * per)
        return raw.reshape(slot.n_elem, NV + 3, self.nq)[:, :NV]

    def _write_connections(self, first):
        """Re-pack the connection lists from solve `first` on (the lists stay compact)."""
        con_start = sum(len(s.con) for s in self.slots[:first])
        bc_start = sum(len(s.bc) for s in self.slots[:first])
        tail = self.slots[first:]
        if tail:
            con = np.concatenate([s.con for s in tail])
            bc = np.concatenate([s.bc for s in tail])
            bc[:, 1] = self.cap * 4 + bc_start + np.arange(len(bc))   # ghost slot per row
            nrml = np.concatenate([s.bc_nrml for s in tail])
            self.ctx.write_int_range(abi.INT_CAR_CON, con_start, con)
            self.ctx.write_int_range(abi.INT_BC_CON, bc_start, bc)
            self.ctx.write_range(abi.ARRAY_BC_NRML, bc_start * N_DIM * self.nfq, nrml)
        self.n_con = con_start + sum(len(s.con) for s in tail)
        self.n_bc = bc_start + sum(len(s.bc) for s in tail)

    def _set_active(self):
        self.ctx.set_active(self.elements.used_end(), self.n_con, self.n_bc)

    # -------------------------------------------------------------- batches
    def enqueue_batch(self):
        """Enqueue k updates of every live solve (returns before they run)."""
        if self.slots:
            self.ctx.update_n(self.params, self.k, self.use_graph)
            for s in self.slots:
                s.updates += self.k

    def residuals(self):
        """Residual norms of every live solve after the last batch: [n_live][3]."""
        if not self.slots:
            return np.zeros((0, 3))
        self.ctx.compute_residual(self.params)
        return self.ctx.segment_residual_norms([s.elem_begin for s in self.slots], [s.n_elem for s in self.slots])


def normalized(slot, norms):
    """Case.hil's normalized residual: mean over momentum, density and energy of the residual
    norm over its first measured value (include/Case.hil:23). The first value is the norm
    after the solve's first batch of updates."""
    if slot.r0 is None:
        slot.r0 = np.maximum(norms, 1e-300)
    return float(np.mean(norms / slot.r0))


# ------------------------------------------------------------------ autotuner
LAUNCH_SHAPES = [(v, f) for v in (0, 1, 2) for f in (64, 128, 256)]
_tuned = {}


def autotune(pool, n_probes=4, reps=3, clock=time.perf_counter):
    """Choose the launch shape of a pool's kernels (volume-kernel elements per CTA and
    face-kernel threads per CTA) by timing graph replays of a batch of updates of probe
    solves on the pool itself, for every candidate; keeps the fastest and returns
    {shape: seconds per batch}. The probes are n_probes solves of up to 64 x 64 elements
    (a quarter of the pool at most). Results are cached per (device, row size, precision)."""
    import torch
    key = (torch.cuda.get_device_name(), pool.rs, pool.precision)
    if key in _tuned:
        pool.ctx.set_launch_shape(*_tuned[key][0])
        return _tuned[key][1]
    side = max(4, min(64, int(math.sqrt(pool.cap / (4 * n_probes)))))
    probes = [pool.admit(Request(-1 - i, side, pool.rs, 0.5, 0., seed=i)) for i in range(n_probes)]
    times = {}
    try:
        for shape in LAUNCH_SHAPES:
            pool.ctx.set_launch_shape(*shape)
            pool.ctx.update_n(pool.params, pool.k, True)     # capture for this shape
            pool.ctx.synchronize()
            t0 = clock()
            for _ in range(reps):
                pool.ctx.update_n(pool.params, pool.k, True)
            pool.ctx.synchronize()
            times[shape] = (clock() - t0) / reps
    finally:
        for p in probes:
            if p is not None:
                pool.retire(p)
    best = min(times, key=times.get)
    pool.ctx.set_launch_shape(*best)
    _tuned[key] = (best, times)
    return times


# ------------------------------------------------------------------ server
@dataclass
class Result:
    """Outcome of one request. status: "converged"; "max_updates" (retired unconverged);
    "diverged" (non-finite residual, elements reset to a quiet state); "rejected" (no pool of
    its row size, or larger than its pool); "cancelled"."""
    rid: int
    arrival: float
    admitted: float
    done: float
    updates: int
    residual: float
    converged: bool
    status: str = "converged"

    @property
    def latency(self):
        return self.done - self.arrival


@dataclass
class ServeStats:
    results: list = field(default_factory=list)
    wall: float = 0.
    batches: int = 0

    def summary(self):
        served = [r for r in self.results if r.status not in ("rejected", "cancelled")]
        lat = np.array([r.latency for r in served]) if served else np.zeros(1)
        first = min((r.arrival for r in served), default=0.)
        last = max((r.done for r in served), default=0.)
        return {"solves": len(served), "converged": sum(r.converged for r in served),
                "rejected": sum(r.status == "rejected" for r in self.results),
                "cancelled": sum(r.status == "cancelled" for r in self.results),
                "solves_per_s": len(served) / max(last - first, 1e-9),
                "p50_latency_s": float(np.percentile(lat, 50)), "p99_latency_s": float(np.percentile(lat, 99)),
                "wall_s": self.wall, "batches": self.batches,
                "updates": int(sum(r.updates for r in self.results))}


class Server:
    """Serves a request stream on one pool per row size.

    max_live bounds the number of solves on the device at once (1 gives the
    one-solve-at-a-time loop the batched one is compared with)."""

    def __init__(self, precision=abi.FP64, row_sizes=(4, 6), capacity=None, max_live=None, tol=1e-8,
                 max_updates=400_000, updates_per_batch=None, params=None, memory_fraction=0.5, tune=True,
                 pools=None):
        self.tol, self.max_updates = tol, max_updates
        self.max_live = max_live
        self.cancelled = set()
        k_default = {4: 20, 6: 20}
        if pools is not None:        # pools built by the caller (any objects with the Pool interface)
            self.pools = dict(pools)
            self.tuning = {}
            return
        self.pools = {}
        for rs in row_sizes:
            cap = capacity or capacity_from_free_memory(rs, precision, memory_fraction / len(row_sizes))
            k = (updates_per_batch or {}).get(rs, k_default.get(rs, 20))
            self.pools[rs] = Pool(rs, precision, capacity=cap, params=params, updates_per_batch=k)
        self.tuning = {rs: autotune(p) for rs, p in self.pools.items()} if tune else {}

    def cancel(self, rid):
        """Withdraw a request: dropped if still queued, retired at the next batch if live."""
        self.cancelled.add(rid)

    def close(self):
        for p in self.pools.values():
            p.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def n_live(self):
        return sum(len(p.slots) for p in self.pools.values())

    def run(self, requests, clock=time.perf_counter, on_retire=None, cases=None, sleep=time.sleep):
        """Serve `requests` (arrival times in seconds from the start) to completion. `cases`
        maps request ids to prepared CaseData (otherwise each case is built at admission)."""
        pending = sorted(requests, key=lambda r: r.arrival)
        queue = []
        stats = ServeStats()
        t0 = clock()
        i_next = 0
        cases = cases or {}

        def finish(req, status, now, admitted=0., updates=0, residual=float("nan")):
            stats.results.append(Result(req.rid, req.arrival, admitted, now, updates, residual,
                                        status == "converged", status))

        while i_next < len(pending) or queue or self.n_live():
            now = clock() - t0
            while i_next < len(pending) and pending[i_next].arrival <= now:
                req = pending[i_next]
                i_next += 1
                pool = self.pools.get(req.row_size)
                if pool is None or req.side < 1 or req.side * req.side > pool.cap:
                    finish(req, "rejected", now)
                else:
                    queue.append(req)
            waiting = []
            for req in queue:
                if req.rid in self.cancelled:
                    finish(req, "cancelled", now)
                    continue
                if self.max_live is not None and self.n_live() >= self.max_live:
                    waiting.append(req)
                    continue
                if self.pools[req.row_size].admit(req, case=cases.get(req.rid), now=now) is None:
                    waiting.append(req)
            queue = waiting
            if not self.n_live():
                # an empty device that still cannot take a queued request never will
                for req in queue:
                    finish(req, "rejected", now)
                queue = []
                if i_next < len(pending):
                    # idle until the next arrival
                    sleep(max(0., min(pending[i_next].arrival - now, 0.01)))
                continue
            for p in self.pools.values():
                p.enqueue_batch()
            stats.batches += 1
            for p in self.pools.values():
                if not p.slots:
                    continue
                norms = p.residuals()
                done_now = clock() - t0
                for slot, r in zip(list(p.slots), norms):
                    finite = bool(np.all(np.isfinite(r)))
                    res = normalized(slot, r) if finite else float("nan")
                    slot.residual = res
                    status = ("cancelled" if slot.req.rid in self.cancelled else "diverged" if not finite
                              else "converged" if res <= self.tol else "max_updates" if slot.updates >= self.max_updates
                              else None)
                    if status is not None:
                        finish(slot.req, status, done_now, slot.admitted_at, slot.updates, res)
                        if on_retire is not None:
                            on_retire(p, slot)
                        p.retire(slot, diverged=not finite)
        stats.wall = clock() - t0
        return stats


def capacity_from_free_memory(row_size, precision, fraction):
    """Elements a pool may hold: `fraction` of the device's free memory, at most 2^21."""
    import torch
    free, _ = torch.cuda.mem_get_info()
    return int(min(free * fraction // pool_bytes_per_element(row_size, precision), 1 << 21))
