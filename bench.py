"""Benchmark: GDOF-updates/s per RK stage of the DG spatial operator + stage update.

Workload (default): compressible Navier-Stokes Taylor-Green vortex on 32^3 deformed hexes,
row size 6, Mach 0.1, Re 1600, Pr 0.71, Sutherland transport, FP64 (hexed_gb300.problems).
A step is one Solver::update: max_dt, the viscous LDG stage 0 and the inviscid stage 1
(src/Solver.cpp:834-886). value = element DOFs x 2 stages x steps / device time.

  python bench.py [--gpus N --steps K --warmup W --precision fp64|mixed --impl gb300|reference]
                  [--workload tgv|vortex|mach2|tree --n N --rs RS]
  python bench.py --serving [--solves S --rate R --max-side M --tol T --precision fp64|mixed]

The default line reports the FP64 form (the headline) and, under "mixed", the mixed form of
the same workload with its error against the FP64 state, and under "serving" a bounded
sample of the serving stream (see serving_sample). The K timed updates replay one CUDA graph
(hexed_gpu_update_n) captured in warm-up; the per-kernel table comes from a separate eager,
profiled pass of K updates. --workload selects the other configurations (see Workload);
--serving measures the serving loop alone (see run_serving).

Multi-GPU: the path runs one independent replica per GPU (no data-path collective);
value aggregates all replicas (weak scaling).
--impl reference times the CPU oracle port of the reference's OpenMP hot path on the host
cores (the reference itself cannot be built here: Eigen/HDF5 are absent).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from hexed_gb300 import abi, problems, replicas  # noqa: E402

METRIC = "GDOF-updates/s per RK stage"


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), \
        int(os.environ.get("LOCAL_RANK", "0"))


class Workload:
    """One benchmark configuration: the mesh and initial state, and the update parameters.

    tgv    compressible Navier-Stokes Taylor-Green vortex, n^3 deformed hexes (default 32),
           row size 6, Mach 0.1, Re 1600, Pr 0.71, Sutherland transport (the headline)
    vortex 2D isentropic vortex, n x n Cartesian quads (default 32) on [-5, 5]^2, row size 6,
           Mach 0.5, Riemann-invariant freestream boundaries
    mach2  the deformed n^3 mesh (default 32) with an inviscid Mach 2 flow and a density jump
           of ratio 2.5 at x = pi, with stabilising artificial viscosity
    tree   16^3 base tree refined 2 levels inside a sphere of radius 0.25 (27,224 hexes with
           hanging faces), row size 4 (or 6), Euler Mach 0.3 with a Gaussian pressure pulse
    """
    DEFAULT_N = {"tgv": 32, "vortex": 32, "mach2": 32, "tree": 16}
    DEFAULT_RS = {"tgv": 6, "vortex": 6, "mach2": 6, "tree": 4}

    def __init__(self, kind, n=None, rs=None):
        self.kind = kind
        self.n = n or self.DEFAULT_N[kind]
        self.rs = rs or self.DEFAULT_RS[kind]

    def arena(self):
        """A fresh copy of the workload's arena (generated once: the 32^3 deformed meshes take
        tens of seconds to set up on the host)."""
        if getattr(self, "_arena", None) is None:
            self._arena = self._make()
        return self._arena.copy()

    def _make(self):
        k, n, rs = self.kind, self.n, self.rs
        if k == "tgv":
            return problems.taylor_green_3d(n_per_side=n, row_size=rs)
        if k == "vortex":
            return problems.vortex_2d(n_per_side=n, row_size=rs)
        if k == "mach2":
            return problems.mach2_jump_3d(n_per_side=n, row_size=rs)
        return problems.pulse_tree_3d(n_base=n, row_size=rs, levels=2)

    def params(self, ar):
        if self.kind == "tgv":
            return abi.update_params(max_safety=0.5, visc=ar.visc, cond=ar.cond)
        if self.kind == "mach2":
            return abi.update_params(max_safety=0.5, av_admis_char_speed=ar.av_char_speed)
        return abi.update_params(max_safety=0.5)

    @property
    def name(self):
        return {"tgv": f"taylor_green_3d_ns_{self.n}cube_deformed_rs{self.rs}",
                "vortex": f"isentropic_vortex_2d_{self.n}sq_rs{self.rs}",
                "mach2": f"mach2_density_jump_3d_euler_av_{self.n}cube_deformed_rs{self.rs}",
                "tree": f"pulse_tree_3d_{self.n}base_2levels_rs{self.rs}"}[self.kind]


def initialize(c):
    """Solver::initialize on a context or oracle: traces, then hanging-face mortars."""
    c.write_face()
    c.prolong()


def dofs_per_update(ar):
    return ar.n_elem * ar.nv * ar.nq * 2  # two stages per update


# ------------------------------------------------------------------ algorithmic bytes
def kernel_bytes(name, ar, precision="fp64"):
    """Compulsory bytes per launch of each kernel: every array the kernel must read or
    write, counted once. The state, time-step scale, AV rows and determinant reciprocals are
    double in both forms; traces, residual cache and metric normals are float in the mixed
    form."""
    nd, nq, nfq, nv = ar.n_dim, ar.nq, ar.nfq, ar.nv
    F = 2 * nd
    d, w = 8, (4 if precision == "mixed" else 8)
    # deformed metrics: the normals and 1/J (FP64 form); the float normals with their
    # determinant row, from which the mixed volume kernel forms 1/J (mixed form)
    metric = w * (nd * nd + 1) * nq if precision == "mixed" else w * nd * nd * nq + d * nq
    per_elem = {
        "local_car_euler": d * (2 * nv + 1) * nq + w * nv * nq + w * 2 * F * nv * nfq,
        "local_def_euler": d * (2 * nv + 1) * nq + w * nv * nq + w * 2 * F * nv * nfq + metric,
        "local_car_ns": d * (2 * nv + 3) * nq + w * nv * nq + w * 3 * F * nv * nfq,
        "local_def_ns": d * (2 * nv + 3) * nq + w * nv * nq + w * 3 * F * nv * nfq + metric + w * F * nd * nfq,
        "reconcile_ldg_car": d * (2 * nv + 1) * nq + w * 2 * F * nv * nfq,
        # 1/J: the FP64 array (FP64 form), the float normals' determinant row (mixed form)
        "reconcile_ldg_def": d * (2 * nv + 1) * nq + w * nq + w * 2 * F * nv * nfq,
        "max_dt": d * (nv + 3) * nq + w * 2 ** nd,   # the mixed form reads float vertex scales
    }
    if name in per_elem:
        n = ar.n_def if "def" in name else ar.n_car if "car" in name else ar.n_elem
        return per_elem[name] * n
    per_con = {
        "neighbor_car": w * 4 * nv * nfq,
        "neighbor_def": w * (4 * nv * nfq + nd * nfq),
        "neighbor_bc_fused": w * (4 * nv * nfq + nd * nfq),
    }
    if name in per_con:
        n = {"neighbor_car": len(ar.car_con), "neighbor_def": len(ar.def_con)}.get(name, len(ar.bc_con))
        return per_con[name] * n
    return None


# DRAM bytes per element and launch measured by ncu (dram__bytes_read.sum +
# dram__bytes_write.sum, one launch) on smaller Taylor-Green meshes of the same kernels: FP64
# on the 16^3 mesh, mixed on the 24^3 mesh, row size 6.
NCU_DRAM_BYTES_PER_ELEM = {
    ("local_def_ns", "fp64", 6): 73092.,
    ("local_def_euler", "fp64", 6): 69626.,
    ("local_def_ns", "mixed", 6): (490.465792e6 + 201.874944e6) / 13824,
    ("local_def_euler", "mixed", 6): (514.078720e6 + 149.316096e6) / 13824,
}


# Busiest pipe of the same kernels in those captures (fraction of peak sustained over active cycles).
NCU_PIPE_FRAC = {
    ("local_def_ns", "fp64", 6): ("fp64", 0.940),
    ("local_def_euler", "fp64", 6): ("fp64", 0.930),
}

# FP64 flops per element of the FP64 kernels (2 x DFMA + DADD + DMUL thread instructions
# counted by ncu on the 16^3 Taylor-Green mesh, row size 6): the compute roofline of the FP64
# form, against the FP64 FMA rate hexed_gpu_fp64_peak measures in the same run.
NCU_FP64_FLOPS_PER_ELEM = {
    ("local_def_ns", 6): 419984.,
    ("local_def_euler", 6): 100440.,
    # the smoothness-AV advection volume kernel (3D deformed, row size 6; ncu on the 16^3 mesh)
    ("sav_local_advection", 6): 128952.,
}


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            self.proc.wait(timeout=5)

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for n, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------ CPU oracle timing
def host_threads():
    """OpenMP threads of the CPU baseline: OMP_NUM_THREADS when set, else the rule of the
    reference's hexecute, all hardware threads but two (src/hexecute.cpp:7)."""
    env = os.environ.get("OMP_NUM_THREADS")
    if env and env.isdigit() and int(env) > 0:
        return int(env)
    return max(1, (os.cpu_count() or 1) - 2)


def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo, else the machine type)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        with open("/proc/cpuinfo") as fh:
            for line in fh:
                if line.lower().startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform
    return platform.machine()


def config_of(wl, ar, precision, world):
    """The `config` object of both arms' lines."""
    return {"workload": wl.name, "n_elem": ar.n_elem, "row_size": wl.rs, "precision": precision,
            "parallelism": f"replicas{world}",
            "l2": f"inputs larger than L2 (state alone {ar.elem.nbytes / 1e6:.0f} MB; L2 129 MB)"}


def cpu_baseline(wl, steps=None, target_s=12.):
    """Time the oracle port (OpenMP, host_threads() threads) on the same workload."""
    import oracle
    threads = oracle.set_threads(host_threads())
    ar = wl.arena()
    o = oracle.Oracle(ar)
    initialize(o)
    p = wl.params(ar)
    t0 = time.perf_counter()
    o.update(p)
    one = time.perf_counter() - t0
    if steps is None:
        steps = max(1, min(50, int(target_s / max(one, 1e-6))))
    t0 = time.perf_counter()
    for _ in range(steps):
        o.update(p)
    t = time.perf_counter() - t0
    return {"value": dofs_per_update(ar) * steps / t / 1e9, "unit": "GDOF/s", "cores": threads, "kind": "port",
            "sample": f"{steps} Solver::update steps of the full {wl.name} workload on the CPU oracle "
                      f"({t:.2f} s)", "seconds": t, "cpu_model": cpu_model(), "host_threads": os.cpu_count()}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    import oracle
    oracle.build()
    threads = oracle.set_threads(host_threads())
    wl = Workload(args.workload, args.n, args.rs)
    ar = wl.arena()
    o = oracle.Oracle(ar)
    initialize(o)
    p = wl.params(ar)
    # one update is a fraction of a second of CPU work at full size: each step is one update
    for _ in range(args.warmup):
        o.update(p)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        o.update(p)
    t = time.perf_counter() - t0
    value = dofs_per_update(ar) * args.steps / t / 1e9
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "GDOF/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": config_of(wl, ar, "fp64", world),
            "cpu_baseline": {"value": value, "unit": "GDOF/s", "cores": threads, "kind": "port",
                             "sample": f"{args.steps} Solver::update steps of the full workload on the CPU oracle",
                             "cpu_model": cpu_model(), "host_threads": os.cpu_count()},
            "e2e": {"value": value, "unit": "GDOF/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def state_errors(a, b, nv):
    """L2 and Linf errors of state a against reference b: per variable (each relative to
    that variable's own norm, and relative to its conserved quantity's norm) and per conserved
    quantity (momentum vector, density, energy)."""
    out = {"l2_rel": [], "linf_rel": []}
    for v in range(nv):
        d, r = a[:, v] - b[:, v], b[:, v]
        out["l2_rel"].append(float(np.linalg.norm(d) / max(np.linalg.norm(r), 1e-300)))
        out["linf_rel"].append(float(np.abs(d).max() / max(np.abs(r).max(), 1e-300)))
    # each variable against the L2 norm of its conserved quantity: a momentum component against
    # the momentum vector's (a component that starts at zero has no meaningful own scale)
    mom = float(np.linalg.norm(b[:, :nv - 2]))
    out["l2_rel_quantity_scaled"] = [
        float(np.linalg.norm(a[:, v] - b[:, v]) / (mom if v < nv - 2 else np.linalg.norm(b[:, v])))
        for v in range(nv)]
    groups = {"momentum": slice(0, nv - 2), "density": slice(nv - 2, nv - 1), "energy": slice(nv - 1, nv)}
    out["l2_rel_by_quantity"] = {k: float(np.linalg.norm(a[:, s] - b[:, s]) / np.linalg.norm(b[:, s]))
                                 for k, s in groups.items()}
    return out


def mixed_vs_fp64(wl, steps):
    """Run the same case `steps` updates in FP64 and in mixed precision on the GPU and
    report the mixed state's error against the FP64 state."""
    from hexed_gb300.solver import Context
    states = {}
    base = wl.arena()
    for prec in (abi.FP64, abi.MIXED):
        ar = base.copy()
        with Context(ar, prec) as c:
            initialize(c)
            p = wl.params(ar)
            for _ in range(steps):
                c.update(p, read_dt=False)
            states[prec] = c.download(abi.ARRAY_ELEM)[:, :ar.nv]
    err = state_errors(states[abi.MIXED], states[abi.FP64], ar.nv)
    err["steps"] = steps
    err["reference"] = "FP64 GPU path, same mesh and initial state"
    return err


# ------------------------------------------------------------------ serving stream
def run_serving(args):
    """Continuous-batching serving of a stream of steady 2D Euler solves against the same
    stream served one solve at a time (FP64), both on this GPU, same tolerance.

    The stream: Cartesian meshes of [0, 1]^2 with sides uniform in [8, max_side], row size 4
    or 6, Mach U(0.2, 0.8), angle U(-10, 10) degrees, freestream plus a 5-mode 2% Fourier
    perturbation, local time stepping until the normalized residual reaches `tol`; Poisson
    arrivals at `rate` per second."""
    from hexed_gb300 import serving
    precision = abi.MIXED if args.precision == "mixed" else abi.FP64
    params = abi.update_params(max_safety=0.5, local_time=True)
    reqs = serving.request_stream(args.solves, args.rate, seed=args.seed, sides=(8, args.max_side))
    k = {4: args.batch, 6: args.batch}
    with serving.Server(precision, tol=args.tol, updates_per_batch=k, params=params,
                        max_updates=args.max_updates) as srv:
        srv.run(reqs[:2])   # warm-up: kernels loaded, graphs of the first shapes
        batched = srv.run(reqs).summary()
    base = None
    if not args.no_one_at_a_time:
        with serving.Server(abi.FP64, tol=args.tol, updates_per_batch=k, params=params, max_live=1,
                            max_updates=args.max_updates) as srv:
            srv.run(reqs[:2])
            base = srv.run(reqs).summary()
    line = {
        "metric": "steady solves/s (continuous batching)", "value": batched["solves_per_s"], "unit": "solves/s",
        "n_gpus": 1, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if precision == abi.FP64 else "f32/f64", "data": "synthetic",
        "config": {"workload": "serving_2d_euler_stream", "solves": args.solves, "rate_per_s": args.rate,
                   "sides": [8, args.max_side], "row_sizes": [4, 6], "tol": args.tol, "seed": args.seed,
                   "updates_per_batch": args.batch, "precision": args.precision},
        "p50_latency_s": batched["p50_latency_s"], "p99_latency_s": batched["p99_latency_s"],
        "batched": batched, "one_at_a_time_fp64": base,
        "speedup_vs_one_at_a_time": (batched["solves_per_s"] / base["solves_per_s"]) if base else None,
    }
    print(json.dumps(line))
    return 0


def run_serving_probe(args):
    """Per-batch time, residual-check time and per-kernel launch time of serving pools
    (FP64 and mixed; one 10x10 solve at row sizes 4 and 6, and 24 solves of 16x16 at row
    size 6): 3 warm-up batches, 30 timed batches of 20 updates, 30 timed residual checks,
    then one eager batch under the library's CUDA-event profiler."""
    from hexed_gb300 import serving
    params = abi.update_params(max_safety=0.5, local_time=True)
    out = {}
    for prec, pname in ((abi.FP64, "fp64"), (abi.MIXED, "mixed")):
        for rs, side, n_cases in ((4, 10, 1), (6, 10, 1), (6, 16, 24)):
            pool = serving.Pool(rs, prec, capacity=8192, params=params, updates_per_batch=20)
            for i in range(n_cases):
                pool.admit(serving.Request(i, side, rs, 0.5, 0., seed=1 + i))
            for _ in range(3):
                pool.enqueue_batch()
                pool.residuals()
            pool.ctx.synchronize()
            t0 = time.perf_counter()
            for _ in range(30):
                pool.enqueue_batch()
            pool.ctx.synchronize()
            t_batch = (time.perf_counter() - t0) / 30
            t0 = time.perf_counter()
            for _ in range(30):
                pool.residuals()
            t_res = (time.perf_counter() - t0) / 30
            pool.ctx.profile_enable(True)
            pool.ctx.update_n(params, 20, False)
            prof = pool.ctx.profile_read()
            out[f"{pname}_rs{rs}_side{side}_x{n_cases}"] = {
                "elements": side * side * n_cases, "batch_of_20_ms": round(t_batch * 1e3, 3),
                "residual_check_ms": round(t_res * 1e3, 3),
                "kernel_us_per_launch": {k: round(v[1] / v[0] * 1e3, 2) for k, v in prof.items()}}
            pool.close()
    print(json.dumps(out))
    return 0


# ------------------------------------------------------------------ GPU arm
def timed_updates(ctx, p, args, stream, barrier, local_rank):
    """W eager warm-up updates, then one untimed hexed_gpu_update_n of K updates, which
    captures them as a CUDA graph; the timed region replays that graph (K updates) between
    CUDA events on the library's stream, with the clocks sampled meanwhile. Then an eager pass
    of K updates under the library's per-kernel CUDA-event profiler gives the kernel table
    (same launches as the graph; outside the timed region). Returns (ms, profile, clocks)."""
    import torch
    for _ in range(args.warmup):
        ctx.update(p, read_dt=False)
    ctx.update_n(p, args.steps, use_graph=True)
    ctx.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    torch.cuda.synchronize()
    with ClockSampler(local_rank) as clk:
        e0.record(stream)
        ctx.update_n(p, args.steps, use_graph=True)
        e1.record(stream)
        torch.cuda.synchronize()
    barrier()
    ms = e0.elapsed_time(e1)
    ctx.profile_enable(True)
    for _ in range(args.steps):
        ctx.update(p, read_dt=False)
    prof = ctx.profile_read()
    ctx.profile_enable(False)
    return ms, prof, clk


_FP64_PEAK = []


def fp64_peak_tflops_cached():
    """hexed_gpu_fp64_peak, measured once per run."""
    if not _FP64_PEAK:
        from hexed_gb300.solver import fp64_peak_tflops
        _FP64_PEAK.append(fp64_peak_tflops())
    return _FP64_PEAK[0]


_DGEMM_PEAK = []


def fp64_dgemm_tflops_cached(n=4096, reps=3):
    """A library cross-check of the FP64 rate: cuBLAS DGEMM (torch.matmul in float64) of
    n x n operands, best of `reps` after one warm-up, 2 n^3 flops each, CUDA events on the
    current stream. Measured once per run."""
    if not _DGEMM_PEAK:
        import torch
        a = torch.randn(n, n, dtype=torch.float64, device="cuda")
        b = torch.randn(n, n, dtype=torch.float64, device="cuda")
        torch.matmul(a, b)
        best = None
        for _ in range(reps):
            t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            t0.record()
            torch.matmul(a, b)
            t1.record()
            torch.cuda.synchronize()
            ms = t0.elapsed_time(t1)
            best = ms if best is None else min(best, ms)
        _DGEMM_PEAK.append(2 * n ** 3 / (best * 1e-3) / 1e12)
        del a, b
        torch.cuda.empty_cache()
    return _DGEMM_PEAK[0]


def sav_advection_bytes(ar):
    """Compulsory bytes of one launch of the smoothness-AV advection volume kernel: per element
    the nd velocity rows, the advection state read and written, its residual cache written
    (first stage) or read (second), the time-step scale, the deformed metric rows (nd^2 + 1),
    and the rs flux traces of each of the 2 nd faces; all double."""
    nd, rs, nq, nfq = ar.n_dim, ar.row_size, ar.nq, ar.nfq
    per_elem = 8 * (nd * nq + 3 * rs * nq + nq + 2 * nd * rs * nfq)
    return per_elem * ar.n_elem + 8 * (nd * nd + 1) * nq * ar.n_def


def smooth_av_sample(wl, args, hbm_peak):
    """Solver::update_art_visc_smoothness on the workload's arena (FP64): `sav_iters` advection
    iterations (two stages each) and `sav_iters` / 2 diffusion iterations; the whole call timed
    with CUDA events, then the same call under the per-kernel profiler for the advection volume
    kernel's HBM roofline."""
    import torch
    from hexed_gb300.solver import Context
    ar = wl.arena()
    fs_mass = float(np.mean(ar.elem[:, ar.n_dim]))
    fs_energy = float(np.mean(ar.elem[:, ar.n_dim + 1]))
    length = 2.0 * float(np.mean(ar.nom_size))
    p = abi.sav_params(length, ar.row_size, fs_mass, fs_energy, advect_iters=args.sav_iters,
                       diff_iters=max(1, args.sav_iters // 2))
    with Context(ar, abi.FP64) as c:
        initialize(c)
        stream = torch.cuda.ExternalStream(c.stream_ptr)
        c.update_art_visc_smoothness(p)   # warm-up (allocates the storage)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        c.update_art_visc_smoothness(p)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        c.profile_enable(True)
        c.update_art_visc_smoothness(p)
        prof = c.profile_read()
        c.profile_enable(False)
    launches, total = prof.get("sav_local_advection", (0, 0.))
    per_launch = total / max(launches, 1)
    nbytes = sav_advection_bytes(ar)
    achieved = nbytes / (per_launch * 1e-3) / 1e9 if per_launch else None
    roof = {"bound": "hbm", "kernel": "sav_local_advection", "achieved": achieved, "peak": hbm_peak,
            "unit": "GB/s", "frac": achieved / hbm_peak if achieved else None,
            "algorithmic_bytes_per_launch": nbytes, "launch_ms": per_launch}
    flops = NCU_FP64_FLOPS_PER_ELEM.get(("sav_local_advection", ar.row_size)) if ar.n_dim == 3 else None
    fp64_peak = fp64_peak_tflops_cached()
    if flops and per_launch and fp64_peak:
        # FP64 throughout (parity with the oracle at 1e-12): the kernel's own roof is the FP64 pipe
        tf = flops * ar.n_elem / (per_launch * 1e-3) / 1e12
        roof["fp64"] = {"achieved": tf, "peak": fp64_peak, "unit": "TFLOP/s", "frac": tf / fp64_peak,
                        "flops_per_launch": flops * ar.n_elem,
                        "flops_source": "ncu 2*dfma + dadd + dmul thread instructions per element of one launch "
                                        "on the 16^3 Taylor-Green mesh, scaled by elements"}
        roof["compute_bound"] = {"pipe": "fp64", "frac_of_peak_ncu": 0.877}
    return {"workload": wl.name, "advect_iters": p.advect_iters, "diff_iters": p.diff_iters,
            "advect_length": length, "ms_per_call": ms,
            "ms_per_advection_iteration": ms / (p.advect_iters + p.diff_iters),
            "roofline": roof,
            "kernels": {k: {"launches": v[0], "total_ms": round(v[1], 4)}
                        for k, v in sorted(prof.items(), key=lambda kv: -kv[1][1])}}


def serving_sample(args):
    """A bounded sample of the serving stream (steady 2D Euler solves, Cartesian meshes of
    sides uniform in [8, serving_max_side], row size 4 or 6, Mach U(0.2, 0.8), angle
    U(-10, 10) degrees, 2% five-mode perturbation, local time stepping to a 1e-8 drop of the
    normalized residual, Poisson arrivals): batched in the mixed form, batched in FP64, and
    one solve at a time in FP64 (the same engine with one live solve), each with solves/s,
    p50/p99 latency and the clocks seen."""
    from hexed_gb300 import serving
    params = abi.update_params(max_safety=0.5, local_time=True)
    reqs = serving.request_stream(args.serving_solves, args.rate, seed=args.seed, sides=(8, args.serving_max_side))
    k = {4: args.batch, 6: args.batch}
    out = {"config": {"workload": "serving_2d_euler_stream_sample", "solves": args.serving_solves,
                      "rate_per_s": args.rate, "sides": [8, args.serving_max_side], "row_sizes": [4, 6],
                      "tol": args.tol, "seed": args.seed, "updates_per_batch": args.batch,
                      "sample": "bounded sample of the 512-solve, sides 8-96 stream with the same distributions"}}
    legs = (("batched_mixed", abi.MIXED, None), ("batched_fp64", abi.FP64, None), ("one_at_a_time_fp64", abi.FP64, 1))
    for name, prec, max_live in legs:
        with serving.Server(prec, tol=args.tol, updates_per_batch=k, params=params, max_live=max_live,
                            max_updates=args.max_updates) as srv:
            srv.run(reqs[:2])   # warm-up: kernels loaded, graphs of the first shapes
            with ClockSampler(0) as clk:
                summary = srv.run(reqs).summary()
        out[name] = {k2: summary[k2] for k2 in ("solves", "converged", "solves_per_s", "p50_latency_s",
                                                "p99_latency_s", "updates", "wall_s")}
        out[name]["clocks"] = clk.summary()
    out["speedup_batched_fp64_vs_one_at_a_time"] = (out["batched_fp64"]["solves_per_s"] /
                                                     out["one_at_a_time_fp64"]["solves_per_s"])
    out["speedup_batched_mixed_vs_one_at_a_time"] = (out["batched_mixed"]["solves_per_s"] /
                                                      out["one_at_a_time_fp64"]["solves_per_s"])
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    ap.add_argument("--workload", default="tgv", choices=["tgv", "vortex", "mach2", "tree"])
    ap.add_argument("--n", type=int, default=None, help="elements per side (tree: base elements per side)")
    ap.add_argument("--rs", type=int, default=None, help="row size")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-steps", type=int, default=None)
    ap.add_argument("--err-steps", type=int, default=200, help="updates for the mixed-vs-FP64 error report")
    ap.add_argument("--no-mixed", action="store_true", help="skip the mixed-form measurement beside FP64")
    ap.add_argument("--serving", action="store_true", help="serve a stream of steady 2D solves instead")
    ap.add_argument("--serving-probe", action="store_true", help="time batches and kernels of serving pools")
    ap.add_argument("--solves", type=int, default=64)
    ap.add_argument("--rate", type=float, default=200.)
    ap.add_argument("--max-side", type=int, default=16)
    ap.add_argument("--tol", type=float, default=1e-8)
    ap.add_argument("--batch", type=int, default=20, help="updates per batch (one graph replay)")
    ap.add_argument("--max-updates", type=int, default=400_000)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--no-one-at-a-time", action="store_true")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving sample of the default line")
    ap.add_argument("--serving-solves", type=int, default=24, help="solves in the default line's serving sample")
    ap.add_argument("--serving-max-side", type=int, default=16)
    ap.add_argument("--no-smooth-av", action="store_true", help="skip the smoothness-AV measurement")
    ap.add_argument("--sav-iters", type=int, default=20, help="advection iterations of the smoothness-AV sample")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.serving:
        return run_serving(args)
    if args.serving_probe:
        return run_serving_probe(args)

    import torch
    rank, world, local_rank = dist_env()
    torch.cuda.set_device(local_rank)
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
        pg = dist

    def barrier():
        if pg:
            pg.barrier()

    from hexed_gb300.solver import Context, fp64_peak_tflops
    precision = abi.MIXED if args.precision == "mixed" else abi.FP64
    wl = Workload(args.workload, args.n, args.rs)
    ar = wl.arena()
    ctx = Context(ar, precision)
    initialize(ctx)
    p = wl.params(ar)
    stream = torch.cuda.ExternalStream(ctx.stream_ptr)
    # timed region: inputs resident in HBM (arena ~2 GB >> 129 MB L2, no flush needed)
    ms, prof, clk = timed_updates(ctx, p, args, stream, barrier, local_rank)
    ms = replicas.max_over_ranks(ms, device="cuda")
    value = replicas.job_rate(dofs_per_update(ar) * args.steps, world, ms) / 1e9
    launches = sum(v[0] for v in prof.values())

    # ---- end to end through the C ABI with pinned host buffers: write the conserved state
    # from host memory, one update, read the conserved state back, every step
    host_in = torch.from_numpy(np.ascontiguousarray(ar.elem[:, :ar.nv])).pin_memory()
    host_out = torch.empty_like(host_in).pin_memory()
    lib = ctx.lib
    n_bytes = host_in.numel() * 8

    def e2e_step():
        # a new state from the host, its face traces (Solver::initialize), one update, read back
        abi.check(lib.hexed_gpu_write_state(ctx.handle, abi.ctypes.cast(host_in.data_ptr(), abi.P_double)))
        initialize(ctx)
        ctx.update(p, read_dt=False)
        abi.check(lib.hexed_gpu_read_state(ctx.handle, abi.ctypes.cast(host_out.data_ptr(), abi.P_double)))
    e2e_step()   # untimed: the first write_state allocates its device staging buffer
    ctx.synchronize()
    barrier()
    torch.cuda.synchronize()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    f1.record(stream)
    torch.cuda.synchronize()
    wall_e2e = time.perf_counter() - t0
    ms_e2e = replicas.max_over_ranks(max(f0.elapsed_time(f1), wall_e2e * 1e3), device="cuda")
    e2e_value = replicas.job_rate(dofs_per_update(ar) * args.steps, world, ms_e2e) / 1e9

    # ---- roofline of the dominant kernel
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            peaks = json.load(fh)
    except OSError:
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.)
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    top = max(prof.items(), key=lambda kv: kv[1][1])
    top_name, (top_launches, top_ms) = top
    per_launch_ms = top_ms / max(top_launches, 1)
    nbytes = kernel_bytes(top_name, ar, args.precision)
    achieved = nbytes / (per_launch_ms * 1e-3) / 1e9 if nbytes else None
    fp64_peak = fp64_peak_tflops_cached()
    traffic = None
    # the Mach-2 case runs the same deformed kernels on the same mesh kind (same arrays per
    # element), so the Taylor-Green captures' per-element figures apply to it too
    per_elem = NCU_DRAM_BYTES_PER_ELEM.get((top_name, args.precision, wl.rs)) if wl.kind in ("tgv", "mach2") else None
    if per_elem is not None:
        traffic = per_elem * (ar.n_def if "def" in top_name else ar.n_car if "car" in top_name else ar.n_elem)
    roofline = {"bound": "hbm", "kernel": top_name, "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                "frac": achieved / hbm_peak if achieved else None, "traffic": traffic,
                "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch of the same "
                                  "kernel on a smaller Taylor-Green mesh (16^3 FP64, 24^3 mixed), scaled by "
                                  "elements" if traffic else None,
                "algorithmic_bytes_per_launch": nbytes, "launch_ms": per_launch_ms,
                "peak_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)",
                "fp64_peak_tflops_measured": fp64_peak}
    pipe = NCU_PIPE_FRAC.get((top_name, args.precision, wl.rs)) if wl.kind in ("tgv", "mach2") else None
    if pipe is not None:
        # what bounds this kernel instead of HBM: the busiest pipe in the same ncu capture
        roofline["compute_bound"] = {"pipe": pipe[0], "frac_of_peak_ncu": pipe[1]}
    flops = NCU_FP64_FLOPS_PER_ELEM.get((top_name, wl.rs)) if wl.kind in ("tgv", "mach2") else None
    if flops is not None and precision == abi.FP64 and fp64_peak:
        # the FP64 form's own roof: its FP64 flops per launch over the launch time, against the
        # FP64 FMA rate measured in this run
        n = ar.n_def if "def" in top_name else ar.n_car
        achieved_tf = flops * n / (per_launch_ms * 1e-3) / 1e12
        roofline["fp64"] = {"achieved": achieved_tf, "peak": fp64_peak, "unit": "TFLOP/s",
                            "frac": achieved_tf / fp64_peak, "flops_per_launch": flops * n,
                            "flops_source": "ncu 2*dfma + dadd + dmul thread instructions per element of one "
                                            "launch on the 16^3 Taylor-Green mesh, scaled by elements",
                            "peak_source": "hexed_gpu_fp64_peak, measured in this run"}
        dgemm = fp64_dgemm_tflops_cached()
        roofline["fp64"]["dgemm_tflops"] = dgemm
        roofline["fp64"]["frac_of_dgemm"] = achieved_tf / dgemm
        roofline["fp64"]["dgemm_source"] = "cuBLAS DGEMM 4096^3 (torch.matmul, float64), best of 3, this run"
    kernels = {k: {"launches": v[0], "total_ms": round(v[1], 4), "share": round(v[1] / sum(x[1] for x in prof.values()), 4)}
               for k, v in sorted(prof.items(), key=lambda kv: -kv[1][1])}

    mixed_err = None
    if precision == abi.MIXED and rank == 0 and args.err_steps > 0:
        ctx.close()
        mixed_err = mixed_vs_fp64(wl, args.err_steps)

    # the mixed form of the same workload beside the FP64 headline
    mixed = None
    if precision == abi.FP64 and rank == 0 and not args.no_mixed:
        ctx.close()
        mctx = Context(wl.arena(), abi.MIXED)
        initialize(mctx)
        mstream = torch.cuda.ExternalStream(mctx.stream_ptr)
        mms, mprof, mclk = timed_updates(mctx, p, args, mstream, lambda: None, local_rank)
        mctx.close()
        mvalue = dofs_per_update(ar) * args.steps / (mms / 1e3) / 1e9
        # HBM roofline of the mixed form's dominant kernel, as for the headline
        mtop, (mlaunches, mtop_ms) = max(mprof.items(), key=lambda kv: kv[1][1])
        mlaunch_ms = mtop_ms / max(mlaunches, 1)
        mbytes = kernel_bytes(mtop, ar, "mixed")
        machieved = mbytes / (mlaunch_ms * 1e-3) / 1e9 if mbytes else None
        mper_elem = NCU_DRAM_BYTES_PER_ELEM.get((mtop, "mixed", wl.rs)) if wl.kind in ("tgv", "mach2") else None
        mroof = {"bound": "hbm", "kernel": mtop, "achieved": machieved, "peak": hbm_peak, "unit": "GB/s",
                 "frac": machieved / hbm_peak if machieved else None, "algorithmic_bytes_per_launch": mbytes,
                 "launch_ms": mlaunch_ms,
                 "traffic": mper_elem * (ar.n_def if "def" in mtop else ar.n_car) if mper_elem else None}
        mixed = {"value": mvalue, "unit": "GDOF/s", "ms_per_step": mms / args.steps, "speedup_vs_fp64": mvalue / value,
                 "dtype": "f32/f64", "roofline": mroof, "clocks": mclk.summary(),
                 "kernels": {k: {"launches": v[0], "total_ms": round(v[1], 4)}
                             for k, v in sorted(mprof.items(), key=lambda kv: -kv[1][1])},
                 "error_vs_fp64": mixed_vs_fp64(wl, args.err_steps) if args.err_steps > 0 else None}

    sav_line = None
    if rank == 0 and world == 1 and not args.no_smooth_av:
        ctx.close()
        sav_line = smooth_av_sample(wl, args, hbm_peak)

    serving_line = None
    if rank == 0 and world == 1 and not args.no_serving:
        ctx.close()
        serving_line = serving_sample(args)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        ctx.close()
        try:
            cpu = cpu_baseline(wl, args.cpu_steps)
        except Exception as exc:  # noqa: BLE001
            cpu = {"error": str(exc)}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "GDOF/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64" if precision == abi.FP64 else "f32/f64",
                "data": "synthetic",
                "config": config_of(wl, ar, args.precision, world),
                "timing": f"{args.steps} updates replayed as one CUDA graph captured in warm-up",
                "e2e": {"value": e2e_value, "unit": "GDOF/s", "h2d_bytes_per_step": n_bytes,
                        "d2h_bytes_per_step": n_bytes},
                "gpu_launches": launches,
                "clocks": clk.summary(),
                "roofline": roofline,
                "kernels": kernels,
                "cpu_baseline": cpu}
        if mixed_err is not None:
            line["mixed_vs_fp64"] = mixed_err
        if mixed is not None:
            line["mixed"] = mixed
        if serving_line is not None:
            line["serving"] = serving_line
        if sav_line is not None:
            line["smooth_av"] = sav_line
        print(json.dumps(line))
    if pg:
        pg.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
