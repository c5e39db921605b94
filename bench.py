"""Benchmark: GDOF-updates/s per RK stage of the DG spatial operator + stage update.

Workload (default): compressible Navier-Stokes Taylor-Green vortex on 32^3 deformed hexes,
row size 6, Mach 0.1, Re 1600, Pr 0.71, Sutherland transport, FP64 (hexed_gb300.problems).
A step is one Solver::update: max_dt, the viscous LDG stage 0 and the inviscid stage 1
(src/Solver.cpp:834-886). value = element DOFs x 2 stages x steps / device time.

  python bench.py [--gpus N --steps K --warmup W --precision fp64|mixed --impl gb300|reference]

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

from hexed_gb300 import abi, problems  # noqa: E402

WORKLOAD = "taylor_green_3d_ns_32cube_deformed_rs6"
METRIC = "GDOF-updates/s per RK stage"


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), \
        int(os.environ.get("LOCAL_RANK", "0"))


def make_case(n, rs, seed=0):
    return problems.taylor_green_3d(n_per_side=n, row_size=rs, seed=seed)


def dofs_per_update(ar):
    return ar.n_elem * ar.nv * ar.nq * 2  # two stages per update


# ------------------------------------------------------------------ algorithmic bytes
def kernel_bytes(name, ar):
    """Compulsory bytes per launch of each kernel: every array the kernel must read or
    write, counted once (FP64 arena; face traces stored in double)."""
    nd, nq, nfq, nv = ar.n_dim, ar.nq, ar.nfq, ar.nv
    F = 2 * nd
    met = (nd * nd + 1) * nq
    per_elem = {
        "local_car_euler": (3 * nv + 1) * nq + 2 * F * nv * nfq,
        "local_def_euler": (3 * nv + 1) * nq + 2 * F * nv * nfq + met,
        "local_car_ns": (3 * nv + 3) * nq + 3 * F * nv * nfq,
        "local_def_ns": (3 * nv + 3) * nq + 3 * F * nv * nfq + met + F * nd * nfq,
        "reconcile_ldg_car": (2 * nv + 1) * nq + 2 * F * nv * nfq,
        "reconcile_ldg_def": (2 * nv + 2) * nq + 2 * F * nv * nfq,
        "max_dt": (nv + 3) * nq + 2 ** nd,
    }
    if name in per_elem:
        n = ar.n_def if "def" in name else ar.n_car if "car" in name else ar.n_elem
        return 8 * per_elem[name] * n
    per_con = {
        "neighbor_car": 4 * nv * nfq,
        "neighbor_def": 4 * nv * nfq + nd * nfq,
        "neighbor_bc_fused": 4 * nv * nfq + nd * nfq,
    }
    if name in per_con:
        n = {"neighbor_car": len(ar.car_con), "neighbor_def": len(ar.def_con)}.get(name, len(ar.bc_con))
        return 8 * per_con[name] * n
    return None


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
def cpu_baseline(n, rs, steps=None, target_s=12.):
    """Time the oracle port (OpenMP, all host threads) on the same workload."""
    import oracle
    ar = make_case(n, rs)
    o = oracle.Oracle(ar)
    o.write_face()
    p = abi.update_params(max_safety=0.5, visc=ar.visc, cond=ar.cond)
    t0 = time.perf_counter()
    o.update(p)
    one = time.perf_counter() - t0
    if steps is None:
        steps = max(1, min(50, int(target_s / max(one, 1e-6))))
    t0 = time.perf_counter()
    for _ in range(steps):
        o.update(p)
    t = time.perf_counter() - t0
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    return {"value": dofs_per_update(ar) * steps / t / 1e9, "unit": "GDOF/s", "cores": cores, "kind": "port",
            "sample": f"{steps} Solver::update steps of the full {n}^3 row-size-{rs} workload on the CPU oracle "
                      f"({t:.2f} s)", "seconds": t}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    import oracle
    oracle.build()
    ar = make_case(args.n, args.rs)
    o = oracle.Oracle(ar)
    o.write_face()
    p = abi.update_params(max_safety=0.5, visc=ar.visc, cond=ar.cond)
    # one update is several seconds of CPU work at full size: keep each step one update
    for _ in range(args.warmup):
        o.update(p)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        o.update(p)
    t = time.perf_counter() - t0
    value = dofs_per_update(ar) * args.steps / t / 1e9
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "GDOF/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": {"workload": WORKLOAD, "n_elem": ar.n_elem, "row_size": args.rs,
                                            "precision": "fp64"},
            "cpu_baseline": {"value": value, "unit": "GDOF/s", "cores": cores, "kind": "port",
                             "sample": f"{args.steps} Solver::update steps of the full workload on the CPU oracle"},
            "e2e": {"value": value, "unit": "GDOF/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def state_errors(a, b, nv):
    """L2 and Linf errors of state a against reference b: per variable (each relative to
    that variable's own norm) and per conserved quantity (momentum vector, density, energy)."""
    out = {"l2_rel": [], "linf_rel": []}
    for v in range(nv):
        d, r = a[:, v] - b[:, v], b[:, v]
        out["l2_rel"].append(float(np.linalg.norm(d) / max(np.linalg.norm(r), 1e-300)))
        out["linf_rel"].append(float(np.abs(d).max() / max(np.abs(r).max(), 1e-300)))
    groups = {"momentum": slice(0, nv - 2), "density": slice(nv - 2, nv - 1), "energy": slice(nv - 1, nv)}
    out["l2_rel_by_quantity"] = {k: float(np.linalg.norm(a[:, s] - b[:, s]) / np.linalg.norm(b[:, s]))
                                 for k, s in groups.items()}
    return out


def mixed_vs_fp64(n, rs, steps):
    """Run the same case `steps` updates in FP64 and in mixed precision on the GPU and
    report the mixed state's error against the FP64 state."""
    from hexed_gb300.solver import Context
    states = {}
    base = make_case(n, rs)
    for prec in (abi.FP64, abi.MIXED):
        ar = base.copy()
        with Context(ar, prec) as c:
            c.write_face()
            p = abi.update_params(max_safety=0.5, visc=ar.visc, cond=ar.cond)
            for _ in range(steps):
                c.update(p, read_dt=False)
            states[prec] = c.download(abi.ARRAY_ELEM)[:, :ar.nv]
    err = state_errors(states[abi.MIXED], states[abi.FP64], ar.nv)
    err["steps"] = steps
    err["reference"] = "FP64 GPU path, same mesh and initial state"
    return err


# ------------------------------------------------------------------ GPU arm
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    ap.add_argument("--n", type=int, default=32, help="elements per side")
    ap.add_argument("--rs", type=int, default=6, help="row size")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-steps", type=int, default=None)
    ap.add_argument("--err-steps", type=int, default=200, help="updates for the mixed-vs-FP64 error report")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)

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
    ar = make_case(args.n, args.rs)
    ctx = Context(ar, precision)
    ctx.write_face()
    p = abi.update_params(max_safety=0.5, visc=ar.visc, cond=ar.cond)
    stream = torch.cuda.ExternalStream(ctx.stream_ptr)
    for _ in range(args.warmup):
        ctx.update(p, read_dt=False)
    ctx.synchronize()

    # ---- timed region: inputs resident in HBM (arena ~2 GB >> 129 MB L2, no flush needed)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ctx.profile_enable(True)
    barrier()
    torch.cuda.synchronize()
    with ClockSampler(local_rank) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            ctx.update(p, read_dt=False)
        e1.record(stream)
        torch.cuda.synchronize()
    barrier()
    ms = e0.elapsed_time(e1)
    prof = ctx.profile_read()
    ms_t = torch.tensor([ms], device="cuda")
    if pg:
        pg.all_reduce(ms_t, op=pg.ReduceOp.MAX)
    ms = float(ms_t.item())
    value = dofs_per_update(ar) * args.steps * world / (ms / 1e3) / 1e9
    launches = sum(v[0] for v in prof.values())

    # ---- end to end through the C ABI with pinned host buffers: upload the state, one
    # update, download the state, every step
    host_in = torch.from_numpy(ar.elem.copy()).pin_memory()
    host_out = torch.empty_like(host_in).pin_memory()
    lib = ctx.lib
    n_bytes = host_in.numel() * 8
    ctx.synchronize()
    barrier()
    torch.cuda.synchronize()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        abi.check(lib.hexed_gpu_upload(ctx.handle, abi.ARRAY_ELEM,
                                       abi.ctypes.cast(host_in.data_ptr(), abi.P_double)))
        ctx.update(p, read_dt=False)
        abi.check(lib.hexed_gpu_download(ctx.handle, abi.ARRAY_ELEM,
                                         abi.ctypes.cast(host_out.data_ptr(), abi.P_double)))
    f1.record(stream)
    torch.cuda.synchronize()
    wall_e2e = time.perf_counter() - t0
    ms_e2e = max(f0.elapsed_time(f1), wall_e2e * 1e3)
    e2e_value = dofs_per_update(ar) * args.steps * world / (ms_e2e / 1e3) / 1e9

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
    nbytes = kernel_bytes(top_name, ar)
    achieved = nbytes / (per_launch_ms * 1e-3) / 1e9 if nbytes else None
    fp64_peak = fp64_peak_tflops()
    roofline = {"bound": "hbm", "kernel": top_name, "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                "frac": achieved / hbm_peak if achieved else None, "traffic": None,
                "algorithmic_bytes_per_launch": nbytes, "launch_ms": per_launch_ms,
                "peak_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)",
                "fp64_peak_tflops_measured": fp64_peak}
    kernels = {k: {"launches": v[0], "total_ms": round(v[1], 4), "share": round(v[1] / sum(x[1] for x in prof.values()), 4)}
               for k, v in sorted(prof.items(), key=lambda kv: -kv[1][1])}

    mixed_err = None
    if precision == abi.MIXED and rank == 0:
        ctx.close()
        mixed_err = mixed_vs_fp64(args.n, args.rs, args.err_steps)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        ctx.close()
        try:
            cpu = cpu_baseline(args.n, args.rs, args.cpu_steps)
        except Exception as exc:  # noqa: BLE001
            cpu = {"error": str(exc)}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "GDOF/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64" if precision == abi.FP64 else "f32/f64",
                "data": "synthetic",
                "config": {"workload": WORKLOAD, "n_elem": ar.n_elem, "row_size": args.rs,
                           "precision": args.precision, "parallelism": f"replicas{world}",
                           "l2": "inputs larger than L2 (arena ~2 GB)"},
                "e2e": {"value": e2e_value, "unit": "GDOF/s", "h2d_bytes_per_step": n_bytes,
                        "d2h_bytes_per_step": n_bytes},
                "gpu_launches": launches,
                "clocks": clk.summary(),
                "roofline": roofline,
                "kernels": kernels,
                "cpu_baseline": cpu}
        if mixed_err is not None:
            line["mixed_vs_fp64"] = mixed_err
        print(json.dumps(line))
    if pg:
        pg.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
