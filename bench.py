#!/usr/bin/env python
"""Benchmark of the GB300 GMGS-3D solve.

Metric: seconds for one V-cycle-preconditioned CG solve to relative residual
1e-3 on the 337 x 294 x 512 voxel block with 120 seeded spherical voids,
6 multigrid levels, mixed precision (FP32 V-cycle, FP64 outer CG vectors,
dots and coarsest solve), next to the plain FP64 GPU path and the CPU oracle.

A step is one full solve from x = 0 with the model, hierarchy and boundary
conditions resident in HBM.  The vectors (>1 GB each) are larger than L2, so
no L2 flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gmgs|reference]

Under torchrun with N > 1 every rank solves its own replica of the workload
on its own GPU (the solve does not shard: replicas only); rank 0 prints.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
for _p in (ROOT / "gmgs-3d_gb300", ROOT / "oracle"):
    if str(_p) not in sys.path:
        sys.path.insert(0, str(_p))

METRIC = "Solve s to rel-res 1e-3 at 52M DOF: mixed vs FP64 V-cycle; matvec GB/s vs HBM"
WORKLOAD = "block337_mixed_L6"
CLOCK_FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")


# DRAM bytes (read + write) per solid node of one k_fine<FM_CG_UPDATE_JACOBI>
# launch (its TMA-staged form): 984,017,664 B over 6,360,481 nodes in an ncu
# --set full capture of the same kernel on the same generator at half
# resolution (--scale 0.5); the traffic grows with the node count.
UJ_TRAFFIC_PER_NODE = 154.7


# Iterations the reference algorithm takes to relres < 1e-3 (omega 0.4) on the
# full-size workloads: the FP64 GPU path, whose iteration counts equal the
# oracle's, measured 32 / 58 / 18.  The CPU sample runs a few iterations of
# a reduced model and is extrapolated to this count.
REF_ITERATIONS = {"block337_mixed_L6": 32, "block428_mixed_adjoint_L7": 58, "block84_adjoint": 18}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gmgs", choices=["gmgs", "reference"])
    ap.add_argument("--workload", default=WORKLOAD)
    ap.add_argument("--scale", type=float, default=1.0, help="linear resolution scale (tests only)")
    ap.add_argument("--omega", type=float, default=0.4)
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 comparison solve")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-tc", action="store_true", help="skip the tensor-core down-sweep comparison")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU oracle sample")
    ap.add_argument("--cpu-scale", type=float, default=0.25,
                    help="linear scale of the reduced model the CPU oracle is timed on")
    ap.add_argument("--cpu-threads", type=int, default=0, help="BLAS/OpenMP threads of the CPU oracle (0: all cores)")
    ap.add_argument("--no-cpu-config1", action="store_true",
                    help="skip the measured CPU solve of the 42 x 37 x 64 workload")
    # a real mesh instead of the synthetic workload: the reference's demo inputs
    # (data/<model>.ply, data/demo_BC_<model>_<res>_fixedNodes.dat / _loadingVec.dat)
    ap.add_argument("--mesh", default=None, help="ASCII .ply triangle mesh (CreateVoxilizedModel input)")
    ap.add_argument("--res", type=int, default=512, help="finestResolutionControl_ for --mesh")
    ap.add_argument("--fixed", default=None, help="fixingCond_ file (node ids) for --mesh")
    ap.add_argument("--loads", default=None, help="loadingCond_ file (id fx fy fz rows) for --mesh")
    ap.add_argument("--published-s", type=float, default=None,
                    help="published seconds for this model (vs_baseline = value / published)")
    return ap.parse_args()


# --------------------------------------------------------------------------
# clocks during the timed region
# --------------------------------------------------------------------------
class ClockSampler:
    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={CLOCK_FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        rows = []
        try:
            for line in open(self.path):
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9 and parts[1].replace(".", "").isdigit():
                    rows.append(parts)
        except OSError:
            pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[1]) for r in rows]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in rows for n, v in zip(names, r[5:9]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": float(rows[0][2]), "reasons": reasons,
                "samples": len(rows), "power_w_max": max(float(r[3]) for r in rows if r[3].replace(".", "").isdigit())}


# --------------------------------------------------------------------------
# CPU oracle (the reference's algorithm restated in NumPy) in a child process
# --------------------------------------------------------------------------
# Two modes.  "iters": set up a reduced model of the workload once (timed, with
# the coarsest factorisation timed on its own), then time `n` single PCG
# iterations from x = 0 (CG_solver.m's loop body: Jacobi step, V-cycle, K p,
# the vector updates).  "full": set up and solve a workload to tolerance and
# save U for the GPU comparison.  The child's BLAS and OpenMP thread counts are
# set from the parent (--cpu-threads, default every host core) and reported.
CPU_WORKER = r"""
import json, os, sys, time
cfg = json.loads(sys.argv[2])
sys.path[:0] = [sys.argv[1] + '/gmgs-3d_gb300', sys.argv[1] + '/oracle']
import numpy as np
from gmgs import synthetic
from gmgs_oracle import Oracle, Params
w = synthetic.WORKLOADS[cfg["workload"]]
scale = cfg["scale"]
nelx, nely, nelz = (max(2, int(round(n * scale))) for n in (w.nelx, w.nely, w.nelz))
if scale == 1.0:
    voids, L = w.voids, synthetic.level_count(nely, nelx, nelz, w.num_levels)
else:
    # the void volume fraction is kept; dropping one level per halving keeps
    # the coarsest level (and its dense factorisation) the size of the full model's
    voids = max(1, round(w.voids * scale ** 3))
    L = max(2, synthetic.level_count(w.nely, w.nelx, w.nelz, w.num_levels) - int(round(-np.log2(scale))))
vox = synthetic.sphere_voids(nelx, nely, nelz, voids, w.seed)
fixed, loads = synthetic.boundary_conditions(vox, L)
t0 = time.perf_counter()
o = Oracle(vox, Params(omega=cfg["omega"], num_levels=L, tol=w.tol))
o.apply_boundary_condition(fixed, loads)
if w.rho_range is not None and cfg.get("density", True):
    o.set_density(synthetic.density(int(vox.sum()), w.rho_range, w.seed), w.penal)
t_fact = [0.0]
_fact = o._factorize_coarsest
def _timed_fact():
    t = time.perf_counter(); _fact(); t_fact[0] += time.perf_counter() - t
o._factorize_coarsest = _timed_fact
o.setup()
t1 = time.perf_counter()
out = {"dofs": int(o.levels[0].numDOFs), "setup_s": t1 - t0, "coarsest_factor_s": t_fact[0],
       "shape": list(vox.shape), "voids": voids, "levels": L,
       "threads": {k: os.environ.get(k) for k in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS")}}
try:
    from threadpoolctl import threadpool_info
    out["blas_threads"] = [i.get("num_threads") for i in threadpool_info() if i.get("user_api") == "blas"]
except ImportError:
    pass
if cfg["mode"] == "iters":
    times = []
    with np.errstate(all='ignore'):
        for _ in range(cfg["n"]):
            t = time.perf_counter()
            o.cg(o.F, max_it=0)              # one iteration of the loop from x = 0
            times.append(time.perf_counter() - t)
    out["iter_times_s"] = times
else:
    u = o.get_deformation()
    t2 = time.perf_counter()
    out.update({"solve_s": t2 - t1, "iterations": int(o.iterations), "relres": float(o.relres)})
    np.save(cfg["u_path"], u)
print(json.dumps(out))
"""


def cpu_threads(a) -> int:
    return a.cpu_threads or os.cpu_count() or 1


def cpu_worker(cfg: dict, threads: int, timeout: float = 1200) -> dict:
    env = dict(os.environ)
    for k in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS"):
        env[k] = str(threads)
    res = subprocess.run([sys.executable, "-c", CPU_WORKER, str(ROOT), json.dumps(cfg)], capture_output=True,
                         text=True, timeout=timeout, env=env)
    if res.returncode != 0:
        raise RuntimeError(res.stderr[-2000:])
    return json.loads(res.stdout.strip().splitlines()[-1])


def cpu_extrapolate(sample: dict, iter_s: float, dofs_full: int, its_full: int) -> float:
    """Seconds for the full solve from a reduced-model sample: the per-iteration
    time and the setup without the coarsest factorisation scale with the DOF
    count; the coarsest factorisation is the same size in the sample (one level
    fewer per halving) and is counted once."""
    ratio = dofs_full / sample["dofs"]
    setup = (sample["setup_s"] - sample["coarsest_factor_s"]) * ratio + sample["coarsest_factor_s"]
    return setup + iter_s * its_full * ratio


# --------------------------------------------------------------------------
def max_over_ranks(value: float, device: str = "cpu") -> float:
    """The slowest rank's value (the job finishes when its last replica does)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return value
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def run_reference(a):
    """The reference's CPU path (the NumPy oracle port; MATLAB cannot run
    here) on the host cores.  The full workload would take about two hours on
    the CPU, so every step is one measured PCG iteration of a reduced model of
    the same generator (a quarter of the resolution, two levels fewer: the same
    coarsest level), set up once beforehand.  `value` is the full solve
    extrapolated from those measurements and is labelled as such; the measured
    figures are reported beside it."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    import numpy as np
    from gmgs import synthetic
    vox, fixed, loads, L, _ = synthetic.make(a.workload, scale=a.scale)
    # DOFs of the full workload, from the node mask of the padded grid
    nely, nelx, nelz = vox.shape
    pad = synthetic.padded_shape(nely, nelx, nelz, L)
    p = np.zeros(pad, np.int32)
    p[:nely, :nelx, :nelz] = vox
    dofs_full = 3 * int(synthetic.solid_node_mask(p).sum())
    its_full = int(os.environ.get("GMGS_REF_ITERS", "0")) or REF_ITERATIONS.get(a.workload, 60)
    threads = cpu_threads(a)
    smp = cpu_worker({"mode": "iters", "workload": a.workload, "scale": a.cpu_scale, "omega": a.omega,
                      "n": a.warmup + a.steps}, threads)
    iter_times = smp["iter_times_s"][a.warmup:]
    iter_s = statistics.median(iter_times)
    v = cpu_extrapolate(smp, iter_s, dofs_full, its_full)
    sample = (f"NumPy oracle ({threads} BLAS/OpenMP threads): {a.steps} timed PCG iterations from x = 0 on the same "
              f"generator at {smp['shape']} (y, x, z; {smp['voids']} voids, {smp['levels']} levels, {smp['dofs']} DOFs), "
              f"median {iter_s:.3f} s per iteration; setup {smp['setup_s']:.2f} s of which the coarsest factorisation "
              f"{smp['coarsest_factor_s']:.2f} s; extrapolated to {dofs_full} DOFs and {its_full} iterations")
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "s", "n_gpus": a.gpus, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": v * 1e3, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": a.workload, "dofs": dofs_full, "levels": L, "omega": a.omega, "tol": 1e-3},
        "extrapolated": True,
        "measured": {"sample_dofs": smp["dofs"], "sample_shape_y_x_z": smp["shape"], "sample_levels": smp["levels"],
                     "iteration_s_median": iter_s, "iteration_s": iter_times, "setup_s": smp["setup_s"],
                     "coarsest_factor_s": smp["coarsest_factor_s"], "threads": threads,
                     "thread_env": smp["threads"], "blas_threads": smp.get("blas_threads"),
                     "timed_s": float(sum(iter_times))},
        "cpu_baseline": {"value": v, "unit": "s", "cores": threads, "kind": "port", "extrapolated": True,
                         "sample": sample},
        "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def pinned_like(arr):
    """A copy of `arr` (same shape, dtype and memory order) in pinned host memory."""
    import numpy as np
    import torch

    arr = np.asarray(arr)
    flat = torch.empty(arr.size, dtype=torch.from_numpy(np.zeros(1, arr.dtype)).dtype, pin_memory=True).numpy()
    order = "F" if arr.flags.f_contiguous and not arr.flags.c_contiguous else "C"
    out = flat.reshape(arr.shape, order=order)
    out[...] = arr
    return out


def config1_comparison(a, threads: int, stream) -> dict:
    """The 42 x 37 x 64 workload (20 voids, 4 levels) solved to tolerance by
    the CPU oracle on the host cores (measured, not extrapolated) and by the
    GPU in both precisions on the same inputs, with the GPU displacements'
    error against the oracle's."""
    import numpy as np
    import torch
    from gmgs import Solver, synthetic

    name = "block42_fp64"
    fd, u_path = tempfile.mkstemp(suffix=".npy")
    os.close(fd)
    try:
        ref = cpu_worker({"mode": "full", "workload": name, "scale": 1.0, "omega": a.omega, "u_path": u_path},
                         threads)
        u_ref = np.load(u_path)
    finally:
        os.unlink(u_path)
    vox, fixed, loads, L, _ = synthetic.make(name)
    out = {"workload": name, "dofs": ref["dofs"], "levels": ref["levels"], "cpu_threads": threads,
           "cpu_setup_s": ref["setup_s"], "cpu_solve_s": ref["solve_s"], "cpu_total_s": ref["setup_s"] + ref["solve_s"],
           "cpu_iterations": ref["iterations"], "cpu_relres": ref["relres"], "thread_env": ref["threads"],
           "blas_threads": ref.get("blas_threads")}
    for prec in ("fp64", "mixed"):
        s = Solver(vox, omega=a.omega, num_levels=L, tol=1e-3, precision=prec)
        s.set_stream(stream.cuda_stream)
        s.set_bc(fixed, loads)
        u = s.solve()
        for _ in range(2):
            s.solve_dev(None)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(5):
            s.solve_dev(None)
        e1.record(stream)
        torch.cuda.synchronize()
        out[f"gpu_{prec}_solve_s"] = e0.elapsed_time(e1) / 5 / 1e3
        out[f"gpu_{prec}_iterations"] = s.iterations
        out[f"gpu_{prec}_displacement_rel_err_vs_cpu"] = float(np.linalg.norm(u - u_ref) / np.linalg.norm(u_ref))
        s.close()
    out["speedup_cpu_solve_vs_gpu_mixed"] = out["cpu_solve_s"] / out["gpu_mixed_solve_s"]
    return out


def run_gmgs(a):
    import numpy as np
    import torch

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    from gmgs import Solver, synthetic

    w = synthetic.WORKLOADS[a.workload]
    t0 = time.perf_counter()
    vox, fixed, loads, L, rho = synthetic.make(a.workload, scale=a.scale)
    t_gen = time.perf_counter() - t0

    stream = torch.cuda.Stream()
    s = Solver(vox, omega=a.omega, num_levels=L, tol=w.tol, precision="mixed")
    s.set_stream(stream.cuda_stream)
    s.set_bc(fixed, loads)
    if rho is not None:
        s.set_density(rho, 3.0)
    nn = s.num_nodes(1)
    dofs = 3 * nn

    def timed(solver, k):
        solver.set_profiling(True)
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(k):
            solver.solve_dev(None)
        e1.record(stream)
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()
        return e0.elapsed_time(e1) / k

    for _ in range(a.warmup):
        s.solve_dev(None)
    l0 = s.launch_count
    with ClockSampler(local) as clk:
        ms = timed(s, a.steps)
    launches = s.launch_count - l0
    its = s.iterations
    relres = s.relres
    nl, mv_ms, mv_bytes = s.kernel_time(3)    # finest CG update + Jacobi: the largest share of the launch list
    phase_names = {1: "vcycle", 2: "cg_iteration", 3: "fine_update_jacobi", 4: "fine_vcycle_down",
                   5: "fine_direction", 6: "fine_prolong_post", 7: "coarse_levels"}
    breakdown = {}
    for k, name in phase_names.items():
        n_k, ms_k, b_k = s.kernel_time(k)
        breakdown[name] = {"launches": n_k, "ms_per_solve": ms_k / a.steps,
                           "ms_per_launch": ms_k / max(n_k, 1),
                           "gbs": (b_k / (ms_k / 1e3) / 1e9) if (b_k and ms_k) else None}
    if ws > 1:
        ms = max_over_ranks(ms, "cuda")

    out = {}
    if rank == 0 and not a.no_tc:
        # the V-cycle down-sweep on the tensor cores (element form, tcgen05 kind::tf32;
        # GMGS_TC=1) on the same handle, against the CUDA-core second-difference kernel
        # timed above; the outer CG's kernels are the same in both
        import numpy as np
        u_cc = s.solve()
        os.environ["GMGS_TC"] = "1"
        try:
            s.solve_dev(None)
            ms_tc = timed(s, max(2, a.steps // 2))
            n_tc, t_tc, _ = s.kernel_time(4)
            u_tc = s.solve()
            its_tc = s.iterations
        finally:
            os.environ.pop("GMGS_TC", None)
        out["tensor_core_downsweep"] = {
            "kernel": "k_tc_vdown (tcgen05 kind::tf32, warp-specialized, element form)",
            "finest_downsweep_ms_per_launch": t_tc / max(n_tc, 1),
            "cuda_core_downsweep_ms_per_launch": breakdown["fine_vcycle_down"]["ms_per_launch"],
            "solve_s": ms_tc / 1e3, "iterations": its_tc,
            "displacement_rel_diff_vs_cuda_core": float(np.linalg.norm(u_tc - u_cc) / np.linalg.norm(u_cc))}
    if rank == 0:
        # stress recovery on the solved state: nodal (f64) + per-voxel (6 f32)
        s.solve_dev(None)
        ne = s.num_elements(1)
        nod = torch.empty((nn, 6), dtype=torch.float64, device="cuda")
        vox6 = torch.empty((ne, 6), dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        s.stress_dev(nod.data_ptr(), vox6.data_ptr())      # warm-up
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        s.stress_dev(nod.data_ptr(), vox6.data_ptr())
        ev1.record(stream)
        torch.cuda.synchronize()
        st_ms = ev0.elapsed_time(ev1)
        st_bytes = nn * (24 + 48) + ne * 24
        out["stress"] = {"ms": st_ms, "algorithmic_bytes": st_bytes, "gbs": st_bytes / (st_ms / 1e3) / 1e9}
        del nod, vox6
    if rho is not None and rank == 0:
        # adjoint: compliance gradient (no extra solve) and the z-displacement of
        # the first loaded node (one adjoint PCG solve), both on the solved state
        s.solve_dev(None)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        g = s.grad()
        t_c = time.perf_counter() - t0
        ell = np.zeros(dofs)
        ell[3 * (int(loads[0, 0]) - 1) + 2] = 1.0
        t0 = time.perf_counter()
        s.grad(ell)
        t_t = time.perf_counter() - t0
        out["adjoint"] = {"compliance_grad_s": t_c, "tip_grad_s_incl_adjoint_solve": t_t,
                          "adjoint_iterations": s.iterations, "grad_max_abs": float(np.abs(g).max()),
                          "grad_all_nonpositive": bool(np.all(g <= 0))}
    mem_now, mem_peak = Solver.memory_stats()
    out["memory"] = {"held_bytes": mem_now, "peak_bytes": mem_peak}
    if rank == 0 and not a.no_fp64:
        u_mixed = s.solve()
        sig_mixed = s.stress(per_voxel=False)
        s64 = Solver(vox, omega=a.omega, num_levels=L, tol=w.tol, precision="fp64")
        s64.set_stream(stream.cuda_stream)
        s64.set_bc(fixed, loads)
        if rho is not None:
            s64.set_density(rho, 3.0)
        ms64 = timed(s64, 1)
        u64 = s64.solve()
        sig64 = s64.stress(per_voxel=False)
        out["fp64"] = {"seconds": ms64 / 1e3, "iterations": s64.iterations, "relres": s64.relres,
                       "speedup_mixed_vs_fp64": ms64 / ms,
                       "displacement_rel_err_mixed_vs_fp64": float(np.linalg.norm(u_mixed - u64) / np.linalg.norm(u64)),
                       "displacement_max_err_mixed_vs_fp64": float(np.abs(u_mixed - u64).max() / np.abs(u64).max()),
                       "stress_rel_err_mixed_vs_fp64": float(np.linalg.norm(sig_mixed - sig64) / np.linalg.norm(sig64))}
        n64, ms64_mv, b64 = s64.kernel_time(0)
        out["fp64"]["fine_matvec_ms_per_launch"] = ms64_mv / max(n64, 1)
        s64.close()

    e2e = None
    if rank == 0 and not a.no_e2e:
        occ_bytes = vox.size * 4
        bc_bytes = fixed.size * 4 + loads.size * 8 + (rho.size * 8 if rho is not None else 0)
        # the step's inputs and its result live in pinned host memory (allocated
        # once, outside the timed region): the occupancy in the reference's
        # int32 column-major layout and the displacement output buffer
        vox_pin = pinned_like(np.asfortranarray(vox, dtype=np.int32))
        rho_pin = pinned_like(rho) if rho is not None else None
        u_pin = None
        times = []
        for i in range(2):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            se = Solver(vox_pin, omega=a.omega, num_levels=L, tol=w.tol, precision="mixed")
            t1 = time.perf_counter()
            se.set_bc(fixed, loads)
            if rho_pin is not None:
                se.set_density(rho_pin, 3.0)
            t2 = time.perf_counter()
            if u_pin is None:
                u_pin = torch.empty(3 * se.num_nodes(1), dtype=torch.float64, pin_memory=True).numpy()
            u = se.solve(out=u_pin)
            torch.cuda.synchronize()
            t3 = time.perf_counter()
            times.append(t3 - t0)
            phases = se.phase_times_ms
            phases.update({"call_create_ms": (t1 - t0) * 1e3, "call_set_bc_ms": (t2 - t1) * 1e3,
                           "call_solve_ms": (t3 - t2) * 1e3})
            se.close()
        e2e = {"value": times[-1], "unit": "s", "h2d_bytes_per_step": int(occ_bytes + bc_bytes),
               "d2h_bytes_per_step": int(u.nbytes), "phases_ms": phases}

    cpu = None
    cpu_config1 = None
    if rank == 0 and not a.no_cpu:
        threads = cpu_threads(a)
        smp = cpu_worker({"mode": "iters", "workload": a.workload, "scale": a.cpu_scale, "omega": a.omega, "n": 3},
                         threads)
        iter_s = statistics.median(smp["iter_times_s"][1:])
        v = cpu_extrapolate(smp, iter_s, dofs, its)
        cpu = {"value": v, "unit": "s", "cores": threads, "kind": "port", "extrapolated": True,
               "sample": f"NumPy oracle ({threads} BLAS/OpenMP threads): setup {smp['setup_s']:.2f} s (coarsest "
                         f"factorisation {smp['coarsest_factor_s']:.2f} s) + 2 timed PCG iterations "
                         f"({iter_s:.3f} s each) on the same generator at {smp['shape']} (y, x, z; {smp['levels']} "
                         f"levels, {smp['dofs']} DOFs), extrapolated to {dofs} DOFs and {its} iterations",
               "measured": {"sample_dofs": smp["dofs"], "iteration_s": iter_s, "setup_s": smp["setup_s"],
                            "coarsest_factor_s": smp["coarsest_factor_s"], "thread_env": smp["threads"],
                            "blas_threads": smp.get("blas_threads")}}
        if not a.no_cpu_config1:
            cpu_config1 = config1_comparison(a, threads, stream)

    if rank != 0:
        return
    peaks = {}
    try:
        peaks = json.load(open(ROOT / "MEASURED_PEAKS.json"))
    except OSError:
        pass
    hbm = peaks.get("hbm_gbs")
    peak_note = "measured" if hbm else "fallback"
    hbm = hbm or 6800.0
    achieved = mv_bytes / (mv_ms / 1e3) / 1e9 if mv_ms > 0 else None
    line = {
        "metric": METRIC, "value": ms / 1e3, "unit": "s", "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": ms, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 V-cycle; x, r double-f32; dots f32 products, f64 sums; f64 coarsest solve", "data": "synthetic",
        "config": {"workload": a.workload, "resolution": [w.nelx, w.nely, w.nelz], "voids": w.voids,
                   "levels": L, "padded": list(s.padded_dims), "dofs": dofs, "omega": a.omega, "tol": w.tol,
                   "iterations": its, "relres": relres, "l2": "inputs larger than L2 (no flush)",
                   "parallelism": "replicas" if ws > 1 else "single GPU"},
        "dof_iterations_per_s": dofs * its / (ms / 1e3),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm if achieved else None,
                     "traffic": UJ_TRAFFIC_PER_NODE * nn if UJ_TRAFFIC_PER_NODE else None,
                     "kernel": "k_fine<FM_CG_UPDATE_JACOBI> (finest CG update + Jacobi step + K dx)",
                     "algorithmic_bytes_per_node": (mv_bytes / max(nl, 1) / nn) if nl else None, "launches_timed": nl,
                     "ms_per_launch": mv_ms / max(nl, 1), "peak_source": peak_note},
        "gpu_launches": launches,
        "breakdown": breakdown,
        "clocks": clk.summary(),
        "cpu_baseline": cpu,
        "cpu_config1": cpu_config1,
        "e2e": e2e,
        "device_bytes": s.device_bytes,
        "generate_s": t_gen,
    }
    line.update(out)
    print(json.dumps(line))
    s.close()


def run_mesh(a):
    """The reference's own demo flow (Demo.m:67-77) on one GPU: voxelise the
    mesh, discretise, apply the demo boundary conditions, solve to tol 1e-3
    with the reference's default controls (omega 0.4, the level rule), in the
    mixed and the FP64 path.  `value` is the mixed solve on device-resident
    data; `e2e` runs from the host mesh and boundary-condition arrays to U on
    the host."""
    import numpy as np
    import torch
    from gmgs import Solver, mesh as M

    v, f = M.read_ply(a.mesh)
    fixed = np.loadtxt(a.fixed, ndmin=1).astype(np.int32)
    loads = np.loadtxt(a.loads, ndmin=2)
    stream = torch.cuda.Stream()
    res = {}
    u_pin = None
    for prec in ("mixed", "fp64"):
        if prec == "mixed":
            # one untimed pass of the whole flow sizes the pinned output buffer
            vol, ele = M.voxelize(v, f, a.res)
            s = Solver(vol, ele_size=ele, precision=prec)
            s.set_bc(fixed, loads)
            u_pin = torch.empty(3 * s.num_nodes(1), dtype=torch.float64, pin_memory=True).numpy()
            s.solve(out=u_pin)
            s.close()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        vol, ele = M.voxelize(v, f, a.res)
        t1 = time.perf_counter()
        s = Solver(vol, ele_size=ele, precision=prec)
        s.set_bc(fixed, loads)
        u = s.solve(out=u_pin if prec == "mixed" else None)
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        s.set_stream(stream.cuda_stream)
        k = a.steps if prec == "mixed" else 1
        for _ in range(a.warmup if prec == "mixed" else 0):
            s.solve_dev(None)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        with ClockSampler(0) as clk:
            e0.record(stream)
            for _ in range(k):
                s.solve_dev(None)
            e1.record(stream)
            torch.cuda.synchronize()
        res[prec] = {"solve_s": e0.elapsed_time(e1) / k / 1e3, "e2e_s": t2 - t0, "voxelize_s": t1 - t0,
                     "iterations": s.iterations, "relres": s.relres, "u": u, "dofs": 3 * s.num_nodes(1),
                     "levels": s.num_levels, "phases_ms": s.phase_times_ms, "device_bytes": s.device_bytes,
                     "clocks": clk.summary(), "grid": list(vol.shape)}
        s.close()
    mx, fp = res["mixed"], res["fp64"]
    err = float(np.linalg.norm(mx["u"] - fp["u"]) / np.linalg.norm(fp["u"]))
    line = {
        "metric": METRIC + " (reference demo mesh)", "value": mx["solve_s"], "unit": "s", "n_gpus": 1,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": mx["solve_s"] * 1e3, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": (mx["solve_s"] / a.published_s) if a.published_s else None,
        "dtype": "f32 V-cycle; x, r double-f32; dots f32 products, f64 sums; f64 coarsest solve", "data": f"mesh {Path(a.mesh).name} with its demo boundary conditions",
        "config": {"workload": f"{Path(a.mesh).stem}_{a.res}", "grid_ny_nx_nz": mx["grid"], "dofs": mx["dofs"],
                   "levels": mx["levels"], "omega": 0.4, "tol": 1e-3, "iterations": mx["iterations"],
                   "relres": mx["relres"], "published_s": a.published_s},
        "e2e": {"value": mx["e2e_s"], "unit": "s", "voxelize_s": mx["voxelize_s"], "phases_ms": mx["phases_ms"]},
        "fp64": {"seconds": fp["solve_s"], "e2e_s": fp["e2e_s"], "iterations": fp["iterations"],
                 "relres": fp["relres"], "speedup_mixed_vs_fp64": fp["solve_s"] / mx["solve_s"],
                 "displacement_rel_err_mixed_vs_fp64": err},
        "clocks": mx["clocks"], "device_bytes": mx["device_bytes"],
    }
    print(json.dumps(line))


def main():
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    elif a.mesh:
        run_mesh(a)
    else:
        run_gmgs(a)


if __name__ == "__main__":
    main()
