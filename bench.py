"""Benchmark: DOF-stage updates per second of the semi-discrete residual.

Default workload (the headline line): 3-D Euler Taylor-Green, 16^3 x 6 =
24,576 curved tetrahedra, ModalTensor(4), FluxDifferencingForm with the
entropy-conservative volume flux and Lax-Friedrichs interface dissipation,
CarpenterKennedy2N54.  The line also carries the mixed FP32/FP64 form on the
same handle, the discrete adjoint (cost against the forward) and the 2-D
vortex gradient check.  ``--workload`` selects the other configurations:
``advection_tri`` (512 triangles, StandardForm, RK4), ``vortex_tri`` (8,192
triangles, FD + LF), ``tgv_p5`` (82,944 tets at p = 5, mixed forward plus the
adjoint of the kinetic energy over 200 stages).

One step = one Runge-Kutta time step (5 residual evaluations and stage
updates for CarpenterKennedy2N54, 4 for RK4) on the whole mesh; DOF =
N_p * N_c * N_e (get_dof).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload tgv_p4|advection_tri|vortex_tri|tgv_p5]

``--impl reference`` times the reference's residual restated in C (OpenMP
over elements on all host cores, the reference's ``Threaded()`` strategy)
on the same workload; Julia is not available to run the reference itself.
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

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import __graft_entry__  # noqa: E402

METRIC = "DOF-stage updates/s, 3D Euler p4 tets, FP64 vs mixed at fixed err; adj/fwd cost"
UNIT = "DOF-stage updates/s"

WORKLOADS = {
    "tgv_p4": {
        "workload": "3-D Euler Taylor-Green vortex, Mach 0.1, periodic [0,2pi]^3",
        "mesh": "16^3 hexahedra x 6 = 24576 curved tetrahedra (Chan warp 0.05)",
        "approximation": "ModalTensor(4) on Tet, N_p=35, N_q=125, N_f=100",
        "form": "FluxDifferencingForm, entropy-conservative (Ranocha) volume flux + Lax-Friedrichs",
        "metrics": "ChanWilcox (conservative curl)",
        "time_integrator": "CarpenterKennedy2N54 (5 stages per step)",
        "l2_policy": "inputs larger than L2: metric terms and states ~0.7 GB read per stage"},
    "advection_tri": {
        "workload": "2-D linear advection, velocity (1,1), sine initial data, periodic [0,1]^2",
        "mesh": "16^2 quadrilaterals x 2 = 512 curved triangles (Chan warp 0.1)",
        "approximation": "ModalTensor(4) on Tri, N_p=15, N_q=25, N_f=15",
        "form": "StandardForm, Lax-Friedrichs",
        "metrics": "exact",
        "time_integrator": "RK4 (4 stages per step)",
        "l2_policy": "working set (~2 MB) is L2-resident: launch-latency bound, reported as is"},
    "vortex_tri": {
        "workload": "2-D Euler isentropic vortex (strength 5, free stream (1,1)), periodic [0,10]^2",
        "mesh": "64^2 quadrilaterals x 2 = 8192 curved triangles (Chan warp 0.1)",
        "approximation": "ModalTensor(4) on Tri, N_p=15, N_q=25, N_f=15",
        "form": "FluxDifferencingForm, entropy-conservative volume flux + Lax-Friedrichs",
        "metrics": "ChanWilcox (conservative curl)",
        "time_integrator": "CarpenterKennedy2N54 (5 stages per step)",
        "l2_policy": "working set ~40 MB fits in L2; reported as is"},
    "tgv_multi_p3": {
        "workload": "3-D Euler Taylor-Green vortex, Mach 0.1, periodic [0,2pi]^3",
        "mesh": "16^3 hexahedra x 6 = 24576 curved tetrahedra (Chan warp 0.05)",
        "approximation": "ModalMulti(3) on Tet (dense V, D, R; collapsed LG x LG x GJ(1,0) rules), "
                         "N_p=20, N_q=64, N_f=64",
        "form": "FluxDifferencingForm, entropy-conservative (Ranocha) volume flux + Lax-Friedrichs",
        "metrics": "ChanWilcox (conservative curl)",
        "time_integrator": "CarpenterKennedy2N54 (5 stages per step)",
        "l2_policy": "inputs larger than L2: metric terms and states ~0.5 GB read per stage"},
    "tgv_p5": {
        "workload": "3-D Euler Taylor-Green vortex, Mach 0.1, periodic [0,2pi]^3",
        "mesh": "24^3 hexahedra x 6 = 82944 curved tetrahedra (Chan warp 0.05)",
        "approximation": "ModalTensor(5) on Tet, N_p=56, N_q=216, N_f=144",
        "form": "FluxDifferencingForm, entropy-conservative (Ranocha) volume flux + Lax-Friedrichs",
        "metrics": "ChanWilcox (conservative curl)",
        "time_integrator": "CarpenterKennedy2N54 (5 stages per step)",
        "l2_policy": "inputs larger than L2: ~4 GB read per stage"},
}

# DRAM bytes (read + write) per element of one fd_time_derivative_kernel<3,5>
# / nodal_values_kernel<3,5> launch at p = 4, from ncu captures of the same
# kernels on the 8^3 x 6 = 3,072-tet case (145.7 MB and 37.9 MB per launch);
# reads scale with the element count
TRAFFIC_PER_ELEMENT = {"tgv_p4": {"B": 47_429, "A": 12_341}}


def env_rank():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), \
        int(os.environ.get("LOCAL_RANK", "0"))


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(prefix=f"clocks_rank{self.idx}_", suffix=".csv")
            self.f = os.fdopen(fd, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as fh:
            lines = fh.readlines()
        os.unlink(self.path)
        for line in lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def replica_time_ms(ms: float, world: int, device: str = "cuda") -> float:
    """Timed region of the slowest rank (replicas only: one independent
    solver per GPU, no exchange; the job's time is the maximum over ranks)."""
    if world == 1:
        return ms
    import torch
    import torch.distributed as dist
    t = torch.tensor([ms], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(dof: int, stages: int, steps: int, ms_max: float, world: int) -> float:
    """Whole-job DOF-stage updates per second: every rank advances its own
    copy of the workload (weak scaling)."""
    return world * dof * stages * steps / (ms_max * 1e-3)


def build_problem(workload: str, cells: int | None, p: int | None = None):
    pkg = __graft_entry__.load_package()
    s = pkg.setups
    if workload == "tgv_p4":
        pb = s.tgv_tet(cells=cells or 16, p=p or 4, lf=True)
    elif workload == "tgv_p5":
        pb = s.tgv_tet(cells=cells or 24, p=p or 5, lf=True)
    elif workload == "tgv_multi_p3":
        pb = s.tgv_tet(cells=cells or 16, p=p or 3, approx="ModalMulti", lf=True)
    elif workload == "vortex_tri":
        pb = s.vortex_tri(cells=cells or 64, p=p or 4)
    elif workload == "advection_tri":
        pb = s.advection_tri(cells=cells or 16, p=p or 4)
    else:
        raise KeyError(workload)
    return pkg, pb, pb.host_arrays()


def workload_config(args, host, world):
    cfg = dict(WORKLOADS[args.workload], dof=host.dof, elements=host.N_e,
               form_precision="FP64 (drop-in form)",
               parallelism="replicas only" if world > 1 else "1 GPU")
    if args.cells:
        cfg["mesh"] = f"{args.cells}^d cells (--cells override)"
    if args.p:
        cfg["approximation"] = f"degree {args.p} (--p override), N_p={host.N_p}, N_q={host.N_q}, N_f={host.N_f}"
    return cfg


def run_reference(args):
    rank, world, _ = env_rank()
    if rank != 0:
        return
    from oracle.oracle import Oracle
    pkg, pb, host = build_problem(args.workload, args.cells, args.p)
    o = Oracle(host)
    u = pb.u0.copy()
    for _ in range(args.warmup):
        u = o.rk_steps(u, 1, pb.dt, pb.scheme)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        u = o.rk_steps(u, 1, pb.dt, pb.scheme)
    dt = time.perf_counter() - t0
    value = host.dof * pb.stages_per_step * args.steps / dt
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(args, host, world), "impl": "reference",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": o.nthreads, "kind": "port",
                             "sample": f"{args.steps} full time steps on the whole mesh; reference "
                                       f"restated in C (OpenMP), not the Julia reference itself"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def cpu_baseline(pb, host, budget_s: float, nthreads: int | None = None):
    """The reference's residual restated in C, timed on the host cores with
    OpenMP over elements (the reference's Threaded() strategy), on all
    cores or on nthreads."""
    from oracle.oracle import Oracle
    o = Oracle(host, nthreads=nthreads)
    u = pb.u0
    o.residual(u)
    n, t0 = 0, time.perf_counter()
    while True:
        o.residual(u)
        n += 1
        if time.perf_counter() - t0 > budget_s:
            break
    t = (time.perf_counter() - t0) / n
    return {"value": host.dof / t, "unit": UNIT, "cores": o.nthreads, "kind": "port",
            "sample": f"{n} residual evaluations (one stage each) on the whole {host.N_e}-element "
                      f"mesh; reference restated in C with OpenMP over elements"}


def timed(stream, fn):
    """Device milliseconds of fn() by CUDA events on the launching stream."""
    import torch
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    out = fn()
    b.record(stream)
    torch.cuda.synchronize()
    return a.elapsed_time(b), out


def adjoint_workload(pkg, gpu, host, u0_np, dt, steps, fwd_ms, stream):
    """Pullback of the volume-averaged kinetic energy after `steps`
    CarpenterKennedy2N54 steps, w.r.t. the initial state (its momentum block
    is the gradient w.r.t. the initial velocity field), at two checkpoint
    intervals.  Cost relative to the plain forward of the same steps."""
    import torch
    out = {"objective": "volume-averaged kinetic energy at T, gradient w.r.t. the initial state",
           "steps": steps, "stages": 5 * steps, "forward_ms": fwd_ms}
    grads = {}
    # every = 0: segments sized from free HBM (here the whole trajectory, no
    # recomputation); every = 2: five segments, four recomputed
    for every, key in ((0, "memory_sized"), (2, "every_2_steps")):
        gpu.rk_record(torch.from_numpy(u0_np).cuda(), steps, dt, 0, every)   # warm-up / allocation
        u = torch.from_numpy(u0_np).cuda()
        rec_ms, _ = timed(stream, lambda: gpu.rk_record(u, steps, dt, 0, every))
        ke, dke = pkg.objectives.kinetic_energy(host, u.cpu().numpy())
        lamT = torch.from_numpy(dke).cuda()
        lam0 = torch.empty_like(lamT)
        adj_ms, info = timed(stream, lambda: gpu.rk_adjoint(lamT, lam0))
        grads[key] = lam0.cpu().numpy()
        out[key] = {"record_ms": rec_ms, "adjoint_ms": adj_ms,
                    "adjoint_over_forward": adj_ms / fwd_ms, "record_over_forward": rec_ms / fwd_ms,
                    "gradient_over_forward": (rec_ms + adj_ms) / fwd_ms,
                    "checkpoint_every_steps": info["checkpoint_every"], "segments": info["segments"],
                    "segments_recomputed": info["recomputed"], "recording_bytes": info["bytes"]}
        out["kinetic_energy_T"] = ke
    # the binomial (revolve) schedule with three checkpoints: a fraction of
    # the memory, more recomputation, the same gradient
    out["binomial_3_checkpoints"] = binomial_leg(pkg, gpu, host, u0_np, dt, steps, 3, fwd_ms, stream)
    grads["binomial"] = out["binomial_3_checkpoints"].pop("lam_0")
    g = grads["memory_sized"]
    out["grad_norm_momentum"] = float(np.linalg.norm(g[:, 1:-1]))
    out["gradients_identical_across_intervals"] = bool(np.array_equal(g, grads["every_2_steps"]))
    out["binomial_gradient_identical"] = bool(np.array_equal(g, grads["binomial"]))
    out["adjoint_over_forward"] = out["every_2_steps"]["adjoint_over_forward"]
    # the same pullback of a mixed-form recording (mixed-form VJP), against
    # the mixed forward of the same steps
    abi = pkg.abi
    try:
        gpu.set_precision(abi.SSE_MIXED)
        gpu.rk_steps(torch.from_numpy(u0_np).cuda(), 2, dt)                   # warm-up / graph capture
        mfwd_ms, _ = timed(stream, lambda: gpu.rk_steps(torch.from_numpy(u0_np).cuda(), steps, dt))
        gpu.rk_record(torch.from_numpy(u0_np).cuda(), steps, dt, 0, 0)        # warm-up / allocation
        u = torch.from_numpy(u0_np).cuda()
        rec_ms, _ = timed(stream, lambda: gpu.rk_record(u, steps, dt, 0, 0))
        ke, dke = pkg.objectives.kinetic_energy(host, u.cpu().numpy())
        lamT = torch.from_numpy(dke).cuda()
        lam0 = torch.empty_like(lamT)
        adj_ms, info = timed(stream, lambda: gpu.rk_adjoint(lamT, lam0))
        gm = lam0.cpu().numpy()
        out["mixed"] = {"forward_ms": mfwd_ms, "record_ms": rec_ms, "adjoint_ms": adj_ms,
                        "adjoint_over_forward": adj_ms / mfwd_ms,
                        "segments": info["segments"], "segments_recomputed": info["recomputed"],
                        "gradient_rel_err_vs_fp64_adjoint": float(np.linalg.norm(gm - g) / np.linalg.norm(g))}
    except pkg.SSEError as ex:
        out["mixed"] = {"unavailable": str(ex)}
    finally:
        gpu.set_precision(abi.SSE_FP64)
    return out


def binomial_leg(pkg, gpu, host, u0_np, dt, steps, n_checkpoints, fwd_ms, stream):
    """Kinetic-energy pullback recorded on the binomial schedule
    (sse_rk_record_binomial) with n_checkpoints checkpoints."""
    import torch
    gpu.rk_record_binomial(torch.from_numpy(u0_np).cuda(), min(steps, 2), dt, 0, n_checkpoints)  # warm-up
    u = torch.from_numpy(u0_np).cuda()
    rec_ms, _ = timed(stream, lambda: gpu.rk_record_binomial(u, steps, dt, 0, n_checkpoints))
    ke, dke = pkg.objectives.kinetic_energy(host, u.cpu().numpy())
    lamT = torch.from_numpy(dke).cuda()
    lam0 = torch.empty_like(lamT)
    adj_ms, info = timed(stream, lambda: gpu.rk_adjoint(lamT, lam0))
    extra, first = pkg.gb300.binomial_schedule(steps, n_checkpoints)
    return {"checkpoints": n_checkpoints, "record_ms": rec_ms, "adjoint_ms": adj_ms,
            "adjoint_over_forward": adj_ms / fwd_ms, "record_over_forward": rec_ms / fwd_ms,
            "steps_recomputed": info["recomputed"], "schedule_extra_steps": extra,
            "first_checkpoint_step": first, "recording_bytes": info["bytes"],
            "lam_0": lam0.cpu().numpy()}


def adjoint_mixed_workload(pkg, gpu, host, u0_np, dt, steps, stream):
    """Mixed-form forward plus the adjoint of the volume-averaged kinetic
    energy over `steps` CarpenterKennedy2N54 steps (checkpoints sized from
    free HBM), against the same pullback of an FP64 recording."""
    import torch
    abi = pkg.abi
    out = {"objective": "volume-averaged kinetic energy at T, gradient w.r.t. the initial velocity "
                        "(momentum block of the initial-state gradient)",
           "steps": steps, "stages": 5 * steps}
    grads = {}
    for prec, key in ((abi.SSE_MIXED, "mixed"), (abi.SSE_FP64, "fp64")):
        gpu.set_precision(prec)
        fwd_ms, _ = timed(stream, lambda: gpu.rk_steps(torch.from_numpy(u0_np).cuda(), steps, dt))
        u = torch.from_numpy(u0_np).cuda()
        rec_ms, _ = timed(stream, lambda: gpu.rk_record(u, steps, dt, 0, 0))
        ke, dke = pkg.objectives.kinetic_energy(host, u.cpu().numpy())
        lamT = torch.from_numpy(dke).cuda()
        lam0 = torch.empty_like(lamT)
        adj_ms, info = timed(stream, lambda: gpu.rk_adjoint(lamT, lam0))
        grads[key] = lam0.cpu().numpy()
        out[key] = {"forward_ms": fwd_ms, "forward_value": host.dof * 5 * steps / (fwd_ms * 1e-3),
                    "record_ms": rec_ms, "adjoint_ms": adj_ms,
                    "adjoint_over_forward": adj_ms / fwd_ms,
                    "checkpoint_every_steps": info["checkpoint_every"], "segments": info["segments"],
                    "segments_recomputed": info["recomputed"], "recording_bytes": info["bytes"],
                    "kinetic_energy_T": ke}
    gpu.set_precision(abi.SSE_FP64)
    # the FP64 pullback again on the binomial schedule with eight checkpoints
    # (a few GB instead of the uniform recording's block)
    out["fp64_binomial_8_checkpoints"] = binomial_leg(pkg, gpu, host, u0_np, dt, steps, 8,
                                                      out["fp64"]["forward_ms"], stream)
    gb = out["fp64_binomial_8_checkpoints"].pop("lam_0")
    out["fp64_binomial_8_checkpoints"]["gradient_identical_to_uniform"] = bool(np.array_equal(gb, grads["fp64"]))
    gm, g64 = grads["mixed"][:, 1:-1], grads["fp64"][:, 1:-1]
    out["gradient_rel_err_mixed_vs_fp64_adjoint"] = float(np.linalg.norm(gm - g64) / np.linalg.norm(g64))
    out["adjoint_over_forward"] = out["mixed"]["adjoint_over_forward"]
    return out


def adjoint_gradient_check(pkg, stream, n_dirs: int = 8):
    """2-D Euler vortex (64^2 x 2 = 8192 curved triangles, ModalTensor(4),
    FD + LF): J = 1/2 ||u(T) - u_target||^2_M after 400 CarpenterKennedy2N54
    stages, checkpoints every 20 stages; the adjoint gradient against
    central differences (step 1e-6) of J through the GPU forward along
    seeded unit directions."""
    import torch
    setups, obj = pkg.setups, pkg.objectives
    pb = setups.vortex_tri(cells=64, p=4)
    host = pb.host_arrays()
    tgt = setups.perturbed(setups.vortex_tri(cells=64, p=4, strength=5.5, shift=0.3).u0, 20261207, 1e-3)
    g = pkg.GB300Solver(host)
    g.set_stream(stream.cuda_stream)
    n_steps = 80
    u0 = torch.from_numpy(pb.u0).cuda()

    def J(x):
        x = x.clone()
        g.rk_steps(x, n_steps, pb.dt)
        return obj.mass_misfit(host, x.cpu().numpy(), tgt)[0]

    u = u0.clone()
    fwd_ms, _ = timed(stream, lambda: g.rk_steps(u.clone(), n_steps, pb.dt))
    g.rk_record(u0.clone(), n_steps, pb.dt, 0, 4)   # warm-up / allocation
    u = u0.clone()
    rec_ms, _ = timed(stream, lambda: g.rk_record(u, n_steps, pb.dt, 0, 4))
    Jv, dJ = obj.mass_misfit(host, u.cpu().numpy(), tgt)
    lamT = torch.from_numpy(dJ).cuda()
    lam0 = torch.empty_like(lamT)
    adj_ms, info = timed(stream, lambda: g.rk_adjoint(lamT, lam0))
    grad = lam0.cpu().numpy()
    rng = np.random.default_rng(20261204)
    errs = []
    for _ in range(n_dirs):
        v = rng.standard_normal(grad.shape)
        v /= np.linalg.norm(v)
        vd = torch.from_numpy(v).cuda()
        fd = (J(u0 + 1e-6 * vd) - J(u0 - 1e-6 * vd)) / 2e-6
        ad = float(np.vdot(grad, v))
        errs.append(abs(fd - ad) / max(abs(ad), 1e-300))
    return {"workload": "2-D Euler isentropic vortex, 8192 curved tris, ModalTensor(4), FD + LF, "
                        "400 CarpenterKennedy2N54 stages, checkpoints every 20 stages",
            "objective": "1/2 ||u(T) - u_target||^2_M, u_target = perturbed vortex (strength 5.5, "
                         "centre shifted by 0.3)",
            "J": Jv, "forward_ms": fwd_ms, "record_ms": rec_ms, "adjoint_ms": adj_ms,
            "adjoint_over_forward": adj_ms / fwd_ms, "segments": info["segments"],
            "segments_recomputed": info["recomputed"],
            "fd_directions": n_dirs, "fd_step": 1e-6,
            "fd_rel_err_max": max(errs), "fd_rel_err_median": float(np.median(errs))}


def geometry_workload(pkg, pb, fp64_peak):
    """GeometricFactors + project_jacobian! of the workload's mesh
    (mesh.jl:229-506, SpatialDiscretizations.jl:310-317): the host numpy
    restatement against sse_geometric_factors, whose FP64 kernel builds every
    element's metric terms in shared memory.  Device buffers: CUDA events
    around the whole call (operator upload, kernel, synchronisation); host
    buffers: wall clock including the copies of coordinates and results."""
    import torch
    sd = pb.sd
    mesh, ra, metrics = sd.mesh, sd.reference_approximation, sd.metrics
    project = metrics == "Exact"
    t0 = time.perf_counter()
    want = pkg.mesh.spatial_discretization(mesh, ra, metrics=metrics, project_jac=project).geometric_factors
    host_s = time.perf_counter() - t0
    xyz = [torch.from_numpy(x).cuda() for x in mesh.xyz]
    pkg.gb300.geometric_factors(mesh, ra, metrics, project, xyz=xyz)
    torch.cuda.synchronize()
    times = []
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        pkg.gb300.geometric_factors(mesh, ra, metrics, project, xyz=xyz)
        e1.record()
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    dev_ms = float(np.median(times))
    t0 = time.perf_counter()
    got = pkg.gb300.geometric_factors(mesh, ra, metrics, project)
    hostbuf_s = time.perf_counter() - t0
    err = max(float(np.abs(getattr(got, f) - getattr(want, f)).max() / np.abs(getattr(want, f)).max())
              for f in ("J_q", "Lambda_q", "J_f", "nJf", "nJq"))
    mo = pkg.mesh.metric_operators(ra, metrics, project)
    flops = pkg.flops_model.geometric_factors_flops(
        ra.d, metrics, mesh.xyz[0].shape[1], mo.Vq.shape[0], mo.Vf.shape[0], mo.num_faces,
        0 if mo.N_to_N1 is None else mo.N_to_N1.shape[0], project) * sd.N_e
    tflops = flops / (dev_ms * 1e-3) / 1e12
    kernel = ("curl_metrics_3d_kernel" if ra.d == 3 else "curl_metrics_2d_kernel") \
        if metrics != "Exact" else "exact_metrics_kernel"
    # project_function (initialize) on the same mesh: host numpy vs the GPU kernel
    ic = pb.initial_data
    uq = np.ascontiguousarray(ic.evaluate(mesh.xyzq, 0.0).transpose(0, 2, 1))
    t0 = time.perf_counter()
    u0_host = pkg.solver.initialize(ic, sd)
    init_host_s = time.perf_counter() - t0
    init = None
    if ra.V is not None:
        Jd, uqd = torch.from_numpy(sd.geometric_factors.J_q).cuda(), torch.from_numpy(uq).cuda()
        pkg.gb300.project_function(ra, Jd, uqd)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        u0_dev = pkg.gb300.project_function(ra, Jd, uqd)
        e1.record()
        torch.cuda.synchronize()
        init = {"host_numpy_s": init_host_s, "gpu_device_buffers_ms": e0.elapsed_time(e1),
                "max_rel_err_vs_host": float(np.abs(u0_dev.cpu().numpy() - u0_host).max() / np.abs(u0_host).max()),
                "note": "host time includes evaluating the initial data at the volume nodes"}
    return {"metrics": metrics, "project_jacobian": project, "elements": sd.N_e, "initialize": init,
            "host_numpy_s": host_s, "gpu_device_buffers_ms": dev_ms,
            "gpu_host_buffers_ms": hostbuf_s * 1e3, "speedup_device_buffers": host_s / (dev_ms * 1e-3),
            "max_field_rel_err_vs_host": err,
            "roofline": {"kernel": kernel, "bound": "fp64", "achieved": tflops, "peak": fp64_peak,
                         "unit": "TFLOP/s", "frac": tflops / fp64_peak,
                         "algorithmic_flops_per_element": flops / sd.N_e}}


def rel2(got, want) -> float:
    return float(np.linalg.norm(got - want) / np.linalg.norm(want))


def e2e_drop_in(pkg, gpu, pb, host, steps, world):
    """The drop-in end to end: the Runge-Kutta loop on the host calling the
    residual through the C-ABI with pinned host buffers once per stage
    (sse_residual(..., SSE_HOST): H2D of u, both phases, D2H of dudt), the
    stage arithmetic in place on the host -- what OrdinaryDiffEq does with
    the ODEProblem of semidiscretize.  Wall-clock seconds over ``steps``."""
    import torch
    alg = "RK4" if pb.scheme == 1 else "CarpenterKennedy2N54"
    ode = pkg.gb300.ODEProblem(pkg.gb300.semi_discrete_residual, torch.from_numpy(pb.u0.copy()).pin_memory(),
                               (0.0, 1.0), gpu)
    pkg.timestepping.solve(ode, pb.dt, 1, alg)            # warm-up (pinned buffers, first launches)
    u = ode.u0.clone().pin_memory()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    pkg.timestepping.solve(ode, pb.dt, steps, alg, u=u)
    secs = time.perf_counter() - t0
    nbytes = host.dof * 8 * pb.stages_per_step
    return {"value": world * host.dof * pb.stages_per_step * steps / secs, "unit": UNIT,
            "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
            "call": f"{alg} on the host, sse_residual(u_host, dudt_host, SSE_HOST) once per stage, "
                    f"stage updates in place on pinned torch CPU tensors "
                    f"({torch.get_num_threads()} threads)",
            "steps": steps, "seconds": secs}


def vortex_exact_error(pkg, pb, states, T):
    """L2 error (ErrorAnalysis, volume quadrature, normalised by the domain
    volume) of each state against the isentropic vortex advected exactly by
    the free stream to time T (the reference's ``evaluate`` ignores t)."""
    ic = pb.initial_data
    exact = lambda x, t: ic.evaluate(x, t, translated=True)
    out = {"T": T, "norm": "sqrt(sum_k sum_q W J (u_exact - V u)^2 / |Omega|) per conserved variable"}
    for key, st in states.items():
        out[key] = [float(x) for x in pkg.timestepping.l2_error(pb.sd, st, exact, T, normalize=True)]
    out["l2_err_at_t0"] = [float(x) for x in pkg.timestepping.l2_error(pb.sd, pb.u0, exact, 0.0, normalize=True)]
    f, m = np.array(out["fp64"]), np.array(out["mixed"])
    out["mixed_minus_fp64_rel"] = float(np.abs(m - f).max() / np.abs(f).max())
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="tgv_p4", choices=sorted(WORKLOADS))
    ap.add_argument("--cells", type=int, default=None, help="override the mesh resolution")
    ap.add_argument("--p", type=int, default=None, help="override the polynomial degree")
    ap.add_argument("--cpu-budget", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-geometry", action="store_true")
    ap.add_argument("--adjoint-steps", type=int, default=40,
                    help="time steps of the tgv_p5 adjoint leg (40 = 200 stages)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)

    import torch
    rank, world, local = env_rank()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    pkg, pb, host = build_problem(args.workload, args.cells, args.p)
    pkg.build.build()
    gpu = pkg.GB300Solver(host)
    stream = torch.cuda.current_stream()
    gpu.set_stream(stream.cuda_stream)
    u = torch.from_numpy(pb.u0).cuda()
    dt, scheme, stages = pb.dt, pb.scheme, pb.stages_per_step
    fd = pkg.abi.SSE_FLUX_DIFFERENCING_FORM == host.cfg.form

    # ---- device-resident throughput (value): the K steps are one call, as a
    # time loop on the device runs them (one captured step replayed K times)
    gpu.rk_steps(u, args.warmup, dt, scheme)
    sampler = ClockSampler(local)
    sampler.start()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    gpu.rk_steps(u, args.steps, dt, scheme)
    ev1.record(stream)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks = sampler.stop()
    ms = replica_time_ms(ev0.elapsed_time(ev1), world)
    value = replica_value(host.dof, stages, args.steps, ms, world)

    # ---- per-kernel timings (CUDA events on the launching stream) and roofline
    phases = gpu.phase_timings(u, 5)
    work = pkg.flops_model.model(host)
    fp64_peak, fp32_peak = pkg.gb300.measure_fma_peaks()
    ne = host.N_e
    one_kernel = gpu.kernel_path() == pkg.abi.SSE_PATH_ONE_KERNEL
    dom = "B" if phases[1] >= phases[0] else "A"
    dom_ms = phases[1] if dom == "B" else phases[0]
    dom_flops = (work.flops_B if dom == "B" else work.flops_A) * ne
    dom_bytes = (work.bytes_B if dom == "B" else work.bytes_A) * ne
    if one_kernel:
        # one kernel evaluates the whole residual: both phases' algorithmic work
        dom_flops = work.flops * ne
        dom_bytes = pkg.flops_model.one_kernel_bytes(host) * ne
    achieved = dom_flops / (dom_ms * 1e-3) / 1e12
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) \
        if os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    kernel_B = "fd_time_derivative_kernel" if fd else (
        "std_compact_kernel" if one_kernel else "std_time_derivative_kernel")
    traffic = TRAFFIC_PER_ELEMENT.get(args.workload) if not (args.cells or args.p) else None
    roofline = {"bound": "fp64", "achieved": achieved, "peak": fp64_peak, "unit": "TFLOP/s",
                "frac": achieved / fp64_peak,
                "kernel": kernel_B if dom == "B" else "nodal_values_kernel",
                "peak_source": "measured live: FP64 FMA-chain microbenchmark on this GPU",
                "hbm_achieved_gbs": dom_bytes / (dom_ms * 1e-3) / 1e9,
                "hbm_frac_of_measured": dom_bytes / (dom_ms * 1e-3) / 1e9 / hbm_peak,
                "traffic": traffic[dom] * ne if traffic else None,
                "traffic_source": ("ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch on "
                                   "the 3,072-tet case, scaled by the element count") if traffic
                else "no ncu capture of this workload",
                "phase_ms": {"nodal_values": phases[0], "time_derivative": phases[1],
                             "rk_stage_update": phases[2]},
                "algorithmic_flops_per_element": {"nodal_values": work.flops_A,
                                                  "time_derivative": work.flops_B},
                "whole_stage_frac": (work.flops * ne) / ((phases[0] + phases[1]) * 1e-3) / 1e12 / fp64_peak,
                "kernel_path": "one kernel per residual and per stage (std_compact_kernel)" if one_kernel
                else "two phases (nodal values, time derivative)",
                "fp32_peak_tflops": fp32_peak}

    # ---- mixed FP32/FP64 form on the same handle: same steps from the same
    # initial state, error against the FP64 trajectory at equal step count
    abi = pkg.abi
    mixed = None
    exact_err = None
    try:
        gpu.set_precision(abi.SSE_MIXED)
        um = torch.from_numpy(pb.u0).cuda()
        torch.cuda.synchronize()
        gpu.rk_steps(um, args.warmup, dt, scheme)
        torch.cuda.synchronize()
        m0, m1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        m0.record(stream)
        gpu.rk_steps(um, args.steps, dt, scheme)
        m1.record(stream)
        torch.cuda.synchronize()
        mms = m0.elapsed_time(m1)
        mphases = gpu.phase_timings(um, 5)
        u0d = torch.from_numpy(pb.u0).cuda()
        torch.cuda.synchronize()
        r_mixed = gpu.residual(u0d).cpu().numpy()
        gpu.set_precision(abi.SSE_FP64)
        r_fp64 = gpu.residual(u0d).cpu().numpy()
        state_err = float(torch.linalg.norm(um - u) / torch.linalg.norm(u))
        res_err = float(np.linalg.norm(r_mixed - r_fp64) / np.linalg.norm(r_fp64))
        # the increment u(T) - u(0): a short run moves the state little, so
        # the state error alone would hide the error of the residual
        du64, dum = (u - u0d).cpu().numpy(), (um - u0d).cpu().numpy()
        inc_err = rel2(dum, du64)
        inc_comp = [rel2(dum[:, c], du64[:, c]) for c in range(host.N_c)]
        res_comp = [rel2(r_mixed[:, c], r_fp64[:, c]) for c in range(host.N_c)]
        if args.workload == "vortex_tri":
            exact_err = vortex_exact_error(pkg, pb, {"fp64": u.cpu().numpy(), "mixed": um.cpu().numpy()},
                                           (args.warmup + args.steps) * dt)
        cons = gpu.conservation_residual(u0d, torch.from_numpy(r_mixed).cuda())
        mvalue = world * host.dof * stages * args.steps / (mms * 1e-3)
        # roofline of the FP32 phase B: max(FP32 pipe, HBM) with the
        # algorithmic flops and the FP32 bytes (half the FP64 bytes)
        mB = mphases[1] * 1e-3
        m_fp32 = work.flops_B * ne / mB / 1e12
        m_hbm = 0.5 * work.bytes_B * ne / mB / 1e9
        mixed_roofline = {"kernel": "fd_time_derivative_mixed_kernel", "bound": "max(fp32, hbm)",
                          "fp32_achieved_tflops": m_fp32, "fp32_peak_tflops": fp32_peak,
                          "fp32_frac": m_fp32 / fp32_peak, "hbm_achieved_gbs": m_hbm,
                          "hbm_peak_gbs": hbm_peak, "hbm_frac": m_hbm / hbm_peak,
                          "frac": max(m_fp32 / fp32_peak, m_hbm / hbm_peak),
                          "note": "neither roof binds: latency (dependent FP32 chains, table loads)"}
        mixed = {"value": mvalue, "unit": UNIT, "ms_per_step": mms / args.steps, "roofline": mixed_roofline,
                 "speedup_vs_fp64": mvalue / value,
                 "state_rel_err_vs_fp64": state_err,
                 "state_err_after_steps": args.warmup + args.steps,
                 "increment_rel_err_vs_fp64": inc_err,
                 "increment_rel_err_per_variable": inc_comp,
                 "residual_rel_err_vs_fp64": res_err,
                 "residual_rel_err_per_variable": res_comp,
                 "conservation_residual_fp64_reduction": [float(x) for x in cons[: host.N_c]],
                 "entropy_production_fp64_reduction": float(cons[host.N_c]),
                 "phase_ms": {"nodal_values_fp32": mphases[0], "time_derivative_fp32": mphases[1],
                              "rk_stage_update_compensated": mphases[2]},
                 "precision": "entropy projection (V, entropy-variable maps, weight-adjusted projection, "
                              "R) FP32 on perturbations from a constant reference state, the projection "
                              "of the constant function FP64; fluxes, flux differencing, facet "
                              "correction, lifting and mass solve FP32 on perturbations; FP64 "
                              "compensated stage accumulation and reductions"}
        if exact_err is not None:
            mixed["exact_solution_error"] = exact_err
    except pkg.SSEError as ex:
        mixed = {"unavailable": str(ex)}
        gpu.set_precision(abi.SSE_FP64)

    # ---- discrete adjoint
    adjoint = None
    if not args.no_adjoint:
        if args.workload == "tgv_p4":
            adjoint = adjoint_workload(pkg, gpu, host, pb.u0, dt, args.steps, ms, stream)
            adjoint["gradient_check"] = adjoint_gradient_check(pkg, stream)
        elif args.workload == "tgv_p5":
            adjoint = adjoint_mixed_workload(pkg, gpu, host, pb.u0, dt, args.adjoint_steps, stream)

    geometry = None if args.no_geometry else geometry_workload(pkg, pb, fp64_peak)

    # ---- end to end through the C-ABI with host (pinned) buffers: the
    # drop-in as OrdinaryDiffEq drives it (sse_residual on host arrays once
    # per stage, stage arithmetic on the host), and beside it the fused
    # device time loop called with a host state once per step
    e2e_steps = max(2, args.steps // 2)
    e2e = e2e_drop_in(pkg, gpu, pb, host, e2e_steps, world)
    u_host = torch.from_numpy(pb.u0.copy()).pin_memory()
    gpu.rk_steps(u_host, 1, dt, scheme)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        gpu.rk_steps(u_host, 1, dt, scheme)   # H2D copy, all stages, D2H copy
    e2e_s = time.perf_counter() - t0
    nbytes = host.dof * 8
    e2e_fused = {"value": world * host.dof * stages * e2e_steps / e2e_s, "unit": UNIT,
                 "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
                 "call": "sse_rk_steps(u_host, 1 step) per step: one H2D and one D2H of the state "
                         "per step, every stage on the device"}

    # per stage: phase A, phase B and one stage-update kernel, or the one
    # kernel that evaluates the stage's residual and applies its update
    launches = args.steps * stages * (1 if one_kernel else 3)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(args, host, world),
            "clocks": clocks, "e2e": e2e, "e2e_fused_time_loop": e2e_fused,
            "gpu_launches": launches, "roofline": roofline,
            "mixed": mixed, "adjoint": adjoint, "geometric_factors": geometry}
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(pb, host, args.cpu_budget)
        line["cpu_baseline_1_core"] = cpu_baseline(pb, host, args.cpu_budget / 2, nthreads=1)
    if rank == 0:
        print(json.dumps(line))


if __name__ == "__main__":
    main()
