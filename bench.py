"""Benchmark: Jacobian-vector product throughput (GDOF/s) of the quasi-static
Neo-Hookean solid, 32x32x32 hexahedra, H1 Q2 vector (823,875 DOF), 3x3x3
Gauss points, FP64, interior vertices perturbed by U(-0.1h, 0.1h) (seed 1),
shear modulus 0.25, bulk modulus 5.0, linearised at load step 1 of the
z-compression (u_z = -0.005 z) plus a seeded perturbation.

One step = one Jacobian action over the whole mesh (sfx_jvp: fused element
kernel + deterministic node-owner scatter).  `value` is timed with CUDA events
around each step with the inputs resident in HBM and the L2 flushed between
steps; `e2e` runs the same call through the C ABI with the direction vector
copied from pinned host memory and the result copied back inside the timed
region.  `--impl reference` times the CPU path (serac's stored-derivative
Jacobian action, as restated by the oracle) on the host cores.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl sfx|reference]
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

METRIC = "Jv GDOF/s"
UNIT = "GDOF/s"
NX = 32
ORDER = 2
K_BULK, G_SHEAR = 5.0, 0.25
WORKLOAD = "neohookean_q2_vector_32cubed_jvp"


def config(n_gpus, flush):
    return {
        "workload": WORKLOAD,
        "mesh": f"{NX}x{NX}x{NX} hex, interior vertices perturbed +-0.1h (seed 1)",
        "space": "H1 Q2, 3 components, byNODES",
        "dofs": 3 * (ORDER * NX + 1) ** 3,
        "quadrature": "3x3x3 Gauss",
        "material": {"model": "NeoHookean", "K": K_BULK, "G": G_SHEAR},
        "linearisation": "u_z = -0.005 z + 1e-4 N(0,1) (seed 2)",
        "l2": flush,
        "parallelism": f"replicas x{n_gpus}" if n_gpus > 1 else "single GPU",
    }


def problem():
    from serac_gb300 import box_vertices

    V = box_vertices(NX, NX, NX, perturb=0.1, seed=1)
    return V


def linearisation_state(mesh):
    X = mesh.node_coordinates(ORDER)
    n = X.shape[0]
    u = np.zeros((3, n))
    u[2] = -0.005 * X[:, 2]
    u += 1e-4 * np.random.default_rng(2).standard_normal((3, n))
    return u.ravel()


# ------------------------------------------------------------------ clocks
class ClockSampler:
    def __init__(self):
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self, device_index=0):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9 or not parts[0].isdigit() or int(parts[0]) != device_index:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9]):
                if flag.lower() == "active":
                    reasons.add(name)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------ CPU baseline
def cpu_jvp_rate(V, seconds=10.0, threads=None, min_reps=1):
    """The oracle's stored-derivative Jacobian action (serac's
    action_of_gradient_kernel restated, sum-factorised) with gather and
    node-owner scatter in C, on all host cores.  Returns (GDOF/s, reps, threads, s)."""
    import ctypes

    from oracle import oracle as O

    threads = threads or os.cpu_count() or 1
    mesh = O.StructuredHexMesh(NX, NX, NX, V)
    lib = O.lib()
    dp = ctypes.POINTER(ctypes.c_double)
    i64p = ctypes.POINTER(ctypes.c_int64)
    lib.orc_linearize.argtypes = [ctypes.c_int] * 3 + [ctypes.c_double] + [dp] * 5 + [dp, ctypes.c_int]
    lib.orc_apply_linearization.argtypes = [ctypes.c_int] * 3 + [dp, dp, dp, ctypes.c_int]
    lib.orc_gather.argtypes = [ctypes.c_int64, ctypes.c_int, ctypes.c_int, ctypes.c_int64, i64p, dp, dp, ctypes.c_int]
    lib.orc_scatter.argtypes = [ctypes.c_int64, ctypes.c_int, ctypes.c_int, i64p, i64p, dp, dp, ctypes.c_int]
    conn = np.ascontiguousarray(mesh.elem_nodes(ORDER))
    nn = mesh.num_nodes(ORDER)
    npe = conn.shape[1]
    order = np.argsort(conn.ravel(), kind="stable")
    node_ent = np.ascontiguousarray(order.astype(np.int64))
    node_ptr = np.zeros(nn + 1, dtype=np.int64)
    np.add.at(node_ptr, conn.ravel() + 1, 1)
    node_ptr = np.cumsum(node_ptr)
    Xq, Jq = O.geometric_factors(mesh.elem_coords(), ORDER + 1)
    ndofs = 3 * nn
    ne = mesh.ne

    u = linearisation_state(_mesh_proxy(V))
    du = np.random.default_rng(0).standard_normal(ndofs)
    uE = np.zeros((ne, 3 * npe))
    lib.orc_gather(ne, npe, 3, nn, conn.ctypes.data_as(i64p), u.ctypes.data_as(dp), uE.ctypes.data_as(dp), threads)
    params = np.ascontiguousarray(np.tile([K_BULK, G_SHEAR], (ne, 1)))
    nq = (ORDER + 1) ** 3
    D = np.zeros((ne, nq, 12, 12))
    rc = lib.orc_linearize(O.MAT_NEOHOOKEAN, ORDER, ne, 0.0, params.ctypes.data_as(dp), uE.ctypes.data_as(dp),
                           Xq.ctypes.data_as(dp), Jq.ctypes.data_as(dp), None, D.ctypes.data_as(dp), threads)
    assert rc == 0
    duE = np.zeros_like(uE)
    dE = np.zeros_like(uE)
    out = np.zeros(ndofs)

    def one():
        lib.orc_gather(ne, npe, 3, nn, conn.ctypes.data_as(i64p), du.ctypes.data_as(dp), duE.ctypes.data_as(dp),
                       threads)
        lib.orc_apply_linearization(ORDER, 3, ne, D.ctypes.data_as(dp), duE.ctypes.data_as(dp),
                                    dE.ctypes.data_as(dp), threads)
        lib.orc_scatter(nn, npe, 3, node_ptr.ctypes.data_as(i64p), node_ent.ctypes.data_as(i64p),
                        dE.ctypes.data_as(dp), out.ctypes.data_as(dp), threads)

    one()
    reps = 0
    t0 = time.perf_counter()
    while True:
        one()
        reps += 1
        el = time.perf_counter() - t0
        if reps >= min_reps and el >= seconds:
            break
    return ndofs * reps / el / 1e9, reps, threads, el


class _mesh_proxy:
    """node_coordinates() of serac_gb300.Mesh without creating a device mesh."""

    def __init__(self, V):
        self.nx = self.ny = self.nz = NX
        self.vertices = V

    def node_coordinates(self, order):
        from serac_gb300.functional import Mesh

        return Mesh.node_coordinates(self, order)


# ----------------------------------------------------------------- GPU arm
def max_over_ranks(seconds, world, device):
    """The slowest rank's time (replicas run the same workload independently)."""
    if world <= 1:
        return seconds
    import torch

    t = torch.tensor([seconds], device=device, dtype=torch.float64)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(world, dofs, steps, seconds):
    """Whole-job GDOF/s: every replica applied the operator `steps` times to
    `dofs` unknowns in at most `seconds`."""
    return world * dofs * steps / seconds / 1e9


def run_sfx(args, rank, world):
    import torch

    import serac_gb300 as sg

    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    V = problem()
    mesh = sg.Mesh.structured_hex(NX, NX, NX, V)
    f = sg.Functional(mesh, sg.H1(ORDER, 3))
    f.AddDomainIntegral(sg.NEOHOOKEAN, [K_BULK, G_SHEAR])
    ndofs = f.ndofs
    u = torch.tensor(linearisation_state(mesh), device=dev)
    grad = f.linearize(0.0, u)
    du = torch.tensor(np.random.default_rng(0).standard_normal(ndofs), device=dev)
    dr = torch.empty_like(du)
    du32 = du.float()
    dr32 = torch.empty_like(du32)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream()

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    for _ in range(args.warmup):
        if not (args.kernels_only and args.precision == "f32"):
            grad.mult(du, dr)
        if not args.kernels_only or args.precision == "f32":
            grad.mult(du32, dr32)
    torch.cuda.synchronize()
    if args.kernels_only:
        # only the Jacobian actions of one precision (for profiler captures)
        for _ in range(args.steps):
            if args.precision == "f32":
                grad.mult(du32, dr32)
            else:
                grad.mult(du, dr)
        torch.cuda.synchronize()
        if rank == 0:
            print(json.dumps({"kernels_only": True, "steps": args.steps, "finite": bool(torch.isfinite(dr).all())}))
        return

    def timed(fn, K):
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
        for k in range(K):
            flush.fill_(k & 0xFF)
            starts[k].record(stream)
            fn()
            ends[k].record(stream)
        torch.cuda.synchronize()
        return [s.elapsed_time(e) * 1e-3 for s, e in zip(starts, ends)]

    # ---- headline: FP64 Jv, inputs resident
    clocks = ClockSampler()
    clocks.start()
    barrier()
    torch.cuda.synchronize()
    t_fp64 = timed(lambda: grad.mult(du, dr), args.steps)
    barrier()
    torch.cuda.synchronize()
    clk = clocks.stop(dev.index)
    total = sum(t_fp64)
    total = max_over_ranks(total, world, dev)
    value = replica_throughput(world, ndofs, args.steps, total)

    # ---- FP32 Jv (inner Krylov operator)
    t_fp32 = timed(lambda: grad.mult(du32, dr32), args.steps)
    # ---- FP64 residual (q-function evaluated at every point, no derivative)
    r_buf = torch.empty_like(du)
    t_res = timed(lambda: f.residual(0.0, u, r_buf), args.steps)
    # ---- dominant kernels alone (element kernels, no scatter)
    dE = torch.empty(mesh.num_elements * 81, dtype=torch.float64, device=dev)
    t_elem = timed(lambda: grad.element_action(du, dE), args.steps)
    dE32 = torch.empty(mesh.num_elements * 81, dtype=torch.float32, device=dev)
    t_elem32 = timed(lambda: grad.element_action(du32, dE32), args.steps)
    # ---- the same Jacobian action without the stored tangent (q-function on duals every call)
    f.set_jvp_mode(f.RECOMPUTE)
    f.linearize(0.0, u)
    t_recompute = timed(lambda: grad.mult(du, dr), args.steps)
    t_recompute32 = timed(lambda: grad.mult(du32, dr32), args.steps)
    f.set_jvp_mode(f.STORED_TANGENT)
    f.linearize(0.0, u)
    # ---- adjoint-side operators: transposed action from the same stored tangent,
    # and the stored-energy quantity of interest (value and gradient dQ/du)
    t_jt = timed(lambda: grad.mult_transpose(du, dr), args.steps)
    t_jt32 = timed(lambda: grad.mult_transpose(du32, dr32), args.steps)
    qoi = sg.QoI(mesh, sg.H1(ORDER, 3))
    qoi.AddDomainIntegral(sg.QOI_NEOHOOKEAN_ENERGY, [K_BULK, G_SHEAR])
    q_val = torch.empty(1, dtype=torch.float64, device=dev)
    t_qv = timed(lambda: qoi.value(0.0, u, q_val), args.steps)
    t_qg = timed(lambda: qoi.gradient(0.0, u, r_buf), args.steps)

    # ---- end to end through the C ABI with host buffers
    h_du = torch.from_numpy(np.random.default_rng(0).standard_normal(ndofs)).pin_memory()
    h_dr = torch.empty(ndofs, dtype=torch.float64).pin_memory()
    d_du = torch.empty(ndofs, dtype=torch.float64, device=dev)

    def e2e_step():
        d_du.copy_(h_du, non_blocking=True)
        grad.mult(d_du, dr)
        h_dr.copy_(dr, non_blocking=True)

    for _ in range(max(1, args.warmup)):
        e2e_step()
    t_e2e = timed(e2e_step, args.steps)

    # parity spot check of the timed path against the C ABI's own FP64 result
    ok = bool(torch.isfinite(dr).all().item())

    # ---- roofline of the dominant kernel
    n_vert = (NX + 1) ** 3
    ne = mesh.num_elements
    nq = ne * (ORDER + 1) ** 3
    # stored-tangent action: read du, write dr, read the 9x9 flux-gradient tangent per point
    alg_bytes = 2 * 8 * ndofs + 81 * 8 * nq
    t_k = statistics.mean(t_elem)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except OSError:
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    prof = load_profile_numbers()
    traffic = prof.get("dram_bytes_per_launch")
    # algorithmic FP64 work of the stored-tangent action per element: per point,
    # interpolate grad du (3 x 24 FMA), apply the 9x9 tangent (81), integrate (3 x 27)
    flops_per_elem = 2 * (72 + 81 + 81) * (ORDER + 1) ** 3
    fp64_peak = measure_fp64_peak(dev)
    roofline = {
        "bound": "hbm",
        "kernel": "sfx::kernels::jvp_stored_kernel<2,3,false,false,double>",
        "achieved": alg_bytes / t_k / 1e9,
        "peak": hbm_peak,
        "unit": "GB/s",
        "frac": alg_bytes / t_k / 1e9 / hbm_peak,
        "traffic": traffic,
        "algorithmic_bytes": alg_bytes,
        "kernel_ms": t_k * 1e3,
        "peak_source": "MEASURED_PEAKS.json hbm_gbs" if "hbm_gbs" in peaks else "fallback 6.8 TB/s",
    }
    alg_bytes32 = 2 * 4 * ndofs + 81 * 4 * nq
    t_k32 = statistics.mean(t_elem32)
    roofline32 = {
        "bound": "hbm",
        "kernel": "sfx::kernels::jvp_stored_tma_kernel<3,false,false,12,2> (FP32, bulk-copy staged)",
        "achieved": alg_bytes32 / t_k32 / 1e9,
        "peak": hbm_peak,
        "unit": "GB/s",
        "frac": alg_bytes32 / t_k32 / 1e9 / hbm_peak,
        "traffic": prof.get("dram_bytes_per_launch_f32"),
        "algorithmic_bytes": alg_bytes32,
        "kernel_ms": t_k32 * 1e3,
    }
    compute = None
    if flops_per_elem:
        ach = flops_per_elem * ne / t_k / 1e12
        compute = {"bound": "fp64", "achieved": ach, "peak": fp64_peak, "unit": "TFLOP/s", "frac": ach / fp64_peak,
                   "flops_per_element": flops_per_elem,
                   "peak_source": "cuBLAS DGEMM 4096^3 measured in this run"}

    result = {
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": total / args.steps * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded mesh perturbation and linearisation state)",
        "config": config(world, "flushed between steps (256 MB write) and working set > L2"),
        "e2e": {"value": ndofs * args.steps / sum(t_e2e) / 1e9, "unit": UNIT, "h2d_bytes_per_step": 8 * ndofs,
                "d2h_bytes_per_step": 8 * ndofs},
        "roofline": roofline,
        "compute_roofline": compute,
        "jv_fp32": {"value": ndofs * args.steps / sum(t_fp32) / 1e9, "unit": UNIT, "dtype": "f32",
                    "ms_per_step": statistics.mean(t_fp32) * 1e3, "roofline": roofline32},
        "residual": {"value": ndofs * args.steps / sum(t_res) / 1e9, "unit": UNIT, "dtype": "f64",
                     "ms_per_step": statistics.mean(t_res) * 1e3,
                     "note": "R(u): fused element kernel (Neo-Hookean q-function, FP64) + node-owner scatter"},
        "jv_recompute": {"value_f64": ndofs * args.steps / sum(t_recompute) / 1e9,
                         "value_f32": ndofs * args.steps / sum(t_recompute32) / 1e9, "unit": UNIT,
                         "note": "q-function re-evaluated on dual numbers in every action; no stored tangent"},
        "adjoint": {"jv_transpose_f64": ndofs * args.steps / sum(t_jt) / 1e9,
                    "jv_transpose_f32": ndofs * args.steps / sum(t_jt32) / 1e9, "unit": UNIT,
                    "qoi_energy_value_ms": statistics.mean(t_qv) * 1e3,
                    "qoi_energy_gradient_ms": statistics.mean(t_qg) * 1e3,
                    "note": "J^T v from the stored tangent (adjoint solves); Neo-Hookean stored-energy QoI"},
        "gpu_launches": 2 * args.steps,
        "clocks": clk,
        "finite": ok,
    }
    if args.newton_steps > 0 and rank == 0:
        result["newton"] = newton_leg(args.newton_steps)
    if rank == 0:
        gd, reps, thr, el = cpu_jvp_rate(V, seconds=args.cpu_seconds)
        result["cpu_baseline"] = {"value": gd, "unit": UNIT, "cores": thr, "kind": "port",
                                  "sample": f"full workload, {reps} Jacobian actions in {el:.1f} s "
                                            "(stored-derivative form, derivative computed once untimed)"}
        print(json.dumps(result))


NEWTON_N = 32
NEWTON_SEED = 2000  # held out from the training seeds
WEIGHTS = os.path.join(ROOT, "serac_gb300", "weights", "lnet_j2_q2.npy")


def newton_leg(steps, only=None):
    """Newton time-to-1e-8 relative residual on the heterogeneous J2 problem
    (32^3 hexes, Q2 vector, per-element lognormal E, held-out seed), over the
    first `steps` load steps (warm-start predictor, Newton, state commit):
    plain FP64 GMRES(50) + Jacobi-Chebyshev against FP32-inner mixed precision
    and, when trained weights are present, the learned preconditioner on top of
    mixed precision.  Every variant reaches the same converged answer."""
    import torch

    import serac_gb300 as sg
    from serac_gb300 import learned as LP

    prob = LP.j2_problem(NEWTON_N, NEWTON_SEED)
    base = dict(newton_rel_tol=1e-8, newton_abs_tol=0.0, krylov_rel_tol=1e-8, krylov_abs_tol=0.0,
                max_krylov_iterations=5000)
    variants = [("plain_fp64", sg.SolverOptions.defaults(precond=sg.JACOBI_CHEBYSHEV, **base)),
                ("mixed", sg.SolverOptions.defaults(precond=sg.JACOBI_CHEBYSHEV, mixed_precision=1, **base)),
                ("mixed_f16", sg.SolverOptions.defaults(precond=sg.JACOBI_CHEBYSHEV, mixed_precision=1, **base))]
    net = None
    if os.path.exists(WEIGHTS):
        net = LP.LearnedPreconditioner()
        net.load(WEIGHTS)
        variants.append(("learned_mixed", sg.SolverOptions.defaults(precond=sg.LEARNED, mixed_precision=1, **base)))
    out = {"metric": "Newton time-to-1e-8 relative residual", "unit": "s", "higher_is_better": False,
           "workload": f"j2_q2_vector_{NEWTON_N}cubed_lognormal_E (seed {NEWTON_SEED}), load steps 1-{steps} of "
                       f"{prob.steps}, strain {prob.strain}",
           "dofs": 3 * (2 * NEWTON_N + 1) ** 3}
    if only is not None:
        variants = [v for v in variants if v[0] in only]
    ref = None
    for name, opts in variants:
        S = LP.SolidSetup(prob)
        if name.endswith("f16"):  # FP16 copy of the tangent for the inner FP32 operator
            S.f.set_tangent_storage(S.f.TANGENT_F16)
        solver = sg.NewtonSolver(S.f, opts)
        solver.set_essential(S.ess)
        if name.startswith("learned"):
            solver.set_learned(net, S.grid, S.features)
        u = torch.zeros(S.f.ndofs, dtype=torch.float64, device="cuda")
        tot = {}
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for step in range(1, steps + 1):
            pre = S.predictor(solver, u, step)
            st = solver.solve(0.0, u, raise_on_failure=False)
            for k in ("newton_iterations", "krylov_iterations", "inner_iterations", "learned_applications",
                      "learned_fallbacks"):
                tot[k] = tot.get(k, 0) + st[k]
            tot["predictor_krylov_iterations"] = tot.get("predictor_krylov_iterations", 0) + pre["krylov_iterations"]
            tot["converged"] = min(tot.get("converged", 1), st["converged"])
            tot["final_rel_residual"] = st["final_residual"] / st["initial_residual"]
            S.commit(u)
        torch.cuda.synchronize()
        tot["seconds"] = time.perf_counter() - t0
        if ref is None:
            ref = u.clone()
        tot["rel_diff_vs_plain"] = float(torch.linalg.norm(u - ref) / torch.linalg.norm(ref))
        out[name] = tot
        del solver, S
    for name in ("mixed", "mixed_f16", "learned_mixed"):
        if name in out and "plain_fp64" in out:
            out[f"speedup_{name}_vs_plain"] = out["plain_fp64"]["seconds"] / out[name]["seconds"]
    if net is None:
        out["learned_mixed"] = {"unavailable": f"no trained weights at {os.path.relpath(WEIGHTS, ROOT)}"}
    else:
        out["weights"] = {"file": os.path.relpath(WEIGHTS, ROOT), "trained_on": "J2 16^3 Q2, seeds 1000-1031 "
                          "(python -m serac_gb300.train_lnet), applied here on the 32^3 node grid"}
    return out


def _solve_step(S, opts, net=None, step=1):
    """Warm start + Newton for one load step from rest; returns (u, stats, seconds)."""
    import torch

    import serac_gb300 as sg

    solver = sg.NewtonSolver(S.f, opts)
    solver.set_essential(S.ess)
    if net is not None:
        solver.set_learned(net, S.grid, S.features)
    u = torch.zeros(S.f.ndofs, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    pre = S.predictor(solver, u, step)
    st = solver.solve(0.0, u, raise_on_failure=False)
    torch.cuda.synchronize()
    st = dict(st)
    st["predictor_krylov_iterations"] = pre["krylov_iterations"]
    st["seconds"] = time.perf_counter() - t0
    return u, st, solver


def _jv_rates(f, u, steps=10):
    """FP64 and FP32 Jacobian-action GDOF/s at the linearisation u (CUDA events)."""
    import torch

    grad = f.linearize(0.0, u)
    du = torch.randn(f.ndofs, dtype=torch.float64, device="cuda")
    dr = torch.empty_like(du)
    du32, dr32 = du.float(), torch.empty(f.ndofs, dtype=torch.float32, device="cuda")
    out = {}
    for name, a, b in (("jv_f64", du, dr), ("jv_f32", du32, dr32)):
        for _ in range(3):
            grad.mult(a, b)
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        for _ in range(steps):
            grad.mult(a, b)
        e.record()
        torch.cuda.synchronize()
        out[name] = f.ndofs * steps / (s.elapsed_time(e) * 1e-3) / 1e9
    return out


def config3_leg():
    """Mixed precision on the 64^3 Q2 heterogeneous Neo-Hookean problem
    (6,440,067 DOF; shear modulus 0.25 exp(g), g a unit Gaussian field of
    correlation length 0.1 (seed 2), bulk modulus 20 G; z = 0 clamped, first of
    10 compression steps to u_z = -0.05): error of the mixed-precision
    displacement against the FP64 solve, and both times to 1e-8."""
    import torch

    import serac_gb300 as sg
    from serac_gb300 import learned as LP

    prob = LP.neohookean_problem(64, 2, sigma_log=1.0, ell=0.1, strain=0.05, steps=10, bulk_ratio=20.0)
    S = LP.SolidSetup(prob, 2)
    base = dict(newton_rel_tol=1e-8, newton_abs_tol=0.0, krylov_rel_tol=1e-8, krylov_abs_tol=0.0,
                max_krylov_iterations=20000)
    u64, st64, _ = _solve_step(S, sg.SolverOptions.defaults(precond=sg.JACOBI_CHEBYSHEV, **base))
    u32, st32, _ = _solve_step(S, sg.SolverOptions.defaults(precond=sg.JACOBI_CHEBYSHEV, mixed_precision=1, **base))
    err = float(torch.linalg.norm(u32 - u64) / torch.linalg.norm(u64))
    return {"workload": "neohookean_q2_vector_64cubed_lognormal_G (seed 2), load step 1 of 10", "dofs": S.f.ndofs,
            "plain_fp64": st64, "mixed": st32, "rel_error_mixed_vs_fp64": err,
            "speedup_mixed_vs_plain": st64["seconds"] / st32["seconds"]}


def large_leg(with_plain=False):
    """The large combined sizes: 128^3 Q1 (6,440,067 DOF, 2x2x2 Gauss) and 96^3
    Q2 (21,567,171 DOF) heterogeneous Neo-Hookean (the 64^3 problem's material
    distribution): time to 1e-8 for the first load step with mixed precision
    (and learned + mixed when weights exist), Jacobian-action throughput at the
    converged state, and the device memory the problem holds."""
    import torch

    import serac_gb300 as sg
    from serac_gb300 import learned as LP

    out = {}
    net = None
    if os.path.exists(WEIGHTS):
        net = LP.LearnedPreconditioner()
        net.load(WEIGHTS)
    base = dict(newton_rel_tol=1e-8, newton_abs_tol=0.0, krylov_rel_tol=1e-8, krylov_abs_tol=0.0,
                max_krylov_iterations=20000)
    for order, n in ((1, 128), (2, 96)):
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        prob = LP.neohookean_problem(n, 2, sigma_log=1.0, ell=0.1, strain=0.05, steps=10, bulk_ratio=20.0)
        S = LP.SolidSetup(prob, order)
        rec = {"dofs": S.f.ndofs, "order": order, "hexes_per_direction": n}
        u, st, solver = _solve_step(S, sg.SolverOptions.defaults(precond=sg.JACOBI_CHEBYSHEV, mixed_precision=1,
                                                                   **base))
        rec["mixed"] = st
        rec.update(_jv_rates(S.f, u))
        torch.cuda.synchronize()
        rec["device_bytes_held"] = free0 - torch.cuda.mem_get_info()[0]
        del solver
        if net is not None:
            ul, stl, solver = _solve_step(S, sg.SolverOptions.defaults(precond=sg.LEARNED, mixed_precision=1, **base),
                                          net)
            stl["rel_diff_vs_mixed"] = float(torch.linalg.norm(ul - u) / torch.linalg.norm(u))
            rec["learned_mixed"] = stl
            del solver
        if with_plain:
            up, stp, solver = _solve_step(S, sg.SolverOptions.defaults(precond=sg.JACOBI_CHEBYSHEV, **base))
            stp["rel_diff_vs_mixed"] = float(torch.linalg.norm(up - u) / torch.linalg.norm(u))
            rec["plain_fp64"] = stp
            rec["speedup_mixed_vs_plain"] = stp["seconds"] / st["seconds"]
            del solver
        out[f"q{order}_{n}cubed"] = rec
        del S
        torch.cuda.synchronize()
    return out


def lnet_leg():
    """The learned preconditioner's kernels: one inference pass and one
    training step (batch 8) on the node grids of the 16^3 and 32^3 Q2 meshes."""
    import torch

    from serac_gb300 import learned as LP

    net = LP.LearnedPreconditioner(seed=0)
    out = {}
    for nodes in (33, 65):
        grid = (nodes,) * 3
        n = nodes ** 3
        r = torch.randn(3 * n, device="cuda")
        feat = torch.zeros(2 * n, device="cuda")
        R = torch.randn(8, 3 * n, device="cuda")
        T = torch.randn(8, 3 * n, device="cuda")
        F = torch.zeros(8, 2 * n, device="cuda")
        rec = {}
        for name, fn, reps in (("apply_ms", lambda: net.apply(grid, r, feat), 20),
                               ("train_step_batch8_ms", lambda: net.train_step(grid, R, T, F, 8, 0.0), 5)):
            for _ in range(3):
                fn()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for _ in range(reps):
                fn()
            torch.cuda.synchronize()
            rec[name] = (time.perf_counter() - t0) / reps * 1e3
        out[f"grid_{nodes}"] = rec
    return out


def measure_fp64_peak(dev):
    import torch

    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device=dev)
    b = torch.randn(n, n, dtype=torch.float64, device=dev)
    for _ in range(2):
        a @ b
    torch.cuda.synchronize()
    best = 0.0
    for _ in range(3):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        a @ b
        e.record()
        torch.cuda.synchronize()
        best = max(best, 2 * n ** 3 / (s.elapsed_time(e) * 1e-3) / 1e12)
    return best


def load_profile_numbers():
    """Per-launch DRAM traffic of the FP64 and FP32 element kernels, read from
    the committed ncu summaries (profiles/), if present."""
    out = {}
    for name, key in (("jvp_stored_f64_neohookean_q2_32cubed.json", "dram_bytes_per_launch"),
                      ("jvp_stored_tma_f32_neohookean_q2_32cubed.json", "dram_bytes_per_launch_f32")):
        try:
            d = json.load(open(os.path.join(ROOT, "profiles", name)))
        except (OSError, ValueError):
            continue
        if key == "dram_bytes_per_launch":
            out.update(d)
        elif "dram_bytes_per_launch" in d:
            out[key] = d["dram_bytes_per_launch"]
    return out


# ------------------------------------------------------------ reference arm
def run_reference(args, rank, world):
    if rank != 0:
        return
    V = problem()
    threads = os.cpu_count() or 1
    # warm-up and timed steps: each step is one full-workload Jacobian action
    _, _, _, _ = cpu_jvp_rate(V, seconds=0.0, threads=threads, min_reps=max(1, args.warmup))
    gd, reps, thr, el = cpu_jvp_rate(V, seconds=0.0, threads=threads, min_reps=args.steps)
    ndofs = 3 * (ORDER * NX + 1) ** 3
    result = {
        "impl": "reference",
        "metric": METRIC,
        "value": gd,
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": el / reps * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded mesh perturbation and linearisation state)",
        "config": config(1, "host memory (CPU path)"),
        "cpu_baseline": {"value": gd, "unit": UNIT, "cores": thr, "kind": "port",
                         "sample": f"full workload, {reps} Jacobian actions ({ndofs} DOF each)"},
        "e2e": {"value": gd, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "serac's reference build needs mfem/hypre/axom (absent); its element kernels are timed through "
                "the oracle's restatement of action_of_gradient_kernel with the same sum factorisation",
    }
    print(json.dumps(result))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["sfx", "reference"], default="sfx")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--kernels-only", action="store_true", help="run only the Jacobian actions (profiling)")
    ap.add_argument("--precision", choices=["f64", "f32"], default="f64", help="precision of --kernels-only")
    ap.add_argument("--newton-steps", type=int, default=1,
                    help="load steps of the Newton time-to-1e-8 leg (0 = skip)")
    ap.add_argument("--extra", choices=["config3", "large", "large-plain", "newton-mixed", "newton-f16", "lnet"],
                    default=None,
                    help="run only an extra configuration (64^3 mixed-precision error, or the large sizes) "
                         "and print its JSON record")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        backend = "nccl" if args.impl == "sfx" else "gloo"
        dist.init_process_group(backend)
    if args.extra is not None:
        import torch

        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
        if args.extra == "newton-mixed":  # the mixed-precision Newton leg alone (for profiler launch lists)
            rec = newton_leg(1, only=("mixed",))
        elif args.extra == "newton-f16":  # mixed precision with the FP32 and the FP16 inner tangent
            rec = newton_leg(1, only=("mixed", "mixed_f16"))
        elif args.extra == "lnet":
            rec = lnet_leg()
        elif args.extra == "config3":
            rec = config3_leg()
        else:
            rec = large_leg(with_plain=args.extra == "large-plain")
        if rank == 0:
            print(json.dumps({"extra": args.extra, **rec}))
    elif args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_sfx(args, rank, world)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
