"""Train the learned preconditioner on seeded J2 problems and save its
parameters (the file bench.py and the solver load):

    python -m serac_gb300.train_lnet --n 16 --seeds 1000:1032 --epochs 40 \\
        --out serac_gb300/weights/lnet_j2_q2.npy

Training problems (--material): small-strain J2 with linear hardening on
n^3 Q2 meshes, per-element lognormal Young's modulus (sigma_log in
[0.5, 1.5], correlation length in [0.05, 0.3], drawn per seed), compression
in load steps; or the heterogeneous Neo-Hookean solid of the large
configurations (shear modulus 0.25 exp(g), sigma_log 1, correlation length
0.1, bulk modulus 20 G), its first load steps (--strain per --steps).  Pairs:
every Newton (residual, correction) of the mixed-precision solve plus probe
pairs (smooth random x, r = J x) at each converged step.  Runs on the GPU with
the library's own BF16 training kernels.
"""
from __future__ import annotations

import argparse
import json
import os
import time


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=16, help="hexes per direction of the training meshes")
    ap.add_argument("--seeds", default="1000:1032", help="first:last (exclusive) training seeds")
    ap.add_argument("--probes", type=int, default=8, help="probe pairs per converged load step")
    ap.add_argument("--epochs", type=int, default=40)
    ap.add_argument("--batch", type=int, default=8)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--init-seed", type=int, default=0)
    ap.add_argument("--steps", type=int, default=4, help="load steps per training problem")
    ap.add_argument("--material", choices=["j2", "neohookean"], default="j2")
    ap.add_argument("--strain", type=float, default=None,
                    help="compression reached after --steps (default: 0.02 for J2, 0.005 for Neo-Hookean)")
    ap.add_argument("--eval-seeds", default=None,
                    help="first:last held-out seeds: after training, solve them with and without the network")
    ap.add_argument("--eval-fp64-seeds", default=None,
                    help="first:last subset of the held-out seeds also solved by the FP64 methods (Chebyshev "
                         "alone and the two-level step); default: all of --eval-seeds")
    ap.add_argument("--eval-steps", type=int, default=None,
                    help="load steps of the held-out problems (default: --steps)")
    ap.add_argument("--eval-strain", type=float, default=None,
                    help="compression of the held-out problems after their load steps (default: --strain)")
    ap.add_argument("--load", default=None,
                    help="evaluate these trained parameters (.npy) instead of harvesting and training")
    ap.add_argument("--out", required=True)
    args = ap.parse_args(argv)

    import torch

    from . import learned as L

    make_eval = problem_factory(args.material, args.strain if args.eval_strain is None else args.eval_strain,
                                args.steps if args.eval_steps is None else args.eval_steps)
    if args.load:
        net = L.LearnedPreconditioner(seed=args.init_seed)
        net.load(args.load)
        info = {"material": args.material, "weights": args.load, "n": args.n,
                "evaluation": evaluate(net, args.n, args.eval_seeds, make_eval, args.eval_fp64_seeds)}
        with open(args.out, "w") as fh:
            json.dump(info, fh, indent=1)
        print(json.dumps(info))
        return

    lo, hi = (int(x) for x in args.seeds.split(":"))
    t0 = time.time()
    make = problem_factory(args.material, args.strain, args.steps)
    problems = [make(args.n, s) for s in range(lo, hi)]
    n_prob = len(problems)

    def progress(done, pairs):
        if done % 32 == 0 or done == n_prob:
            print(f"harvest {done}/{n_prob} problems, {pairs} pairs, {time.time() - t0:.0f} s", flush=True)

    R, T, F = L.harvest(problems, probes_per_step=args.probes, log=progress)
    torch.cuda.synchronize()
    t_harvest = time.time() - t0
    grid = (2 * args.n + 1,) * 3
    net = L.LearnedPreconditioner(seed=args.init_seed)
    t0 = time.time()
    hist = L.train(net, grid, R, T, F, epochs=args.epochs, batch=args.batch, lr=args.lr,
                   log=lambda e, l: print(f"epoch {e} loss {l:.4f}", flush=True))
    torch.cuda.synchronize()
    os.makedirs(os.path.dirname(os.path.abspath(args.out)), exist_ok=True)
    net.save(args.out)
    info = {"material": args.material, "pairs": int(R.shape[0]), "seeds": args.seeds, "n": args.n,
            "steps": args.steps, "epochs": args.epochs, "batch": args.batch,
            "lr": args.lr, "harvest_s": round(t_harvest, 1), "train_s": round(time.time() - t0, 1),
            "final_loss": hist[-1], "loss_history": [round(h, 4) for h in hist]}
    if args.eval_seeds:
        info["evaluation"] = evaluate(net, args.n, args.eval_seeds, make_eval, args.eval_fp64_seeds)
    with open(os.path.splitext(args.out)[0] + ".json", "w") as fh:
        json.dump(info, fh, indent=1)
    print(json.dumps(info))


def problem_factory(material, strain, steps):
    """(n, seed) -> SolidProblem of the chosen family."""
    from . import learned as L

    if material == "neohookean":
        st = 0.005 if strain is None else strain
        return lambda n, seed: L.neohookean_problem(n, seed, sigma_log=1.0, ell=0.1, strain=st, steps=steps,
                                                    bulk_ratio=20.0)
    st = 0.02 if strain is None else strain
    return lambda n, seed: L.j2_problem(n, seed, strain=st, steps=steps)


def evaluate(net, n, seeds, make, fp64_seeds=None):
    """Held-out seeds: Krylov iterations and seconds of flexible GMRES with
    Jacobi-Chebyshev alone against the network's two-level step
    (Chebyshev, network, Chebyshev) on the fp64_seeds subset (default: all),
    and of mixed precision against learned + mixed precision on every seed;
    every solve of a seed must reach the same answer."""
    import torch

    from . import learned as L
    from .solver import FGMRES, JACOBI_CHEBYSHEV, LEARNED, NewtonSolver, SolverOptions

    tol = dict(newton_rel_tol=1e-8, newton_abs_tol=0.0, krylov_rel_tol=1e-8, krylov_abs_tol=0.0,
               max_krylov_iterations=20000)
    variants = {
        "chebyshev": (SolverOptions.defaults(precond=JACOBI_CHEBYSHEV, krylov=FGMRES, **tol), False),
        "learned_two_level": (SolverOptions.defaults(precond=LEARNED, learned_cycle=1, **tol), True),
        "mixed": (SolverOptions.defaults(precond=JACOBI_CHEBYSHEV, mixed_precision=1, **tol), False),
        "learned_mixed": (SolverOptions.defaults(precond=LEARNED, mixed_precision=1, **tol), True),
    }
    lo, hi = (int(x) for x in seeds.split(":"))
    flo, fhi = (int(x) for x in fp64_seeds.split(":")) if fp64_seeds else (lo, hi)
    totals = {k: {"krylov_iterations": 0, "seconds": 0.0, "seeds": 0} for k in variants}
    per_seed = []
    worst_diff = 0.0
    for seed in range(lo, hi):
        prob = make(n, seed)
        sols = {}
        row = {"seed": seed}
        for name, (opts, use_net) in variants.items():
            if name in ("chebyshev", "learned_two_level") and not flo <= seed < fhi:
                continue
            S = L.SolidSetup(prob)
            solver = NewtonSolver(S.f, opts)
            solver.set_essential(S.ess)
            if use_net:
                solver.set_learned(net, S.grid, S.features)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            u, tot = L.solve_load_steps(S, solver)
            torch.cuda.synchronize()
            dt = time.perf_counter() - t0
            its = tot["krylov_iterations"] + tot["predictor_krylov_iterations"]
            totals[name]["seconds"] += dt
            totals[name]["krylov_iterations"] += its
            totals[name]["seeds"] += 1
            row[name] = {"krylov_iterations": its, "seconds": round(dt, 3), "converged": int(tot.get("converged", 0)),
                         "newton_iterations": tot.get("newton_iterations", 0),
                         "learned_fallbacks": tot.get("learned_fallbacks", 0),
                         "learned_skipped": tot.get("learned_skipped", 0),
                         "learned_applications": tot.get("learned_applications", 0)}
            sols[name] = u
        ref = sols.get("chebyshev", sols["mixed"])
        for name, u in sols.items():
            d = float(torch.linalg.norm(u - ref) / torch.linalg.norm(ref))
            row[name]["rel_diff"] = d
            if all(row[k]["converged"] for k in sols):
                worst_diff = max(worst_diff, d)
        per_seed.append(row)
    converged = sum(all(v["converged"] for k, v in r.items() if k != "seed") for r in per_seed)
    out = {"seeds": seeds, "fp64_seeds": f"{flo}:{fhi}", "n": n, "totals": totals,
           "seeds_all_converged": converged, "max_rel_diff_converged": worst_diff,
           "time_ratio_learned_mixed": totals["learned_mixed"]["seconds"] / totals["mixed"]["seconds"],
           "iteration_ratio_learned_mixed": totals["learned_mixed"]["krylov_iterations"]
           / max(1, totals["mixed"]["krylov_iterations"]),
           "per_seed": per_seed}
    if totals["chebyshev"]["seeds"]:
        out["iteration_ratio_two_level"] = (totals["learned_two_level"]["krylov_iterations"]
                                            / max(1, totals["chebyshev"]["krylov_iterations"]))
        out["time_ratio_two_level"] = totals["learned_two_level"]["seconds"] / totals["chebyshev"]["seconds"]
    return out


if __name__ == "__main__":
    main()
