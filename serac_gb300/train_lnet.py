"""Train the learned preconditioner on seeded J2 problems and save its
parameters (the file bench.py and the solver load):

    python -m serac_gb300.train_lnet --n 16 --seeds 1000:1032 --epochs 40 \\
        --out serac_gb300/weights/lnet_j2_q2.npy

Training problems: small-strain J2 with linear hardening on n^3 Q2 meshes,
per-element lognormal Young's modulus (sigma_log in [0.5, 1.5], correlation
length in [0.05, 0.3], drawn per seed), compression in load steps.  Pairs:
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
    ap.add_argument("--out", required=True)
    args = ap.parse_args(argv)

    import torch

    from . import learned as L

    lo, hi = (int(x) for x in args.seeds.split(":"))
    t0 = time.time()
    problems = [L.j2_problem(args.n, s) for s in range(lo, hi)]
    R, T, F = L.harvest(problems, probes_per_step=args.probes)
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
    info = {"pairs": int(R.shape[0]), "seeds": args.seeds, "n": args.n, "epochs": args.epochs, "batch": args.batch,
            "lr": args.lr, "harvest_s": round(t_harvest, 1), "train_s": round(time.time() - t0, 1),
            "final_loss": hist[-1], "loss_history": [round(h, 4) for h in hist]}
    with open(os.path.splitext(args.out)[0] + ".json", "w") as fh:
        json.dump(info, fh, indent=1)
    print(json.dumps(info))


if __name__ == "__main__":
    main()
