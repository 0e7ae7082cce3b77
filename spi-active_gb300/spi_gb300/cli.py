"""Command-line identification on logged Go2 trajectories (npz files in the reference's format).

    python -m spi_gb300.cli landscape --data a.npz b.npz --horizon 5 [--env-batch 4096]
    python -m spi_gb300.cli identify  --data a.npz --horizon 20 [--params 0 1 2 4] [--samples 4096]

``landscape`` is scripts/mass_landscape.py (20 base-mass scales in [0.5, 2.0], weighted
10/5/1 cost, argmin, results text) with every scale in one GPU launch. ``identify`` replaces
the Optuna loop of scripts/mass_opt.py with the device CEM over any subset of the 13 theta
slots. Both write a results file next to the reference's (``landscape_results.txt`` /
``optimization_results.txt``).
"""
from __future__ import annotations

import argparse
from datetime import datetime
from pathlib import Path

import numpy as np
import torch

from . import eval_compat as ec
from .cem import CEM
from .data import init_states, load_dataset, target_states
from .engine import COST_REF, Engine
from .robot import THETA_NAMES, THETA_NOMINAL, THETA_PRIOR_HI, THETA_PRIOR_LO, SimConfig

MASS_SCALE_MIN, MASS_SCALE_MAX, MASS_SAMPLES = 0.5, 2.0, 20


def _cfg(args):
    return SimConfig.reference_compatible(kp=args.kp, kd=args.kd, sim_dt=args.sim_dt, decimation=args.decimation)


def landscape(args):
    n, ds_np = ec.load_dataset([Path(p) for p in args.data], args.horizon)
    env = ec.instantiate_env(None, min(args.env_batch, n, 8192), cfg=_cfg(args))
    ds = ec.to_device(ds_np, env.device)
    masses = ec.capture_reference_masses(env.simulator)
    scales = np.linspace(MASS_SCALE_MIN, MASS_SCALE_MAX, MASS_SAMPLES)
    costs = ec.mass_sweep(env, ds, args.horizon, masses, scales)
    total = np.array([ec.compute_cost(c) for c in costs])
    best = int(np.argmin(total))
    base = float(masses[0])
    out = Path(args.out) / f"{datetime.now():%Y%m%d-%H%M%S}_h{args.horizon}"
    out.mkdir(parents=True, exist_ok=True)
    with open(out / "landscape_results.txt", "w", encoding="utf-8") as f:
        f.write(f"Mass Landscape Results\n{'=' * 60}\nHorizon: {args.horizon}\n")
        f.write(f"Cost coefficients: {ec.COST_COEFF}\nNumber of samples: {MASS_SAMPLES}\n\n")
        f.write(f"Nominal base mass: {base:.3f} kg\nOptimal base mass: {base * scales[best]:.3f} kg\n")
        f.write(f"Minimum total cost: {total[best]:.6f}\nAll samples:\n")
        f.write("scale,base_mass_kg,base_pos,base_quat,joint_pos,total_cost\n")
        for s, c, t in zip(scales, costs, total):
            f.write(f"{s:.4f},{base * s:.3f},{c[0]:.6f},{c[1]:.6f},{c[2]:.6f},{t:.6f}\n")
    print(f"Optimal: scale={scales[best]:.4f}, base={base * scales[best]:.3f} kg, cost={total[best]:.6f}")
    return out


def identify(args):
    n, ds = load_dataset([Path(p) for p in args.data], args.horizon, causal=args.causal)
    eng = Engine(_cfg(args))
    eng.load_windows(torch.from_numpy(init_states(ds)), torch.from_numpy(ds["action_sequences"]),
                     torch.from_numpy(target_states(ds)))
    if args.reference_cost:
        eng.set_cost(COST_REF)
    ids = list(args.params)
    cem = CEM(eng, args.samples, ids, THETA_PRIOR_LO[ids], THETA_PRIOR_HI[ids], THETA_NOMINAL,
              elite_frac=args.elite_frac, seed=args.seed)
    cem.run(args.iterations, graph=True)
    r = cem.read()
    out = Path(args.out) / f"{datetime.now():%Y%m%d-%H%M%S}_h{args.horizon}"
    out.mkdir(parents=True, exist_ok=True)
    with open(out / "optimization_results.txt", "w", encoding="utf-8") as f:
        f.write(f"Identification results (device CEM)\n{'=' * 60}\nHorizon: {args.horizon}\n")
        f.write(f"Windows: {n}\nSamples: {args.samples}\nIterations: {args.iterations}\n\n")
        for d, i in enumerate(ids):
            f.write(f"{THETA_NAMES[i]}: mean {r['mu'][d]:.6f}, best {r['best_theta'][i]:.6f}\n")
        f.write(f"Best cost: {r['best_cost']:.6g}\n")
    print(f"Best cost {r['best_cost']:.6g}; " + ", ".join(f"{THETA_NAMES[i]}={r['best_theta'][i]:.4f}" for i in ids))
    return out, r


def main(argv=None):
    ap = argparse.ArgumentParser(prog="spi_gb300")
    sub = ap.add_subparsers(dest="cmd", required=True)
    for name in ("landscape", "identify"):
        p = sub.add_parser(name)
        p.add_argument("--data", nargs="+", required=True, help="npz trajectories (scripts/data/common.py format)")
        p.add_argument("--horizon", type=int, default=5)
        p.add_argument("--out", default="logs")
        p.add_argument("--kp", type=float, default=20.0)
        p.add_argument("--kd", type=float, default=0.5)
        p.add_argument("--sim-dt", type=float, default=0.00125)
        p.add_argument("--decimation", type=int, default=4)
    sub.choices["landscape"].add_argument("--env-batch", type=int, default=4096)
    p = sub.choices["identify"]
    p.add_argument("--params", type=int, nargs="+", default=list(range(13)))
    p.add_argument("--samples", type=int, default=4096)
    p.add_argument("--iterations", type=int, default=30)
    p.add_argument("--elite-frac", type=float, default=0.1)
    p.add_argument("--seed", type=int, default=0)
    p.add_argument("--causal", action="store_true", help="pair each window with the actions after its state")
    p.add_argument("--reference-cost", action="store_true", help="10/5/1 L2 cost instead of weighted squares")
    args = ap.parse_args(argv)
    return landscape(args) if args.cmd == "landscape" else identify(args)


if __name__ == "__main__":
    main()
