"""Train the crystal-pass surrogate on solver-generated pairs, then time the OPO with it.

    python -m optifax_gb300.train_surrogate --cavities 38 --trips 160 --epochs 120 --out DIR

Writes DIR/fno_params.npy (the FP32 parameter vector) and DIR/train_summary.json
(data generation and training figures, the fast-forward OPO run against the
solver-only run and the plain FP64 solver's trip rate).
"""
from __future__ import annotations

import argparse
import json
import os
import time

import numpy as np
import torch


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--cavities", type=int, default=38)
    ap.add_argument("--trips", type=int, default=160)
    ap.add_argument("--epochs", type=int, default=120)
    ap.add_argument("--batch", type=int, default=32)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=3)
    ap.add_argument("--crystal-length", type=float, default=5e-3)
    ap.add_argument("--eval-trips", type=int, default=200)
    ap.add_argument("--check-tol", type=float, default=0.05)
    ap.add_argument("--fp64-trips", type=int, default=2)
    ap.add_argument("--no-eval", action="store_true")
    ap.add_argument("--out", default="surrogate_out")
    args = ap.parse_args(argv)
    from . import fastforward as ff, opo
    from .surrogate import FNO
    os.makedirs(args.out, exist_ok=True)
    summary = {"args": vars(args)}
    base = opo.CavitySpec(crystal_length=args.crystal_length)
    crop = ff.reference_crop(base)
    summary["crop"] = {"k0": crop.k0, "n_bins": crop.n_bins, "split": crop.split, "pump_scale": crop.pump_scale}
    t0 = time.perf_counter()
    specs = ff.training_specs(args.cavities, seed=args.seed, base=base)
    X, T, trip_idx, attempts = ff.generate_pairs(specs, args.trips, crop)
    torch.cuda.synchronize()
    summary["generation"] = {"pairs": int(X.shape[0]), "seconds": time.perf_counter() - t0,
                             "solver_attempts": attempts}
    print(json.dumps(summary["generation"]), flush=True)
    net = FNO(n_bins=crop.n_bins, max_batch=args.batch, seed=args.seed)
    hist = ff.train(net, X, T, epochs=args.epochs, batch=args.batch, lr=args.lr, seed=args.seed,
                    trip_idx=trip_idx, log=lambda s: print(s, flush=True))
    summary["training"] = hist
    print(json.dumps({k: hist[k] for k in ("seconds", "steps", "val_signal_rel_l2_quantiles")
                      + (("val_by_trip",) if "val_by_trip" in hist else ())}), flush=True)
    params = net.params().cpu().numpy()
    np.save(os.path.join(args.out, "fno_params.npy"), params)
    del X, T
    torch.cuda.empty_cache()
    if not args.no_eval:
        spec = base                       # the evaluation cavity: 2 W, 200 fs, noise seed 1
        infer = FNO(n_bins=crop.n_bins, max_batch=1, params=params)
        solo = ff.run_fast_forward(opo.OpticalSim(spec), None, crop, max_trips=args.eval_trips)
        fast = ff.run_fast_forward(opo.OpticalSim(spec), infer, crop, max_trips=args.eval_trips,
                                   check_tol=args.check_tol)
        fp64 = ff.fp64_plain_trips(spec, args.fp64_trips)
        fp64.pop("field")
        a_s, a_f = solo.pop("field"), fast.pop("field")
        for r in (solo, fast):
            r["energies_head"] = r["energies"][:60:3]
            r["energies"] = r["energies"][-20:]
        summary["eval"] = {"solver_only": solo, "surrogate_plus_solver": fast, "fp64_plain": fp64,
                           "field_rel_l2_vs_solver_only": float((a_f - a_s).norm() / a_s.norm()),
                           "speedup_vs_fp64_plain": fast["trips_per_s"] / fp64["trips_per_s"],
                           "speedup_vs_solver_only_wall": solo["wall_s"] / fast["wall_s"],
                           "final_energy_rel_diff": abs(fast["final_output_signal_energy"] -
                                                        solo["final_output_signal_energy"]) /
                           abs(solo["final_output_signal_energy"])}
        print(json.dumps(summary["eval"], default=float), flush=True)
    with open(os.path.join(args.out, "train_summary.json"), "w") as f:
        json.dump(summary, f, indent=1, default=float)


if __name__ == "__main__":
    main()
