"""Train the crystal-pass surrogate on solver-generated pairs, then time the OPO with it.

    python -m optifax_gb300.train_surrogate --cavities 38 --trips 160 --epochs 120 --repr env --out DIR

Writes DIR/fno_params_<repr>.npy (the FP32 parameter vector of each trained
representation) and DIR/train_summary.json (data generation and training figures,
the identity-map baseline, the fast-forward OPO runs, optionally the solver-only
run, and the plain FP64 solver's trip rate).
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
    ap.add_argument("--repr", default="env", help="comma list of representations: env (band envelopes), bins")
    ap.add_argument("--eval-trips", type=int, default=100)
    ap.add_argument("--solver-only-trips", type=int, default=0)
    ap.add_argument("--check-tol", type=float, default=0.05)
    ap.add_argument("--fp64-trips", type=int, default=1)
    ap.add_argument("--out", default="surrogate_out")
    ap.add_argument("--no-align", action="store_true",
                    help="keep each target's global signal-phase change (default: remove it, as the check does)")
    ap.add_argument("--weight-decay", type=float, default=0.0)
    ap.add_argument("--power", default="0.5,3.0", help="pump power range of the training cavities [W]")
    ap.add_argument("--oc-output", type=float, default=0.10, help="output-coupler transmission of the cavities")
    ap.add_argument("--eval-power", type=float, default=2.0, help="pump power of the evaluation cavity [W]")
    ap.add_argument("--check", default="field", choices=["field", "energy"])
    ap.add_argument("--save-params", default="", help="also write the trained parameters here (float16 .npy)")
    args = ap.parse_args(argv)
    from . import fastforward as ff, opo
    from .surrogate import FNO
    os.makedirs(args.out, exist_ok=True)
    summary = {"args": vars(args), "runs": {}}
    base = opo.CavitySpec(crystal_length=args.crystal_length, oc_output=args.oc_output)
    evalspec = opo.CavitySpec(crystal_length=args.crystal_length, oc_output=args.oc_output,
                              pump_power=args.eval_power)
    t0 = time.perf_counter()
    pw = tuple(float(x) for x in args.power.split(","))
    specs = ff.training_specs(args.cavities, seed=args.seed, base=base, power=pw)
    ins, outs, trip_idx, attempts = ff.generate_raw(specs, args.trips)
    torch.cuda.synchronize()
    summary["generation"] = {"pairs": int(ins.shape[0]), "seconds": time.perf_counter() - t0,
                             "solver_attempts": attempts}
    print(json.dumps(summary["generation"]), flush=True)
    for rep in [r.strip() for r in args.repr.split(",") if r.strip()]:
        crop = ff.reference_env_crop(base) if rep == "env" else ff.reference_crop(base)
        tgt = outs
        if rep == "env" and not args.no_align:
            tgt = ff.align_signal_phase(ins, outs, ff.signal_mask(crop, ins.shape[1], ins.device))
        X, T = ff.encode_pairs(ins, tgt, crop)
        net = FNO(n_bins=crop.n_bins, max_batch=args.batch, seed=args.seed)
        hist = ff.train(net, X, T, epochs=args.epochs, batch=args.batch, lr=args.lr, seed=args.seed,
                        weight_decay=args.weight_decay, trip_idx=trip_idx,
                        log=lambda s: print(f"[{rep}] {s}", flush=True))
        run = {"training": hist}
        print(json.dumps({"repr": rep, **{k: hist[k] for k in hist if k not in ("train_loss", "val_signal_rel_l2")}}),
              flush=True)
        params = net.params().cpu().numpy()
        np.save(os.path.join(args.out, f"fno_params_{rep}.npy"), params)
        if args.save_params:
            np.save(args.save_params, params.astype(np.float16))
        del X, T, net
        torch.cuda.empty_cache()
        if args.eval_trips > 0:
            infer = FNO(n_bins=crop.n_bins, max_batch=1, params=params)
            fast = ff.run_fast_forward(opo.OpticalSim(evalspec), infer, crop, max_trips=args.eval_trips,
                                       check_tol=args.check_tol, check=args.check)
            summary["_fast_field"] = fast.pop("field")
            fast["energies"] = fast["energies"][-10:]
            run["fast_forward"] = fast
            print(json.dumps({"repr": rep, "fast_forward": {k: fast[k] for k in
                                                            ("trips", "surrogate_trips", "solver_trips",
                                                             "fallback_blocks", "wall_s", "trips_per_s",
                                                             "reached_steady_state", "final_output_signal_energy")},
                              "checks": fast["checks"]}), flush=True)
            del infer
        summary["runs"][rep] = run
    if args.solver_only_trips > 0:
        solo = ff.run_fast_forward(opo.OpticalSim(evalspec), None, ff.reference_crop(base),
                                   max_trips=args.solver_only_trips)
        solo_field = solo.pop("field")
        solo["energies"] = solo["energies"][-10:]
        summary["solver_only"] = solo
        print(json.dumps({"solver_only": {k: solo[k] for k in ("trips", "wall_s", "trips_per_s", "reached_steady_state",
                                                               "final_output_signal_energy")}}), flush=True)
        fast_field = summary.pop("_fast_field", None)
        if fast_field is not None:
            # final crystal inputs of the two runs, fed-back band, after the best global signal phase
            sim = opo.OpticalSim(evalspec)
            band = sim.feedback.abs() > 0
            Xa = torch.from_numpy(np.fft.fft(fast_field.cpu().numpy().astype(np.complex128)))
            Xb = torch.from_numpy(np.fft.fft(solo_field.cpu().numpy().astype(np.complex128)))
            summary["final_state_fed_back_band_rel_l2"] = ff.phase_aligned_err(Xa, Xb, band.cpu())
            print(json.dumps({"final_state_fed_back_band_rel_l2": summary["final_state_fed_back_band_rel_l2"]}),
                  flush=True)
    if args.fp64_trips > 0:
        fp64 = ff.fp64_plain_trips(base, args.fp64_trips)
        fp64.pop("field")
        summary["fp64_plain"] = fp64
        print(json.dumps({"fp64_plain": fp64}), flush=True)
    summary.pop("_fast_field", None)
    with open(os.path.join(args.out, "train_summary.json"), "w") as f:
        json.dump(summary, f, indent=1, default=float)


if __name__ == "__main__":
    main()
