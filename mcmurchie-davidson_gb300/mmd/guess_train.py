"""Train and evaluate the learned initial guess on seeded water clusters (6-31G).

    python -m mmd.guess_train --train 20000 --eval 500 --out DIR
    python -m mmd.guess_train --basis 6-31gss --train 8000 --eval 64 --out DIR

1. training data: converged RHF densities (direct, conver 1e-8) of seeded (H2O)n,
   n ~ U{1..6}, computed by the batched GPU path (1024 molecules per launch);
2. features/targets per atom pair (mmd.guess), Adam training on the GPU with the
   project's MLP kernels;
3. evaluation on held-out seeded (H2O)8: SCF iterations and wall time to
   convergence from the learned guess vs the core-Hamiltonian guess (both batched),
   and the energy differences.
Writes the weights (npz) and a JSON report into DIR (and the weights into mmd/data).
"""
from __future__ import annotations

import argparse
import json
import os
import time

import numpy as np

from . import guess as G
from .batch import BatchRHF
from .clusters import water_cluster


def converged_densities(geoms, basis="6-31g", chunk=1024, log=print):
    out = []
    for s in range(0, len(geoms), chunk):
        br = BatchRHF(geoms[s:s + chunk], basis)
        br.run(conver=1e-8)
        Ph = br.P.cpu().numpy()
        out.extend(Ph[b, :n, :n].copy() for b, n in enumerate(br.N))
        log(f"  densities {s + len(br.N)}/{len(geoms)} (converged {int(br.converged.sum())}/{len(br.N)})")
    return out


def dataset(mols, dens, gb=G.B631G):
    F, Y, M = [], [], []
    for m, P in zip(mols, dens):
        _, f, y, k, _ = G.molecule_samples(m, P, gb)
        F.append(f)
        Y.append(y)
        M.append(k)
    return np.concatenate(F), np.concatenate(Y), np.concatenate(M)


def evaluate(net, geoms, log=print, basis="6-31g"):
    """Core vs learned guess on the same molecules (batched, FP64, conver 1e-8): SCF
    iterations and wall time; then both again at conver 1e-10 with an FP64 polish
    build (BatchRHF.run(polish=True)) for the energy comparison."""
    from .molecule import Molecule
    mols = [Molecule(g, basis) for g in geoms]
    t0 = time.perf_counter()
    guesses = [G.predict_density(net, m) for m in mols]
    t_pred = time.perf_counter() - t0
    res = {}
    for name, gs in (("core", None), ("learned", guesses)):
        br = BatchRHF(geoms, basis)
        t0 = time.perf_counter()
        br.run(conver=1e-8, guess=gs)
        t = time.perf_counter() - t0
        r = {"energies": br.energies_raw.copy(), "iterations": br.iterations.copy(), "time_s": t,
             "converged": int(br.converged.sum()), "reverted": int(br.reverted.sum())}
        r["polished"] = br.run(conver=1e-10, guess=gs, polish=True).copy()
        r["converged_tight"] = int(br.converged.sum())
        res[name] = r
        log(f"  {name}: mean iterations {r['iterations'].mean():.2f}, time {t:.2f} s")
    dE = np.abs(res["learned"]["energies"] - res["core"]["energies"])
    dEp = np.abs(res["learned"]["polished"] - res["core"]["polished"])
    return {
        "molecules": len(geoms),
        "core_mean_iterations": float(res["core"]["iterations"].mean()),
        "learned_mean_iterations": float(res["learned"]["iterations"].mean()),
        "core_time_s": res["core"]["time_s"], "learned_time_s": res["learned"]["time_s"] + t_pred,
        "guess_prediction_s": t_pred,
        "max_abs_energy_difference_conver_1e-8": float(dE.max()),
        "max_abs_energy_difference_polished": float(dEp.max()),
        "reverted_to_core": res["learned"]["reverted"],
        "converged": [res["core"]["converged"], res["learned"]["converged"]],
        "converged_tight": [res["core"]["converged_tight"], res["learned"]["converged_tight"]],
        "iterations_core": res["core"]["iterations"].tolist(),
        "iterations_learned": res["learned"]["iterations"].tolist(),
        "energies_polished_core": res["core"]["polished"].tolist(),
    }


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--train", type=int, default=20000)
    ap.add_argument("--eval", type=int, default=500)
    ap.add_argument("--epochs", type=int, default=30)
    ap.add_argument("--out", default="guess_out")
    ap.add_argument("--eval-only", action="store_true", help="evaluate the committed weights only")
    ap.add_argument("--basis", default="6-31g", choices=sorted(G.BASES), help="basis of the network")
    args = ap.parse_args(argv)
    gb = G.BASES[args.basis]
    from .molecule import Molecule
    eval_geoms = [water_cluster(8, seed=900000 + k) for k in range(args.eval)]
    if args.eval_only:
        ev = evaluate(G.DensityMLP.load(gb.weights), eval_geoms, basis=args.basis)
        os.makedirs(args.out, exist_ok=True)
        with open(os.path.join(args.out, "guess_eval.json"), "w") as f:
            json.dump(ev, f, indent=1)
        print(json.dumps({k: v for k, v in ev.items() if not isinstance(v, list)}))
        return
    rng = np.random.default_rng(2025)
    sizes = rng.integers(1, 7, size=args.train)
    train_geoms = [water_cluster(int(n), seed=200000 + k) for k, n in enumerate(sizes)]
    t0 = time.perf_counter()
    dens = converged_densities(train_geoms, args.basis)
    t_data = time.perf_counter() - t0
    mols = [Molecule(g, args.basis) for g in train_geoms]
    F, Y, M = dataset(mols, dens, gb)
    print(f"dataset: {len(F)} pair blocks from {len(mols)} clusters ({t_data:.1f} s of SCF)")
    t0 = time.perf_counter()
    net = G.train(F, Y, M, epochs=args.epochs, log=print, gb=gb)
    t_train = time.perf_counter() - t0
    os.makedirs(args.out, exist_ok=True)
    net.save(os.path.join(args.out, os.path.basename(gb.weights)))
    net.save()
    ev = evaluate(net, eval_geoms, basis=args.basis)
    report = {"train_molecules": len(mols), "pair_blocks": int(len(F)), "data_scf_s": t_data, "train_s": t_train,
              "epochs": args.epochs, "loss_history": net.history, "evaluation": ev}
    with open(os.path.join(args.out, "guess_report.json"), "w") as f:
        json.dump(report, f, indent=1)
    print(json.dumps({k: v for k, v in ev.items() if not isinstance(v, list)}))


if __name__ == "__main__":
    main()
