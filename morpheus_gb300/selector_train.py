"""Train and evaluate the learned format selector on the GPU.

    python -m morpheus_gb300.selector_train --train 2000 --test 400 \
        --out morpheus_gb300/selector_weights.bin --report selector_report.json

Builds the synthetic corpus (morpheus_gb300/corpus.py: every format timed
with CUDA events), trains the 12 -> 64 -> 64 -> 6 network with the project's
own gradient and Adam kernels, and evaluates on held-out seeds against
exhaustive timing (regret), against CSR-only, and against the rule-based
selector (DIA / HDC / ELL / CSR by three feature thresholds tuned on the
training set, selector.rule_select).

--select picks epochs, learning rate and initialisation seed from a small
grid by the mean regret on the last fifth of the training matrices (the
held-out test matrices play no part), then trains on all of them.
--corpus-in reuses a corpus saved by --corpus-out instead of timing a new one.
"""
from __future__ import annotations

import argparse
import collections
import json
import time

import numpy as np

from . import corpus, selector


GRID = {"epochs": (400, 1000, 2000), "lr": (1e-3, 3e-3), "seed": (0, 1, 2)}
def load_corpus(path: str):
    """The training and test parts of a corpus saved with --corpus-out."""
    d = np.load(path)

    def part(X, F, T, D):
        desc = [{"family": str(f)} for f in d[D]] if D in d.files else [{"family": "?"}] * len(d[X])
        return {"X": d[X], "feasible": d[F], "times": d[T], "labels": np.argmin(d[T], axis=1), "desc": desc}
    return part("Xtr", "Ftr", "Ttr", "Dtr"), part("Xte", "Fte", "Tte", "Dte")


def select_hyperparameters(tr, mu, sigma) -> dict:
    """Grid over epochs x learning rate x seed, scored by mean regret on the
    last fifth of the training matrices after training on the rest."""
    n = len(tr["labels"])
    cut = n - n // 5
    fit = {k: tr[k][:cut] for k in ("X", "labels", "feasible", "times")}
    val = {k: tr[k][cut:] for k in ("X", "labels", "feasible", "times")}
    best = None
    for epochs in GRID["epochs"]:
        for lr in GRID["lr"]:
            for seed in GRID["seed"]:
                sel = selector.Selector.random(mu, sigma, seed=seed)
                sel.train(fit["X"], fit["labels"], fit["feasible"], epochs=epochs, lr=lr, seed=seed)
                r = selector.evaluate(val["times"], sel.predict(val["X"], val["feasible"]))["mean_regret"]
                if best is None or r < best["validation_mean_regret"]:
                    best = {"epochs": epochs, "lr": lr, "seed": seed, "validation_mean_regret": r}
    return best


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--train", type=int, default=2000)
    ap.add_argument("--test", type=int, default=400)
    ap.add_argument("--reps", type=int, default=10)
    ap.add_argument("--epochs", type=int, default=400)
    ap.add_argument("--lr", type=float, default=3e-3)
    ap.add_argument("--out", default=selector.DEFAULT_WEIGHTS)
    ap.add_argument("--report", default="selector_report.json")
    ap.add_argument("--corpus-out", default=None)
    ap.add_argument("--corpus-in", default=None)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--select", action="store_true")
    args = ap.parse_args(argv)

    t0 = time.time()
    if args.corpus_in:
        tr, te = load_corpus(args.corpus_in)
    else:
        tr = corpus.build(args.train, seed0=0, reps=args.reps, log=print)
        te = corpus.build(args.test, seed0=1_000_000, reps=args.reps, log=print)
    t_corpus = time.time() - t0
    if args.corpus_out:
        np.savez_compressed(args.corpus_out, Xtr=tr["X"], Ftr=tr["feasible"], Ttr=tr["times"], Xte=te["X"],
                            Fte=te["feasible"], Tte=te["times"],
                            Dtr=np.array([d["family"] for d in tr["desc"]]),
                            Dte=np.array([d["family"] for d in te["desc"]]))

    mu, sigma = tr["X"].mean(0), tr["X"].std(0) + 1e-3
    selection = None
    if args.select:
        selection = select_hyperparameters(tr, mu, sigma)
        args.epochs, args.lr, args.seed = selection["epochs"], selection["lr"], selection["seed"]
        print("selected", json.dumps(selection), flush=True)
    sel = selector.Selector.random(mu, sigma, seed=args.seed)
    t1 = time.time()
    hist = sel.train(tr["X"], tr["labels"], tr["feasible"], epochs=args.epochs, lr=args.lr, seed=args.seed)
    t_train = time.time() - t1

    pred = sel.predict(te["X"], te["feasible"])
    thr = selector.tune_rule(tr["X"], tr["feasible"], tr["times"])
    rule = selector.rule_select(te["X"], te["feasible"], **thr)
    csr_only = np.full(len(pred), 1)
    names = ["COO", "CSR", "DIA", "ELL", "HYB", "HDC"]
    report = {
        "corpus": {"train": args.train, "test": args.test, "nnz_cap": corpus.NNZ_CAP,
                   "families_train": dict(collections.Counter(d["family"] for d in tr["desc"])),
                   "label_counts_train": {names[k]: int(v) for k, v in
                                          sorted(collections.Counter(tr["labels"].tolist()).items())},
                   "label_counts_test": {names[k]: int(v) for k, v in
                                         sorted(collections.Counter(te["labels"].tolist()).items())},
                   "seconds": t_corpus},
        "training": {"epochs": args.epochs, "lr": args.lr, "seed": args.seed, "selection": selection,
                     "loss_first": hist[0], "loss_last": hist[-1],
                     "seconds": t_train, "train_accuracy": float(np.mean(
                         sel.predict(tr["X"], tr["feasible"]) == tr["labels"]))},
        "test": {"learned": selector.evaluate(te["times"], pred),
                 "rule_based": dict(selector.evaluate(te["times"], rule), **thr),
                 "csr_only": selector.evaluate(te["times"], csr_only)},
    }
    sel.save(args.out, {"report": report["test"], "corpus": report["corpus"]["train"]})
    with open(args.report, "w") as f:
        json.dump(report, f, indent=1)
    print(json.dumps(report["test"], indent=1))


if __name__ == "__main__":
    main()
