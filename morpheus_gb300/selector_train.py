"""Train and evaluate the learned format selector on the GPU.

    python -m morpheus_gb300.selector_train --train 2000 --test 400 \
        --out morpheus_gb300/selector_weights.bin --report selector_report.json

Builds the synthetic corpus (morpheus_gb300/corpus.py: every format timed
with CUDA events), trains the 12 -> 64 -> 64 -> 6 network with the project's
own gradient and Adam kernels, and evaluates on held-out seeds against
exhaustive timing (regret), against CSR-only, and against the rule-based
selector (DIA / HDC / ELL / CSR by three feature thresholds tuned on the
training set, selector.rule_select).
"""
from __future__ import annotations

import argparse
import collections
import json
import time

import numpy as np

from . import corpus, selector


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
    args = ap.parse_args(argv)

    t0 = time.time()
    tr = corpus.build(args.train, seed0=0, reps=args.reps, log=print)
    te = corpus.build(args.test, seed0=1_000_000, reps=args.reps, log=print)
    t_corpus = time.time() - t0
    if args.corpus_out:
        np.savez_compressed(args.corpus_out, Xtr=tr["X"], Ftr=tr["feasible"], Ttr=tr["times"], Xte=te["X"],
                 Fte=te["feasible"], Tte=te["times"])

    mu, sigma = tr["X"].mean(0), tr["X"].std(0) + 1e-3
    sel = selector.Selector.random(mu, sigma, seed=0)
    t1 = time.time()
    hist = sel.train(tr["X"], tr["labels"], tr["feasible"], epochs=args.epochs, lr=args.lr)
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
        "training": {"epochs": args.epochs, "lr": args.lr, "loss_first": hist[0], "loss_last": hist[-1],
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
