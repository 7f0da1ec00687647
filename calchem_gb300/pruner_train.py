"""Generates the pruner's training data on the GPU and trains its network with the library's
kernels: ``python -m calchem_gb300.pruner_train --out calchem_gb300/data/pruner_mlp.json``.

The data (per-atom log10 quadrature errors of every candidate level against the Fine grid, for the
seeded molecules of ``pruner.training_set``) are written beside the model as ``.npz`` when
``--samples`` is given, and read back from there with ``--reuse``."""

import argparse
import json
import sys
import time

import numpy as np

from . import pruner


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=pruner.MODEL_PATH)
    ap.add_argument("--samples", default=None, help=".npz file for the generated samples")
    ap.add_argument("--reuse", action="store_true", help="train on the samples in --samples")
    ap.add_argument("--steps", type=int, default=4000)
    ap.add_argument("--lr", type=float, default=3e-3)
    ap.add_argument("--seed", type=int, default=0)
    a = ap.parse_args(argv)
    log = lambda s: print(s, flush=True)
    t0 = time.time()
    if a.reuse and a.samples:
        z = np.load(a.samples)
        samples = (z["X"], z["Y"], z["mol"])
    else:
        log("generating samples (GPU, FP64 per-atom shares)")
        samples = pruner.generate_samples(log=log)
        if a.samples:
            np.savez(a.samples, X=samples[0], Y=samples[1], mol=samples[2])
    t1 = time.time()
    log(f"{len(samples[0])} atom samples in {t1 - t0:.1f} s; training")
    net, stats = pruner.train(samples, steps=a.steps, lr=a.lr, log=log, seed=a.seed)
    stats["data_seconds"] = round(t1 - t0, 2)
    stats["train_seconds"] = round(time.time() - t1, 2)
    stats["molecules"] = int(samples[2].max() + 1)
    with open(a.out, "w") as f:
        json.dump(net.to_json(training=stats), f)
    log(json.dumps({k: v for k, v in stats.items() if k != "loss_history"}))
    return 0


if __name__ == "__main__":
    sys.exit(main())
