"""Train the learned Delhommeau wave-term surrogate and write its parameters.

    python marinehydro.jl_gb300/data/train_surrogate.py [--out DIR] [--samples N] [--seed S]
                                                       [--epochs E] [--batch B] [--lr LR]

Writes DIR/surrogate_delhommeau.npy (the packed float32 parameters, BF16-rounded) and
DIR/surrogate_delhommeau.json (the training settings and the held-out error report
of mh_surrogate_train).  The defaults are the settings of the parameters shipped in
this directory: 1e7 samples of the exact kernel, seed 2026, 30 epochs of batch 8192,
learning rate 3e-3 with cosine decay.  Needs a CUDA device.
"""
from __future__ import annotations

import argparse
import importlib.util
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)


def _package():
    if "marinehydro_gb300" in sys.modules:
        return sys.modules["marinehydro_gb300"]
    spec = importlib.util.spec_from_file_location("marinehydro_gb300", os.path.join(PKG, "__init__.py"),
                                                  submodule_search_locations=[PKG])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["marinehydro_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--out", default=HERE)
    ap.add_argument("--samples", type=int, default=10_000_000)
    ap.add_argument("--seed", type=int, default=2026)
    ap.add_argument("--epochs", type=int, default=30)
    ap.add_argument("--batch", type=int, default=8192)
    ap.add_argument("--lr", type=float, default=3e-3)
    a = ap.parse_args(argv)
    mh = _package()
    ctx = mh.default_context()
    t0 = time.perf_counter()
    params, report = ctx.surrogate_train(a.samples, a.seed, a.epochs, a.batch, a.lr)
    wall = time.perf_counter() - t0
    os.makedirs(a.out, exist_ok=True)
    np.save(os.path.join(a.out, "surrogate_delhommeau.npy"), params.astype(np.float32))
    meta = {"samples": a.samples, "seed": a.seed, "epochs": a.epochs, "batch": a.batch, "lr": a.lr,
            "wall_seconds": round(wall, 3), "report": report}
    with open(os.path.join(a.out, "surrogate_delhommeau.json"), "w") as f:
        json.dump(meta, f, indent=1)
    print(json.dumps(meta))


if __name__ == "__main__":
    main()
