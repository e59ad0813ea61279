"""Autotune the batched LU's launch shapes on this GPU and write the tile table.

    python marinehydro.jl_gb300/data/autotune_tiles.py [--out FILE] [--sizes 384,768,1536,3072]
                                                       [--batch 16] [--reps 3]

For each precision (fp64, mixed, fp64_tc) and matrix order, mh_autotune times the
factorization of `batch` random complex matrices with every candidate shape (panel
cluster bound 8 / 4 / 2; 1 / 2 / 4 / 8 column tiles per CTA of the BF16x3 update; the
FP64 tensor-core update is a persistent kernel and has no shape to tune) and keeps the
fastest per order bucket.  The defaults are the settings of
the table shipped in this directory (tile_table_gb300.json, made on a GB300).  Load
a table with marinehydro_gb300.load_tile_table(path).  Needs a CUDA device.
"""
from __future__ import annotations

import argparse
import importlib.util
import json
import os
import sys
import time

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


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.join(HERE, "tile_table_gb300.json"))
    ap.add_argument("--sizes", default="384,768,1536,3072")
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--reps", type=int, default=3)
    a = ap.parse_args()
    mh = _package()
    t0 = time.time()
    rep = mh.autotune(sizes=[int(s) for s in a.sizes.split(",")], batch=a.batch, reps=a.reps, path=a.out)
    print(json.dumps({"seconds": round(time.time() - t0, 1), "table": rep["table"], "ms": rep["ms"]}, indent=1))


if __name__ == "__main__":
    main()
