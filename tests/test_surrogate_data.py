"""The shipped surrogate parameters and their training record (CPU only)."""
import json
import os

import numpy as np

DATA = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "marinehydro.jl_gb300", "data")


def test_shipped_parameters():
    p = np.load(os.path.join(DATA, "surrogate_delhommeau.npy"))
    assert p.dtype == np.float32 and p.shape == (8902,)
    assert np.all(np.isfinite(p))
    # BF16-rounded: the low 16 bits of every float32 are zero
    assert np.all((p.view(np.uint32) & 0xFFFF) == 0)
    meta = json.load(open(os.path.join(DATA, "surrogate_delhommeau.json")))
    assert meta["samples"] == 10_000_000 and meta["seed"] == 2026
    rep = meta["report"]
    assert rep["rms_rel_err_G"] < rep["wu_rms_rel_err_G"]
