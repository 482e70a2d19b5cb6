"""Load the golden fixtures (tests/golden/*.npz, made by tests/golden/make_golden.py)."""
import json
import os

import numpy as np

from molflow_sources_gb300.model import FACET_FIELDS, Model

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    meta = json.loads(bytes(z["meta"]).decode())
    vs = z["facet_vertex_start"]
    vi = z["facet_vertex_index"]
    facets = [vi[vs[i]:vs[i + 1]].tolist() for i in range(len(vs) - 1)]
    m = Model(z["vertices"], facets)
    for k in FACET_FIELDS:
        setattr(m, k, np.array(z["f_" + k]))
    for k, v in meta["scalars"].items():
        setattr(m, k, int(v) if k in ("use_maxwell", "constant_flow", "enable_decay", "low_flux_mode", "n_structures") else v)
    ref = {k: z[k] for k in z.files if k.startswith("ref_")}
    return m, ref, meta
