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
        if "f_" + k in z.files:
            setattr(m, k, np.array(z["f_" + k]))
    if "global_histogram" in meta:
        m.global_histogram = dict(meta["global_histogram"])
    for k, v in meta["scalars"].items():
        setattr(m, k, int(v) if k in ("use_maxwell", "constant_flow", "enable_decay", "low_flux_mode", "n_structures") else v)
    if "moment_time" in z.files and len(z["moment_time"]):
        m.set_moments(z["moment_time"], z["moment_window"])
    for k in z.files:
        if k.startswith("desorb_am_"):
            m.desorb_anglemaps[int(k[10:])] = np.array(z[k])
    i = 0
    while "param_%d" % i in z.files:
        tv = z["param_%d" % i]
        lx, ly = z["param_%d_log" % i]
        m.add_param(tv[0], tv[1], logx=bool(lx), logy=bool(ly))
        i += 1
    ref = {k: z[k] for k in z.files if k.startswith("ref_")}
    return m, ref, meta
