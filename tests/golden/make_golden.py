"""Generate the golden fixtures in this folder from the reference's test cases.

Reads the MolFlow+ test cases shipped with the reference
(tests/TestCases/*.zip of szakeetm/molflow_sources: geometry + a converged
GlobalSimuState) with molflow_sources_gb300.xmlio and stores, per case, the
model arrays and a subset of the stored results as a compressed .npz.

Run in a checkout next to the reference sources:
    python tests/golden/make_golden.py /root/reference/tests/TestCases
The .npz files are committed; tests never read the reference tree.
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from molflow_sources_gb300 import xmlio  # noqa: E402
from molflow_sources_gb300.model import FACET_FIELDS  # noqa: E402

# case -> facets whose textures / profiles are kept (all facets' counters are kept)
CASES = {
    "01-quick_pipe_profiles_textures_2sided": {"tex": "all", "prof": "all"},
    "B01-lr1000_pipe": {"tex": [], "prof": "all"},
    "B02-lr10_pipe_tex": {"tex": [2, 252, 502, 752, 1001], "prof": []},
    "B03-lr10_pipe_prof": {"tex": [], "prof": [2, 252, 502, 752, 1001]},
    "B04-lr10_pipe_trans": {"tex": [0, 1, 2, 500, 1001, 1002, 1003, 1004], "prof": []},
}


def save_case(src_dir, name, keep):
    m, st, info = xmlio.load(os.path.join(src_dir, name + ".zip"))
    L = st.L
    out = {
        "vertices": m.vertices,
        "facet_vertex_start": m.facet_vertex_start,
        "facet_vertex_index": m.facet_vertex_index,
        "ref_global": st.global_,
        "ref_facet_counts": st.facet_counts[0],
        "ref_facet_sums": st.facet_sums[0],
    }
    for k in FACET_FIELDS:
        out["f_" + k] = getattr(m, k)
    scalars = {k: float(getattr(m, k)) for k in ("gas_mass", "use_maxwell", "constant_flow", "time_window",
                                                    "enable_decay", "half_life", "low_flux_mode",
                                                    "low_flux_cutoff", "n_structures")}
    tex_f = [i for i in range(m.n_facets) if L["tex_off"][i] >= 0] if keep["tex"] == "all" else keep["tex"]
    prof_f = [i for i in range(m.n_facets) if L["prof_idx"][i] >= 0] if keep["prof"] == "all" else keep["prof"]
    for i in tex_f:
        out["ref_tex_%d" % i] = st.texture_of(i)
    for i in prof_f:
        out["ref_prof_%d" % i] = st.profile_of(i)
    out["meta"] = np.frombuffer(json.dumps({"scalars": scalars, "tex_facets": tex_f, "prof_facets": prof_f,
                                            "source": "tests/TestCases/%s.zip" % name}).encode(), dtype=np.uint8)
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path))


if __name__ == "__main__":
    src = sys.argv[1] if len(sys.argv) > 1 else "/root/reference/tests/TestCases"
    only = sys.argv[2:]
    for name, keep in CASES.items():
        if not only or name in only:
            save_case(src, name, keep)
