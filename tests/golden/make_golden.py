"""Generate the golden fixtures in this folder from the reference's test cases.

Reads the MolFlow+ test cases shipped with the reference
(tests/TestCases/*.zip of szakeetm/molflow_sources: geometry + a converged
GlobalSimuState) with molflow_sources_gb300.xmlio and stores, per case, the
model arrays and a subset of the stored results as a compressed .npz.

Run in a checkout next to the reference sources (the reference's parameter catalog,
copy_to_build/parameter_catalog, is read from the same tree); the test-case folder is a
required argument:
    python tests/golden/make_golden.py <reference>/tests/TestCases [case ...]
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
    # time-dependent parameters, moments, angle maps, decay, sojourn time: per-moment hits kept
    "02-timedependent_with_two_parameters": {"tex": [], "prof": [], "moments": True},
    "02b-timedependent_with_three_parameters": {"tex": [], "prof": [], "moments": True},
    "02c-timedependent_temperature": {"tex": [], "prof": [], "moments": True},
    "03-anglemap_record": {"tex": [], "prof": [], "anglemap": True},
    "03b-anglemap_record_transparent_target": {"tex": [], "prof": [], "anglemap": True},
    "07-volume_decay": {"tex": [], "prof": [], "moments": True},
    "08-wall_sojourn_time": {"tex": [], "prof": [], "moments": True},
    "09-histograms": {"tex": [], "prof": [], "moments": True},
    "05-three_structures_nonsquare_textures": {"tex": "all", "prof": "all"},
    "04-anglemap_desorb": {"tex": [], "prof": []},
    "04b-anglemap_desorb-sticking source": {"tex": [], "prof": []},
}


def save_case(src_dir, name, keep, catalog):
    m, st, info = xmlio.load(os.path.join(src_dir, name + ".zip"), catalog=catalog)
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
    out["moment_time"] = m.moment_time
    out["moment_window"] = m.moment_window
    for i, (t, v, lx, ly) in enumerate(m.params):
        out["param_%d" % i] = np.stack([t, v])
        out["param_%d_log" % i] = np.array([lx, ly], np.int32)
    if keep.get("moments"):
        out["ref_hits_moments"] = st.facet_counts[..., 0].astype(np.float64)   # nbMCHit, moment 0 and each moment
    if keep.get("anglemap"):
        out["ref_anglemap"] = st.anglemap
    if st.histogram.size:
        out["ref_histogram"] = st.histogram
    for f, amap in m.desorb_anglemaps.items():   # recorded maps that angle-map sources desorb by
        out["desorb_am_%d" % f] = amap
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
                                            "global_histogram": {k: (int(v) if k in ("record", "bounce_binsize", "bounce_max") else float(v))
                                                                 for k, v in m.global_histogram.items()},
                                            "source": "tests/TestCases/%s.zip" % name}).encode(), dtype=np.uint8)
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path))


if __name__ == "__main__":
    if len(sys.argv) < 2:
        sys.exit("usage: make_golden.py <reference tests/TestCases folder> [case ...]")
    src = sys.argv[1]
    # the parameter catalog shipped next to the test cases (copy_to_build/parameter_catalog)
    catalog = xmlio.load_catalog(os.path.join(src, "..", "..", "copy_to_build", "parameter_catalog"))
    only = sys.argv[2:]
    for name, keep in CASES.items():
        if not only or name in only:
            save_case(src, name, keep, catalog)
