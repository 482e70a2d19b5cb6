"""The oracle against the reference's stored results of its own test cases (tests/TestCases):
time-dependent sticking and outgassing parameters with moments (02, 02b), angle-map recording
across two structures with transparent facets (03, 03b), volume decay (07), wall sojourn time
(08), a five-moment model (09) three structures joined by link facets (05) and angle-map desorption (04, 04b).  Per-facet hits per desorption in every moment."""
import numpy as np
import pytest

from molflow_sources_gb300 import _abi as A
from oracle import oracle as O
from tests import golden_util
from tests.fixture_compare import assert_hits_agree, hit_rates

SEED = 0x4D6F6C66
NB = 8

CASES = {   # test case -> desorptions per batch (the oracle finishes each case in seconds)
    "02-timedependent_with_two_parameters": 40000,
    "02b-timedependent_with_three_parameters": 20000,
    "03-anglemap_record": 40000,
    "03b-anglemap_record_transparent_target": 40000,
    "07-volume_decay": 20000,
    "08-wall_sojourn_time": 40000,
    "09-histograms": 100000,
    "04-anglemap_desorb": 25000,
    "04b-anglemap_desorb-sticking source": 25000,
    "05-three_structures_nonsquare_textures": 40000,
}


def run_batches(m, n):
    orc = O.Oracle(m)
    return [orc.run(n, seed=SEED, first_particle=b * n)[0] for b in range(NB)]


@pytest.mark.parametrize("case", sorted(CASES))
def test_oracle_hits_per_moment_match_stored_state(case):
    m, ref, _ = golden_util.load(case)
    n = CASES[case]
    states = run_batches(m, n)
    ref_hits = ref["ref_hits_moments"] if "ref_hits_moments" in ref else ref["ref_facet_counts"][None, :, A.FC_NBMCHIT]
    per = hit_rates(states)[:, :ref_hits.shape[0]]
    assert_hits_agree(per, n, ref_hits.astype(np.float64), ref["ref_global"][A.G_NBDESORBED])
    tex = sorted(int(k[8:]) for k in ref if k.startswith("ref_tex_"))
    if tex:   # texture hit counts of the stored facets, every cell
        pt = np.array([np.concatenate([s.texture_of(f)[..., 0].ravel() for f in tex]) / n for s in states])[:, None, :]
        rt = np.concatenate([ref["ref_tex_%d" % f][..., 0].ravel() for f in tex])[None, :]
        assert_hits_agree(pt, n, rt.astype(np.float64), ref["ref_global"][A.G_NBDESORBED])
    if "ref_histogram" in ref:   # bounce / distance / time histograms of absorptions, every moment
        ph = np.array([s.histogram / n for s in states])
        assert_hits_agree(ph, n, ref["ref_histogram"].astype(np.float64), ref["ref_global"][A.G_NBDESORBED])
    if "ref_anglemap" in ref:
        pa = np.array([s.anglemap.astype(np.float64) / n for s in states])[:, None, :]
        assert_hits_agree(pa, n, ref["ref_anglemap"].astype(np.float64)[None, :], ref["ref_global"][A.G_NBDESORBED])
