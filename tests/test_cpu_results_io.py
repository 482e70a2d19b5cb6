"""Results on the host (CPU): the XML writer against the XML reader, the reference's Compare rule,
and the CSV exporter's derived quantities.

* A result written as a MolFlow+ file and read back is the same result (every array), and the
  geometry and settings come back unchanged.
* compare_states (GlobalSimuState::Compare) passes two runs of the same model, flags a run of a
  model with a different outlet sticking, and passes an oracle run against the reference's own
  stored state of test case B02.
* Facet physics (CSVExporter): the density correction's limiting values, and on the wall of the
  L/R = 10 tube the kinetic-gas relations p = n k T, p = J sqrt(2 pi m k T) and the mean speed of a
  Maxwell gas hold to 1 %; the CSV table has one line per facet and a constant column count.
"""
import math

import numpy as np
import pytest

from molflow_sources_gb300 import _abi as A
from molflow_sources_gb300 import compare, physics, xmlio, xmlwriter
from molflow_sources_gb300.model import SimuState
from molflow_sources_gb300.simulation import GpuModel
from molflow_sources_gb300.workloads import config1_tube
from oracle.oracle import Oracle
from tests import golden_util

ARRAYS = ("global_", "facet_counts", "facet_sums", "texture", "profile", "direction", "anglemap", "histogram")


@pytest.mark.parametrize("case", ["01-quick_pipe_profiles_textures_2sided", "02-timedependent_with_two_parameters",
                                  "05-three_structures_nonsquare_textures", "09-histograms", "B02-lr10_pipe_tex"])
def test_written_result_reads_back_the_same(case, tmp_path):
    m, _, _ = golden_util.load(case)
    st, _ = Oracle(m).run(20000, seed=5)
    gm = GpuModel(m)
    path = str(tmp_path / (case + ".zip"))
    xmlwriter.save(path, m, st, gm.outgassing(), gm.facet_geometry()[1])
    m2, st2, info = xmlio.load(path)
    for k in ARRAYS:
        assert np.array_equal(getattr(st, k), getattr(st2, k)), k
    for k in ("sticking", "opacity", "outgassing", "temperature", "desorb_type", "tex_width", "tex_height",
              "count_flags", "profile_type", "structure", "link_dest", "is_2sided", "sticking_param",
              "outgassing_param", "opacity_param", "hist_record", "anglemap_record"):
        assert np.array_equal(getattr(m, k), getattr(m2, k)), k
    np.testing.assert_array_equal(m.vertices, m2.vertices)
    assert m.facets == m2.facets
    np.testing.assert_array_equal(m.moment_time, m2.moment_time)
    assert [tuple(map(tuple, p[:2])) for p in m.params] == [tuple(map(tuple, p[:2])) for p in m2.params]
    assert compare.compare_states(st, st2)[:3] == (0, 0, 0)


def _stored_state(m, ref):
    """A stored test-case state (global counters, facet buffers, the kept textures) as a SimuState."""
    st = SimuState(m)
    st.global_[:] = ref["ref_global"]
    fc = ref["ref_facet_counts"].reshape(-1, m.n_facets, A.FC_N)
    fs = ref["ref_facet_sums"].reshape(-1, m.n_facets, A.FS_N)
    st.facet_counts[:fc.shape[0]] = fc
    st.facet_sums[:fs.shape[0]] = fs
    L = st.L
    for k in ref:
        if k.startswith("ref_tex_"):
            f = int(k.split("_")[-1])
            o, n = int(L["tex_off"][f]), int(L["tex_w"][f] * L["tex_h"][f])
            t = ref[k].reshape(-1, n, 3)
            st.texture[:t.shape[0], o:o + n] = t
    return st


def test_compare_rule_passes_same_model_and_flags_a_different_one():
    m, ref, _ = golden_util.load("B02-lr10_pipe_tex")
    a, _ = Oracle(m).run(200000, seed=5)
    b, _ = Oracle(m).run(200000, seed=5, first_particle=10 ** 9)
    assert compare.compare_states(a, b)[:2] == (0, 0)
    m2, _, _ = golden_util.load("B02-lr10_pipe_tex")
    m2.sticking[1] = 0.5   # outlet half as absorbing
    c, _ = Oracle(m2).run(200000, seed=5)
    g, f, fine, msgs = compare.compare_states(a, c)
    assert g > 0 and any("absRatio" in s or "hits/des" in s for s in msgs)


def test_compare_rule_oracle_against_stored_b02():
    m, ref, _ = golden_util.load("B02-lr10_pipe_tex")
    run, _ = Oracle(m).run(400000, seed=5)
    stored = _stored_state(m, ref)
    g, f, fine, msgs = compare.compare_states(stored, run, 0.009, 0.07)
    assert (g, f) == (0, 0), msgs[:5]


def test_is_equal_is_relative_to_the_larger_value():
    assert compare.is_equal(0.0, 0.0, 0.01)
    assert compare.is_equal(100.0, 100.9, 0.01)
    assert not compare.is_equal(100.0, 101.1, 0.01)
    assert not compare.is_equal(0.0, 1e-30, 0.01)


def test_density_correction_limits():
    # no desorption and no absorption: 1; only desorption: 0.5; absorbing half the hits: 0.75
    np.testing.assert_allclose(physics.density_correction([10, 0, 10], [0, 10, 0], [10.0, 0.0, 10.0], [0.0, 0.0, 5.0]),
                               [1.0, 0.5, 0.75])
    assert physics.density_correction([0], [0], [0.0], [0.0])[0] == 1.0


def test_facet_physics_follow_kinetic_gas_relations(tmp_path):
    m = config1_tube()
    st, _ = Oracle(m).run(200000, seed=3)
    gm = GpuModel(m)
    og = gm.outgassing()
    area = gm.facet_geometry()[1]
    q = physics.facet_quantities(m, st, area, og)
    walls = np.arange(2, 66)
    mass = m.gas_mass / 1000.0 / 6e23
    kt = 1.38e-23 * 293.15
    p = q["pressure_mbar"][walls] * 100.0
    assert abs(np.mean(p / (q["density_1p"][walls] * kt)) - 1) < 0.01
    assert abs(np.mean(p / q["impingement_rate"][walls]) / math.sqrt(2 * math.pi * mass * kt) - 1) < 0.01
    assert abs(np.mean(q["avg_speed"][walls]) / math.sqrt(8 * kt / (math.pi * mass)) - 1) < 0.01
    # the molecules one test particle stands for, constant flow: final outgassing rate / desorptions
    assert physics.molecules_per_tp(st, og) == pytest.approx(og["final_outgassing_rate"] / st.n_desorbed)
    path = str(tmp_path / "facet_physics.csv")
    assert physics.write_facet_physics_csv(path, m, st, area, og) == 0
    assert physics.validate_csv(path) == len(physics.PHYSICS_COLUMNS) - 1
    lines = open(path).read().splitlines()
    assert lines[0] == "#,Imping.rate,Pressure [mbar],Density [1/m3],Density [kg/m3],Av.mol.speed[m/s]"
    assert len(lines) == m.n_facets + 1 and lines[1].startswith("1,")
