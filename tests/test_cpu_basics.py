"""CPU tests: oracle known answers, golden pins, library boundary (no GPU needed)."""
import ctypes as C
import math
import os
import re

import numpy as np
import pytest

from molflow_sources_gb300 import _abi as A
from molflow_sources_gb300.model import SimuState, build_pipe, config1_tube
from oracle import oracle as O
from tests import golden_util
from tests.stats import batch_means, binom_sigma, z_threshold

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SEED = 0x4D6F6C66


def test_philox_known_answers():
    # Random123 philox4x32-10 known-answer vectors
    assert O.philox4x32([0, 0, 0, 0], [0, 0]) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert O.philox4x32([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert O.philox4x32([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0]) == \
        [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def test_maxwell_cdf_matches_closed_form():
    v, p = O.maxwell_cdf(28.0)
    assert v[0] == 0 and p[0] == 0 and np.all(np.diff(p) > 0) and p[-1] > 0.99999
    a = math.sqrt(1.38e-23 / (28.0 * 1.67e-27))
    y = v ** 2 / (2 * a * a)
    np.testing.assert_allclose(p, 1 - np.exp(-y) * (1 + y), rtol=1e-12, atol=1e-15)


def test_oracle_pipe_geometry():
    m = config1_tube()
    geo, area = O.Oracle(m).facet_geometry()
    assert np.allclose(geo[0, 9:12], [0, 0, 1]) and np.allclose(geo[1, 9:12], [0, 0, -1])
    # wall normals point inward, U along the tube axis (first polygon edge)
    c = np.array([0.0, 0.0, 5.0])
    for i in range(2, 66):
        cen = geo[i, 0:3] + 0.5 * geo[i, 3:6] + 0.5 * geo[i, 6:9]
        assert np.dot(geo[i, 9:12], c - cen) > 0
        assert np.allclose(geo[i, 3:6], [0, 0, 10])
    np.testing.assert_allclose(area[0], 0.5 * 64 * math.sin(2 * math.pi / 64), rtol=1e-12)


def test_oracle_is_thread_count_independent():
    m = build_pipe(step=12)
    orc = O.Oracle(m)
    a, _ = orc.run(3000, seed=SEED, threads=1)
    b, _ = orc.run(3000, seed=SEED, threads=4)
    assert np.array_equal(a.facet_counts, b.facet_counts)
    np.testing.assert_allclose(a.facet_sums, b.facet_sums, rtol=1e-12)


def test_oracle_pinned_to_quick_pipe_fixture():
    """01-quick_pipe: transmission, per-facet hits/des, U profile vs the reference's converged state."""
    m, ref, _ = golden_util.load("01-quick_pipe_profiles_textures_2sided")
    n = 200000
    st, _ = O.Oracle(m).run(n, seed=SEED)
    n_ref = ref["ref_global"][A.G_NBDESORBED]
    p_ref = ref["ref_facet_counts"][1, A.FC_NBABSORBED] / n_ref
    p = st.transmission(1)
    assert abs(p - p_ref) < 3 * math.hypot(binom_sigma(p, n), binom_sigma(p_ref, n_ref))
    hits_ref = ref["ref_facet_counts"][:, A.FC_NBMCHIT] / n_ref
    hits = st.facet_counts[0, :, A.FC_NBMCHIT] / n
    assert np.all(np.abs(hits - hits_ref) < 4 * np.sqrt(hits / n) + 1e-12)
    # pressure-like sums per hit are pinned by the Maxwell speeds and the cosine law
    for f in (2, 3, 4, 5, 6):
        a = st.facet_sums[0, f, A.FS_SUM_V_ORT] / st.facet_counts[0, f, A.FC_NBMCHIT]
        b = ref["ref_facet_sums"][f, A.FS_SUM_V_ORT] / ref["ref_facet_counts"][f, A.FC_NBMCHIT]
        assert abs(a / b - 1) < 0.01, (f, a, b)
    prof = st.profile_of(4)[:, 0] / n
    pr = ref["ref_prof_4"][:, 0] / n_ref
    z = (prof - pr) / np.sqrt(prof / n + pr / n_ref)
    assert np.abs(z).max() < z_threshold(100) + 1.0
    tex = st.texture_of(3)[..., 0] / n
    tr = ref["ref_tex_3"][..., 0] / n_ref
    zt = (tex - tr) / np.sqrt(tex / n + tr / n_ref + 1e-30)
    assert np.abs(zt).max() < z_threshold(600) + 1.0


def test_oracle_pinned_to_b02_transmission():
    m, ref, _ = golden_util.load("B02-lr10_pipe_tex")
    n = 100000
    st, _ = O.Oracle(m).run(n, seed=SEED)
    n_ref = ref["ref_global"][A.G_NBDESORBED]
    p_ref = ref["ref_facet_counts"][1, A.FC_NBABSORBED] / n_ref
    p = st.transmission(1)
    assert abs(p - p_ref) < 3 * math.hypot(binom_sigma(p, n), binom_sigma(p_ref, n_ref))
    assert st.global_[A.G_NBLEAK] == 0


def test_oracle_pinned_to_b01_long_tube():
    m, ref, _ = golden_util.load("B01-lr1000_pipe")
    n = 30000
    st, s = O.Oracle(m).run(n, seed=SEED)
    n_ref = ref["ref_global"][A.G_NBDESORBED]
    p_ref = ref["ref_facet_counts"][1, A.FC_NBABSORBED] / n_ref
    p = st.transmission(1)
    assert abs(p - p_ref) < 3 * math.hypot(binom_sigma(p, n), binom_sigma(p_ref, n_ref))


def b04_compare(st, n, ref):
    """Per-desorption hits on B04's transparent and opaque facets against the stored state.

    B04 stacks three identical L/R=10 tubes: the first two are transparent (opacity 0),
    the third opaque.  Transparent passes are counted as hits (RegisterTransparentPass)."""
    n_ref = ref["ref_global"][A.G_NBDESORBED]
    fc_ref = ref["ref_facet_counts"]
    fc = st.facet_counts[0]
    groups = {"in1": [0], "out1": [1], "in2": [1002], "out2": [1003], "in3": [2004], "out3": [2005],
              "walls1": list(range(2, 1002)), "walls2": list(range(1004, 2004))}
    z = {}
    for name, fs in groups.items():
        a = fc[fs, A.FC_NBMCHIT].sum() / n
        b = fc_ref[fs, A.FC_NBMCHIT].sum() / n_ref
        z[name] = (a - b) / math.sqrt(a / n + b / n_ref)
    # texture of a transparent facet counts the passes (countTrans)
    for f in (0, 1002):
        a = st.texture_of(f)[..., 0].sum() / n
        b = ref["ref_tex_%d" % f][..., 0].sum() / n_ref
        z["tex%d" % f] = (a - b) / math.sqrt(a / n + b / n_ref)
    return z


def test_oracle_pinned_to_b04_transparent_tubes():
    m, ref, _ = golden_util.load("B04-lr10_pipe_trans")
    assert (m.opacity[:2004] == 0).all() and (m.opacity[2004:] == 1).all()
    n = 200000
    st, s = O.Oracle(m).run(n, seed=SEED)
    assert s["leaks"] == 0
    z = b04_compare(st, n, ref)
    assert max(abs(v) for v in z.values()) < z_threshold(len(z)), z


def test_oracle_negative_control_detects_wrong_sticking():
    """The comparator must reject a wrong model (cf. the reference's ResultsWrong test)."""
    m, ref, _ = golden_util.load("01-quick_pipe_profiles_textures_2sided")
    m.sticking[2:] = 0.01
    n = 100000
    st, _ = O.Oracle(m).run(n, seed=SEED)
    n_ref = ref["ref_global"][A.G_NBDESORBED]
    p_ref = ref["ref_facet_counts"][1, A.FC_NBABSORBED] / n_ref
    assert abs(st.transmission(1) - p_ref) > 3 * math.hypot(binom_sigma(p_ref, n), binom_sigma(p_ref, n_ref))


def test_xml_reader_matches_fixture_arrays():
    m, ref, meta = golden_util.load("01-quick_pipe_profiles_textures_2sided")
    assert m.n_facets == 7 and m.is_2sided[5] == 1 and m.profile_type[4] == A.PROFILE_U
    assert m.tex_width[3] == 50 and abs(m.tex_height[3] - 11.7557) < 1e-3
    L = m.layout()
    assert L["texture_cells"] == 600 and L["profile_facets"] == 1


# ------------------------------------------------------------------ ABI ---
def _declared_functions():
    src = open(os.path.join(ROOT, "include", "mfg.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(mfg_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    from molflow_sources_gb300.simulation import load_library
    L = load_library()
    names = _declared_functions()
    assert len(names) >= 19
    for n in names:
        assert hasattr(L, n), n
    assert L.mfg_abi_version() == A.MFG_ABI_VERSION


def test_library_model_prep_matches_oracle_and_layout():
    from molflow_sources_gb300.simulation import GpuModel
    for m in (config1_tube(), golden_util.load("01-quick_pipe_profiles_textures_2sided")[0]):
        g = GpuModel(m)
        o = O.Oracle(m)
        ga, aa = g.facet_geometry()
        oa, ob = o.facet_geometry()
        np.testing.assert_allclose(ga, oa, atol=1e-12)
        np.testing.assert_allclose(aa, ob, rtol=1e-12)
        lg, lo = g.layout(), o.layout()
        assert lg == lo
        L = m.layout()
        assert lg["texture_cells"] == L["texture_cells"] and lg["profile_facets"] == L["profile_facets"]


def test_library_rejects_bad_models_without_gpu():
    from molflow_sources_gb300.simulation import GpuModel, MfgError
    m = config1_tube()
    m.facet_vertex_index[0] = 10 ** 6
    with pytest.raises(MfgError) as e:
        GpuModel(m)
    assert e.value.code == A.MFG_ERR_INVALID_MODEL
    bad = build_pipe(step=8)
    bad.structure[0] = 5
    with pytest.raises(MfgError):
        GpuModel(bad)


def test_sim_create_without_device_fails_cleanly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from molflow_sources_gb300.simulation import GpuSimulation, MfgError
    with pytest.raises(MfgError) as e:
        GpuSimulation(config1_tube())
    assert e.value.code == A.MFG_ERR_NO_DEVICE


def test_counts_for_unsigned_arguments():
    """Particle counts and ids go to unsigned 64-bit C arguments: a negative number is refused
    instead of wrapping to 2^64 - n."""
    from molflow_sources_gb300.simulation import _count
    assert _count(0) == 0 and _count(2 ** 64 - 1) == 2 ** 64 - 1
    for bad in (-1, 2 ** 64):
        with pytest.raises(ValueError):
            _count(bad)
