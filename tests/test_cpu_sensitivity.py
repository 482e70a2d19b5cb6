"""The score-function estimator of the sensitivity kernel, restated in the oracle, against central
finite differences of the oracle with common random numbers (CPU).

A short tube whose wall is 4 rings of 8 facets: the 8 facets of ring 1 are the parameters
(sticking 0.02-0.2), two facets of ring 3 are gauges.  Large facets see many hits, so the finite
differences have enough flipped stick/reflect decisions to be precise."""
import math

import numpy as np

from molflow_sources_gb300 import _abi as A
from molflow_sources_gb300.model import Model
from oracle.oracle import Oracle
from tests.stats import z_threshold

SEED = 0x4D6F6C66


def ring_tube(n_around=8, n_rings=4, L=4.0, R=1.0):
    ang = np.arange(n_around) / n_around * 2 * math.pi
    zs = np.linspace(0.0, L, n_rings + 1)
    V = np.array([[R * math.cos(a), R * math.sin(a), z] for z in zs for a in ang])
    vid = lambda k, i: k * n_around + (i % n_around)
    facets = [[vid(0, i) for i in range(n_around)], [vid(n_rings, n_around - 1 - i) for i in range(n_around)]]
    for k in range(n_rings):
        for i in range(n_around):
            facets.append([vid(k, i), vid(k + 1, i), vid(k + 1, i + 1), vid(k, i + 1)])
    m = Model(V, facets)
    m.sticking[0] = m.sticking[1] = 1.0
    m.desorb_type[0] = A.DES_COSINE
    m.outgassing[0] = 1.0
    m.neg = np.arange(2 + n_around, 2 + 2 * n_around)
    m.sticking[m.neg] = np.linspace(0.02, 0.2, n_around)
    m.gauges = np.array([2 + 3 * n_around, 2 + 3 * n_around + n_around // 2])
    return m


def outputs(st, m, n):
    y = np.zeros(9)
    y[:len(m.gauges)] = st.facet_sums[0, m.gauges, A.FS_SUM_V_ORT] / n
    y[8] = st.facet_counts[0, m.neg, A.FC_NBABSORBED].sum() / n
    return y


def test_score_function_outputs_equal_plain_tallies():
    m = ring_tube()
    n = 50000
    y, _ = Oracle(m).run_sens(n, m.neg, m.gauges, m.neg, seed=SEED)
    st, _ = Oracle(m).run(n, seed=SEED)
    np.testing.assert_allclose(y, outputs(st, m, n), rtol=1e-12, atol=1e-15)


def test_score_function_matches_central_differences():
    m = ring_tube()
    orc = Oracle(m)
    nb, n = 8, 100000
    js = np.array([orc.run_sens(n, m.neg, m.gauges, m.neg, seed=SEED, first_particle=b * n)[1] for b in range(nb)])
    jm, jse = js.mean(0), js.std(0, ddof=1) / math.sqrt(nb)
    zs = []
    for k, f in enumerate(m.neg):
        s0 = float(m.sticking[f])
        ds = 0.25 * s0
        fd = []
        for b in range(nb):
            ys = []
            for s in (s0 + ds, s0 - ds):
                mm = ring_tube()
                mm.sticking[f] = s
                st, _ = Oracle(mm).run(n, seed=SEED, first_particle=b * n)   # common random numbers
                ys.append(outputs(st, mm, n))
            fd.append((ys[0] - ys[1]) / (2 * ds))
        fd = np.array(fd)
        fm, fse = fd.mean(0), fd.std(0, ddof=1) / math.sqrt(nb)
        for j in (0, 1, 8):
            zs.append((jm[k, j] - fm[j]) / math.hypot(jse[k, j], fse[j]))
            assert abs(jm[k, j]) > 3 * jse[k, j]    # every gradient here is resolved
    zs = np.array(zs)
    assert np.abs(zs).max() < z_threshold(len(zs)) + 0.5, np.round(zs, 2)
