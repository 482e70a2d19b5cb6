"""Parity on the other benchmark workloads as configured, through the C ABI.

* Transient tube (1 ms pulse, 100 log-spaced moments with 1e-5 s windows): FP64 kernel equals
  the oracle on the same particles in every moment block; FP32R hits per moment and facet
  within 3 standard errors of oracle batches.
* The 256-instance batch (tubes, elbows, T-junctions of 1k-50k facets): FP64 tallies of every
  instance equal the oracle's run of that instance.
* The 1000-parameter sensitivity tube: score-function gradients of all 9 outputs against
  central differences with common random numbers, for the strongest parameters and 20 drawn at
  random.
"""
import math

import numpy as np
import pytest

from molflow_sources_gb300 import _abi as A
from molflow_sources_gb300 import batch_workloads as BW
from molflow_sources_gb300.sensitivity import SensitivityFunction, config5_neg_tube
from molflow_sources_gb300.simulation import GpuBatch, GpuSimulation
from molflow_sources_gb300.workloads import config3_transient
from oracle.oracle import Oracle
from tests.stats import z_threshold

pytestmark = pytest.mark.gpu
SEED = 0x4D6F6C66


def test_c3_fp64_equals_oracle_in_every_moment():
    m = config3_transient()
    assert len(m.moment_time) == 100
    n = 30000
    sim = GpuSimulation(m)
    sim.SimulationMCStep(n, precision=A.PREC_FP64, seed=SEED)
    g = sim.fetch()
    r, _ = Oracle(m).run(n, seed=SEED)
    assert g.facet_counts.shape[0] == 101
    assert g.facet_counts[1:, :, A.FC_NBMCHIT].sum() > 0
    assert np.array_equal(g.facet_counts, r.facet_counts)
    assert np.array_equal(g.texture[..., 0], r.texture[..., 0])
    np.testing.assert_allclose(g.facet_sums, r.facet_sums, rtol=1e-8, atol=1e-6)
    sim.close()


def test_c3_fp32r_hits_per_moment_within_3_sigma():
    m = config3_transient()
    sim = GpuSimulation(m)
    nb_g, n_g = 8, 1_000_000
    gpu = []
    for b in range(nb_g):
        sim.ResetSimulation()
        sim.set_particle_offset(10 ** 10 + b * n_g)
        sim.SimulationMCStep(n_g, precision=A.PREC_FP32R, seed=SEED)
        gpu.append(sim.fetch().facet_counts[..., A.FC_NBMCHIT].astype(np.float64) / n_g)
    sim.close()
    orc = Oracle(m)
    nb_o, n_o = 8, 250_000
    ora = [orc.run(n_o, seed=SEED, first_particle=10 ** 12 + b * n_o)[0].facet_counts[..., A.FC_NBMCHIT]
           .astype(np.float64) / n_o for b in range(nb_o)]
    gpu, ora = np.array(gpu), np.array(ora)
    # hits per moment (all facets): batch-means errors with a Poisson floor (late windows hold
    # few hits, where a batch variance of a handful of counts says little)
    a, b = gpu.sum(2), ora.sum(2)
    ma, mb = a.mean(0), b.mean(0)
    ng, no = nb_g * n_g, nb_o * n_o
    floor = np.maximum(np.maximum(ma, mb), 1.0 / no)
    sa = np.maximum(a.std(0, ddof=1) / math.sqrt(nb_g), np.sqrt(floor / ng))
    sb = np.maximum(b.std(0, ddof=1) / math.sqrt(nb_o), np.sqrt(floor / no))
    z = (ma - mb) / np.sqrt(sa ** 2 + sb ** 2)
    live = (ma + mb) > 0
    w = int(np.argmax(np.abs(z) * live))
    print("C3 hits per moment: %d live moments, max |z| %.2f at block %d (FP32R %.4g, oracle %.4g hits per desorption)"
          % (int(live.sum()), np.abs(z[live]).max(), w, ma[w], mb[w]))
    assert live.sum() > 50
    assert np.abs(z[live]).max() < z_threshold(int(live.sum())) + 0.5, np.abs(z[live]).max()
    # per moment and facet: pooled Poisson
    cg, co = gpu.sum(0) * n_g, ora.sum(0) * n_o
    pool = (cg + co) / (ng + no)
    zz = np.where(cg + co > 0, (cg / ng - co / no) / np.sqrt(np.maximum(pool, 1e-300) * (1 / ng + 1 / no)), 0.0)
    k = int(((cg + co) > 0).sum())
    spread = float(np.mean(zz[(cg + co) > 0] ** 2))
    print("C3 hits per moment and facet: %d cells, mean z^2 %.3f, max |z| %.2f" % (k, spread, np.abs(zz).max()))
    assert spread < 1.3
    assert np.abs(zz).max() < (z_threshold(k) + 0.5) * math.sqrt(max(1.0, spread))


def test_c4_fp64_every_instance_equals_oracle():
    models = BW.config4_batch()
    assert len(models) == 256
    b = GpuBatch(models)
    n = 200
    b.run(n, precision=A.PREC_FP64, seed=SEED)
    assert b.last_stats["kernel_launches"] == 1
    bad = []
    for i, m in enumerate(models):
        g = b.fetch_instance(i)
        r, _ = Oracle(m).run(n, seed=SEED, instance=i)
        if g.n_desorbed != n or not np.array_equal(g.facet_counts, r.facet_counts):
            bad.append(i)
    b.close()
    assert not bad, "instances differing from the oracle: %s" % bad[:20]


def _outputs(st, m, n):
    y = np.zeros(9)
    y[:8] = st.facet_sums[0, m.gauges, A.FS_SUM_V_ORT] / n
    y[8] = st.facet_counts[0, m.neg, A.FC_NBABSORBED].sum() / n
    return y


def test_c5_fp64_jacobian_equals_oracle_score_function():
    """The sensitivity kernel (FP64) and the oracle's restatement of its bookkeeping on the same
    particles: outputs and all 1000 x 9 Jacobian entries agree (up to the order of the FP64
    atomic sums, and the rare particle whose path splits at a last-bit difference)."""
    m = config5_neg_tube()
    sim = GpuSimulation(m)
    sf = SensitivityFunction(sim, m.neg, m.gauges, m.neg)
    n = 100000
    y = sf.forward(n, precision=A.PREC_FP64, seed=SEED)
    js, _, _ = sf.jacobian()
    sim.close()
    yo, jo = Oracle(m).run_sens(n, m.neg, m.gauges, m.neg, seed=SEED)
    scale = np.abs(jo).max()
    diff = np.abs(js - jo)
    off = int((diff > 1e-9 * scale + 1e-9 * np.abs(jo)).sum())
    print("C5 FP64 Jacobian vs oracle: %d of %d entries differ beyond 1e-9, max difference %.2e of the largest"
          % (off, jo.size, diff.max() / scale))
    np.testing.assert_allclose(y, yo, rtol=1e-6)
    assert off <= 0.02 * jo.size
    assert diff.max() <= 2e-3 * scale


def test_c5_gradients_of_all_outputs_match_central_differences():
    """Strongest parameters and 20 drawn at random, all 9 outputs, against central differences
    with common random numbers (step 0.5 s).  With common random numbers a difference comes only
    from the particles whose stick/reflect decision flips; for a far gauge and a weak parameter
    most batches see none, and a batch variance of zeros says nothing, so a (parameter, output)
    pair is compared when at least 6 of the 16 batches saw a change."""
    m = config5_neg_tube()
    sim = GpuSimulation(m)
    sf = SensitivityFunction(sim, m.neg, m.gauges, m.neg)
    nb, n = 16, 2_000_000
    js = []
    for b in range(nb):
        sim.ResetSimulation()
        sim.set_particle_offset(b * n)
        sf.forward(n, seed=SEED)
        js.append(sf.jacobian()[0])
    js = np.array(js)
    # parameters chosen on batch 0, gradients estimated on the other batches (the largest of 1000
    # noisy estimates is biased upwards)
    jm, jse = js[1:].mean(0), js[1:].std(0, ddof=1) / math.sqrt(nb - 1)
    rng = np.random.default_rng(11)
    top = list(np.argsort(-np.abs(js[0, :, 8]))[:2]) + [int(np.argmax(np.abs(js[0, :, 3])))]
    pick = sorted(set(top) | set(rng.choice(len(m.neg), 20, replace=False).tolist()))
    zs, skipped = [], 0
    for k in pick:
        f = int(m.neg[k])
        s0 = float(m.sticking[f])
        ds = 0.5 * s0
        fd = []
        for b in range(nb):
            ys = []
            for s in (s0 + ds, s0 - ds):
                sim.update_sticking([f], [s])
                sim.ResetSimulation()
                sim.set_particle_offset(b * n)   # common random numbers
                sim.SimulationMCStep(n, precision=A.PREC_FP32R, seed=SEED)
                ys.append(_outputs(sim.fetch(), m, n))
            fd.append((ys[0] - ys[1]) / (2 * ds))
        sim.update_sticking([f], [s0])
        fd = np.array(fd)
        fm, fse = fd.mean(0), fd.std(0, ddof=1) / math.sqrt(nb)
        for j in range(9):
            if (fd[:, j] != 0).sum() < 6:
                skipped += 1
                continue
            zs.append((jm[k, j] - fm[j]) / math.hypot(jse[k, j], fse[j]))
    zs = np.array(zs)
    print("C5: %d parameters x 9 outputs, %d pairs compared (%d with too few flipped decisions), max |z| %.2f, "
          "mean z^2 %.2f" % (len(pick), len(zs), skipped, np.abs(zs).max(), np.mean(zs ** 2)))
    assert len(zs) >= 0.4 * len(pick) * 9
    assert np.abs(zs).max() < z_threshold(zs.size) + 0.5
    assert np.mean(zs ** 2) < 2.0
    sim.close()
