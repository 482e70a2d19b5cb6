"""Batched instances in one persistent launch (mfg_model_merge / mfg_run_batch), through the C ABI."""
import math

import numpy as np
import pytest

from molflow_sources_gb300 import _abi as A
from molflow_sources_gb300 import batch_workloads as BW
from molflow_sources_gb300.model import build_pipe
from molflow_sources_gb300.simulation import GpuBatch, GpuSimulation
from oracle.oracle import Oracle
from tests.stats import binom_sigma

pytestmark = pytest.mark.gpu
SEED = 0x4D6F6C66


@pytest.fixture(scope="module")
def models():
    rng = np.random.default_rng(7)
    return [build_pipe(step=24), BW.make_instance("tube", 2000, rng), BW.make_instance("elbow", 3000, rng),
            BW.make_instance("tee", 2500, rng)]


def test_batch_fp64_equals_oracle_per_instance(models):
    b = GpuBatch(models)
    n = 8000
    b.run(n, precision=A.PREC_FP64, seed=SEED)
    assert b.last_stats["kernel_launches"] == 1
    for i, m in enumerate(models):
        g = b.fetch_instance(i)
        r, _ = Oracle(m).run(n, seed=SEED, instance=i)
        assert g.n_desorbed == n
        assert np.array_equal(g.facet_counts, r.facet_counts), "instance %d" % i
        np.testing.assert_allclose(g.facet_sums, r.facet_sums, rtol=1e-8, atol=1e-6)


def test_batch_graph_launch_matches_plain_launch(models):
    a = GpuBatch(models)
    b = GpuBatch(models)
    counts = [3000, 5000, 2000, 4000]
    for _ in range(2):   # the second graph launch replays the captured graph
        a.run(counts, precision=A.PREC_FP64, seed=SEED, use_graph=False)
        b.run(counts, precision=A.PREC_FP64, seed=SEED, use_graph=True)
    for i in range(len(models)):
        assert np.array_equal(a.fetch_instance(i).facet_counts, b.fetch_instance(i).facet_counts)


def test_batch_fp32r_matches_single_runs(models):
    n = 200000
    b = GpuBatch(models)
    b.run(n, precision=A.PREC_FP32R, seed=SEED)
    for i, m in enumerate(models):
        s = GpuSimulation(m)
        s.set_particle_offset(10 ** 12)
        s.SimulationMCStep(n, precision=A.PREC_FP32R, seed=SEED + 1)
        ga, gb = b.fetch_instance(i), s.fetch()
        pump = np.atleast_1d(getattr(m, "pump_facets", np.array([1])))
        pa = ga.facet_counts[0, pump, A.FC_NBABSORBED].sum() / n
        pb = gb.facet_counts[0, pump, A.FC_NBABSORBED].sum() / n
        assert abs(pa - pb) <= 3 * math.sqrt(2) * binom_sigma(max(pa, pb, 1.0 / n), n) + 1e-12, (i, pa, pb)
