"""Histograms of absorbed particles on the GPU (RecordHistograms, Particle.cpp:926-975): fixture
09 records global distance and time histograms and bounce, distance and time histograms on one
facet, in five moments.  The FP64 kernel and the oracle trace the same particles and must fill
the same bins."""
import numpy as np
import pytest

from molflow_sources_gb300 import _abi as A
from molflow_sources_gb300.simulation import GpuSimulation
from oracle.oracle import Oracle
from tests import golden_util

pytestmark = pytest.mark.gpu
SEED = 0x4D6F6C66


def test_fp64_histograms_equal_oracle():
    m, ref, _ = golden_util.load("09-histograms")
    L = m.layout()
    assert L["histogram_bins"] > 0
    n = 100000
    sim = GpuSimulation(m)
    sim.SimulationMCStep(n, precision=A.PREC_FP64, seed=SEED)
    g = sim.fetch()
    r, _ = Oracle(m).run(n, seed=SEED)
    assert np.array_equal(g.facet_counts, r.facet_counts)
    assert g.histogram.sum() > 0
    assert np.array_equal(g.histogram, r.histogram)
    # every absorption lands in each recorded global histogram once (moment 0)
    dist, time_ = g.histograms_of(None)[1:]
    assert dist.sum() == time_.sum() == g.global_[A.G_NBABSEQUIV]
