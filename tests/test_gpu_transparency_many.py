"""Rays that cross more transparent facets than one pass list holds (32) on the GPU: the tracer
takes the nearest passes, then traces the same ray again for the ones beyond, so the run completes
and every pass is counted.  48 disks across the tube, fully transparent or of opacity 0.5."""
import math

import numpy as np
import pytest

from molflow_sources_gb300 import _abi as A
from molflow_sources_gb300.simulation import GpuSimulation
from molflow_sources_gb300.workloads import stacked_disk_tube
from oracle.oracle import Oracle
from tests.stats import binom_sigma

pytestmark = pytest.mark.gpu
SEED = 0x4D6F6C66


@pytest.mark.parametrize("opacity", [0.0, 0.5])
def test_fp64_many_passes_equal_oracle(opacity):
    m = stacked_disk_tube(48, opacity=opacity)
    n = 20000
    sim = GpuSimulation(m)
    sim.SimulationMCStep(n, precision=A.PREC_FP64, seed=SEED)
    g = sim.fetch()
    r, _ = Oracle(m).run(n, seed=SEED)
    assert np.array_equal(g.facet_counts, r.facet_counts)
    assert g.facet_counts[0, m.disks, A.FC_NBMCHIT].min() > 0
    sim.close()


def test_fp32r_many_passes_transmission_within_3_sigma():
    m = stacked_disk_tube(48, opacity=0.0)
    n = 2_000_000
    sim = GpuSimulation(m)
    sim.SimulationMCStep(n, precision=A.PREC_FP32R, seed=SEED)
    g = sim.fetch()
    no = 400000
    r, _ = Oracle(m).run(no, seed=SEED, first_particle=10 ** 9)
    p, q = g.transmission(1), r.transmission(1)
    assert abs(p - q) < 3 * math.hypot(binom_sigma(p, n), binom_sigma(q, no)), (p, q)
    # passes per desorption on each disk
    a = g.facet_counts[0, m.disks, A.FC_NBMCHIT] / n
    b = r.facet_counts[0, m.disks, A.FC_NBMCHIT] / no
    assert np.abs(a / b - 1).max() < 0.02
    sim.close()
