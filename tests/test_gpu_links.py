"""Structure links on the GPU (PerformBounce's link branch, Particle.cpp:698-724): fixture 05
joins three structures with two link facets; the FP64 kernel and the oracle trace the same
particles and must give the same integer tallies."""
import numpy as np
import pytest

from molflow_sources_gb300 import _abi as A
from molflow_sources_gb300.simulation import GpuSimulation
from oracle.oracle import Oracle
from tests import golden_util

pytestmark = pytest.mark.gpu
SEED = 0x4D6F6C66


def test_fp64_linked_structures_equal_oracle():
    m, ref, _ = golden_util.load("05-three_structures_nonsquare_textures")
    assert (m.link_dest != 0).sum() == 2
    n = 50000
    sim = GpuSimulation(m)
    sim.SimulationMCStep(n, precision=A.PREC_FP64, seed=SEED)
    g = sim.fetch()
    r, _ = Oracle(m).run(n, seed=SEED)
    links = np.nonzero(m.link_dest)[0]
    assert (g.facet_counts[0, links, A.FC_NBMCHIT] > 1000).all()
    assert np.array_equal(g.facet_counts, r.facet_counts)
    assert np.array_equal(g.texture[..., 0], r.texture[..., 0])
    assert np.array_equal(g.profile[..., 0], r.profile[..., 0])
    assert g.global_[A.G_NBMCHIT] == r.global_[A.G_NBMCHIT]
