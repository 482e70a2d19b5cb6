"""Angle-map desorption on the GPU (AnglemapGeneration.cpp; Particle.cpp:598-622): the sources of
test cases 04 and 04b desorb by the incident-angle map recorded on them.

The FP64 kernel and the oracle trace the same particles and must give the same integer tallies.
In the stored models a particle makes thousands of bounces in a closed tube, and along such a
trajectory the last-bit differences between the device's and the host's sin, cos and acos grow
until, after about 5000 bounces, one hit lands on the other side of a wall edge.  The exact check
therefore makes the tube walls absorb (sticking 0.2, a few bounces per particle); the stored
models themselves are checked statistically against the reference's results in
test_gpu_fixtures.py."""
import numpy as np
import pytest

from molflow_sources_gb300 import _abi as A
from molflow_sources_gb300.simulation import GpuSimulation
from oracle.oracle import Oracle
from tests import golden_util

pytestmark = pytest.mark.gpu
SEED = 0x4D6F6C66
CASES = ["04-anglemap_desorb", "04b-anglemap_desorb-sticking source"]


def _short_trajectories(case):
    m, _, _ = golden_util.load(case)
    walls = (m.sticking == 0) & (m.opacity == 1)
    m.sticking = np.where(walls, 0.2, m.sticking)
    return m


@pytest.mark.parametrize("case", CASES)
def test_fp64_anglemap_desorption_equals_oracle(case):
    m = _short_trajectories(case)
    src = [i for i in range(m.n_facets) if m.desorb_type[i] == A.DES_ANGLEMAP]
    assert src and all(i in m.desorb_anglemaps for i in src)
    n = 40000
    sim = GpuSimulation(m)
    sim.SimulationMCStep(n, precision=A.PREC_FP64, seed=SEED)
    g = sim.fetch()
    r, _ = Oracle(m).run(n, seed=SEED)
    assert g.facet_counts[0, src, A.FC_NBDESORBED].sum() > 500
    assert g.global_[A.G_NBLEAK] == 0 and r.global_[A.G_NBLEAK] == 0
    assert np.array_equal(g.facet_counts, r.facet_counts)
    assert np.array_equal(g.texture[..., 0], r.texture[..., 0])
    # velocity sums: fixed-point device sums against FP64 host sums
    np.testing.assert_allclose(g.facet_sums, r.facet_sums, rtol=1e-6, atol=1e-6)


def test_fp32r_anglemap_source_does_not_leak():
    """FP32 start points near the rim of a source whose rim lies on the tube walls are decided in
    FP64, so no particle starts outside the walls."""
    m, _, _ = golden_util.load("04b-anglemap_desorb-sticking source")
    sim = GpuSimulation(m)
    for b in range(4):
        sim.ResetSimulation()
        sim.set_particle_offset(b * 1_000_000)
        sim.SimulationMCStep(1_000_000, precision=A.PREC_FP32R, seed=SEED + 7)
        assert sim.fetch().global_[A.G_NBLEAK] == 0
