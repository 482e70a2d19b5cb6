"""Outgassing maps on the GPU (StartFromSource with useOutgassingFile, Particle.cpp:425-446 and
513-535): the FP64 kernel picks the same cells and start points as the oracle, particle by
particle; the FP32R kernel's desorption cells follow the map."""
import numpy as np
import pytest

from molflow_sources_gb300 import _abi as A
from molflow_sources_gb300.simulation import GpuSimulation
from oracle.oracle import Oracle
from tests.og_model import GRID, og_tube
from tests.stats import z_threshold

pytestmark = pytest.mark.gpu
SEED = 0x4D6F6C66


def test_fp64_outgassing_map_equals_oracle():
    m, _ = og_tube()
    n = 40000
    sim = GpuSimulation(m)
    sim.SimulationMCStep(n, precision=A.PREC_FP64, seed=SEED)
    g = sim.fetch()
    r, _ = Oracle(m).run(n, seed=SEED)
    assert g.global_[A.G_NBLEAK] == 0
    assert np.array_equal(g.facet_counts, r.facet_counts)
    assert np.array_equal(g.texture[..., 0], r.texture[..., 0])
    np.testing.assert_allclose(g.facet_sums, r.facet_sums, rtol=1e-6, atol=1e-6)


def test_fp32r_desorption_cells_follow_the_map():
    m, vals = og_tube()
    n = 4_000_000
    sim = GpuSimulation(m)
    sim.SimulationMCStep(n, precision=A.PREC_FP32R, seed=SEED)
    g = sim.fetch()
    assert g.global_[A.G_NBLEAK] == 0
    tex = g.texture_of(0)[..., 0].reshape(GRID, GRID)
    assert tex.sum() == n
    p = vals / vals.sum()
    assert (tex[p == 0] == 0).all()
    z = (tex / n - p)[p > 0] / np.sqrt(p[p > 0] * (1 - p[p > 0]) / n)
    assert np.abs(z).max() < z_threshold(int((p > 0).sum())), np.abs(z).max()
