"""Moving facets (TreatMovingFacet, Physics.cpp:25-39) and background-gas scattering
(PerformScatter, Particle.cpp:840-886) on the GPU: the FP64 kernel and the oracle trace the same
particles (same Philox draws in the same order) and must give the same integer tallies; the
FP32 traversal path agrees within 3 standard errors."""
import math

import numpy as np
import pytest

from molflow_sources_gb300 import _abi as A
from molflow_sources_gb300.model import config1_tube
from molflow_sources_gb300.simulation import GpuSimulation
from oracle.oracle import Oracle
from tests.stats import binom_sigma

pytestmark = pytest.mark.gpu
SEED = 0x4D6F6C66


def rotating_tube():
    """Tube whose walls rotate about its axis at 2000 rad/s (20 m/s at the wall)."""
    m = config1_tube()
    m.is_moving[2:] = 1
    m.motion_type = 2
    m.motion_vector1 = (0.0, 0.0, 0.0)
    m.motion_vector2 = (0.0, 0.0, 2000.0)
    return m


def scattering_tube():
    """Tube filled with background gas: 5 cm mean free path, slow particles stop below 50 m/s."""
    m = config1_tube()
    m.scatter_enabled = 1
    m.scatter_mean_free_path_cm = 5.0
    m.scatter_rho = 1e-8
    m.scatter_mass_ratio = 1.0
    m.scatter_cutoff_enabled = 1
    m.scatter_cutoff_speed = 50.0
    return m


@pytest.mark.parametrize("make", [rotating_tube, scattering_tube])
def test_fp64_equals_oracle(make):
    m = make()
    n = 30000
    sim = GpuSimulation(m)
    sim.SimulationMCStep(n, precision=A.PREC_FP64, seed=SEED)
    g = sim.fetch()
    r, _ = Oracle(m).run(n, seed=SEED)
    assert g.global_[A.G_NBMCHIT] == r.global_[A.G_NBMCHIT]
    assert np.array_equal(g.facet_counts, r.facet_counts)
    assert np.array_equal(g.texture[..., 0], r.texture[..., 0])
    np.testing.assert_allclose(g.facet_sums, r.facet_sums, rtol=1e-6, atol=1e-6)
    np.testing.assert_allclose(g.global_[A.G_DIST_TOTAL], r.global_[A.G_DIST_TOTAL], rtol=1e-9)


@pytest.mark.parametrize("make", [rotating_tube, scattering_tube])
def test_fp32r_transmission_within_3_sigma(make):
    m = make()
    n_g, n_o = 2_000_000, 200_000
    sim = GpuSimulation(m)
    sim.SimulationMCStep(n_g, precision=A.PREC_FP32R, seed=SEED)
    g = sim.fetch()
    r, _ = Oracle(m).run(n_o, seed=SEED + 1)
    p_g, p_o = g.transmission(1), r.transmission(1)
    z = (p_g - p_o) / math.hypot(binom_sigma(p_g, n_g), binom_sigma(p_o, n_o))
    assert abs(z) < 3, (p_g, p_o)
    hg, ho = g.n_hits / n_g, r.n_hits / n_o
    assert abs(hg / ho - 1) < 0.01, (hg, ho)
