"""Teleports on the GPU (PerformTeleport, Particle.cpp:76-183): the FP64 kernel equals the oracle
particle by particle on the teleport pair (two tubes joined by teleport facets both ways); the
FP32R kernel's transmission agrees with the oracle's within 3 sigma."""
import math

import numpy as np
import pytest

from molflow_sources_gb300 import _abi as A
from molflow_sources_gb300.simulation import GpuSimulation
from oracle.oracle import Oracle
from tests.stats import binom_sigma
from tests.teleport_model import teleport_pair

pytestmark = pytest.mark.gpu
SEED = 0x4D6F6C66


def test_fp64_teleport_equals_oracle():
    m, b_in, b_out = teleport_pair()
    n = 40000
    sim = GpuSimulation(m)
    sim.SimulationMCStep(n, precision=A.PREC_FP64, seed=SEED)
    g = sim.fetch()
    r, _ = Oracle(m).run(n, seed=SEED)
    assert g.global_[A.G_NBLEAK] == 0
    assert g.global_[A.G_NBMCHIT] == r.global_[A.G_NBMCHIT]
    assert np.array_equal(g.facet_counts, r.facet_counts)
    assert np.array_equal(g.texture[..., 0], r.texture[..., 0])
    assert np.array_equal(g.profile[..., 0], r.profile[..., 0])
    np.testing.assert_allclose(g.facet_sums, r.facet_sums, rtol=1e-6, atol=1e-6)
    assert g.facet_counts[0, 1, A.FC_NBMCHIT] > 5000


def test_fp32r_teleport_transmission_within_3_sigma():
    m, b_in, b_out = teleport_pair()
    n_g, n_o = 4_000_000, 400_000
    sim = GpuSimulation(m)
    sim.SimulationMCStep(n_g, precision=A.PREC_FP32R, seed=SEED)
    g = sim.fetch()
    r, _ = Oracle(m).run(n_o, seed=SEED + 1)
    assert g.global_[A.G_NBLEAK] == 0
    p_g = g.facet_counts[0, b_out, A.FC_NBABSORBED] / n_g
    p_o = r.facet_counts[0, b_out, A.FC_NBABSORBED] / n_o
    z = (p_g - p_o) / math.hypot(binom_sigma(p_g, n_g), binom_sigma(p_o, n_o))
    assert abs(z) < 3, (p_g, p_o)
