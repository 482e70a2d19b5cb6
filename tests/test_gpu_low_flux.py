"""Low-flux mode on the GPU (Particle.cpp:338-356): a particle hitting a facet of sticking s is
split into an absorbed part of weight ori*s and a reflected part ori*(1-s), traced on while its
weight stays above the cutoff.  Counters keep Monte Carlo counts; the equivalent counts and the
velocity sums carry the weights."""
import numpy as np
import pytest

from molflow_sources_gb300 import _abi as A
from molflow_sources_gb300.model import config1_tube
from molflow_sources_gb300.simulation import GpuSimulation
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu
SEED = 0x4D6F6C66


def low_flux_tube():
    m = config1_tube()
    m.sticking[2:] = 0.2            # absorbing walls: every wall hit splits the particle
    m.profile_type[5] = A.PROFILE_U
    m.count_flags[2] |= A.COUNT_DIR
    m.low_flux_mode = 1
    m.low_flux_cutoff = 1e-3
    return m


def test_fp64_low_flux_equals_oracle():
    m = low_flux_tube()
    n = 20000
    sim = GpuSimulation(m)
    sim.SimulationMCStep(n, precision=A.PREC_FP64, seed=SEED)
    g = sim.fetch()
    r, _ = Oracle(m).run(n, seed=SEED)
    assert np.array_equal(g.facet_counts, r.facet_counts)
    assert g.global_[A.G_NBMCHIT] == r.global_[A.G_NBMCHIT]
    # equivalent counts and sums: FP64 atomics and fixed-point samples, not bit-exact
    np.testing.assert_allclose(g.global_[A.G_NBHITEQUIV], r.global_[A.G_NBHITEQUIV], rtol=1e-9)
    np.testing.assert_allclose(g.global_[A.G_NBABSEQUIV], r.global_[A.G_NBABSEQUIV], rtol=1e-9)
    np.testing.assert_allclose(g.facet_sums, r.facet_sums, rtol=1e-6, atol=1e-6)
    np.testing.assert_allclose(g.texture[..., 0], r.texture[..., 0], rtol=1e-9, atol=1e-9)
    np.testing.assert_allclose(g.texture[..., 2], r.texture[..., 2], rtol=1e-6, atol=1e-6)
    # sum of v_ort per area: each sample is quantized to 2^-20 m/s before the 1/area increment of
    # its cell (~4e3 /cm2 on the 64x64 wall texture), and low-flux weights make samples small
    np.testing.assert_allclose(g.texture[..., 1], r.texture[..., 1], rtol=1e-3, atol=1e-6)
    np.testing.assert_allclose(g.profile, r.profile, rtol=1e-6, atol=1e-6)
    np.testing.assert_allclose(g.direction, r.direction, rtol=1e-6, atol=1e-6)
    # the split conserves weight: what desorbs is absorbed or dropped below the cutoff
    assert 0.999 * n < g.global_[A.G_NBABSEQUIV] <= n


def test_fp32r_low_flux_transmission_matches_oracle():
    m = low_flux_tube()
    n_g, n_o = 2_000_000, 200_000
    sim = GpuSimulation(m)
    sim.SimulationMCStep(n_g, precision=A.PREC_FP32R, seed=SEED)
    g = sim.fetch()
    r, _ = Oracle(m).run(n_o, seed=SEED + 1)
    # weighted transmission: absorbed equivalents on the outlet per desorbed particle
    tg = g.facet_sums[0, 1, A.FS_NBABSEQUIV] / n_g
    to = r.facet_sums[0, 1, A.FS_NBABSEQUIV] / n_o
    assert abs(tg - to) < 4 * np.sqrt(to / n_o) + 1e-12, (tg, to)
