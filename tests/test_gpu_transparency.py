"""Transparent and semi-transparent facets on the GPU (RegisterTransparentPass,
Particle.cpp:1232-1257; opacity decisions in Intersect).

The opacity of a facet is decided per (particle, trace step, facet) by a Philox draw in a
stream of its own, the oracle's scheme, so the FP64 kernel and the oracle make the same
decisions and their integer tallies agree exactly.
"""
import math

import numpy as np
import pytest

from molflow_sources_gb300 import _abi as A
from molflow_sources_gb300.simulation import GpuSimulation
from molflow_sources_gb300.workloads import transparent_tube
from oracle.oracle import Oracle
from tests import golden_util
from tests.stats import binom_sigma, z_threshold
from tests.test_cpu_basics import b04_compare

pytestmark = pytest.mark.gpu
SEED = 0x4D6F6C66


@pytest.mark.parametrize("transient", [False, True])
def test_fp64_transparent_tube_equals_oracle(transient):
    m = transparent_tube(transient=transient)
    n = 40000
    sim = GpuSimulation(m)
    sim.SimulationMCStep(n, precision=A.PREC_FP64, seed=SEED)
    g = sim.fetch()
    r, _ = Oracle(m).run(n, seed=SEED)
    assert g.global_[A.G_NBLEAK] == 0
    assert np.array_equal(g.facet_counts, r.facet_counts)
    assert np.array_equal(g.texture[..., 0], r.texture[..., 0])
    assert np.array_equal(g.profile[..., 0], r.profile[..., 0])
    assert np.array_equal(g.direction[..., 3], r.direction[..., 3])
    assert np.array_equal(g.anglemap, r.anglemap)
    # velocity sums: the device adds fixed-point samples (2^-20 m/s and 2^-32 s/m quanta), so a
    # cell holding a few samples times a large area increment differs by up to ~1e-7 relative
    np.testing.assert_allclose(g.facet_sums, r.facet_sums, rtol=1e-6, atol=1e-6)
    np.testing.assert_allclose(g.texture, r.texture, rtol=1e-6, atol=1e-6)
    np.testing.assert_allclose(g.profile, r.profile, rtol=1e-6, atol=1e-6)
    np.testing.assert_allclose(g.direction[..., :3], r.direction[..., :3], rtol=1e-9, atol=1e-6)
    # every disk saw passes; the semi-transparent ones also hard hits (reflections)
    for d in m.disks:
        assert g.facet_counts[0, d, A.FC_NBMCHIT] > 1000


def test_fp32r_transparent_tube_within_3_sigma():
    m = transparent_tube()
    n_gpu, n_o = 4_000_000, 400_000
    sim = GpuSimulation(m)
    sim.SimulationMCStep(n_gpu, precision=A.PREC_FP32R, seed=SEED)
    g = sim.fetch()
    r, _ = Oracle(m).run(n_o, seed=SEED + 1)
    p_g, p_o = g.transmission(1), r.transmission(1)
    z = (p_g - p_o) / math.hypot(binom_sigma(p_g, n_gpu), binom_sigma(p_o, n_o))
    assert abs(z) < 3, (p_g, p_o)
    zs = []
    for d in m.disks:
        a = g.facet_counts[0, d, A.FC_NBMCHIT] / n_gpu
        b = r.facet_counts[0, d, A.FC_NBMCHIT] / n_o
        zs.append((a - b) / math.sqrt(a / n_gpu + b / n_o))
    assert max(abs(x) for x in zs) < z_threshold(3), zs


def test_b04_transparent_tubes_vs_reference_state():
    """B04 on the GPU (FP32 traversal + FP64 recheck) against the reference's stored state."""
    m, ref, _ = golden_util.load("B04-lr10_pipe_trans")
    n = 2_000_000
    sim = GpuSimulation(m)
    sim.SimulationMCStep(n, precision=A.PREC_FP32R, seed=SEED)
    g = sim.fetch()
    assert g.global_[A.G_NBLEAK] == 0
    z = b04_compare(g, n, ref)
    assert max(abs(v) for v in z.values()) < z_threshold(len(z)), z


def test_opacity_parameter_only_model_is_traced():
    """A model whose only non-opaque facet has an opacity parameter is traced, not rejected."""
    m = transparent_tube()
    m.opacity[m.disks[0]] = 1.0
    m.opacity[m.disks[1]] = 1.0
    sim = GpuSimulation(m)
    st = sim.SimulationMCStep(20000, precision=A.PREC_FP32R, seed=SEED)
    g = sim.fetch()
    assert g.facet_counts[0, m.disks[2], A.FC_NBMCHIT] > 0
    assert g.global_[A.G_NBLEAK] == 0
