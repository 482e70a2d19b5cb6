"""Force measurement on the GPU (IncreaseFacetCounter's impulse sums, Particle.cpp:1194-1230):
the FP64 kernel's impulse, impulse-square and torque sums per facet equal the oracle's (same
particles, FP64 atomics in another order); the FP32R kernel keeps the wall identity
impulse . N = -sum_v_ort."""
import numpy as np
import pytest

from molflow_sources_gb300 import _abi as A
from molflow_sources_gb300.model import build_pipe
from molflow_sources_gb300.simulation import GpuSimulation
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu
SEED = 0x4D6F6C66


def _tube():
    m = build_pipe(L=10.0, R=1.0, step=16)
    m.enable_force_measurement = 1
    m.torque_ref_point = (0.3, -0.2, 5.0)
    m.set_moments([1e-4, 3e-4], [1e-4, 1e-4])
    m.constant_flow = 0
    m.time_window = 1e-3
    return m


def test_fp64_forces_equal_oracle():
    m = _tube()
    n = 40000
    sim = GpuSimulation(m)
    sim.SimulationMCStep(n, precision=A.PREC_FP64, seed=SEED)
    g = sim.fetch()
    r, _ = Oracle(m).run(n, seed=SEED)
    assert np.array_equal(g.facet_counts, r.facet_counts)
    assert g.force.shape == r.force.shape and np.abs(r.force).sum() > 0
    scale = np.abs(r.force).max(axis=(0, 1), keepdims=True)
    np.testing.assert_allclose(g.force, r.force, rtol=1e-9, atol=1e-12 * scale.max())


def test_fp32r_wall_identity():
    m = _tube()
    n = 400000
    sim = GpuSimulation(m)
    sim.SimulationMCStep(n, precision=A.PREC_FP32R, seed=SEED)
    g = sim.fetch()
    basis, _ = Oracle(m).facet_geometry()
    N = basis[:, 9:12]
    walls = np.arange(2, m.n_facets)
    imp_n = np.einsum("fk,fk->f", g.force[0, walls, 0:3], N[walls])
    # FP32 directions and fixed-point velocity sums: agreement to a few 1e-6
    np.testing.assert_allclose(imp_n, -g.facet_sums[0, walls, A.FS_SUM_V_ORT], rtol=2e-5)
