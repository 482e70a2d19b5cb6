"""Particle logger on the GPU (LogHit, Particle.cpp:1088-1102; mfg_fetch_log): the FP64 kernel logs
the same events as the oracle (the same records, in another order); the limit holds."""
import numpy as np
import pytest

from molflow_sources_gb300 import _abi as A
from molflow_sources_gb300.model import build_pipe
from molflow_sources_gb300.simulation import GpuSimulation
from oracle.oracle import Oracle
from tests.teleport_model import teleport_pair

pytestmark = pytest.mark.gpu
SEED = 0x4D6F6C66


def _sorted(log):
    return log[np.lexsort((log[:, 1], log[:, 0], log[:, 6]))]


@pytest.mark.parametrize("facet", [0, 1])
def test_fp64_log_equals_oracle(facet):
    m = build_pipe(step=16)
    m.log_facet, m.log_limit = facet, 200000
    n = 20000
    sim = GpuSimulation(m)
    sim.SimulationMCStep(n, precision=A.PREC_FP64, seed=SEED)
    g = _sorted(sim.fetch_log())
    st, r = Oracle(m).run_logged(n, seed=SEED)
    r = _sorted(r)
    assert len(g) == len(r) > 1000
    np.testing.assert_allclose(g[:, [0, 1, 4, 6, 7]], r[:, [0, 1, 4, 6, 7]], rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(g[:, 2:4], r[:, 2:4], rtol=1e-9, atol=1e-9)
    sim.ResetSimulation()
    assert len(sim.fetch_log()) == 0


def test_log_limit_on_a_teleport_source():
    m, b_in, b_out = teleport_pair()
    m.log_facet, m.log_limit = 1, 1000
    sim = GpuSimulation(m)
    sim.SimulationMCStep(40000, precision=A.PREC_FP32R, seed=SEED)
    log = sim.fetch_log()
    assert len(log) == 1000
    assert int(sim.fetch().facet_counts[0, 1, A.FC_NBMCHIT]) > 1000
