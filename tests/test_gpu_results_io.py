"""A GPU run of the reference's test case B02 (L/R = 10 tube, 1000 walls with 100x1 textures),
written as a MolFlow+ file and read back, passes the reference's own acceptance rule against the
stored state: GlobalSimuState::Compare(stored, run, 0.009, 0.07) with no global and no facet
differences (tests/testsuite.cpp:460)."""
import numpy as np
import pytest

from molflow_sources_gb300 import _abi as A
from molflow_sources_gb300 import compare, physics, xmlio, xmlwriter
from molflow_sources_gb300.simulation import GpuSimulation
from tests import golden_util
from tests.test_cpu_results_io import _stored_state

pytestmark = pytest.mark.gpu
SEED = 0x4D6F6C66


def test_gpu_b02_written_and_reread_passes_reference_compare(tmp_path):
    m, ref, _ = golden_util.load("B02-lr10_pipe_tex")
    sim = GpuSimulation(m)
    sim.SimulationMCStep(40_000_000, precision=A.PREC_FP32R, seed=SEED)
    run = sim.fetch()
    og = sim.gmodel.outgassing()
    area = sim.gmodel.facet_geometry()[1]
    path = str(tmp_path / "B02_gpu.zip")
    xmlwriter.save(path, m, run, og, area)
    m2, back, _ = xmlio.load(path)
    for k in ("global_", "facet_counts", "facet_sums", "texture"):
        assert np.array_equal(getattr(run, k), getattr(back, k)), k
    stored = _stored_state(m, ref)
    walls = back.facet_counts[0, 2:, A.FC_NBMCHIT]
    assert walls.min() >= 40000   # every wall takes part in the facet comparisons
    g, f, fine, msgs = compare.compare_states(stored, back, 0.009, 0.07)
    print("B02 GPU run vs stored state: %d global, %d facet, %d fine differences" % (g, f, fine))
    assert (g, f) == (0, 0), msgs[:10]
    # the facet-physics table of the re-read result
    csv = str(tmp_path / "facet_physics.csv")
    assert physics.write_facet_physics_csv(csv, m2, back, area, og) == 0
    assert physics.validate_csv(csv) == 5
    sim.close()
