"""Rays that cross more transparent facets than one pass list holds (32) on the GPU: the tracer
takes the nearest passes, then traces the same ray again for the ones beyond, so the run completes
and every pass is counted.  48 disks across the tube, fully transparent or of opacity 0.5."""
import math

import numpy as np
import pytest

from molflow_sources_gb300 import _abi as A
from molflow_sources_gb300.simulation import GpuSimulation
from molflow_sources_gb300.workloads import stacked_disk_tube
from oracle.oracle import Oracle
from tests.stats import binom_sigma, z_threshold

pytestmark = pytest.mark.gpu
SEED = 0x4D6F6C66


def test_fp64_many_passes_equal_oracle():
    """Fully transparent disks: every ray along the tube crosses up to 48 of them (up to two
    extra rounds per ray), paths are as short as in the plain tube, and the FP64 kernel's tallies
    equal the oracle's on the same particles."""
    m = stacked_disk_tube(48, opacity=0.0)
    n = 20000
    sim = GpuSimulation(m)
    sim.SimulationMCStep(n, precision=A.PREC_FP64, seed=SEED)
    g = sim.fetch()
    r, _ = Oracle(m).run(n, seed=SEED)
    assert np.array_equal(g.facet_counts, r.facet_counts)
    assert g.facet_counts[0, m.disks, A.FC_NBMCHIT].min() > 0
    sim.close()


def test_fp64_semi_transparent_disks_within_3_sigma():
    """Disks of opacity 0.5 make a maze of long paths (hundreds of bounces between neighbouring
    disks), where last-bit differences between CUDA's and glibc's trigonometry split paths, so the
    FP64 kernel is compared with the oracle statistically (batch means): transmission and the
    hits per desorption on every disk, family-wise."""
    m = stacked_disk_tube(48, opacity=0.5)
    sim = GpuSimulation(m)
    nb, n = 16, 25000
    gpu = []
    for b in range(nb):
        sim.ResetSimulation()
        sim.set_particle_offset(10 ** 10 + b * n)
        sim.SimulationMCStep(n, precision=A.PREC_FP64, seed=SEED)
        st = sim.fetch()
        gpu.append(np.concatenate([[st.transmission(1)], st.facet_counts[0, m.disks, A.FC_NBMCHIT] / n]))
    sim.close()
    orc = Oracle(m)
    ora = []
    for b in range(16):
        st, _ = orc.run(6250, seed=SEED, first_particle=10 ** 12 + b * 6250)
        ora.append(np.concatenate([[st.transmission(1)], st.facet_counts[0, m.disks, A.FC_NBMCHIT] / 6250]))
    gpu, ora = np.array(gpu), np.array(ora)
    z = (gpu.mean(0) - ora.mean(0)) / np.sqrt(gpu.var(0, ddof=1) / len(gpu) + ora.var(0, ddof=1) / len(ora))
    # 16 batches a side: t-distributed scores, hence the margin over the normal family threshold
    assert np.abs(z).max() < z_threshold(len(z)) + 1.0, np.round(z, 2)


def test_fp32r_many_passes_transmission_within_3_sigma():
    m = stacked_disk_tube(48, opacity=0.0)
    n = 2_000_000
    sim = GpuSimulation(m)
    sim.SimulationMCStep(n, precision=A.PREC_FP32R, seed=SEED)
    g = sim.fetch()
    no = 400000
    r, _ = Oracle(m).run(no, seed=SEED, first_particle=10 ** 9)
    p, q = g.transmission(1), r.transmission(1)
    assert abs(p - q) < 3 * math.hypot(binom_sigma(p, n), binom_sigma(q, no)), (p, q)
    # passes per desorption on each disk
    a = g.facet_counts[0, m.disks, A.FC_NBMCHIT] / n
    b = r.facet_counts[0, m.disks, A.FC_NBMCHIT] / no
    assert np.abs(a / b - 1).max() < 0.02
    sim.close()
