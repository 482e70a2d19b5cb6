"""Rays that cross many transparent facets (the oracle, CPU): a tube crossed by 48 fully transparent
disks transmits like the same tube without them, and every pass is counted (the reference keeps
every transparent hit of a ray, Particle.cpp:246-253, 293-309)."""
import math

import numpy as np

from molflow_sources_gb300 import _abi as A
from molflow_sources_gb300.workloads import config1_tube, stacked_disk_tube
from oracle.oracle import Oracle
from tests.stats import binom_sigma

SEED = 0x4D6F6C66


def test_transparent_disks_leave_transmission_unchanged():
    n = 200000
    m = stacked_disk_tube(48, opacity=0.0)
    st, _ = Oracle(m).run(n, seed=SEED)
    plain, _ = Oracle(config1_tube(texture_facet=None)).run(n, seed=SEED)
    p, q = st.transmission(1), plain.transmission(1)
    assert abs(p - q) < 3 * math.hypot(binom_sigma(p, n), binom_sigma(q, n))
    # every transmitted particle crossed every disk at least once
    passes = st.facet_counts[0, m.disks, A.FC_NBMCHIT]
    assert passes.min() >= st.absorbed(1)
    assert st.global_[A.G_NBLEAK] == 0
