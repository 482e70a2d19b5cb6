"""Teleports in the oracle (PerformTeleport, Particle.cpp:76-183; the hit dispatch at :326-329)."""
import numpy as np

from molflow_sources_gb300 import _abi as A
from molflow_sources_gb300.model import build_pipe
from oracle.oracle import Oracle
from tests.stats import binom_sigma
from tests.teleport_model import teleport_pair

SEED = 0x4D6F6C66


def test_teleport_pair_transmits_like_one_long_tube():
    m, b_in, b_out = teleport_pair()
    n = 400_000
    r, _ = Oracle(m).run(n, seed=SEED)
    assert r.global_[A.G_NBLEAK] == 0
    p_pair = r.facet_counts[0, b_out, A.FC_NBABSORBED] / n
    t = build_pipe(L=10.0, R=1.0, step=32)                # one L/R = 10 tube of the same polygon
    q, _ = Oracle(t).run(n, seed=SEED + 1)
    p_long = q.facet_counts[0, 1, A.FC_NBABSORBED] / n
    assert abs(p_pair - p_long) < 4 * np.hypot(binom_sigma(p_pair, n), binom_sigma(p_long, n)), (p_pair, p_long)
    # the global hit count leaves the teleports out (Particle.cpp:176-182)
    tele = int(r.facet_counts[0, 1, A.FC_NBMCHIT]) + int(r.facet_counts[0, b_in, A.FC_NBMCHIT])
    assert tele > 0.15 * n
    per_facet = int(r.facet_counts[0, :, A.FC_NBMCHIT].sum())
    assert int(r.global_[A.G_NBMCHIT]) == per_facet - tele
    assert int(r.facet_counts[0, 1, A.FC_NBABSORBED]) == 0 and int(r.facet_counts[0, b_in, A.FC_NBABSORBED]) == 0


def test_teleport_source_records_passes():
    m, b_in, b_out = teleport_pair()
    n = 100_000
    r, _ = Oracle(m).run(n, seed=SEED)
    tele = int(r.facet_counts[0, 1, A.FC_NBMCHIT])
    tex = r.texture_of(1)[..., 0]
    assert int(tex.sum()) == tele                      # countTrans cells: one per teleport
    assert r.facet_sums[0, 1, 0] > 0                   # velocity sums of the outgoing direction
