"""Per-facet, per-moment hit rates of a run against a reference test case's stored state.

The run is split into batches (independent particle ranges); a rate's standard error is the
larger of its batch-means error and the Poisson error of the null hypothesis (the larger of
the two rates), and the reference's own error is that of the same per-particle variance over
its (larger) number of desorptions.  The family threshold covers every non-empty cell.  It is
the normal quantile unless `student` is set; then, since the standard error comes from the batch
means, it is Student's t quantile with one degree of freedom fewer than the batches (the normal
quantile is the stricter of the two and rejects a correct run more often).

No systematic allowance is added by default (`rel_sys` = 0): the comparisons are the 3-standard-
error rule of the combined estimate.  A case with a measured, named cause of a systematic
difference may pass a relative allowance `rel_sys`, added in quadrature (the reference's own
acceptance rule, GlobalSimuState::Compare, MolflowSimGeom.cpp:559-1148, called with 0.9 % global
and 7 % per-facet relative thresholds in tests/testsuite.cpp:460, is far looser).
"""
import math

import numpy as np

from molflow_sources_gb300 import _abi as A
from tests.stats import z_threshold


def hit_rates(states):
    """[batches, 1+moments, facets] hits per desorption of each batch's state."""
    return np.array([s.facet_counts[..., A.FC_NBMCHIT].astype(np.float64) / s.global_[A.G_NBDESORBED]
                     for s in states])


def zscores(per, n_per_batch, ref, ref_desorbed, rel_sys=0.0):
    nb = per.shape[0]
    ntot = nb * n_per_batch
    a = per.mean(0)
    se = per.std(0, ddof=1) / math.sqrt(nb)
    b = ref / ref_desorbed
    sa = np.maximum(se, np.sqrt(np.maximum(np.maximum(a, b), 1.0 / ntot) / ntot))
    sig = np.sqrt((sa * sa) * (1.0 + ntot / ref_desorbed) + (rel_sys * b) ** 2)
    mask = (a > 0) | (b > 0)
    z = np.where(mask, (a - b) / sig, 0.0)
    return z, int(mask.sum())


def assert_hits_agree(per, n_per_batch, ref, ref_desorbed, extra=0.0, rel_sys=0.0, label="", student=False):
    z, k = zscores(per, n_per_batch, ref, ref_desorbed, rel_sys)
    thr = z_threshold(max(k, 1), df=per.shape[0] - 1 if student else None) + extra
    worst = np.unravel_index(np.argmax(np.abs(z)), z.shape)
    if label:
        print("%s: max |z| %.2f against %.2f over %d cells (rel_sys %g)" % (label, np.abs(z).max(), thr, k, rel_sys))
    assert np.abs(z).max() < thr, ("max |z| %.2f >= %.2f at (moment, facet) %s: run %.5g, stored %.5g"
                                   % (np.abs(z).max(), thr, worst, per.mean(0)[worst], (ref / ref_desorbed)[worst]))
    return np.abs(z).max(), thr
