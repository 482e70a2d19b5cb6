"""Test model for teleports (PerformTeleport, Particle.cpp:76-183): two L/R = 5 tubes side by side.
Tube A's outlet (facet 1) teleports to tube B's entry facet, which has the same shape and
orientation, and B's entry (two-sided) teleports back to A's outlet, so a particle crossing the
joint either way goes on as if the tubes were one: the pair transmits like one L/R = 10 tube.
B's outlet absorbs."""
import numpy as np

from molflow_sources_gb300 import _abi as A
from molflow_sources_gb300.model import FACET_FIELDS, Model, build_pipe

STEP = 32
SHIFT = 10.0


def teleport_pair():
    a = build_pipe(L=5.0, R=1.0, step=STEP)
    na = len(a.vertices)
    vb = a.vertices + np.array([SHIFT, 0.0, 0.0])
    fb = [[i + na for i in f] for f in a.facets]
    # B's entry at z = 0: A's outlet polygon (odd vertices, z = L) moved to the even vertices below
    # them, so it has the outlet's orientation and basis
    fb[0] = [i - 1 + na for i in a.facets[1]]
    m = Model(np.concatenate([a.vertices, vb]), [list(f) for f in a.facets] + fb)
    nf = a.n_facets
    for k in FACET_FIELDS:
        getattr(m, k)[:nf] = getattr(a, k)
        getattr(m, k)[nf:] = getattr(a, k)
    b_in, b_out = nf, nf + 1
    m.teleport_dest[1] = b_in + 1                  # 1-based destination (teleportDest)
    m.sticking[1] = 0.0
    m.desorb_type[b_in] = A.DES_NONE
    m.outgassing[b_in] = 0.0
    m.is_2sided[b_in] = 1
    m.teleport_dest[b_in] = 1 + 1                  # back to A's outlet
    m.sticking[b_out] = 1.0
    # transparent-pass recordings on the teleport source: 8x8 texture and a U profile
    m.tex_width[1] = 8.0
    m.tex_height[1] = 8.0
    m.count_flags[1] = A.COUNT_TRANS
    m.profile_type[1] = A.PROFILE_U
    return m, b_in, b_out
