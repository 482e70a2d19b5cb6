"""Test model with an outgassing map: the config-1 tube whose inlet (facet 0) desorbs from a
10 x 10 map instead of uniformly.  The map's grid spans 9.5 x 9.5 cells over the inlet's
bounding rectangle (so its last row and column are half cells, Particle.cpp:518-533), only
cells lying wholly inside the 64-gon have rates, and the inlet's desorption texture uses the
same grid (texture 9.5 x 9.5), so texture cell k counts the particles started in map cell k."""
import numpy as np

from molflow_sources_gb300 import _abi as A
from molflow_sources_gb300.workloads import config1_tube
from oracle.oracle import Oracle

GRID = 10
EXTENT = 9.5


def og_tube(seed=3):
    m = config1_tube()
    basis, _ = Oracle(m).facet_geometry()
    nu, nv = np.linalg.norm(basis[0, 3:6]), np.linalg.norm(basis[0, 6:9])
    rng = np.random.default_rng(seed)
    vals = np.zeros((GRID, GRID))
    for h in range(GRID):
        for w in range(GRID):
            # cell corners in (u,v) in [0,1], then distance from the inlet's centre in cm
            us = np.array([w, w + 1]) / EXTENT
            vs = np.array([h, h + 1]) / EXTENT
            cu, cv = np.meshgrid((us - 0.5) * nu, (vs - 0.5) * nv)
            if np.hypot(cu, cv).max() < 0.98 * np.cos(np.pi / 64):
                vals[h, w] = rng.uniform(0.2, 1.0) * (3.0 if (h + w) % 4 == 0 else 1.0)
    m.outgassing_maps[0] = dict(width=GRID, height=GRID, ratio_u=EXTENT / nu, ratio_v=EXTENT / nv, values=vals)
    m.tex_width[0] = EXTENT
    m.tex_height[0] = EXTENT
    m.count_flags[0] = A.COUNT_DES
    return m, vals
