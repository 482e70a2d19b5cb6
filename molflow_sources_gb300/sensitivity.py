"""Sticking / outgassing sensitivities by the score-function method (config 5).

Geometry: the config-1 tube (L/R = 10, R = 1 cm) re-meshed to 64 x 16 = 1024 wall quads; 1000
of them are non-evaporable-getter (NEG) facets whose sticking ~U[0.001, 0.05] are the
parameters and which outgas uniformly per area; 8 are pressure gauges (sticking 0) spaced
along the tube; the rest are inert walls.  Inlet disk: cosine source, sticking 1; outlet: pump,
sticking 1.

Outputs per desorbed test particle: the 8 gauges' Sum v_ort (pressure up to the factor
MolPerTP/area) and the NEG pumped flux (absorptions on NEG facets).  Gradients with respect to
each NEG sticking coefficient come from the score of every stick/reflect decision (1/s on stick,
-1/(1-s) on reflect) accumulated along each trajectory; gradients with respect to each source's
outgassing come from the per-source conditional means (the output is linear in the rates).
The library exposes a forward/backward pair (mfg_sens_forward / mfg_sens_backward) shaped like
an autograd Function.
"""
import ctypes as C
import math

import numpy as np

from . import _abi as A
from .model import Model
from .simulation import GpuSimulation, _check, _count, load_library

N_OUT = 9   # 8 gauges + pumped flux


def config5_neg_tube(n_around=64, n_rings=16, L=10.0, R=1.0, seed=20260505, n_gauges=8, n_neg=1000):
    rng = np.random.default_rng(seed)
    ang = np.arange(n_around) / n_around * 2 * math.pi
    zs = np.linspace(0.0, L, n_rings + 1)
    V = np.zeros(((n_rings + 1) * n_around, 3))
    for k, z in enumerate(zs):
        V[k * n_around:(k + 1) * n_around, 0] = R * np.cos(ang)
        V[k * n_around:(k + 1) * n_around, 1] = R * np.sin(ang)
        V[k * n_around:(k + 1) * n_around, 2] = z
    vid = lambda k, i: k * n_around + (i % n_around)
    facets = [[vid(0, i) for i in range(n_around)], [vid(n_rings, n_around - 1 - i) for i in range(n_around)]]
    walls = []
    for k in range(n_rings):
        for i in range(n_around):
            walls.append(len(facets))
            facets.append([vid(k, i), vid(k + 1, i), vid(k + 1, i + 1), vid(k, i + 1)])
    m = Model(V, facets)
    walls = np.array(walls)
    m.sticking[0] = 1.0
    m.sticking[1] = 1.0
    m.desorb_type[0] = A.DES_COSINE
    m.outgassing[0] = 1.0
    # gauges: one wall quad per two rings, at azimuth 0
    gauges = np.array([2 + (2 * g + 1) * n_around for g in range(n_gauges)])
    rest = np.setdiff1d(walls, gauges)
    neg = np.sort(rng.choice(rest, size=n_neg, replace=False))
    m.sticking[neg] = rng.uniform(0.001, 0.05, n_neg)
    area = 2 * R * math.sin(math.pi / n_around) * (L / n_rings)
    m.outgassing[neg] = 1e-3 * area     # uniform NEG outgassing per area, small next to the inlet
    m.desorb_type[neg] = A.DES_COSINE
    m.gauges = gauges
    m.neg = neg
    return m


class SensitivityFunction:
    """forward(n) -> outputs[9] (per desorbed particle); backward(dL/dY) -> (dL/ds[1000], dL/dQ[sources])."""

    def __init__(self, sim: GpuSimulation, params, gauges, pumps):
        self.sim = sim
        self.params = np.ascontiguousarray(params, np.int32)
        self.gauges = np.ascontiguousarray(gauges, np.int32)
        self.pumps = np.ascontiguousarray(pumps, np.int32)
        L = load_library()
        _check(L.mfg_sens_setup(sim.h, len(self.params), A.ptr(self.params, C.c_int32), len(self.gauges),
                                A.ptr(self.gauges, C.c_int32), len(self.pumps), A.ptr(self.pumps, C.c_int32)))

    def forward(self, n, precision=A.PREC_FP32R, seed=0x4D6F6C66, block_size=0, blocks_per_sm=0):
        out = np.zeros(N_OUT)
        st = A.RunStats()
        o = A.RunOptions(precision=precision, seed=seed, block_size=block_size, blocks_per_sm=blocks_per_sm)
        _check(load_library().mfg_sens_forward(self.sim.h, _count(n, "n"), C.byref(o), A.ptr(out, C.c_double), C.byref(st)))
        self.last_stats = {f: getattr(st, f) for f, _ in A.RunStats._fields_}
        return out

    def jacobian(self):
        """(d outputs / d sticking [P, 9], d outputs / d outgassing [S, 9], source facet ids [S])."""
        L = load_library()
        ns = L.mfg_sens_sources(self.sim.h)
        js = np.zeros((len(self.params), N_OUT))
        jq = np.zeros((ns, N_OUT))
        src = np.zeros(ns, np.int32)
        _check(L.mfg_sens_jacobian(self.sim.h, A.ptr(js, C.c_double), A.ptr(jq, C.c_double), A.ptr(src, C.c_int32)))
        return js, jq, src

    def backward(self, dl_dy):
        dl_dy = np.ascontiguousarray(dl_dy, np.float64)
        L = load_library()
        ns = L.mfg_sens_sources(self.sim.h)
        ds = np.zeros(len(self.params))
        dq = np.zeros(ns)
        _check(L.mfg_sens_backward(self.sim.h, A.ptr(dl_dy, C.c_double), A.ptr(ds, C.c_double), A.ptr(dq, C.c_double)))
        return ds, dq
