"""Config-4 batch: 256 independent vacuum components traced together.

Straight tubes, 90-degree elbows and T-junctions with 1k-50k facets each (log-uniform),
walls with their own sticking ~U[0, 0.1], one pump with sticking ~U[0.1, 1] and one
cosine-desorbing inlet.  All geometry is generated here with a fixed seed.
"""
import math

import numpy as np

from . import _abi as A
from .model import Model


def _newell(P):
    """Newell normals of polygons P[n, k, 3] (k vertices each)."""
    Q = np.roll(P, -1, axis=1)
    return np.cross(P, Q).sum(axis=1)


def _orient(V, polys, refs):
    """polys: int array [n, k]; flip rows whose right-hand normal points away from refs[n]."""
    P = V[polys]
    n = _newell(P)
    c = P.mean(axis=1)
    flip = np.einsum("ij,ij->i", n, refs - c) < 0
    polys = polys.copy()
    polys[flip] = polys[flip, ::-1]
    return polys


def _sweep(k, centres, tangents, normals, radius):
    """Ring vertices [len(centres) * k, 3] and wall quads [(len-1) * k, 4]."""
    binorm = np.cross(tangents, normals)
    a = 2 * np.pi * np.arange(k) / k
    V = (centres[:, None, :] + radius * (np.cos(a)[None, :, None] * normals[:, None, :] +
                                         np.sin(a)[None, :, None] * binorm[:, None, :])).reshape(-1, 3)
    r = np.arange(len(centres) - 1)[:, None]
    j = np.arange(k)[None, :]
    j1 = (j + 1) % k
    quads = np.stack([r * k + j, (r + 1) * k + j, (r + 1) * k + j1, r * k + j1], axis=-1).reshape(-1, 4)
    return V, quads


def straight_tube(n_facets, rng):
    k = max(8, int(round(math.sqrt(n_facets / 6))))
    m = max(2, int(round((n_facets - 2) / k)))
    L, R = rng.uniform(5, 50), rng.uniform(0.5, 3)
    z = np.linspace(0, L, m + 1)
    C = np.stack([np.zeros_like(z), np.zeros_like(z), z], axis=1)
    T = np.tile([0.0, 0.0, 1.0], (m + 1, 1))
    N = np.tile([1.0, 0.0, 0.0], (m + 1, 1))
    V, Q = _sweep(k, C, T, N, R)
    refs = np.stack([np.zeros(len(Q)), np.zeros(len(Q)), V[Q].mean(axis=1)[:, 2]], axis=1)
    Q = _orient(V, Q, refs)
    ends = [np.arange(k), m * k + np.arange(k)]
    ends = [e if np.dot(_newell(V[e][None])[0], [0, 0, L / 2] - V[e].mean(0)) > 0 else e[::-1] for e in ends]
    return V, [list(q) for q in Q] + [list(e) for e in ends]


def elbow(n_facets, rng):
    k = max(8, int(round(math.sqrt(n_facets / 6))))
    m = max(4, int(round((n_facets - 2) / k)))
    Rb = rng.uniform(4, 20)
    R = min(rng.uniform(0.5, 2), 0.5 * Rb)
    phi = 0.5 * np.pi * np.arange(m + 1) / m
    C = np.stack([Rb * np.cos(phi), Rb * np.sin(phi), np.zeros_like(phi)], axis=1)
    T = np.stack([-np.sin(phi), np.cos(phi), np.zeros_like(phi)], axis=1)
    N = np.tile([0.0, 0.0, 1.0], (m + 1, 1))
    V, Q = _sweep(k, C, T, N, R)
    c = V[Q].mean(axis=1)
    ang = np.arctan2(c[:, 1], c[:, 0])
    refs = np.stack([Rb * np.cos(ang), Rb * np.sin(ang), np.zeros_like(ang)], axis=1)
    Q = _orient(V, Q, refs)
    mid = C[len(C) // 2]
    ends = [np.arange(k), m * k + np.arange(k)]
    ends = [e if np.dot(_newell(V[e][None])[0], mid - V[e].mean(0)) > 0 else e[::-1] for e in ends]
    return V, [list(q) for q in Q] + [list(e) for e in ends]


def tee(n_facets, rng):
    """Square-duct T: three arms (-x inlet, +x pump, +y closed end) on a central cube."""
    q = max(2, int(round(math.sqrt(n_facets / 60.0))))
    r = max(2, int(round((n_facets - 6 * q * q) / (12.0 * q))))
    w, La = rng.uniform(1, 4), rng.uniform(5, 30)
    h = w / 2
    quads_xyz, refs, groups = [], [], []
    X, Y, Z = np.eye(3)

    def grid(origin, e1, e2, n1, n2, ref_fn):
        i = np.arange(n1)[:, None]
        j = np.arange(n2)[None, :]
        def pt(a, b):
            return (origin[None, None, :] + e1[None, None, :] * (a / n1)[..., None] + e2[None, None, :] * (b / n2)[..., None])
        a = pt(i + 0 * j, j + 0 * i)
        b = pt(i + 1 + 0 * j, j + 0 * i)
        c = pt(i + 1 + 0 * j, j + 1 + 0 * i)
        d = pt(i + 0 * j, j + 1 + 0 * i)
        qd = np.stack([a, b, c, d], axis=2).reshape(-1, 4, 3)
        quads_xyz.append(qd)
        refs.append(ref_fn(qd.mean(axis=1)))
        return len(qd)

    zero = lambda c: np.zeros_like(c)
    grid(np.array([-h, -h, -h]), 2 * h * X, 2 * h * Z, q, q, zero)   # -y face
    grid(np.array([-h, -h, -h]), 2 * h * X, 2 * h * Y, q, q, zero)   # -z face
    grid(np.array([-h, -h, h]), 2 * h * X, 2 * h * Y, q, q, zero)    # +z face
    caps = []
    for axis, sign in ((X, -1.0), (X, 1.0), (Y, 1.0)):
        o1, o2 = [a for a in (X, Y, Z) if not np.allclose(a, axis)]
        base = sign * h * axis
        onaxis = lambda c, axis=axis: (c @ axis)[:, None] * axis[None, :]
        for e, f_ in ((o1, o2), (o2, o1)):
            for side in (-1, 1):
                grid(base + side * h * e - h * f_, sign * axis * La, 2 * h * f_, r, q, onaxis)
        start = sum(len(x) for x in quads_xyz)
        n = grid(sign * (h + La) * axis - h * o1 - h * o2, 2 * h * o1, 2 * h * o2, q, q, zero)
        caps.append(np.arange(start, start + n))
    P = np.concatenate(quads_xyz)
    R = np.concatenate(refs)
    flat = np.round(P.reshape(-1, 3), 9)
    V, inv = np.unique(flat, axis=0, return_inverse=True)
    Qi = inv.reshape(-1, 4)
    Qi = _orient(V, Qi, R)
    return V, [list(x) for x in Qi], caps


def make_instance(kind, n_facets, rng, gas_mass=28.0):
    caps = None
    if kind == "tube":
        V, F = straight_tube(n_facets, rng)
    elif kind == "elbow":
        V, F = elbow(n_facets, rng)
    else:
        V, F, caps = tee(n_facets, rng)
    m = Model(V, F)
    nf = m.n_facets
    m.sticking[:] = rng.uniform(0.0, 0.1, nf)
    if caps is None:
        inlet, pump = np.array([nf - 2]), np.array([nf - 1])
    else:
        inlet, pump = caps[0], caps[1]
    m.sticking[inlet] = 1.0
    m.desorb_type[inlet] = A.DES_COSINE
    m.outgassing[inlet] = 1.0
    m.sticking[pump] = rng.uniform(0.1, 1.0)
    m.gas_mass = gas_mass
    m.pump_facets = pump
    m.inlet_facets = inlet
    m.kind_name = kind
    return m


def config4_batch(n_instances=256, min_facets=1000, max_facets=50000, seed=20260404):
    """n_instances components, facet counts log-uniform in [min, max], kinds cycling tube/elbow/tee."""
    rng = np.random.default_rng(seed)
    kinds = ("tube", "elbow", "tee")
    out = []
    for i in range(n_instances):
        nfac = int(round(math.exp(rng.uniform(math.log(min_facets), math.log(max_facets)))))
        out.append(make_instance(kinds[i % 3], nfac, rng))
    return out
