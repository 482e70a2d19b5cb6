"""Synthetic workloads: the benchmark geometries, generated with fixed seeds.

config1_tube          — L/R=10 tube (R=1 cm, 64-gon prism), cosine inlet, 64x64 wall texture.
config2_beam_chamber  — elliptical 60x30 mm chamber, 5 m, ~200k triangles (50 points around x
                        2000 rings, Gaussian vertex jitter 0.2 mm), 20 baffles with 10 mm apertures, 4 pumping ports
                        (sticking 0.3), walls sticking ~U[0,0.05] with uniform outgassing per
                        area, 128x128 textures on 50 facets, 90x180 angle map on port 1.
config3_transient     — config 1 with a 1 ms desorption pulse and 100 log-spaced moments.
No public dataset is involved: every input is generated here.
"""
import math

import numpy as np

from . import _abi as A
from .model import FACET_FIELDS, Model, build_pipe


def config1_tube(texture_facet=2, tex=64):
    """Steady-state L/R=10 tube: 64 wall quads (sticking 0, diffuse), inlet 64-gon desorbing
    with a cosine law (sticking 1), outlet 64-gon (sticking 1), 64x64 texture on one wall,
    Maxwell speeds at 28 g/mol and 293.15 K, constant flow."""
    m = build_pipe(L=10.0, R=1.0, step=64)
    if texture_facet is not None:
        m.tex_width[texture_facet] = float(tex)
        m.tex_height[texture_facet] = float(tex)
        m.count_flags[texture_facet] = A.COUNT_REFL | A.COUNT_ABS
    return m


def config3_transient(n_moments=100, window=1e-5, pulse=1e-3):
    """Transient variant of config 1: 1 ms square desorption pulse from the inlet and
    n_moments log-spaced moments from 1e-5 s to 1 s with `window`-wide time windows
    (windows that overlap count an event in each of them)."""
    m = config1_tube()
    m.constant_flow = 0
    m.set_moments(np.logspace(-5, 0, n_moments), window)
    pid = m.add_param([0.0, pulse, pulse * (1 + 1e-9), 10.0], [10.0, 10.0, 0.0, 0.0])
    m.outgassing_param[0] = pid
    return m


def _newell(p):
    n = np.zeros(3)
    for i in range(len(p)):
        a, b = p[i], p[(i + 1) % len(p)]
        n += np.array([(a[1] - b[1]) * (a[2] + b[2]), (a[2] - b[2]) * (a[0] + b[0]), (a[0] - b[0]) * (a[1] + b[1])])
    return n


def config2_beam_chamber(n_around=50, n_rings=2000, length=500.0, a=3.0, b=1.5, n_baffles=20,
                         aperture_r=0.5, n_aperture=32, jitter=0.02, seed=20260101, n_textures=50, tex=128):
    """~200k-triangle beam chamber (units cm)."""
    rng = np.random.default_rng(seed)
    th = np.arange(n_around) / n_around * 2 * math.pi
    zs = np.arange(n_rings + 1) * (length / n_rings)
    X = np.zeros((n_rings + 1, n_around, 3))
    X[:, :, 0] = a * np.cos(th)[None, :]
    X[:, :, 1] = b * np.sin(th)[None, :]
    X[:, :, 2] = zs[:, None]
    X += rng.normal(0.0, jitter, X.shape)
    baffle_rings = sorted(set(int(round((j + 1) * n_rings / (n_baffles + 1))) for j in range(n_baffles)))
    for k in (0, n_rings, *baffle_rings):
        X[k, :, 2] = zs[k]                       # planar end caps and baffles
    # pumping ports: flat 10-segment x 10-ring patches on the bottom (y = -b)
    bottom = int(round(0.75 * n_around))
    port_i = (bottom - 5, bottom + 5)
    port_len = 20   # rings (5 cm)
    port_k = [int(round(f * n_rings)) for f in (0.125, 0.375, 0.625, 0.875)]
    port_cells = set()
    for k0 in port_k:
        for k in range(k0, k0 + port_len + 1):
            for i in range(port_i[0], port_i[1] + 1):
                X[k, i, 0] = a * math.cos(th[i])
                X[k, i, 1] = -b
                X[k, i, 2] = zs[k]
        for k in range(k0, k0 + port_len):
            for i in range(port_i[0], port_i[1]):
                port_cells.add((k, i))
    vid = lambda k, i: k * n_around + (i % n_around)
    nv = (n_rings + 1) * n_around
    facets, kind = [], []   # kind: 0 wall, 1 baffle, 2 end cap, 3+j port j

    allv = X.reshape(-1, 3)
    for k in range(n_rings):
        for i in range(n_around):
            if (k, i) in port_cells:
                continue
            facets.append([vid(k, i), vid(k + 1, i), vid(k + 1, i + 1)])
            kind.append(0)
            facets.append([vid(k, i), vid(k + 1, i + 1), vid(k, i + 1)])
            kind.append(0)
    for j, k0 in enumerate(port_k):
        i0, i1 = port_i
        k1 = k0 + port_len
        loop = [vid(k0, i) for i in range(i0, i1 + 1)] + [vid(k, i1) for k in range(k0 + 1, k1 + 1)] + \
               [vid(k1, i) for i in range(i1 - 1, i0 - 1, -1)] + [vid(k, i0) for k in range(k1 - 1, k0, -1)]
        facets.append(loop)
        kind.append(3 + j)
    # baffles: annulus between the wall ring and a circular aperture, triangulated by zipping the loops
    extra = []
    base = nv
    for k in baffle_rings:
        ap = np.stack([aperture_r * np.cos(np.arange(n_aperture) / n_aperture * 2 * math.pi),
                       aperture_r * np.sin(np.arange(n_aperture) / n_aperture * 2 * math.pi),
                       np.full(n_aperture, zs[k])], axis=1)
        extra.append(ap)
        ai = lambda q: base + (q % n_aperture)
        i = q = 0
        while i < n_around or q < n_aperture:
            # advance along the loop whose next point has the smaller angle fraction
            fi = (i + 1) / n_around
            fq = (q + 1) / n_aperture
            if q >= n_aperture or (i < n_around and fi <= fq):
                facets.append([vid(k, i), vid(k, i + 1), ai(q)])
                i += 1
            else:
                facets.append([vid(k, i), ai(q + 1), ai(q)])
                q += 1
            kind.append(1)
        base += n_aperture
    for k, sgn in ((0, 1), (n_rings, -1)):
        facets.append([vid(k, i) for i in range(n_around)])
        kind.append(2)
    V = np.concatenate([allv] + extra, axis=0)
    kind = np.array(kind)
    # orient walls, ports and end caps toward the chamber axis
    for f in range(len(facets)):
        if kind[f] == 1:
            continue
        p = V[facets[f]]
        n = _newell(p)
        c = p.mean(axis=0)
        ref = np.array([0.0, 0.0, c[2]])
        if kind[f] == 2:
            ref = np.array([0.0, 0.0, length / 2])
        if np.dot(n, ref - c) < 0:
            facets[f] = facets[f][::-1]
    m = Model(V, facets)
    nf = len(facets)
    m.sticking[:] = rng.uniform(0.0, 0.05, nf)
    ports = np.where(kind >= 3)[0]
    m.sticking[ports] = 0.3
    m.is_2sided[kind == 1] = 1
    walls = np.where(kind == 0)[0]
    # uniform outgassing per unit area on the wall facets (1e-9 Pa m3/s per cm2)
    areas = np.array([0.5 * np.linalg.norm(_newell(V[facets[f]])) for f in walls])
    m.outgassing[walls] = 1e-9 * areas
    m.desorb_type[walls] = A.DES_COSINE
    tex_f = walls[np.linspace(0, len(walls) - 1, n_textures).astype(int)]
    m.tex_width[tex_f] = float(tex)
    m.tex_height[tex_f] = float(tex)
    m.count_flags[tex_f] = A.COUNT_REFL | A.COUNT_ABS
    p1 = ports[0]
    m.anglemap_record[p1] = 1
    m.anglemap_phi_width[p1] = 180
    m.anglemap_theta_lower_res[p1] = 90
    m.anglemap_theta_higher_res[p1] = 0
    m.anglemap_theta_limit[p1] = math.pi / 2
    m.kind = kind
    return m


def transparent_tube(transient=False, n_disk=48):
    """Config-1 tube with three two-sided disks across it: z = 2.5 cm fully transparent
    (opacity 0), z = 5 cm semi-transparent (opacity 0.5), z = 7.5 cm with a time-dependent
    opacity parameter (0.2 -> 0.8 over 1 ms).  Each disk has an 8x8 texture counting
    transparent passes, a U profile, and the middle one direction vectors and an angle map.
    With `transient`, the 1 ms inlet pulse and 40 log-spaced moments of config 3 are added."""
    base = config1_tube()
    V = [base.vertices]
    facets = [list(f) for f in base.facets]
    r = 1.0 * math.cos(math.pi / 64) * 0.999          # inside the 64-gon's inscribed circle
    ang = np.arange(n_disk) / n_disk * 2 * math.pi
    nv = len(base.vertices)
    disks = []
    for z in (2.5, 5.0, 7.5):
        ring = np.stack([r * np.cos(ang), r * np.sin(ang), np.full(n_disk, z)], axis=1)
        V.append(ring)
        disks.append(len(facets))
        facets.append(list(range(nv, nv + n_disk)))
        nv += n_disk
    m = Model(np.concatenate(V), facets)
    for k in FACET_FIELDS:
        getattr(m, k)[:base.n_facets] = getattr(base, k)
    d0, d1, d2 = disks
    for d in disks:
        m.is_2sided[d] = 1
        m.sticking[d] = 0.0
        m.tex_width[d] = 8.0
        m.tex_height[d] = 8.0
        m.count_flags[d] = A.COUNT_TRANS | A.COUNT_REFL | A.COUNT_ABS
        m.profile_type[d] = A.PROFILE_U
    m.opacity[d0] = 0.0
    m.opacity[d1] = 0.5
    m.count_flags[d1] |= A.COUNT_DIR
    m.anglemap_record[d1] = 1
    m.anglemap_phi_width[d1] = 36
    m.anglemap_theta_limit[d1] = math.pi / 4
    m.anglemap_theta_lower_res[d1] = 9
    m.anglemap_theta_higher_res[d1] = 9
    m.opacity_param[d2] = m.add_param([0.0, 1e-3], [0.2, 0.8])
    m.disks = disks
    if transient:
        m.constant_flow = 0
        m.set_moments(np.logspace(-5, -1, 40), 1e-5)
        m.outgassing_param[0] = m.add_param([0.0, 1e-3, 1e-3 * (1 + 1e-9), 10.0], [10.0, 10.0, 0.0, 0.0])
    return m


def stacked_disk_tube(n_disks=48, opacity=0.0, n_disk=48, L=10.0):
    """Config-1 tube (L/R = 10) crossed by `n_disks` two-sided disks spaced evenly along it, all of
    the given opacity (0: fully transparent): a ray along the tube crosses more transparent facets
    than one pass list holds."""
    base = config1_tube(texture_facet=None)
    V = [base.vertices]
    facets = [list(f) for f in base.facets]
    r = 1.0 * math.cos(math.pi / 64) * 0.999
    ang = np.arange(n_disk) / n_disk * 2 * math.pi
    nv = len(base.vertices)
    disks = []
    for z in (np.arange(n_disks) + 0.5) * (L / n_disks):
        V.append(np.stack([r * np.cos(ang), r * np.sin(ang), np.full(n_disk, z)], axis=1))
        disks.append(len(facets))
        facets.append(list(range(nv, nv + n_disk)))
        nv += n_disk
    m = Model(np.concatenate(V), facets)
    for k in FACET_FIELDS:
        getattr(m, k)[:base.n_facets] = getattr(base, k)
    for d in disks:
        m.is_2sided[d] = 1
        m.sticking[d] = 0.0
        m.opacity[d] = opacity
    m.disks = np.array(disks)
    return m
