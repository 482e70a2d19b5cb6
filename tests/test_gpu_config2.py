"""Parity on the headline workload: the full ~200k-triangle beam chamber (elliptical 60x30 mm
section, 5 m, 20 baffles, 4 pumping ports, 50 textures of 128x128 cells, a 90x180 angle map on
port 1), through the C ABI.

* FP64 kernel against the CPU oracle on the same particles: tallies equal up to rare last-bit
  splits of a path at a shared triangle edge (bounded).
* FP32 traversal + FP64 recheck against oracle batches: pumped flux per port, facet hits
  (grouped along the chamber), the 50 textures (8x8-cell blocks) and the angle map (10x10-bin
  blocks) within 3 standard errors of the combined estimate, family-wise.
* Replay of rays recorded by the oracle on the full mesh: FP64 facet ids bit-exact, FP32R
  misclassifies none.
"""
import math

import numpy as np
import pytest

from molflow_sources_gb300 import _abi as A
from molflow_sources_gb300.simulation import GpuSimulation
from molflow_sources_gb300.workloads import config2_beam_chamber
from oracle.oracle import Oracle
from tests.stats import binom_sigma, z_threshold

pytestmark = pytest.mark.gpu
SEED = 0x4D6F6C66


@pytest.fixture(scope="module")
def chamber():
    return config2_beam_chamber()


@pytest.fixture(scope="module")
def sim(chamber):
    s = GpuSimulation(chamber)
    yield s
    s.close()


def ports_of(m):
    return np.where(m.kind >= 3)[0]


def pooled_poisson_z(cg, ng, co, no):
    """Two-sample z of per-desorption rates of counts cg (over ng desorptions) and co (over no),
    with the pooled rate as the Poisson variance under the null hypothesis."""
    cg = np.asarray(cg, np.float64)
    co = np.asarray(co, np.float64)
    pool = (cg + co) / (ng + no)
    s = np.sqrt(np.maximum(pool, 1e-300) * (1.0 / ng + 1.0 / no))
    return np.where(cg + co > 0, (cg / ng - co / no) / s, 0.0)


def facet_groups(m, band_cm=5.0):
    """Group id per facet: (kind, 5 cm band along the chamber)."""
    zc = np.array([m.vertices[f, 2].mean() for f in m.facets])
    band = np.floor(zc / band_cm).astype(np.int64)
    key = m.kind.astype(np.int64) * 100000 + band
    _, gid = np.unique(key, return_inverse=True)
    return gid


def test_fp64_equals_oracle_on_the_same_particles(chamber, sim):
    """Same particles (Philox streams) in the FP64 kernel and the oracle.  Their arithmetic differs
    in the last bits (CUDA's and glibc's acos/sin/cos, fused multiply-adds), so now and then a
    hit within ~1e-15 of an edge shared by two of the chamber's 200k triangles goes to the
    neighbour, and that particle's path continues differently.  Bound: the global counts agree
    to 1e-4, and the facets, texture cells and angle-map bins whose counts differ hold at most
    5e-4 of the hits."""
    n = 20000
    sim.ResetSimulation()
    sim.set_particle_offset(0)
    sim.SimulationMCStep(n, precision=A.PREC_FP64, seed=SEED)
    g = sim.fetch()
    r, st = Oracle(chamber).run(n, seed=SEED)
    assert g.n_desorbed == n and st["leaks"] == 0
    hits = float(st["hits"])
    for k in (A.G_NBMCHIT, A.G_NBABSEQUIV):
        assert abs(g.global_[k] - r.global_[k]) <= 1e-4 * hits, (k, g.global_[k], r.global_[k])
    gc = g.facet_counts.astype(np.int64)
    rc = r.facet_counts.astype(np.int64)
    nd = int((gc != rc).any(axis=-1).sum())
    dh = int(np.abs(gc[..., A.FC_NBMCHIT] - rc[..., A.FC_NBMCHIT]).sum())
    dt = float(np.abs(g.texture[..., 0] - r.texture[..., 0]).sum())
    da = int(np.abs(g.anglemap.astype(np.int64) - r.anglemap.astype(np.int64)).sum())
    print("C2 FP64 vs oracle, %d desorptions, %d hits: %d facets differ (%d hits), texture cells %d hits, "
          "angle map %d" % (n, hits, nd, dh, dt, da))
    assert dh <= 5e-4 * hits and dt <= 5e-4 * hits and da <= 5e-4 * hits
    # the ports' absorptions: the transmission of the two runs agrees to the same bound
    p = ports_of(chamber)
    assert abs(int(gc[0, p, A.FC_NBABSORBED].sum()) - int(rc[0, p, A.FC_NBABSORBED].sum())) <= max(2, 5e-4 * n)


def test_replay_on_full_mesh_bit_exact_and_no_misclassification(chamber, sim):
    orc = Oracle(chamber)
    o, d, last, hf, ht = orc.record_rays(12000, 400000, seed=SEED + 3)
    assert len(hf) > 300000
    gf, gt, _ = sim.replay(o, d, last, precision=A.PREC_FP64)
    assert np.array_equal(gf, hf), "FP64 replay differs on %d of %d rays" % ((gf != hf).sum(), len(hf))
    ok = hf >= 0
    np.testing.assert_allclose(gt[ok], ht[ok], rtol=1e-9, atol=1e-9)
    ff, ft, nre = sim.replay(o, d, last, precision=A.PREC_FP32R)
    mis = int((ff != hf).sum())
    print("C2 replay: %d rays, FP32R misclassified %d, rechecked %d (%.2e)" % (len(hf), mis, nre, nre / len(hf)))
    assert mis == 0, "FP32R misclassified %d of %d rays" % (mis, len(hf))
    np.testing.assert_allclose(ft[ok], ht[ok], rtol=1e-7, atol=1e-7)
    assert nre < 0.01 * len(hf)


@pytest.fixture(scope="module")
def fp32r_and_oracle(chamber, sim):
    nb_g, n_g = 8, 2_500_000
    gpu = []
    for b in range(nb_g):
        sim.ResetSimulation()
        sim.set_particle_offset(10 ** 10 + b * n_g)
        sim.SimulationMCStep(n_g, precision=A.PREC_FP32R, seed=SEED)
        st = sim.last_stats
        assert st["leaks"] == 0 and st["dropped"] == 0
        gpu.append(sim.fetch())
    orc = Oracle(chamber)
    nb_o, n_o = 8, 250_000
    ora = [orc.run(n_o, seed=SEED, first_particle=10 ** 12 + b * n_o)[0] for b in range(nb_o)]
    return gpu, ora


def _sum(states, f):
    return sum(f(s) for s in states)


def test_fp32r_pumped_flux_per_port_within_3_sigma(chamber, fp32r_and_oracle):
    gpu, ora = fp32r_and_oracle
    ng = _sum(gpu, lambda s: s.n_desorbed)
    no = _sum(ora, lambda s: s.n_desorbed)
    ports = ports_of(chamber)
    pg = _sum(gpu, lambda s: s.facet_counts[0, ports, A.FC_NBABSORBED].astype(np.float64)) / ng
    po = _sum(ora, lambda s: s.facet_counts[0, ports, A.FC_NBABSORBED].astype(np.float64)) / no
    z = np.array([(a - b) / math.hypot(binom_sigma(a, ng), binom_sigma(b, no)) for a, b in zip(pg, po)])
    tg, to = pg.sum(), po.sum()
    zt = (tg - to) / math.hypot(binom_sigma(tg, ng), binom_sigma(to, no))
    print("C2 pumped fraction: FP32R %.6f (n %d), oracle %.6f (n %d), difference %.2e +- %.2e (z %.2f); per port z %s"
          % (tg, ng, to, no, tg - to, math.hypot(binom_sigma(tg, ng), binom_sigma(to, no)), zt, np.round(z, 2)))
    assert abs(zt) < 3.0
    assert np.abs(z).max() < z_threshold(len(ports))


def test_fp32r_facet_hits_within_3_sigma(chamber, fp32r_and_oracle):
    """Hits per desorption summed over groups of facets (kind x 5 cm band), batch-means errors;
    and per facet, pooled Poisson z-scores whose spread stays near 1."""
    gpu, ora = fp32r_and_oracle
    gid = facet_groups(chamber)
    ng_ = gid.max() + 1

    def grouped(s):
        return np.bincount(gid, weights=s.facet_counts[0, :, A.FC_NBMCHIT].astype(np.float64), minlength=ng_) / s.n_desorbed

    a = np.array([grouped(s) for s in gpu])
    b = np.array([grouped(s) for s in ora])
    ma, sa = a.mean(0), a.std(0, ddof=1) / math.sqrt(len(a))
    mb, sb = b.mean(0), b.std(0, ddof=1) / math.sqrt(len(b))
    z = (ma - mb) / np.sqrt(sa ** 2 + sb ** 2)
    assert np.abs(z).max() < z_threshold(ng_) + 0.5, (np.abs(z).max(), int(np.argmax(np.abs(z))))
    # per facet
    cg = _sum(gpu, lambda s: s.facet_counts[0, :, A.FC_NBMCHIT].astype(np.float64))
    co = _sum(ora, lambda s: s.facet_counts[0, :, A.FC_NBMCHIT].astype(np.float64))
    zf = pooled_poisson_z(cg, _sum(gpu, lambda s: s.n_desorbed), co, _sum(ora, lambda s: s.n_desorbed))
    k = int(((cg + co) > 0).sum())
    spread = float(np.mean(zf[(cg + co) > 0] ** 2))
    print("C2 per-facet hits: %d facets, mean z^2 %.3f, max |z| %.2f" % (k, spread, np.abs(zf).max()))
    assert spread < 1.3     # repeated hits of one particle on a facet widen the spread a little
    assert np.abs(zf).max() < (z_threshold(k) + 0.5) * math.sqrt(max(1.0, spread))


def _blocks(tex, w, h, bw):
    """Sum a (h, w) array of cell counts into bw x bw blocks."""
    return tex.reshape(h // bw, bw, w // bw, bw).sum(axis=(1, 3))


def test_fp32r_textures_within_3_sigma(chamber, fp32r_and_oracle):
    gpu, ora = fp32r_and_oracle
    L = chamber.layout()
    tex_f = np.where(L["tex_off"] >= 0)[0]
    assert len(tex_f) == 50
    ng = _sum(gpu, lambda s: s.n_desorbed)
    no = _sum(ora, lambda s: s.n_desorbed)
    cg, co = [], []
    for f in tex_f:
        w, h = int(L["tex_w"][f]), int(L["tex_h"][f])
        cg.append(_blocks(_sum(gpu, lambda s: s.texture_of(f)[..., 0]), w, h, 16).ravel())
        co.append(_blocks(_sum(ora, lambda s: s.texture_of(f)[..., 0]), w, h, 16).ravel())
    cg, co = np.concatenate(cg), np.concatenate(co)
    z = pooled_poisson_z(cg, ng, co, no)
    k = int(((cg + co) > 0).sum())
    spread = float(np.mean(z[(cg + co) > 0] ** 2))
    print("C2 textures: %d blocks of 16x16 cells, mean z^2 %.3f, max |z| %.2f" % (k, spread, np.abs(z).max()))
    assert k > 1500     # a triangle covers about half of its texture's cells
    assert spread < 1.3
    assert np.abs(z).max() < (z_threshold(k) + 0.5) * math.sqrt(max(1.0, spread))
    # texture totals per facet
    zt = pooled_poisson_z(cg.reshape(50, -1).sum(1), ng, co.reshape(50, -1).sum(1), no)
    assert np.abs(zt).max() < z_threshold(50) * math.sqrt(max(1.0, spread)) + 0.5


def test_fp32r_angle_map_within_3_sigma(chamber, fp32r_and_oracle):
    gpu, ora = fp32r_and_oracle
    ng = _sum(gpu, lambda s: s.n_desorbed)
    no = _sum(ora, lambda s: s.n_desorbed)
    am_g = _sum(gpu, lambda s: s.anglemap.astype(np.float64)).reshape(90, 180)
    am_o = _sum(ora, lambda s: s.anglemap.astype(np.float64)).reshape(90, 180)
    assert am_g.sum() > 0 and am_o.sum() > 0
    for bw, name in ((10, "10x10-bin blocks"), (1, "bins")):
        cg, co = _blocks(am_g, 180, 90, bw).ravel(), _blocks(am_o, 180, 90, bw).ravel()
        z = pooled_poisson_z(cg, ng, co, no)
        k = int(((cg + co) > 0).sum())
        spread = float(np.mean(z[(cg + co) > 0] ** 2))
        print("C2 angle map (%s): %d, mean z^2 %.3f, max |z| %.2f" % (name, k, spread, np.abs(z).max()))
        assert spread < 1.2
        assert np.abs(z).max() < (z_threshold(k) + 0.5) * math.sqrt(max(1.0, spread))
