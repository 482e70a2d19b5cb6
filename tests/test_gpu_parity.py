"""GPU parity tests: the CUDA tracer against the CPU oracle and the reference's stored results.

All calls go through the C ABI (libmfg.so).  Integer tallies of the FP64 kernel
must equal the oracle's on the same particles (same Philox streams); FP32R and
fixture comparisons use the 3-standard-error rule of the combined estimate.
"""
import math

import numpy as np
import pytest

from molflow_sources_gb300 import _abi as A
from molflow_sources_gb300.model import build_pipe, config1_tube
from molflow_sources_gb300.simulation import GpuBatch, GpuSimulation, MfgError
from oracle.oracle import Oracle
from tests import golden_util
from tests.stats import batch_means, binom_sigma, z_threshold, zscores

pytestmark = pytest.mark.gpu
SEED = 0x4D6F6C66


@pytest.fixture(scope="module")
def tube():
    return config1_tube()


def test_replay_fp64_facet_ids_bit_exact(tube):
    orc = Oracle(tube)
    o, d, last, hf, ht = orc.record_rays(30000, 300000, seed=SEED)
    assert len(last) > 100000
    sim = GpuSimulation(tube)
    gf, gt, nre = sim.replay(o, d, last, precision=A.PREC_FP64)
    assert np.array_equal(gf, hf), "FP64 replay hit facets differ: %d of %d" % ((gf != hf).sum(), len(hf))
    ok = hf >= 0
    np.testing.assert_allclose(gt[ok], ht[ok], rtol=1e-9, atol=1e-12)
    # FP32 traversal + FP64 recheck: the same facets, recheck rate reported
    ff, ft, nre = sim.replay(o, d, last, precision=A.PREC_FP32R)
    mis = int((ff != hf).sum())
    assert mis == 0, "FP32R misclassified %d of %d rays (rechecks %d)" % (mis, len(hf), nre)
    np.testing.assert_allclose(ft[ok], ht[ok], rtol=1e-9, atol=1e-9)
    assert nre < 0.05 * len(hf)


def test_fp64_tallies_equal_oracle_same_particles(tube):
    n = 50000
    sim = GpuSimulation(tube)
    assert sim.SimulationMCStep(n, precision=A.PREC_FP64, seed=SEED) == 0
    g = sim.fetch()
    r, st = Oracle(tube).run(n, seed=SEED)
    assert g.n_desorbed == n
    assert np.array_equal(g.facet_counts, r.facet_counts)
    assert np.array_equal(g.texture[..., 0], r.texture[..., 0])
    assert g.global_[A.G_NBMCHIT] == r.global_[A.G_NBMCHIT] == st["hits"]
    np.testing.assert_allclose(g.facet_sums, r.facet_sums, rtol=1e-8, atol=1e-6)
    np.testing.assert_allclose(g.texture, r.texture, rtol=1e-8, atol=1e-6)
    np.testing.assert_allclose(g.global_[A.G_DIST_TOTAL], r.global_[A.G_DIST_TOTAL], rtol=1e-9)
    assert sim.last_stats["kernel_launches"] == 1 and sim.last_stats["hits"] == st["hits"]


def test_fp64_continues_streams_across_calls(tube):
    """Two runs of n/2 give the same tallies as one run of n (particle counter persists)."""
    sim = GpuSimulation(tube)
    sim.SimulationMCStep(10000, seed=SEED)
    sim.SimulationMCStep(10000, seed=SEED)
    a = sim.fetch()
    sim2 = GpuSimulation(tube)
    sim2.SimulationMCStep(20000, seed=SEED)
    b = sim2.fetch()
    assert np.array_equal(a.facet_counts, b.facet_counts)


def _oracle_batches(model, n, k):
    orc = Oracle(model)
    out = []
    for b in range(k):
        st, _ = orc.run(n // k, seed=SEED, first_particle=10 ** 9 + b * (n // k))
        out.append(st)
    return out


def test_fp32r_agrees_with_oracle_within_3_sigma(tube):
    n_gpu = 2_000_000
    sim = GpuSimulation(tube)
    sim.SimulationMCStep(n_gpu, precision=A.PREC_FP32R, seed=SEED)
    g = sim.fetch()
    assert sim.last_stats["leaks"] == 0
    batches = _oracle_batches(tube, 400000, 8)
    per = np.array([b.facet_counts[0, :, :].astype(np.float64) / b.n_desorbed for b in batches])
    m, s = batch_means(per)
    # transmission (outlet absorbed / desorbed), binomial sigma
    p_o = m[1, A.FC_NBABSORBED]
    p_g = g.transmission(1)
    z = (p_g - p_o) / math.sqrt(binom_sigma(p_o, 400000) ** 2 + binom_sigma(p_g, n_gpu) ** 2)
    assert abs(z) < 3, (p_g, p_o, z)
    # per-facet hits per desorption, family of 66
    gh = g.facet_counts[0, :, A.FC_NBMCHIT] / g.n_desorbed
    ah = per[:, :, A.FC_NBMCHIT]
    zz = zscores(gh, np.sqrt(gh / g.n_desorbed), m[:, A.FC_NBMCHIT], s[:, A.FC_NBMCHIT])
    assert np.abs(zz).max() < z_threshold(66), np.abs(zz).max()
    # texture counts on the 64x64 wall texture, family of 4096 cells
    # (Poisson counts per cell: a particle rarely hits the same cell twice)
    n_o = sum(b.n_desorbed for b in batches)
    co = sum(b.texture[0, :, 0] for b in batches)
    cg = g.texture[0, :, 0]
    pool = (cg + co) / (g.n_desorbed + n_o)   # pooled rate per cell under the null hypothesis
    zt = (cg / g.n_desorbed - co / n_o) / np.sqrt(np.maximum(pool, 1e-300) * (1.0 / g.n_desorbed + 1.0 / n_o))
    assert np.abs(zt).max() < z_threshold(4096) + 0.5, np.abs(zt).max()
    assert abs(np.mean(zt ** 2) - 1.0) < 0.1, np.mean(zt ** 2)
    # pressure-like sums per hit on the walls (Maxwell speeds)
    fs = g.facet_sums[0, 2:, A.FS_SUM_V_ORT].sum() / g.facet_counts[0, 2:, A.FC_NBMCHIT].sum()
    fo = np.mean([b.facet_sums[0, 2:, A.FS_SUM_V_ORT].sum() / b.facet_counts[0, 2:, A.FC_NBMCHIT].sum() for b in batches])
    assert abs(fs / fo - 1) < 3e-3


def test_fp32r_recheck_rate_and_no_leaks(tube):
    sim = GpuSimulation(tube)
    sim.SimulationMCStep(1_000_000, precision=A.PREC_FP32R, seed=SEED + 1)
    st = sim.last_stats
    assert st["leaks"] == 0 and st["dropped"] == 0
    assert st["rechecks"] < 0.02 * (st["hits"] + st["desorbed"])


def test_golden_b02_transmission_and_wall_texture():
    m, ref, meta = golden_util.load("B02-lr10_pipe_tex")
    n = 4_000_000
    sim = GpuSimulation(m)
    sim.SimulationMCStep(n, precision=A.PREC_FP32R, seed=SEED)
    g = sim.fetch()
    n_ref = ref["ref_global"][A.G_NBDESORBED]
    p_ref = ref["ref_facet_counts"][1, A.FC_NBABSORBED] / n_ref
    p = g.transmission(1)
    z = (p - p_ref) / math.sqrt(binom_sigma(p_ref, n_ref) ** 2 + binom_sigma(p, n) ** 2)
    assert abs(z) < 3, (p, p_ref, z)
    # hits per desorption on the walls
    hd = g.facet_counts[0, 2:, A.FC_NBMCHIT].sum() / n
    hd_ref = ref["ref_facet_counts"][2:, A.FC_NBMCHIT].sum() / n_ref
    assert abs(hd / hd_ref - 1) < 5e-3
    # density profile along the tube: all walls' 100x1 textures summed, vs the reference's sampled walls
    L = g.L
    walls = [i for i in range(2, m.n_facets)]
    prof = np.zeros(100)
    for i in walls:
        prof += g.texture_of(i)[0, :, 0]
    prof /= (len(walls) * n)
    kept = [int(k.split("_")[-1]) for k in ref if k.startswith("ref_tex_") and int(k.split("_")[-1]) >= 2]
    rp = np.mean([ref["ref_tex_%d" % i][0, :, 0] for i in kept], axis=0) / n_ref
    sig = np.sqrt(prof / (len(walls) * n) + rp / (len(kept) * n_ref))
    zp = (prof - rp) / sig
    assert np.abs(zp).max() < z_threshold(100), np.abs(zp).max()


def test_golden_quick_pipe_profile_and_two_sided():
    m, ref, meta = golden_util.load("01-quick_pipe_profiles_textures_2sided")
    n = 4_000_000
    sim = GpuSimulation(m)
    sim.SimulationMCStep(n, precision=A.PREC_FP32R, seed=SEED)
    g = sim.fetch()
    n_ref = ref["ref_global"][A.G_NBDESORBED]
    for f in range(m.n_facets):
        a = g.facet_counts[0, f, A.FC_NBMCHIT] / n
        b = ref["ref_facet_counts"][f, A.FC_NBMCHIT] / n_ref
        # hits per desorption: per-particle counts are correlated, allow 4 binomial-sigma of the hit count
        assert abs(a - b) < 4 * math.sqrt(a / n) + 4 * math.sqrt(b / n_ref), (f, a, b)
    pu = g.profile_of(4)[:, 0] / n
    pr = ref["ref_prof_4"][:, 0] / n_ref
    zp = (pu - pr) / np.sqrt(pu / n + pr / n_ref)
    assert np.abs(zp).max() < z_threshold(100) + 1.0


def test_fp64_quick_pipe_all_tallies_equal_oracle():
    """Fixture 01 geometry (5-gon tube, 2-sided facet, U profile, 50x12 texture with direction
    cells): FP64 kernel and oracle on the same particles give the same integer tallies."""
    m, ref, meta = golden_util.load("01-quick_pipe_profiles_textures_2sided")
    n = 50000
    sim = GpuSimulation(m)
    sim.SimulationMCStep(n, precision=A.PREC_FP64, seed=SEED)
    g = sim.fetch()
    r, _ = Oracle(m).run(n, seed=SEED)
    assert np.array_equal(g.facet_counts, r.facet_counts)
    assert np.array_equal(g.texture[..., 0], r.texture[..., 0])
    assert np.array_equal(g.profile[..., 0], r.profile[..., 0])
    assert np.array_equal(g.direction[..., 3], r.direction[..., 3])
    np.testing.assert_allclose(g.direction[..., :3], r.direction[..., :3], rtol=1e-9, atol=1e-6)
    np.testing.assert_allclose(g.profile, r.profile, rtol=1e-8, atol=1e-6)
    np.testing.assert_allclose(g.texture, r.texture, rtol=1e-8, atol=1e-6)


def clausing_santeler(l_over_r):
    """Transmission probability of a circular tube, Santeler's approximation (J. Vac. Sci.
    Technol. A 4, 1986): 1/(1 + 3L/8R (1 + 1/(3(1 + L/7R)))), within ~0.6 % for all L/R."""
    x = l_over_r
    return 1.0 / (1.0 + 3.0 * x / 8.0 * (1.0 + 1.0 / (3.0 * (1.0 + x / 7.0))))


def test_long_tube_clausing():
    """L/R=1000 tube: transmission vs the reference's stored run (B01) and the Clausing factor."""
    m, ref, meta = golden_util.load("B01-lr1000_pipe")
    n = 4_000_000
    sim = GpuSimulation(m)
    sim.SimulationMCStep(n, precision=A.PREC_FP32R, seed=SEED, time_limit_s=300)
    g = sim.fetch()
    p = g.transmission(1)
    sp = binom_sigma(p, n)
    n_ref = ref["ref_global"][A.G_NBDESORBED]
    p_ref = ref["ref_facet_counts"][1, A.FC_NBABSORBED] / n_ref
    z = (p - p_ref) / math.sqrt(sp ** 2 + binom_sigma(p_ref, n_ref) ** 2)
    assert abs(z) < 3, (p, p_ref)
    w = clausing_santeler(1000.0)
    assert abs(p - w) < 3 * sp + 0.01 * w, (p, w)
    assert g.global_[A.G_NBLEAK] == 0


def test_transient_moments_fp64_match_oracle():
    m = build_pipe(L=10.0, R=1.0, step=16)
    m.constant_flow = 0
    m.set_moments(np.linspace(1e-4, 2e-3, 20), 1e-4)
    pid = m.add_param([0.0, 1e-3, 1.0000001e-3, 1.0], [1.0, 1.0, 0.0, 0.0])
    m.outgassing_param[0] = pid
    m.tex_width[2] = 8
    m.tex_height[2] = 4
    m.count_flags[2] = A.COUNT_REFL
    n = 30000
    sim = GpuSimulation(m)
    sim.SimulationMCStep(n, precision=A.PREC_FP64, seed=SEED)
    g = sim.fetch()
    r, _ = Oracle(m).run(n, seed=SEED)
    assert np.array_equal(g.facet_counts, r.facet_counts)
    assert np.array_equal(g.texture[..., 0], r.texture[..., 0])
    assert g.facet_counts[5].sum() > 0


def test_kernel_time_limit_returns_status_and_context_survives():
    """A closed box without any sink never ends: the kernel stops at its time limit."""
    m = build_pipe(L=10.0, R=1.0, step=8)
    m.sticking[:] = 0.0
    sim = GpuSimulation(m)
    with pytest.raises(MfgError) as e:
        sim.SimulationMCStep(1000, precision=A.PREC_FP32R, time_limit_s=1.0)
    assert e.value.code == A.MFG_ERR_TIMEOUT
    assert sim.last_stats["dropped"] > 0
    # step cap: every particle is dropped after 1000 bounces, run ends normally
    sim.ResetSimulation()
    sim.SimulationMCStep(1000, precision=A.PREC_FP64, max_steps=1000)
    assert sim.last_stats["dropped"] == 1000
    # the context is still usable
    t = GpuSimulation(config1_tube())
    t.SimulationMCStep(1000)
    assert t.fetch().n_desorbed == 1000


def test_autotune_and_occupancy_variants_agree(tube):
    """Every launch shape (block size, register budget, BVH levels staged in shared memory, particles
    per work-queue request) gives identical FP32R tallies for the same particles."""
    sim = GpuSimulation(tube)
    ref = None
    shapes = [(256, b, -1, 0) for b in (2, 3, 4, 6, 8)] + [(512, 4, -1, 0), (1024, 2, -1, 0), (256, 8, 5, 0),
                                                          (256, 8, 9, 0), (1024, 2, 7, 0), (1024, 2, 12, 0),
                                                          (1024, 2, -1, 32), (256, 4, -1, 256), (1024, 2, -1, 65536)]
    for block, bps, lv, ppr in shapes:
        sim.ResetSimulation()
        sim.set_particle_offset(0)
        sim.SimulationMCStep(20000, precision=A.PREC_FP32R, seed=SEED, block_size=block, blocks_per_sm=bps,
                             smem_bvh_levels=lv, particles_per_request=ppr)
        st = sim.fetch()
        if ref is None:
            ref = st
        assert np.array_equal(st.facet_counts, ref.facet_counts), (block, bps, lv, ppr)
        assert np.array_equal(st.texture, ref.texture), (block, bps, lv, ppr)
    with pytest.raises(MfgError):
        sim.SimulationMCStep(100, precision=A.PREC_FP32R, seed=SEED, particles_per_request=16)
    best = sim.autotune(20000)
    assert (best["block_size"], best["blocks_per_sm"]) in [(b, k) for b, k, _, _ in shapes]
    assert best["smem_bvh_levels"] in (-1, 5, 7, 9)
    assert best["particles_per_request"] in (32, 64, 256)
    assert sim.fetch().n_desorbed == 0
    # the tuned shape is the default afterwards
    sim.SimulationMCStep(20000, precision=A.PREC_FP32R, seed=SEED)
    assert sim.last_stats["desorbed"] == 20000


def test_unsupported_feature_is_reported():
    """Teleports are traced in single models but not in batches: the merge reports it."""
    m = config1_tube()
    m.teleport_dest[5] = 3
    with pytest.raises(MfgError) as e:
        GpuBatch([config1_tube(), m])
    assert e.value.code == A.MFG_ERR_UNSUPPORTED_FEATURE
