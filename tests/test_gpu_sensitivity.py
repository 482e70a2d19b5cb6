"""Score-function sticking/outgassing gradients (mfg_sens_*) against central finite differences
with common random numbers: on the GPU (same Philox particles for s+ds and s-ds) and with the
CPU oracle."""
import math

import numpy as np
import pytest

from molflow_sources_gb300 import _abi as A
from molflow_sources_gb300.sensitivity import SensitivityFunction, config5_neg_tube
from molflow_sources_gb300.simulation import GpuSimulation
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu
SEED = 0x4D6F6C66
DS = 1e-3


def outputs_from_state(st, m, n):
    y = np.zeros(9)
    y[:8] = st.facet_sums[0, m.gauges, A.FS_SUM_V_ORT] / n
    y[8] = st.facet_counts[0, m.neg, A.FC_NBABSORBED].sum() / n
    return y


@pytest.fixture(scope="module")
def setup():
    m = config5_neg_tube()
    sim = GpuSimulation(m)
    sf = SensitivityFunction(sim, m.neg, m.gauges, m.neg)
    return m, sim, sf


def test_forward_outputs_equal_plain_run(setup):
    """The sensitivity kernel traces the same particles as the plain kernel (FP64, same streams)."""
    m, sim, sf = setup
    n = 200000
    sim.ResetSimulation()
    sim.set_particle_offset(0)
    y = sf.forward(n, precision=A.PREC_FP64, seed=SEED)
    plain = outputs_from_state(sim.fetch(), m, n)
    np.testing.assert_allclose(y, plain, rtol=1e-7, atol=1e-12)


def test_gradients_match_central_differences(setup):
    m, sim, sf = setup
    nb, n = 8, 4_000_000
    js = []
    for b in range(nb):
        sim.ResetSimulation()
        sim.set_particle_offset(b * n)
        sf.forward(n, seed=SEED)
        js.append(sf.jacobian()[0])
    js = np.array(js)
    # parameters with the largest pumped-flux sensitivity, and the one most coupled to gauge 0,
    # chosen on batch 0 and estimated on the other batches (the largest of 1000 noisy
    # estimates is biased upwards)
    pick = list(np.argsort(-np.abs(js[0, :, 8]))[:3]) + [int(np.argmax(np.abs(js[0, :, 0])))]
    jm, jse = js[1:].mean(0), js[1:].std(0, ddof=1) / math.sqrt(nb - 1)
    for k in pick:
        f = int(m.neg[k])
        s0 = float(m.sticking[f])
        fd = []
        for b in range(nb):
            ys = []
            for s in (s0 + DS, s0 - DS):
                sim.update_sticking([f], [s])
                sim.ResetSimulation()
                sim.set_particle_offset(b * n)   # common random numbers: the same particles
                sim.SimulationMCStep(n, precision=A.PREC_FP32R, seed=SEED)
                ys.append(outputs_from_state(sim.fetch(), m, n))
            fd.append((ys[0] - ys[1]) / (2 * DS))
        sim.update_sticking([f], [s0])
        fd = np.array(fd)
        fm, fse = fd.mean(0), fd.std(0, ddof=1) / math.sqrt(nb)
        for j in (0, 8):
            sig = math.sqrt(jse[k, j] ** 2 + fse[j] ** 2)
            assert abs(jm[k, j] - fm[j]) < 3.5 * sig + 1e-9, (k, j, jm[k, j], fm[j], sig)


def test_outgassing_gradient_is_the_conditional_mean(setup):
    m, sim, sf = setup
    sim.ResetSimulation()
    y = sf.forward(2_000_000, seed=SEED)
    js, jq, src = sf.jacobian()
    # the inlet (facet 0) dominates the desorptions: its conditional pumped flux is close to the mean
    k = int(np.where(src == 0)[0][0])
    assert abs(jq[k, 8] / y[8] - 1) < 0.05
    ds, dq = sf.backward(np.eye(9)[8])
    np.testing.assert_allclose(ds, js[:, 8])
    np.testing.assert_allclose(dq, jq[:, 8])


def test_gradient_cost_over_forward(setup):
    """Kernel time of the forward run with gradients against the plain forward run on the same
    particles, both at the register budget of 2 resident blocks of 256 threads per SM."""
    m, sim, sf = setup
    n = 4_000_000
    t_fwd, t_sens = [], []
    for _ in range(3):
        sim.ResetSimulation()
        sim.set_particle_offset(0)
        sim.SimulationMCStep(n, precision=A.PREC_FP32R, seed=SEED, block_size=256, blocks_per_sm=2)
        t_fwd.append(sim.last_stats["kernel_ms"])
        sim.set_particle_offset(0)
        sf.forward(n, seed=SEED, block_size=256, blocks_per_sm=2)
        t_sens.append(sf.last_stats["kernel_ms"])
    t_fwd, t_sens = min(t_fwd), min(t_sens)
    print("sensitivity / forward kernel time: %.3f" % (t_sens / t_fwd))
    assert t_sens / t_fwd < 1.3   # the target cost of the gradients: at most 1.3 forward runs


def test_gradient_matches_oracle_finite_difference(setup):
    """Finite difference of the CPU oracle (common random numbers) for the strongest pumped-flux parameter."""
    m, sim, sf = setup
    nb, nj = 4, 4_000_000
    est = []
    for b in range(nb + 1):
        sim.ResetSimulation()
        sim.set_particle_offset(b * nj)
        sf.forward(nj, seed=SEED)
        est.append(sf.jacobian()[0][:, 8])
    # parameter chosen on the first batch, gradient estimated on the others (no selection bias)
    k = int(np.argmax(np.abs(est[0])))
    jk = np.array([e[k] for e in est[1:]])
    jm, jse = jk.mean(), jk.std(ddof=1) / math.sqrt(nb)
    f = int(m.neg[k])
    s0 = float(m.sticking[f])
    n = 4_000_000
    vals = []
    for s in (s0 + 5 * DS, s0 - 5 * DS):
        mm = config5_neg_tube()
        mm.sticking[f] = s
        st, _ = Oracle(mm).run(n, seed=SEED)
        vals.append(outputs_from_state(st, mm, n)[8])
        hits_f = st.facet_counts[0, f, A.FC_NBMCHIT] / n
    fd = (vals[0] - vals[1]) / (10 * DS)
    # common random numbers: only particles whose stick/reflect decision at facet f flips
    # (about hits_f * 10 DS per desorption) can change the output, each by at most one
    sigma = math.sqrt(hits_f * 10 * DS * n) / (n * 10 * DS)
    assert abs(fd - jm) < 0.1 * abs(jm) + 3 * math.hypot(sigma, jse), (fd, jm, sigma, jse)


def _neg_tube_extended(opacity=0.5, n_disk=48):
    """The config-5 tube with a two-sided semi-transparent disk across it between two rings
    (z = 5.3125 cm): the pass list makes the model run on the extended kernel variants."""
    from molflow_sources_gb300.model import FACET_FIELDS, Model
    base = config5_neg_tube()
    r = math.cos(math.pi / 64) * 0.999
    ang = np.arange(n_disk) / n_disk * 2 * math.pi
    ring = np.stack([r * np.cos(ang), r * np.sin(ang), np.full(n_disk, 5.3125)], axis=1)
    nv = len(base.vertices)
    m = Model(np.concatenate([base.vertices, ring]), [list(f) for f in base.facets] + [list(range(nv, nv + n_disk))])
    for k in FACET_FIELDS:
        getattr(m, k)[:base.n_facets] = getattr(base, k)
    d = base.n_facets
    m.is_2sided[d] = 1
    m.opacity[d] = opacity
    m.gauges, m.neg = base.gauges, base.neg
    return m


def test_extended_variant_jacobian_equals_plain_variant():
    """A model that only adds a recorded global histogram runs on the extended kernel variant and
    traces the same particles: FP64 outputs and Jacobians equal the plain variant's."""
    plain = config5_neg_tube()
    ext = config5_neg_tube()
    ext.global_histogram = dict(record=A.HIST_BOUNCE, bounce_binsize=1, bounce_max=100, distance_binsize=1.0,
                                distance_max=0.0, time_binsize=1.0, time_max=0.0)
    out = []
    for m in (plain, ext):
        sim = GpuSimulation(m)
        sf = SensitivityFunction(sim, m.neg, m.gauges, m.neg)
        y = sf.forward(100000, precision=A.PREC_FP64, seed=SEED)
        js, jq, _ = sf.jacobian()
        out.append((y, js, jq))
        sim.close()
    (y0, js0, jq0), (y1, js1, jq1) = out
    assert np.abs(js1[:, 8]).max() > 0 and np.abs(js1[:, :8]).max() > 0
    np.testing.assert_allclose(y1, y0, rtol=1e-9, atol=1e-15)
    np.testing.assert_allclose(js1, js0, rtol=1e-8, atol=1e-9 * np.abs(js0).max())
    np.testing.assert_allclose(jq1, jq0, rtol=1e-8, atol=1e-12)


def test_extended_variant_gradient_matches_central_differences():
    """Semi-transparent disk in the tube (extended variant, FP32R): the strongest pumped-flux
    gradient and the gauge-0 gradient of that parameter against central differences with
    common random numbers."""
    m = _neg_tube_extended()
    sim = GpuSimulation(m)
    sf = SensitivityFunction(sim, m.neg, m.gauges, m.neg)
    nb, n = 6, 2_000_000
    js = []
    for b in range(nb):
        sim.ResetSimulation()
        sim.set_particle_offset(b * n)
        sf.forward(n, seed=SEED)
        js.append(sf.jacobian()[0])
    js = np.array(js)
    k = int(np.argmax(np.abs(js[0, :, 8])))    # chosen on batch 0, estimated on the others
    jm, jse = js[1:].mean(0), js[1:].std(0, ddof=1) / math.sqrt(nb - 1)
    f = int(m.neg[k])
    s0 = float(m.sticking[f])
    fd = []
    for b in range(nb):
        ys = []
        for s in (s0 + DS, s0 - DS):
            sim.update_sticking([f], [s])
            sim.ResetSimulation()
            sim.set_particle_offset(b * n)
            sim.SimulationMCStep(n, precision=A.PREC_FP32R, seed=SEED)
            ys.append(outputs_from_state(sim.fetch(), m, n))
        fd.append((ys[0] - ys[1]) / (2 * DS))
    sim.update_sticking([f], [s0])
    fd = np.array(fd)
    fm, fse = fd.mean(0), fd.std(0, ddof=1) / math.sqrt(nb)
    assert abs(jm[k, 8]) > 5 * jse[k, 8]
    for j in (0, 8):
        sig = math.sqrt(jse[k, j] ** 2 + fse[j] ** 2)
        assert abs(jm[k, j] - fm[j]) < 3.5 * sig + 1e-9, (k, j, jm[k, j], fm[j], sig)
    sim.close()


def test_sensitivity_setup_refuses_low_flux_models():
    from molflow_sources_gb300.simulation import MfgError
    m = config5_neg_tube()
    m.low_flux_mode = 1
    sim = GpuSimulation(m)
    with pytest.raises(MfgError) as e:
        SensitivityFunction(sim, m.neg, m.gauges, m.neg)
    assert e.value.code == A.MFG_ERR_UNSUPPORTED_FEATURE
    sim.close()


def test_gradients_after_autotune(setup):
    """An autotuned plain shape (512- or 1024-thread blocks) does not carry over to the sensitivity
    kernel, which keeps a compiled shape; the outputs are those of an untuned run."""
    m, sim, sf = setup
    sim.ResetSimulation()
    sim.autotune(200000, precision=A.PREC_FP32R, seed=SEED)
    n = 200000
    sim.ResetSimulation()
    sim.set_particle_offset(0)
    y_tuned = sf.forward(n, precision=A.PREC_FP32R, seed=SEED)
    sim.ResetSimulation()
    sim.set_particle_offset(0)
    y_plain = sf.forward(n, precision=A.PREC_FP32R, seed=SEED, block_size=256, blocks_per_sm=2)
    # the same particles; FP64 output sums added in another order
    np.testing.assert_allclose(y_tuned, y_plain, rtol=1e-9, atol=0)


def test_new_setup_drops_the_previous_jacobian():
    """A new mfg_sens_setup (other parameters) drops the Jacobian of the previous one: backward and
    jacobian refuse until the next forward pass, instead of reading the old, smaller matrices."""
    from molflow_sources_gb300.simulation import MfgError
    m = config5_neg_tube()
    sim = GpuSimulation(m)
    try:
        sf = SensitivityFunction(sim, m.neg[:10], m.gauges, m.neg)
        sf.forward(20000, precision=A.PREC_FP32R, seed=SEED)
        sf.backward(np.ones(9))
        sf2 = SensitivityFunction(sim, m.neg, m.gauges, m.neg)
        for call in (lambda: sf2.backward(np.ones(9)), sf2.jacobian):
            with pytest.raises(MfgError) as e:
                call()
            assert e.value.code == A.MFG_ERR_INVALID_ARGUMENT
        sf2.forward(20000, precision=A.PREC_FP32R, seed=SEED)
        js, jq, src = sf2.jacobian()
        assert js.shape == (len(m.neg), 9) and np.isfinite(js).all()
    finally:
        sim.close()
