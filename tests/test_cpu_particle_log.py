"""Particle logger in the oracle (LogHit, Particle.cpp:1088-1102): every desorption from, hit on,
absorption on, link pass through and teleport from the logged facet leaves one record, up to the
limit."""
import numpy as np

from molflow_sources_gb300 import _abi as A
from molflow_sources_gb300.model import build_pipe
from oracle.oracle import Oracle
from tests.teleport_model import teleport_pair

SEED = 0x4D6F6C66


def test_outlet_log_has_one_record_per_absorption():
    m = build_pipe(step=16)
    m.log_facet, m.log_limit = 1, 100000
    st, log = Oracle(m).run_logged(20000, seed=SEED)
    assert len(log) == int(st.facet_counts[0, 1, A.FC_NBABSORBED]) > 0
    assert (log[:, 2] > np.pi / 2).all()          # arriving: against the facet normal
    assert ((log[:, 0] >= 0) & (log[:, 0] <= 1) & (log[:, 1] >= 0) & (log[:, 1] <= 1)).all()
    assert (log[:, 4] == 1.0).all() and (log[:, 7] > 0).all()


def test_inlet_log_has_desorptions_and_returns():
    m = build_pipe(step=16)
    m.log_facet, m.log_limit = 0, 100000
    st, log = Oracle(m).run_logged(20000, seed=SEED)
    n_des, n_abs = int(st.facet_counts[0, 0, A.FC_NBDESORBED]), int(st.facet_counts[0, 0, A.FC_NBABSORBED])
    assert len(log) == n_des + n_abs
    assert int((log[:, 2] < np.pi / 2).sum()) == n_des   # leaving along the normal


def test_log_limit_and_teleports():
    m, b_in, b_out = teleport_pair()
    m.log_facet, m.log_limit = 1, 1000                # A's outlet, a teleport source
    st, log = Oracle(m).run_logged(20000, seed=SEED, threads=1)
    assert len(log) == 1000 < int(st.facet_counts[0, 1, A.FC_NBMCHIT])
