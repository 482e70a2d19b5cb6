"""Model validation of the library and the oracle, without a GPU: models the reference rejects
or cannot trace are refused at model creation with MFG_ERR_INVALID_MODEL, by both sides."""
import numpy as np
import pytest

from molflow_sources_gb300 import _abi as A
from molflow_sources_gb300.model import build_pipe
from molflow_sources_gb300.simulation import GpuModel, MfgError
from oracle.oracle import Oracle, OracleError
from tests.og_model import og_tube


def _both_reject(m):
    with pytest.raises(MfgError) as e:
        GpuModel(m)
    assert e.value.code == A.MFG_ERR_INVALID_MODEL, e.value
    with pytest.raises(OracleError):
        Oracle(m)


def test_teleport_into_a_facet_of_all_structures():
    m = build_pipe(step=8)
    m.structure[1] = -1
    m.desorb_type[1] = A.DES_NONE
    m.teleport_dest[3] = 2          # into facet 1, which is in all structures
    _both_reject(m)


def test_teleport_destination_below_minus_one():
    m = build_pipe(step=8)
    m.teleport_dest[3] = -2
    _both_reject(m)


def test_outgassing_map_larger_than_its_facet():
    m, _ = og_tube()
    g = m.outgassing_maps[0]
    g["ratio_u"] *= 0.5             # the grid now covers 4.75 cells, the map has 10
    _both_reject(m)


def test_negative_outgassing_map_cell():
    m, vals = og_tube()
    v = vals.copy()
    v[5, 5] = -1.0
    m.outgassing_maps[0]["values"] = v
    _both_reject(m)


def test_angle_map_source_without_a_map():
    m = build_pipe(step=8)
    m.desorb_type[0] = A.DES_ANGLEMAP
    m.anglemap_phi_width[0] = 4
    m.anglemap_theta_lower_res[0] = 2
    m.anglemap_theta_higher_res[0] = 2
    _both_reject(m)


def test_desorbing_facet_in_all_structures():
    m = build_pipe(step=8)
    m.structure[0] = -1
    _both_reject(m)
