"""GlobalSimuState::Compare on the C++ host (mfg_compare_states) against the Python restatement
(compare.compare_states) on the same pairs of results: the same error counts and the same
differences, in the same order."""
import ctypes as C

import numpy as np
import pytest

from molflow_sources_gb300 import _abi as A
from molflow_sources_gb300 import compare
from molflow_sources_gb300.simulation import GpuModel, load_library
from oracle.oracle import Oracle
from tests import golden_util
from tests.test_cpu_results_io import _stored_state


def _native(gm, a, b, glob=0.009, loc=0.07):
    L = load_library()
    L.mfg_compare_states.argtypes = [C.c_void_p, C.POINTER(A.StateView), C.POINTER(A.StateView), C.c_double, C.c_double,
                                     C.POINTER(C.c_int64), C.c_char_p, C.c_size_t]
    counts = (C.c_int64 * 3)()
    buf = C.create_string_buffer(1 << 22)
    va, vb = a.view(), b.view()
    assert L.mfg_compare_states(gm.h, C.byref(va), C.byref(vb), glob, loc, counts, buf, len(buf)) == A.MFG_OK
    return tuple(counts), [s for s in buf.value.decode().split("\n") if s]


def _tags(msgs):
    """The position part of each message (the numbers are formatted differently in each language)."""
    return [m.split(" has large difference")[0] for m in msgs]


def _check(gm, a, b, glob=0.009, loc=0.07):
    g, f, fine, msgs = compare.compare_states(a, b, glob, loc)
    counts, nmsgs = _native(gm, a, b, glob, loc)
    assert counts == (g, f, fine)
    assert _tags(nmsgs) == _tags(msgs)
    return counts, nmsgs


def test_same_model_passes_and_a_different_one_is_flagged():
    m, _, _ = golden_util.load("B02-lr10_pipe_tex")
    gm = GpuModel(m)
    a, _ = Oracle(m).run(200000, seed=5)
    b, _ = Oracle(m).run(200000, seed=5, first_particle=10 ** 9)
    counts, _ = _check(gm, a, b)
    assert counts[:2] == (0, 0)
    m2, _, _ = golden_util.load("B02-lr10_pipe_tex")
    m2.sticking[1] = 0.5
    c, _ = Oracle(m2).run(200000, seed=5)
    counts, msgs = _check(gm, a, c)
    assert counts[0] > 0 and any("absRatio" in s or "hits/des" in s for s in msgs)


def test_oracle_against_stored_b02():
    m, ref, _ = golden_util.load("B02-lr10_pipe_tex")
    gm = GpuModel(m)
    run, _ = Oracle(m).run(400000, seed=5)
    counts, _ = _check(gm, _stored_state(m, ref), run)
    assert counts[:2] == (0, 0)


@pytest.mark.parametrize("case", ["01-quick_pipe_profiles_textures_2sided", "09-histograms",
                                  "05-three_structures_nonsquare_textures"])
def test_fine_differences_agree(case):
    """Tight thresholds, so that profiles, textures, directions and histograms report differences."""
    m, _, _ = golden_util.load(case)
    gm = GpuModel(m)
    a, _ = Oracle(m).run(300000, seed=5)
    b, _ = Oracle(m).run(300000, seed=5, first_particle=10 ** 9)
    counts, msgs = _check(gm, a, b, glob=1e-4, loc=1e-4)
    assert sum(max(c, 0) for c in counts) > 0


def test_no_desorptions():
    m, _, _ = golden_util.load("B02-lr10_pipe_tex")
    gm = GpuModel(m)
    a, _ = Oracle(m).run(1000, seed=5)
    from molflow_sources_gb300.model import SimuState
    empty = SimuState(m)
    counts, msgs = _check(gm, a, empty)
    assert counts == (1, -1, -1) and "Second state" in msgs[0]
