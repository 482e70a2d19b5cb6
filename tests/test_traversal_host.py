"""The GPU traversal code compiled for the host (tests/cpp/traversal_host.cpp) on rays recorded
by the oracle: the FP32 traversal with error bounds never returns a wrong facet once its
ambiguous rays go to FP64, the FP64 traversal returns the oracle's facets, and few rays
need the FP64 recheck."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from molflow_sources_gb300 import _abi as A
from molflow_sources_gb300 import workloads
from oracle.oracle import Oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def trav(tmp_path_factory):
    so = str(tmp_path_factory.mktemp("trav") / "libtrav.so")
    subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-w",
                    "-I/usr/local/cuda/include", os.path.join(ROOT, "tests/cpp/traversal_host.cpp"),
                    os.path.join(ROOT, "molflow_sources_gb300/csrc/model_build.cpp"), "-o", so], check=True)
    return C.CDLL(so)


def _run(L, m, n_des, max_rays):
    o, d, last, hf, ht = Oracle(m).record_rays(n_des, max_rays, seed=5)
    n = len(last)
    desc = m.desc()
    h32 = np.zeros(n, np.int32)
    h64 = np.zeros(n, np.int32)
    rs = np.zeros(8, np.int64)
    na = C.c_int64()
    rc = L.trav_run(C.byref(desc), C.c_int64(n), A.ptr(o, C.c_double), A.ptr(d, C.c_double), A.ptr(last, C.c_int32),
                    A.ptr(h32, C.c_int32), A.ptr(h64, C.c_int32), A.ptr(rs, C.c_int64), C.byref(na))
    assert rc == 0
    return hf, h32, h64, na.value / n, rs


@pytest.mark.parametrize("which", ["tube", "chamber"])
def test_fp32_traversal_with_recheck_is_exact(trav, which):
    if which == "tube":
        m = workloads.config1_tube()
    else:
        m = workloads.config2_beam_chamber(n_rings=400, length=100.0, n_baffles=6, n_textures=5)
    hf, h32, h64, amb, rs = _run(trav, m, 20000, 200000)
    assert np.array_equal(h64, hf)
    assert np.array_equal(h32, h64)
    assert amb < 1e-3, (amb, rs.tolist())


def test_hit_weighted_bvh_gives_the_same_hits(trav):
    """ProbSplit-style BVH (facets weighted by a prior run's hits) changes the tree, not the hits."""
    m = workloads.config2_beam_chamber(n_rings=400, length=100.0, n_baffles=6, n_textures=5)
    r, _ = Oracle(m).run(5000, seed=3)
    w = r.facet_sums[0, :, A.FS_NBHITEQUIV]
    m.bvh_facet_weight = w / w.sum()
    hf, h32, h64, amb, rs = _run(trav, m, 20000, 200000)
    assert np.array_equal(h64, hf)
    assert np.array_equal(h32, h64)
    assert amb < 1e-3
