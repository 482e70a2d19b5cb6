"""Angle-map desorption generator (AnglemapGeneration.cpp:14-257) on the CPU.

1. The oracle's generator, drawn many times from the map recorded on the source of test case
   04b, gives back the map's distribution (bin by bin, within counting noise).
2. The GPU generator compiled for the host (tests/cpp/anglemap_host.cpp), with the tables the
   library builds, puts every draw in the same bin as the oracle's generator."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from molflow_sources_gb300 import _abi as A
from oracle import oracle as O
from tests import golden_util

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CASE = "04b-anglemap_desorb-sticking source"


def _map(m, f):
    return (m.desorb_anglemaps[f], int(m.anglemap_phi_width[f]), int(m.anglemap_theta_lower_res[f]),
            int(m.anglemap_theta_higher_res[f]), float(m.anglemap_theta_limit[f]))


def _source(m):
    return [i for i in range(m.n_facets) if m.desorb_type[i] == A.DES_ANGLEMAP][0]


def test_oracle_generator_reproduces_the_recorded_map():
    m, _, _ = golden_util.load(CASE)
    pdf, w, lo, hi, lim = _map(m, _source(m))
    n = 2_000_000
    out = O.anglemap_resample(pdf, w, lo, hi, lim, n).astype(np.float64)
    p = pdf.astype(np.float64) / pdf.sum()
    q = out / n
    # the generator takes the pdf as linear between bin midpoints (and flat in the outer half bins),
    # so it smooths the recorded counts: close in total variation, each well-filled bin within 15 %
    assert 0.5 * np.abs(q - p).sum() < 0.02
    big = p > 0.002
    assert big.sum() > 200
    assert (np.abs(q - p)[big] / p[big]).max() < 0.15
    # and it draws nothing where a whole theta line of the map is empty
    lines = pdf.reshape(lo + hi, w).sum(1)
    assert (out.reshape(lo + hi, w).sum(1)[lines == 0] == 0).all()


@pytest.fixture(scope="module")
def amhost(tmp_path_factory):
    so = str(tmp_path_factory.mktemp("am") / "libamhost.so")
    subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-w",
                    "-I/usr/local/cuda/include", os.path.join(ROOT, "tests/cpp/anglemap_host.cpp"),
                    os.path.join(ROOT, "molflow_sources_gb300/csrc/model_build.cpp"), "-o", so], check=True)
    return C.CDLL(so)


@pytest.mark.parametrize("case", ["04-anglemap_desorb", CASE])
def test_gpu_generator_bins_like_oracle(amhost, case):
    m, _, _ = golden_util.load(case)
    f = _source(m)
    pdf, w, lo, hi, lim = _map(m, f)
    n = 500_000
    r = np.random.default_rng(11).random(2 * n)
    th = np.zeros(n)
    ph = np.zeros(n)
    d = m.desc()
    assert amhost.am_draw(C.byref(d), f, C.c_int64(n), A.ptr(r, C.c_double), A.ptr(th, C.c_double),
                          A.ptr(ph, C.c_double)) == 0
    assert np.isfinite(th).all() and np.isfinite(ph).all()
    assert th.min() >= 0 and th.max() <= np.pi / 2 and ph.min() >= -np.pi and ph.max() < np.pi
    ref = np.zeros((lo + hi) * w, np.uint64)
    O.lib().orc_anglemap_resample(A.ptr(np.ascontiguousarray(pdf, np.uint64), C.c_uint64), w, lo, hi, lim, n,
                                  A.ptr(r, C.c_double), A.ptr(ref, C.c_uint64))
    t = np.where(th < lim, (th / lim * lo).astype(np.int64), lo + ((th - lim) / (np.pi / 2 - lim) * hi).astype(np.int64))
    p = ((ph + 3.1415926) / (2 * np.pi) * w).astype(np.int64)
    t = np.clip(t, 0, lo + hi - 1)
    p = np.clip(p, 0, w - 1)
    mine = np.bincount(t * w + p, minlength=(lo + hi) * w).astype(np.uint64)
    assert np.array_equal(mine, ref)
