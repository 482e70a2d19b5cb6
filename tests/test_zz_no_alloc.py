"""mfg_replay_noalloc: the replay variant that allocates no device memory.

Some callers cannot allocate device memory while they query the tracer (their device memory
belongs to another framework's pool, or they may not block in cudaMalloc/cudaFree).  They pass
device buffers and get the same answers as the allocating mfg_replay.  This file is collected
last and passes on its own in a fresh process as well as after the other tests.
"""
import ctypes as C

import numpy as np
import pytest

from molflow_sources_gb300 import _abi as A
from molflow_sources_gb300.model import config1_tube
from molflow_sources_gb300.simulation import GpuSimulation, load_library
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu


def _bind(L):
    L.mfg_replay_noalloc.argtypes = [C.c_void_p, C.c_int32, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p,
                                     C.c_void_p, C.c_void_p, C.POINTER(C.c_uint64)]
    return L.mfg_replay_noalloc


@pytest.mark.parametrize("precision", [A.PREC_FP32R, A.PREC_FP64])
def test_noalloc_replay_matches_allocating_replay(precision):
    import torch
    L = load_library()
    fn = _bind(L)
    m = config1_tube()
    o, d, last, _, _ = Oracle(m).record_rays(20000, 150000, seed=11)
    n = len(last)
    sim = GpuSimulation(m)
    ref_f, ref_t, ref_n = sim.replay(o, d, last, precision=precision)
    # device buffers owned by the caller (torch here); the entry point allocates none
    d_o = torch.from_numpy(np.ascontiguousarray(o)).cuda()
    d_d = torch.from_numpy(np.ascontiguousarray(d)).cuda()
    d_l = torch.from_numpy(np.ascontiguousarray(last)).cuda()
    for call in range(2):   # the shared array keeps the previous call's contents; results must not depend on it
        out_f = torch.full((n,), -7, dtype=torch.int32, device="cuda")
        out_t = torch.full((n,), -7.0, dtype=torch.float64, device="cuda")
        nre = C.c_uint64(12345)
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        rc = fn(sim.h, precision, n, d_o.data_ptr(), d_d.data_ptr(), d_l.data_ptr(), out_f.data_ptr(),
                out_t.data_ptr(), C.byref(nre))
        assert rc == A.MFG_OK
        torch.cuda.synchronize()
        if call == 1:
            # the first call looked up the array's address; the second allocates no device memory
            assert torch.cuda.mem_get_info()[0] == free_before
        got_f = out_f.cpu().numpy()
        got_t = out_t.cpu().numpy()
        assert np.array_equal(got_f, ref_f), "call %d: %d facets differ" % (call, int((got_f != ref_f).sum()))
        ok = ref_f >= 0
        np.testing.assert_allclose(got_t[ok], ref_t[ok], rtol=1e-9, atol=1e-12)
        assert nre.value == ref_n


def test_noalloc_replay_rejects_too_many_rays():
    L = load_library()
    fn = _bind(L)
    sim = GpuSimulation(config1_tube())
    nre = C.c_uint64(0)
    rc = fn(sim.h, A.PREC_FP32R, (1 << 20) + 1, None, None, None, None, None, C.byref(nre))
    assert rc == A.MFG_ERR_LIMIT
