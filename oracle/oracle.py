"""ctypes binding of the CPU oracle (oracle.c).

TEST INFRASTRUCTURE: imported only by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, as the checker.  The product path never uses it.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from molflow_sources_gb300 import _abi as A
from molflow_sources_gb300.model import Model, SimuState

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")

ORC_RNG_PHILOX, ORC_RNG_MT = 0, 1


def build(force=False):
    """Compile oracle.c with gcc (OpenMP, no FMA contraction so x86 and Arm agree)."""
    src = os.path.join(HERE, "oracle.c")
    deps = [src, os.path.join(HERE, "oracle.h"), os.path.join(os.path.dirname(HERE), "include", "mfg.h")]
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(d) for d in deps):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O2", "-std=c11", "-D_POSIX_C_SOURCE=200809L", "-fPIC", "-shared", "-fopenmp",
           "-ffp-contract=off", "-fno-fast-math", "-Wall", "-Wno-misleading-indentation",
           "-o", tmp, src, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


class OrcRunOpts(C.Structure):
    _fields_ = [("seed", C.c_uint64), ("first_particle", C.c_uint64), ("n_threads", C.c_int32),
                ("rng_mode", C.c_int32), ("max_steps", C.c_uint64), ("instance", C.c_uint32)]


class OrcStats(C.Structure):
    _fields_ = [("desorbed", C.c_uint64), ("hits", C.c_uint64), ("leaks", C.c_uint64), ("dropped", C.c_uint64),
                ("rays", C.c_uint64), ("node_visits", C.c_uint64), ("prim_tests", C.c_uint64),
                ("seconds", C.c_double), ("threads", C.c_int32)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        L.orc_model_create.argtypes = [C.POINTER(A.ModelDesc), C.POINTER(C.c_void_p), C.c_char_p, C.c_size_t]
        L.orc_model_destroy.argtypes = [C.c_void_p]
        L.orc_layout.argtypes = [C.c_void_p, C.POINTER(A.StateLayout)]
        L.orc_facet_geometry.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.orc_run.argtypes = [C.c_void_p, C.c_uint64, C.POINTER(OrcRunOpts), C.POINTER(A.StateView), C.POINTER(OrcStats)]
        L.orc_run_logged.argtypes = [C.c_void_p, C.c_uint64, C.POINTER(OrcRunOpts), C.POINTER(A.StateView),
                                     C.POINTER(OrcStats), C.POINTER(C.c_double), C.c_int64, C.POINTER(C.c_int64)]
        L.orc_run_sens.argtypes = [C.c_void_p, C.c_uint64, C.POINTER(OrcRunOpts), C.POINTER(A.StateView),
                                   C.POINTER(OrcStats), C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                   C.POINTER(C.c_uint8), C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                   C.POINTER(C.c_double), C.POINTER(C.c_uint64)]
        L.orc_replay.argtypes = [C.c_void_p, C.c_int64, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                 C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_double), C.POINTER(OrcStats)]
        L.orc_record_rays.argtypes = [C.c_void_p, C.c_uint64, C.c_uint64, C.c_int64, C.POINTER(C.c_double),
                                      C.POINTER(C.c_double), C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                      C.POINTER(C.c_double)]
        L.orc_record_rays.restype = C.c_int64
        L.orc_philox4x32.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
        L.orc_maxwell_cdf.argtypes = [C.c_double, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.orc_anglemap_resample.argtypes = [C.POINTER(C.c_uint64), C.c_int, C.c_int, C.c_int, C.c_double, C.c_int64,
                                            C.POINTER(C.c_double), C.POINTER(C.c_uint64)]
        _lib = L
    return _lib


class OracleError(RuntimeError):
    pass


class Oracle:
    """CPU FP64 restatement of the reference tracer for one model."""

    def __init__(self, model: Model):
        self.model = model
        self._desc = model.desc()
        h = C.c_void_p()
        err = C.create_string_buffer(512)
        rc = lib().orc_model_create(C.byref(self._desc), C.byref(h), err, 512)
        if rc != 0:
            raise OracleError("%s: %s" % (A.STATUS_NAMES.get(rc, rc), err.value.decode()))
        self.h = h

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_model_destroy(self.h)
            self.h = None

    def layout(self):
        L = A.StateLayout()
        lib().orc_layout(self.h, C.byref(L))
        return {f: getattr(L, f) for f, _ in A.StateLayout._fields_}

    def facet_geometry(self):
        o = np.zeros((self.model.n_facets, 18))
        area = np.zeros(self.model.n_facets)
        lib().orc_facet_geometry(self.h, A.ptr(o, C.c_double), A.ptr(area, C.c_double))
        return o, area

    def run(self, n_des, seed=0x4D6F6C66, first_particle=0, threads=0, rng=ORC_RNG_PHILOX, state=None,
            max_steps=0, instance=0):
        """Trace n_des particles; tallies are added into `state` (new one if None)."""
        st = state if state is not None else SimuState(self.model)
        o = OrcRunOpts(seed=seed, first_particle=first_particle, n_threads=threads, rng_mode=rng, max_steps=max_steps,
                       instance=instance)
        s = OrcStats()
        v = st.view()
        rc = lib().orc_run(self.h, n_des, C.byref(o), C.byref(v), C.byref(s))
        if rc != 0:
            raise OracleError(A.STATUS_NAMES.get(rc, rc))
        return st, {f: getattr(s, f) for f, _ in OrcStats._fields_}

    def run_logged(self, n_des, seed=0x4D6F6C66, first_particle=0, threads=0, capacity=1_000_000):
        """run() that also returns the particle log as an (n, 8) array."""
        st = SimuState(self.model)
        o = OrcRunOpts(seed=seed, first_particle=first_particle, n_threads=threads, rng_mode=ORC_RNG_PHILOX)
        s = OrcStats()
        v = st.view()
        log = np.zeros((capacity, A.LOG_N))
        n = C.c_int64()
        rc = lib().orc_run_logged(self.h, n_des, C.byref(o), C.byref(v), C.byref(s), A.ptr(log, C.c_double),
                                  capacity, C.byref(n))
        if rc != 0:
            raise OracleError(A.STATUS_NAMES.get(rc, rc))
        return st, log[:n.value]

    def run_sens(self, n_des, params, gauges, pumps, seed=0x4D6F6C66, first_particle=0, threads=0):
        """Trace n_des particles with the score-function bookkeeping of the GPU's sensitivity
        kernel.  Returns (outputs[9] per desorbed particle, d outputs / d sticking [P, 9])."""
        nf = self.model.n_facets
        pof = np.full(nf, -1, np.int32)
        gof = np.full(nf, -1, np.int32)
        pump = np.zeros(nf, np.uint8)
        pof[np.asarray(params)] = np.arange(len(params), dtype=np.int32)
        gof[np.asarray(gauges)] = np.arange(len(gauges), dtype=np.int32)
        pump[np.asarray(pumps)] = 1
        P = len(params)
        a = np.zeros(P * 9 + 1)
        b = np.zeros(P * 9 + 1)
        y = np.zeros(9)
        ovf = C.c_uint64(0)
        st = SimuState(self.model)
        v = st.view()
        s = OrcStats()
        o = OrcRunOpts(seed=seed, first_particle=first_particle, n_threads=threads, rng_mode=ORC_RNG_PHILOX)
        rc = lib().orc_run_sens(self.h, n_des, C.byref(o), C.byref(v), C.byref(s), A.ptr(pof, C.c_int32),
                                A.ptr(gof, C.c_int32), A.ptr(pump, C.c_uint8), P, A.ptr(a, C.c_double),
                                A.ptr(b, C.c_double), A.ptr(y, C.c_double), C.byref(ovf))
        if rc != 0:
            raise OracleError(A.STATUS_NAMES.get(rc, rc))
        if ovf.value:
            raise OracleError("reflection list overflowed for %d particles" % ovf.value)
        s_k = np.asarray(self.model.sticking, np.float64)[np.asarray(params)][:, None]
        jac = (-a[:P * 9].reshape(P, 9) / (1.0 - s_k) + b[:P * 9].reshape(P, 9) / s_k) / n_des
        return y / n_des, jac

    def replay(self, origin, direction, last):
        n = len(last)
        origin = np.ascontiguousarray(origin, np.float64)
        direction = np.ascontiguousarray(direction, np.float64)
        last = np.ascontiguousarray(last, np.int32)
        hf = np.zeros(n, np.int32)
        ht = np.zeros(n, np.float64)
        s = OrcStats()
        lib().orc_replay(self.h, n, A.ptr(origin, C.c_double), A.ptr(direction, C.c_double), A.ptr(last, C.c_int32),
                         A.ptr(hf, C.c_int32), A.ptr(ht, C.c_double), C.byref(s))
        return hf, ht, {f: getattr(s, f) for f, _ in OrcStats._fields_}

    def record_rays(self, n_des, max_rays, seed=0x4D6F6C66):
        o = np.zeros((max_rays, 3))
        d = np.zeros((max_rays, 3))
        last = np.zeros(max_rays, np.int32)
        hf = np.zeros(max_rays, np.int32)
        ht = np.zeros(max_rays)
        n = lib().orc_record_rays(self.h, n_des, seed, max_rays, A.ptr(o, C.c_double), A.ptr(d, C.c_double),
                                  A.ptr(last, C.c_int32), A.ptr(hf, C.c_int32), A.ptr(ht, C.c_double))
        return o[:n], d[:n], last[:n], hf[:n], ht[:n]


def philox4x32(ctr, key):
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    out = (C.c_uint32 * 4)()
    lib().orc_philox4x32(c, k, out)
    return list(out)


def anglemap_resample(pdf, w, lo, hi, limit, n, seed=1):
    """Draw n directions from a recorded angle map with the desorption generator and re-bin them."""
    pdf = np.ascontiguousarray(pdf, np.uint64)
    r = np.random.default_rng(seed).random(2 * n)
    out = np.zeros((lo + hi) * w, np.uint64)
    rc = lib().orc_anglemap_resample(A.ptr(pdf, C.c_uint64), w, lo, hi, limit, n, A.ptr(r, C.c_double),
                                     A.ptr(out, C.c_uint64))
    if rc != 0:
        raise OracleError(A.STATUS_NAMES.get(rc, rc))
    return out


def maxwell_cdf(gas_mass):
    v = np.zeros(100)
    p = np.zeros(100)
    lib().orc_maxwell_cdf(gas_mass, A.ptr(v, C.c_double), A.ptr(p, C.c_double))
    return v, p
