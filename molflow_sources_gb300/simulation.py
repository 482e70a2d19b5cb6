"""Host-side mirror of the reference simulation interface over the C ABI (libmfg.so).

`GpuSimulation` stands where `MolflowSimulation` (src/Simulation/MolflowSimulation.h:22-45)
and its `MFSim::ParticleTracer` worker threads (src/Simulation/Particle.h:40-129)
stand in molflowCLI: the model goes in once, `SimulationMCStep` advances the
simulation by a number of desorptions, and `UpdateHitsAndLog` adds the tallies
into a `GlobalSimuState`-shaped `SimuState` (src/Simulation/Particle.cpp:21-73,
1294-1312).  All work runs in the CUDA library; this module never computes
tallies itself and raises when the library is missing.
"""
import ctypes as C
import enum
import os
import threading

import numpy as np

from . import _abi as A
from .model import Model, SimuState

_LIB = None
_LIB_LOCK = threading.Lock()


class MfgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s: %s" % (A.STATUS_NAMES.get(code, code), msg))
        self.code = code


class MCStepResult(enum.IntEnum):
    """MFSim::MCStepResult (src/Simulation/Particle.h:24-28)."""
    Success = 0
    DesorptionError = 1
    MaxReached = 2


def library_path():
    from .build import LIB
    return LIB


def load_library(build_if_missing=True):
    """Load libmfg.so (building it when sources are newer).  Raises if unavailable."""
    global _LIB
    with _LIB_LOCK:
        if _LIB is not None:
            return _LIB
        from . import build as B
        if build_if_missing:
            B.build()
        if not os.path.exists(B.LIB):
            raise MfgError(A.MFG_ERR_NO_DEVICE, "libmfg.so is not built (run molflow_sources_gb300.build.build())")
        L = C.CDLL(B.LIB)
        vp = C.c_void_p
        L.mfg_abi_version.restype = C.c_uint32
        L.mfg_last_error.argtypes = [C.c_char_p, C.c_size_t]
        L.mfg_last_error.restype = C.c_size_t
        L.mfg_model_create.argtypes = [C.POINTER(A.ModelDesc), C.POINTER(vp)]
        L.mfg_model_destroy.argtypes = [vp]
        L.mfg_model_destroy.restype = None
        L.mfg_state_layout_of.argtypes = [vp, C.POINTER(A.StateLayout)]
        L.mfg_model_facet_geometry.argtypes = [vp, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.mfg_model_bvh_info.argtypes = [vp, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
        L.mfg_model_outgassing.argtypes = [vp, C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.mfg_sim_create.argtypes = [vp, C.c_int, C.POINTER(vp)]
        L.mfg_sim_destroy.argtypes = [vp]
        L.mfg_sim_destroy.restype = None
        L.mfg_reset.argtypes = [vp]
        L.mfg_set_particle_offset.argtypes = [vp, C.c_uint64]
        L.mfg_particle_offset.argtypes = [vp]
        L.mfg_particle_offset.restype = C.c_uint64
        L.mfg_run.argtypes = [vp, C.c_uint64, C.POINTER(A.RunOptions), C.POINTER(A.RunStats)]
        L.mfg_run_async.argtypes = [vp, C.c_uint64, C.POINTER(A.RunOptions)]
        L.mfg_poll.argtypes = [vp]
        L.mfg_wait.argtypes = [vp, C.c_int64, C.POINTER(A.RunStats)]
        L.mfg_abort.argtypes = [vp]
        L.mfg_fetch.argtypes = [vp, C.POINTER(A.StateView)]
        L.mfg_fetch_log.argtypes = [vp, C.POINTER(C.c_double), C.c_int64, C.POINTER(C.c_int64)]
        L.mfg_model_merge.argtypes = [C.POINTER(vp), C.c_int32, C.POINTER(vp)]
        L.mfg_model_instances.argtypes = [vp]
        L.mfg_model_instances.restype = C.c_int32
        L.mfg_instance_layout.argtypes = [vp, C.c_int32, C.POINTER(A.StateLayout)]
        L.mfg_fetch_instance.argtypes = [vp, C.c_int32, C.POINTER(A.StateView)]
        L.mfg_run_batch.argtypes = [vp, C.POINTER(C.c_uint64), C.POINTER(A.RunOptions), C.POINTER(A.RunStats)]
        L.mfg_run_batch_async.argtypes = [vp, C.POINTER(C.c_uint64), C.POINTER(A.RunOptions)]
        L.mfg_update_sticking.argtypes = [vp, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_double)]
        L.mfg_sens_setup.argtypes = [vp, C.c_int32, C.POINTER(C.c_int32), C.c_int32, C.POINTER(C.c_int32), C.c_int32,
                                     C.POINTER(C.c_int32)]
        L.mfg_sens_sources.argtypes = [vp]
        L.mfg_sens_sources.restype = C.c_int32
        L.mfg_sens_forward.argtypes = [vp, C.c_uint64, C.POINTER(A.RunOptions), C.POINTER(C.c_double), C.POINTER(A.RunStats)]
        L.mfg_sens_jacobian.argtypes = [vp, C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_int32)]
        L.mfg_sens_backward.argtypes = [vp, C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.mfg_autotune.argtypes = [vp, C.c_uint64, C.c_int32, C.c_uint64, C.POINTER(A.RunOptions)]
        L.mfg_replay.argtypes = [vp, C.c_int32, C.c_int64, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                 C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_double),
                                 C.POINTER(C.c_uint64)]
        if L.mfg_abi_version() != A.MFG_ABI_VERSION:
            raise MfgError(A.MFG_ERR_INVALID_MODEL, "libmfg ABI version mismatch")
        _LIB = L
        return L


def last_error():
    L = load_library()
    buf = C.create_string_buffer(1024)
    L.mfg_last_error(buf, 1024)
    return buf.value.decode(errors="replace")


def _check(rc):
    if rc != A.MFG_OK:
        raise MfgError(rc, last_error())
    return rc


def _count(n, what="count"):
    """A particle count or id for an unsigned 64-bit argument of the C ABI (ctypes would wrap a
    negative number)."""
    n = int(n)
    if n < 0 or n >= 1 << 64:
        raise ValueError("%s must be in [0, 2^64), got %d" % (what, n))
    return n


class GpuModel:
    """Device-independent prepared model (facet basis, BVH, tables) — mfg_model."""

    def __init__(self, model: Model):
        self.model = model
        L = load_library()
        self._desc = model.desc()
        h = C.c_void_p()
        _check(L.mfg_model_create(C.byref(self._desc), C.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            load_library().mfg_model_destroy(self.h)
            self.h = None

    __del__ = close

    def layout(self):
        Lo = A.StateLayout()
        _check(load_library().mfg_state_layout_of(self.h, C.byref(Lo)))
        return {f: getattr(Lo, f) for f, _ in A.StateLayout._fields_}

    def facet_geometry(self):
        o = np.zeros((self.model.n_facets, 18))
        area = np.zeros(self.model.n_facets)
        _check(load_library().mfg_model_facet_geometry(self.h, A.ptr(o, C.c_double), A.ptr(area, C.c_double)))
        return o, area

    def bvh_info(self):
        n, d, l = C.c_int64(), C.c_int64(), C.c_int64()
        _check(load_library().mfg_model_bvh_info(self.h, C.byref(n), C.byref(d), C.byref(l)))
        return {"nodes": n.value, "depth": d.value, "leaves": l.value}

    def outgassing(self):
        """CalcTotalOutgassing: molecules desorbed up to the latest moment, final rate in molecules/s
        and in Pa m3/s."""
        a, b, c = C.c_double(), C.c_double(), C.c_double()
        _check(load_library().mfg_model_outgassing(self.h, C.byref(a), C.byref(b), C.byref(c)))
        return {"total_desorbed_molecules": a.value, "final_outgassing_rate": b.value,
                "final_outgassing_rate_pa_m3_s": c.value}


class GpuSimulation:
    """GPU replacement of MolflowSimulation + its ParticleTracer threads."""

    def __init__(self, model: Model = None, device: int = 0):
        self.device = device
        self.h = None
        self.gmodel = None
        self.last_stats = None
        if model is not None:
            self.LoadSimulation(model)

    # --- MolflowSimulation surface (MolflowSimulation.h:22-45) ---
    def LoadSimulation(self, model: Model):
        """Prepare the model (geometry, BVH, tables) and upload it (MolflowSimulation.cpp:92-154)."""
        self.close()
        self.model = model
        self.gmodel = GpuModel(model)
        self._scratch = None   # host state reused by UpdateHitsAndLog
        h = C.c_void_p()
        _check(load_library().mfg_sim_create(self.gmodel.h, self.device, C.byref(h)))
        self.h = h
        return 0

    def RebuildAccelStructure(self, global_state: SimuState = None):
        """Rebuild the BVHs (MolflowSimulationModel::BuildAccelStructure, MolflowSimGeom.cpp:124-184).
        With a state that holds hits, the splits weigh each facet by its share of the hits
        (SplitMethod::ProbSplit); without one, by surface area.  Tallies start from zero."""
        w = None
        if global_state is not None:
            h = np.asarray(global_state.facet_sums[0, :, A.FS_NBHITEQUIV], np.float64)
            if h.sum() > 0:
                w = h / h.sum()
        self.model.bvh_facet_weight = w
        self.LoadSimulation(self.model)
        return 0

    def ResetSimulation(self):
        _check(load_library().mfg_reset(self.h))

    def GetHitsSize(self):
        L = self.gmodel.layout()
        return 8 * (L["n_global"] + L["n_facet_counts"] + L["n_facet_sums"] + L["n_texture"] + L["n_profile"] +
                    L["n_direction"] + L["n_anglemap"])

    def set_particle_offset(self, first_particle):
        _check(load_library().mfg_set_particle_offset(self.h, _count(first_particle, "first_particle")))

    def particle_offset(self):
        return int(load_library().mfg_particle_offset(self.h))

    # --- ParticleTracer surface (Particle.h:45,86) ---
    def SimulationMCStep(self, n_desorptions, precision=A.PREC_FP64, seed=0x4D6F6C66, block_size=0,
                         blocks_per_sm=0, time_limit_s=0.0, max_steps=0, use_graph=False, smem_bvh_levels=0,
                         particles_per_request=0):
        """Desorb and trace n_desorptions particles on the GPU (blocking)."""
        if not time_limit_s:
            time_limit_s = float(os.environ.get("MFG_TIME_LIMIT_S", "0"))
        o = A.RunOptions(precision=precision, seed=seed, block_size=block_size, blocks_per_sm=blocks_per_sm,
                         time_limit_s=time_limit_s, max_steps_per_particle=max_steps, use_graph=int(use_graph),
                         smem_bvh_levels=smem_bvh_levels, particles_per_request=particles_per_request)
        st = A.RunStats()
        rc = load_library().mfg_run(self.h, _count(n_desorptions, "n_desorptions"), C.byref(o), C.byref(st))
        self.last_stats = {f: getattr(st, f) for f, _ in A.RunStats._fields_}
        if rc == A.MFG_ERR_NO_SOURCE:
            return MCStepResult.DesorptionError
        _check(rc)
        return MCStepResult.Success

    def update_sticking(self, facets, values):
        """Change sticking coefficients in place (between runs)."""
        f = np.ascontiguousarray(facets, np.int32)
        v = np.ascontiguousarray(values, np.float64)
        _check(load_library().mfg_update_sticking(self.h, len(f), A.ptr(f, C.c_int32), A.ptr(v, C.c_double)))

    def autotune(self, n_trial, precision=A.PREC_FP32R, seed=0x4D6F6C66):
        """Pick the fastest launch shape for this model (clears tallies); returns it as a dict."""
        o = A.RunOptions()
        _check(load_library().mfg_autotune(self.h, _count(n_trial, "n_trial"), precision, seed, C.byref(o)))
        return {"block_size": o.block_size, "blocks_per_sm": o.blocks_per_sm, "smem_bvh_levels": o.smem_bvh_levels,
                "particles_per_request": o.particles_per_request}

    def run_async(self, n_desorptions, precision=A.PREC_FP64, seed=0x4D6F6C66, time_limit_s=0.0):
        o = A.RunOptions(precision=precision, seed=seed, time_limit_s=time_limit_s)
        _check(load_library().mfg_run_async(self.h, _count(n_desorptions, "n_desorptions"), C.byref(o)))

    def poll(self):
        return load_library().mfg_poll(self.h)

    def wait(self, timeout_ms=-1):
        st = A.RunStats()
        rc = load_library().mfg_wait(self.h, int(timeout_ms), C.byref(st))
        self.last_stats = {f: getattr(st, f) for f, _ in A.RunStats._fields_}
        return rc

    def abort(self):
        _check(load_library().mfg_abort(self.h))

    def fetch(self, state: SimuState = None):
        """Accumulated tallies since the last reset, as a new (or given) SimuState."""
        st = state if state is not None else SimuState(self.model)
        v = st.view()
        _check(load_library().mfg_fetch(self.h, C.byref(v)))
        return st

    def fetch_log(self, capacity=None):
        """Particle log since the last reset as an (n, 8) array (u, v, theta, phi, oriRatio, decay
        moment, time, speed), in no particular order."""
        cap = int(capacity if capacity is not None else max(int(self.model.log_limit), 0))
        out = np.zeros((max(cap, 1), A.LOG_N))
        n = C.c_int64()
        _check(load_library().mfg_fetch_log(self.h, A.ptr(out, C.c_double), cap, C.byref(n)))
        return out[:n.value]

    def UpdateHitsAndLog(self, global_state: SimuState, lock: threading.Lock = None, timeout_ms=10000):
        """Add this simulation's tallies into global_state and clear them (Particle.cpp:21-73,1294-1312)."""
        if self._scratch is None:
            self._scratch = SimuState(self.model)
        local = self.fetch(self._scratch)   # every field is rewritten by the fetch
        if lock is not None:
            if not lock.acquire(timeout=timeout_ms / 1000.0):
                return False
        try:
            global_state += local
        finally:
            if lock is not None:
                lock.release()
        self.ResetSimulation()
        return True

    def replay(self, origin, direction, last, precision=A.PREC_FP64):
        """Intersect given rays (replay mode); returns (hit_facet, hit_t, n_rechecks)."""
        origin = np.ascontiguousarray(origin, np.float64)
        direction = np.ascontiguousarray(direction, np.float64)
        last = np.ascontiguousarray(last, np.int32)
        n = len(last)
        hf = np.zeros(n, np.int32)
        ht = np.zeros(n, np.float64)
        nr = C.c_uint64()
        _check(load_library().mfg_replay(self.h, precision, n, A.ptr(origin, C.c_double), A.ptr(direction, C.c_double),
                                         A.ptr(last, C.c_int32), A.ptr(hf, C.c_int32), A.ptr(ht, C.c_double),
                                         C.byref(nr)))
        return hf, ht, nr.value

    def close(self):
        if getattr(self, "h", None):
            load_library().mfg_sim_destroy(self.h)
            self.h = None
        if getattr(self, "gmodel", None) is not None:
            self.gmodel.close()
            self.gmodel = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class GpuBatch:
    """Many independent models traced in one persistent launch (mfg_model_merge + mfg_run_batch).

    Each instance keeps its geometry, BVH, sources and tallies; particles of all instances
    share one work queue, so instances of different cost balance across the GPU."""

    def __init__(self, models, device=0):
        L = load_library()
        self.models = list(models)
        self.parts = [GpuModel(m) for m in self.models]
        arr = (C.c_void_p * len(self.parts))(*[p.h.value for p in self.parts])
        h = C.c_void_p()
        _check(L.mfg_model_merge(arr, len(self.parts), C.byref(h)))
        self.merged = h
        s = C.c_void_p()
        _check(L.mfg_sim_create(self.merged, device, C.byref(s)))
        self.h = s
        self.last_stats = None

    def run(self, counts, precision=A.PREC_FP32R, seed=0x4D6F6C66, use_graph=False, time_limit_s=0.0,
            block_size=0, blocks_per_sm=0, smem_bvh_levels=0, particles_per_request=0):
        """counts: particles per instance (int applies to all)."""
        if np.isscalar(counts):
            counts = [int(counts)] * len(self.models)
        c = np.ascontiguousarray([_count(k, "counts") for k in counts], dtype=np.uint64)
        if not time_limit_s:
            time_limit_s = float(os.environ.get("MFG_TIME_LIMIT_S", "0"))
        o = A.RunOptions(precision=precision, seed=seed, block_size=block_size, blocks_per_sm=blocks_per_sm,
                         time_limit_s=time_limit_s, use_graph=int(bool(use_graph)), smem_bvh_levels=smem_bvh_levels,
                         particles_per_request=particles_per_request)
        st = A.RunStats()
        rc = load_library().mfg_run_batch(self.h, A.ptr(c, C.c_uint64), C.byref(o), C.byref(st))
        self.last_stats = {f: getattr(st, f) for f, _ in A.RunStats._fields_}
        _check(rc)
        return self.last_stats

    def autotune(self, n_trial, precision=A.PREC_FP32R, seed=0x4D6F6C66):
        """Fastest launch shape for the batch (n_trial particles per instance per trial); clears tallies."""
        o = A.RunOptions()
        _check(load_library().mfg_autotune(self.h, _count(n_trial, "n_trial"), precision, seed, C.byref(o)))
        return {"block_size": o.block_size, "blocks_per_sm": o.blocks_per_sm, "smem_bvh_levels": o.smem_bvh_levels,
                "particles_per_request": o.particles_per_request}

    def fetch_instance(self, i):
        st = SimuState(self.models[i])
        v = st.view()
        _check(load_library().mfg_fetch_instance(self.h, i, C.byref(v)))
        return st

    def reset(self):
        _check(load_library().mfg_reset(self.h))

    def set_particle_offset(self, first_particle):
        _check(load_library().mfg_set_particle_offset(self.h, _count(first_particle, "first_particle")))

    def close(self):
        L = load_library()
        if getattr(self, "h", None):
            L.mfg_sim_destroy(self.h)
            self.h = None
        if getattr(self, "merged", None):
            L.mfg_model_destroy(self.merged)
            self.merged = None
        for p in getattr(self, "parts", []):
            p.close()
        self.parts = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
