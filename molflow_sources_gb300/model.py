"""Host-side model description: the MolflowSimulationModel fields the tracer reads.

`Model` holds the geometry (vertices3 + polygon index lists, as in
src/Simulation/MolflowSimGeom.h:158-232) and per-facet / global parameters as
numpy arrays, and packs them into the flat `mfg_model_desc` of include/mfg.h.
`SimuState` is the GlobalSimuState-shaped result (src/Simulation/MolflowSimGeom.h:56-154).
"""
import ctypes as C
import math

import numpy as np

from . import _abi as A

# per-facet arrays: name -> (dtype, default)
FACET_FIELDS = {
    "sticking": (np.float64, 0.0),
    "opacity": (np.float64, 1.0),
    "outgassing": (np.float64, 0.0),
    "temperature": (np.float64, 293.15),
    "accommodation": (np.float64, 1.0),
    "desorb_type": (np.int32, A.DES_NONE),
    "desorb_exponent": (np.float64, 0.0),
    "refl_diffuse": (np.float64, 1.0),
    "refl_specular": (np.float64, 0.0),
    "refl_cos_exponent": (np.float64, 0.0),
    "is_2sided": (np.uint8, 0),
    "structure": (np.int32, 0),
    "link_dest": (np.int32, 0),
    "teleport_dest": (np.int32, 0),
    "tex_width": (np.float64, 0.0),
    "tex_height": (np.float64, 0.0),
    "count_flags": (np.uint32, 0),
    "profile_type": (np.int32, A.PROFILE_NONE),
    "max_speed": (np.float64, 0.0),
    "anglemap_phi_width": (np.int32, 0),
    "anglemap_theta_limit": (np.float64, 1.570796326),
    "anglemap_theta_lower_res": (np.int32, 0),
    "anglemap_theta_higher_res": (np.int32, 0),
    "anglemap_record": (np.uint8, 0),
    "sticking_param": (np.int32, -1),
    "opacity_param": (np.int32, -1),
    "outgassing_param": (np.int32, -1),
    "temperature_param": (np.int32, -1),
    "enable_sojourn": (np.uint8, 0),
    "sojourn_freq": (np.float64, 0.0),
    "sojourn_e": (np.float64, 0.0),
    "is_moving": (np.uint8, 0),
    # facet histogram settings (sh.facetHistogramParams): MFG_HIST_* bits and bin sizes / limits
    "hist_record": (np.uint32, 0),
    "hist_bounce_binsize": (np.uint64, 1),
    "hist_bounce_max": (np.uint64, 0),
    "hist_distance_binsize": (np.float64, 1.0),
    "hist_distance_max": (np.float64, 0.0),
    "hist_time_binsize": (np.float64, 1.0),
    "hist_time_max": (np.float64, 0.0),
}
HIST_FIELDS = ("record", "bounce_binsize", "bounce_max", "distance_binsize", "distance_max", "time_binsize", "time_max")
HIST_DTYPE = np.dtype([("record", np.uint32), ("pad", np.uint32), ("bounce_binsize", np.uint64),
                       ("bounce_max", np.uint64), ("distance_binsize", np.float64), ("distance_max", np.float64),
                       ("time_binsize", np.float64), ("time_max", np.float64)])

_CTYPE = {np.float64: C.c_double, np.int32: C.c_int32, np.uint8: C.c_uint8, np.uint32: C.c_uint32}


class Model:
    """Geometry + parameters of one simulation model (units: cm, s, K, g/mol, Pa m3/s)."""

    def __init__(self, vertices, facets, **kw):
        self.vertices = np.ascontiguousarray(vertices, dtype=np.float64).reshape(-1, 3)
        self.facets = [list(map(int, f)) for f in facets]
        nf = len(self.facets)
        self.facet_vertex_start = np.zeros(nf + 1, dtype=np.int32)
        self.facet_vertex_start[1:] = np.cumsum([len(f) for f in self.facets])
        self.facet_vertex_index = np.ascontiguousarray(
            np.concatenate([np.asarray(f, dtype=np.int32) for f in self.facets]) if nf else np.zeros(0, np.int32))
        for name, (dt, default) in FACET_FIELDS.items():
            setattr(self, name, np.full(nf, default, dtype=dt))
        # MolflowSimulationModel::sp / otfParams
        self.gas_mass = 28.0
        self.use_maxwell = 1
        self.constant_flow = 1
        self.time_window = 1e-10
        self.enable_decay = 0
        self.half_life = 1.0
        self.low_flux_mode = 0
        self.low_flux_cutoff = 1e-7
        self.n_structures = 1
        self.moment_time = np.zeros(0)
        self.moment_window = np.zeros(0)
        self.params = []   # list of (t array, v array, logx, logy)
        # sp.motionType / motionVector1 / motionVector2 (moving facets)
        self.motion_type = 0
        self.motion_vector1 = (0.0, 0.0, 0.0)
        self.motion_vector2 = (0.0, 0.0, 0.0)
        # sp.scattering (background-gas collisions)
        self.scatter_enabled = 0
        self.scatter_mass_ratio = 1.0
        self.scatter_mean_free_path_cm = 1e30
        self.scatter_rho = 1e-8
        self.scatter_cutoff_enabled = 0
        self.scatter_cutoff_speed = 0.0
        # recorded angle maps of the facets that desorb by angle map: {facet: uint64 counts}
        self.desorb_anglemaps = {}
        # outgassing maps (useOutgassingFile): {facet: dict(width, height, ratio_u, ratio_v,
        # values = height x width rates in Pa m^3/s)}
        self.outgassing_maps = {}
        # sp.enableForceMeasurement, sp.torqueRefPoint (cm)
        self.enable_force_measurement = 0
        self.torque_ref_point = (0.0, 0.0, 0.0)
        # BVH split weights per facet (ProbSplit), None: surface-area heuristic
        self.bvh_facet_weight = None
        # particle logger: facet (-1 none) and record limit (otfParams.logFacetId, logLimit)
        self.log_facet = -1
        self.log_limit = 0
        # sp.globalHistogramParams
        self.global_histogram = dict(record=0, bounce_binsize=1, bounce_max=0, distance_binsize=1.0,
                                     distance_max=0.0, time_binsize=1.0, time_max=0.0)
        for k, v in kw.items():
            setattr(self, k, v)

    @property
    def n_facets(self):
        return len(self.facets)

    def set_moments(self, times, windows):
        order = np.argsort(times, kind="stable")
        self.moment_time = np.ascontiguousarray(np.asarray(times, np.float64)[order])
        self.moment_window = np.ascontiguousarray(np.broadcast_to(np.asarray(windows, np.float64), (len(order),))[order])

    def add_param(self, t, v, logx=False, logy=False):
        self.params.append((np.asarray(t, np.float64), np.asarray(v, np.float64), int(logx), int(logy)))
        return len(self.params) - 1

    def desc(self):
        """Pack into mfg_model_desc; the returned object keeps the arrays alive."""
        d = A.ModelDesc()
        keep = []

        def p(arr, ct):
            a = np.ascontiguousarray(arr)
            keep.append(a)
            return a.ctypes.data_as(C.POINTER(ct))

        d.abi_version = A.MFG_ABI_VERSION
        d.n_vertices = self.vertices.shape[0]
        d.vertices = p(self.vertices.reshape(-1), C.c_double)
        d.n_facets = self.n_facets
        d.facet_vertex_start = p(self.facet_vertex_start, C.c_int32)
        d.facet_vertex_index = p(self.facet_vertex_index, C.c_int32)
        for name, (dt, _) in FACET_FIELDS.items():
            if name.startswith("hist_"):   # packed into facet_histogram below
                continue
            arr = np.asarray(getattr(self, name), dtype=dt)
            assert arr.shape == (self.n_facets,), name
            setattr(d, name, p(arr, _CTYPE[dt]))
        d.gas_mass = float(self.gas_mass)
        d.use_maxwell = int(self.use_maxwell)
        d.constant_flow = int(self.constant_flow)
        d.time_window = float(self.time_window)
        d.enable_decay = int(self.enable_decay)
        d.half_life = float(self.half_life)
        d.low_flux_mode = int(self.low_flux_mode)
        d.low_flux_cutoff = float(self.low_flux_cutoff)
        d.n_structures = int(self.n_structures)
        d.n_moments = len(self.moment_time)
        d.moment_time = p(np.asarray(self.moment_time, np.float64), C.c_double)
        d.moment_window = p(np.asarray(self.moment_window, np.float64), C.c_double)
        d.n_params = len(self.params)
        starts = np.zeros(len(self.params) + 1, np.int32)
        if self.params:
            starts[1:] = np.cumsum([len(t) for t, _, _, _ in self.params])
            pt = np.concatenate([t for t, _, _, _ in self.params])
            pv = np.concatenate([v for _, v, _, _ in self.params])
        else:
            pt = np.zeros(1)
            pv = np.zeros(1)
        d.param_start = p(starts, C.c_int32)
        d.param_t = p(pt, C.c_double)
        d.param_v = p(pv, C.c_double)
        d.param_log_x = p(np.array([x[2] for x in self.params] or [0], np.uint8), C.c_uint8)
        d.param_log_y = p(np.array([x[3] for x in self.params] or [0], np.uint8), C.c_uint8)
        d.motion_type = int(self.motion_type)
        d.motion_vector1 = (C.c_double * 3)(*map(float, self.motion_vector1))
        d.motion_vector2 = (C.c_double * 3)(*map(float, self.motion_vector2))
        d.scatter_enabled = int(self.scatter_enabled)
        d.scatter_cutoff_enabled = int(self.scatter_cutoff_enabled)
        d.scatter_mass_ratio = float(self.scatter_mass_ratio)
        d.scatter_mean_free_path_cm = float(self.scatter_mean_free_path_cm)
        d.scatter_rho = float(self.scatter_rho)
        d.scatter_cutoff_speed = float(self.scatter_cutoff_speed)
        am_facets = [i for i in range(self.n_facets) if self.desorb_type[i] == A.DES_ANGLEMAP]
        if am_facets:
            parts = []
            for i in am_facets:
                n = int(self.anglemap_phi_width[i]) * int(self.anglemap_theta_lower_res[i] + self.anglemap_theta_higher_res[i])
                a = np.zeros(n, np.uint64)
                src = np.asarray(self.desorb_anglemaps.get(i, []), np.uint64).ravel()
                a[:min(n, src.size)] = src[:n]
                parts.append(a)
            d.desorb_anglemap = p(np.concatenate(parts), C.c_uint64)
        if self.bvh_facet_weight is not None:
            d.bvh_facet_weight = p(np.asarray(self.bvh_facet_weight, np.float64).reshape(self.n_facets), C.c_double)
        d.log_facet = int(self.log_facet)
        d.log_limit = int(self.log_limit)
        d.enable_force_measurement = int(self.enable_force_measurement)
        d.torque_ref_point = (C.c_double * 3)(*map(float, self.torque_ref_point))
        if self.outgassing_maps:
            ow = np.zeros(self.n_facets, np.int32)
            oh = np.zeros(self.n_facets, np.int32)
            oru = np.zeros(self.n_facets, np.float64)
            orv = np.zeros(self.n_facets, np.float64)
            vals = []
            for i in sorted(self.outgassing_maps):
                g = self.outgassing_maps[i]
                v = np.asarray(g["values"], np.float64)
                ow[i], oh[i] = int(g["width"]), int(g["height"])
                oru[i], orv[i] = float(g["ratio_u"]), float(g["ratio_v"])
                vals.append(v.reshape(-1)[:ow[i] * oh[i]])
            d.outgassing_map_width = p(ow, C.c_int32)
            d.outgassing_map_height = p(oh, C.c_int32)
            d.outgassing_map_ratio_u = p(oru, C.c_double)
            d.outgassing_map_ratio_v = p(orv, C.c_double)
            d.outgassing_map = p(np.concatenate(vals), C.c_double)
        gh = A.HistogramParams()
        for k in HIST_FIELDS:
            setattr(gh, k, type(getattr(gh, k))(self.global_histogram[k]))
        d.global_histogram = gh
        if self.hist_record.any():
            fh = np.zeros(self.n_facets, HIST_DTYPE)
            for k in HIST_FIELDS:
                fh[k] = getattr(self, "hist_" + k)
            keep.append(fh)
            d.facet_histogram = fh.ctypes.data_as(C.POINTER(A.HistogramParams))
        d._keep = keep
        return d

    # ------------------------------------------------------------ layout --
    def texture_dims(self):
        """(texWidth, texHeight) per facet: ceil of the precise sizes, 0 when untextured."""
        w = np.zeros(self.n_facets, np.int64)
        h = np.zeros(self.n_facets, np.int64)
        tx = (self.tex_width * self.tex_height) > 0
        w[tx] = np.maximum(1, np.ceil(self.tex_width[tx] - 1e-9)).astype(np.int64)
        h[tx] = np.maximum(1, np.ceil(self.tex_height[tx] - 1e-9)).astype(np.int64)
        return w, h

    def layout(self):
        """Sizes of every GlobalSimuState array (same rule as mfg_state_layout_of)."""
        w, h = self.texture_dims()
        cells = w * h
        nm = len(self.moment_time)
        B = 1 + nm
        tex_off = np.full(self.n_facets, -1, np.int64)
        dir_off = np.full(self.n_facets, -1, np.int64)
        ang_off = np.full(self.n_facets, -1, np.int64)
        prof_idx = np.full(self.n_facets, -1, np.int64)
        tc = dc = ac = pc = 0
        for i in range(self.n_facets):
            if cells[i] > 0:
                tex_off[i] = tc
                tc += cells[i]
                if self.count_flags[i] & A.COUNT_DIR:
                    dir_off[i] = dc
                    dc += cells[i]
            if self.profile_type[i] != A.PROFILE_NONE:
                prof_idx[i] = pc
                pc += 1
            if self.anglemap_record[i] and self.anglemap_phi_width[i] > 0 and \
                    self.anglemap_theta_lower_res[i] + self.anglemap_theta_higher_res[i] > 0:
                ang_off[i] = ac
                ac += int(self.anglemap_phi_width[i]) * int(self.anglemap_theta_lower_res[i] + self.anglemap_theta_higher_res[i])
        # histograms: the global ones, then each recording facet's, bounce / distance / time
        class _H:
            pass
        hb = 0
        g = _H()
        for k in HIST_FIELDS:
            setattr(g, k, self.global_histogram[k])
        gsz = A.histogram_sizes(g)
        hb += sum(gsz)
        hist_off = np.full(self.n_facets, -1, np.int64)
        hist_sz = np.zeros((self.n_facets, 3), np.int64)
        for i in range(self.n_facets):
            if self.hist_record[i]:
                f = _H()
                for k in HIST_FIELDS:
                    setattr(f, k, getattr(self, "hist_" + k)[i])
                hist_sz[i] = A.histogram_sizes(f)
                hist_off[i] = hb
                hb += int(hist_sz[i].sum())
        return dict(n_facets=self.n_facets, n_moments=nm, blocks=B, texture_cells=int(tc), direction_cells=int(dc),
                    anglemap_cells=int(ac), profile_facets=int(pc), tex_off=tex_off, dir_off=dir_off,
                    ang_off=ang_off, prof_idx=prof_idx, tex_w=w, tex_h=h, histogram_bins=int(hb),
                    global_hist_sizes=gsz, hist_off=hist_off, hist_sizes=hist_sz,
                    force=bool(self.enable_force_measurement))


class SimuState:
    """GlobalSimuState-shaped tallies (numpy), filled through an mfg_state_view."""

    def __init__(self, model_or_layout):
        L = model_or_layout.layout() if isinstance(model_or_layout, Model) else model_or_layout
        self.L = L
        B, F = L["blocks"], L["n_facets"]
        self.global_ = np.zeros(A.G_N, np.float64)
        self.facet_counts = np.zeros((B, F, A.FC_N), np.uint64)
        self.facet_sums = np.zeros((B, F, A.FS_N), np.float64)
        self.texture = np.zeros((B, L["texture_cells"], 3), np.float64)
        self.profile = np.zeros((B, L["profile_facets"], A.PROFILE_SIZE, 3), np.float64)
        self.direction = np.zeros((B, L["direction_cells"], 4), np.float64)
        self.anglemap = np.zeros(max(L["anglemap_cells"], 0), np.uint64)
        self.histogram = np.zeros((B, L.get("histogram_bins", 0)), np.float64)
        # impulse, impulse_square, impulse_momentum (x, y, z each) per facet and moment
        self.force = np.zeros((B, F, 9) if L.get("force", False) or L.get("n_force", 0) else (B, 0, 9), np.float64)

    def view(self):
        v = A.StateView()
        v.global_ = A.ptr(self.global_, C.c_double)
        v.facet_counts = A.ptr(self.facet_counts, C.c_uint64)
        v.facet_sums = A.ptr(self.facet_sums, C.c_double)
        v.texture = A.ptr(self.texture, C.c_double)
        v.profile = A.ptr(self.profile, C.c_double)
        v.direction = A.ptr(self.direction, C.c_double)
        v.anglemap = A.ptr(self.anglemap, C.c_uint64)
        v.histogram = A.ptr(self.histogram, C.c_double)
        v.force = A.ptr(self.force, C.c_double) if self.force.size else None
        return v

    def __iadd__(self, other):
        """GlobalSimuState::operator+= (src/Simulation/MolflowSimGeom.cpp:452-458)."""
        for name in ("global_", "facet_counts", "facet_sums", "texture", "profile", "direction", "anglemap", "histogram",
                     "force"):
            getattr(self, name).__iadd__(getattr(other, name))
        return self

    # derived quantities ---------------------------------------------------
    @property
    def n_desorbed(self):
        return float(self.global_[A.G_NBDESORBED])

    @property
    def n_hits(self):
        return float(self.global_[A.G_NBMCHIT])

    def absorbed(self, facet, moment=0):
        return int(self.facet_counts[moment, facet, A.FC_NBABSORBED])

    def transmission(self, facet):
        """absorbed on `facet` / desorbed (the fixtures' 'A2/SUMDES' formula)."""
        return self.absorbed(facet) / max(self.n_desorbed, 1.0)

    def histograms_of(self, facet=None, moment=0):
        """(bounce, distance, time) histograms of a facet, or the global ones (facet None);
        None for the kinds not recorded."""
        L = self.L
        if facet is None:
            o, sz = 0, L["global_hist_sizes"]
        else:
            o, sz = L["hist_off"][facet], L["hist_sizes"][facet]
            if o < 0:
                return (None, None, None)
        out = []
        for n in sz:
            out.append(self.histogram[moment, o:o + n] if n else None)
            o += n
        return tuple(out)

    def texture_of(self, facet, moment=0):
        L = self.L
        o = L["tex_off"][facet]
        if o < 0:
            return None
        w, h = int(L["tex_w"][facet]), int(L["tex_h"][facet])
        return self.texture[moment, o:o + w * h].reshape(h, w, 3)

    def profile_of(self, facet, moment=0):
        k = self.L["prof_idx"][facet]
        return None if k < 0 else self.profile[moment, k]


# ---------------------------------------------------------------- builders --
def build_pipe(L=10.0, R=1.0, step=64, wall_sticking=0.0, **kw):
    """Tube of length L and radius R as a `step`-sided prism, following the
    reference's BuildPipe spec (src/MolflowGeometry.cpp:106-178): facet 0 is the
    inlet disk (DES_COSINE, outgassing 1, sticking 1), facet 1 the outlet
    (sticking 1), facets 2..step+1 the wall quads."""
    ang = np.arange(step) / step * 2.0 * math.pi
    v = np.zeros((2 * step, 3))
    v[0::2, 0] = R * np.cos(ang)
    v[0::2, 1] = R * np.sin(ang)
    v[1::2, 0] = R * np.cos(ang)
    v[1::2, 1] = R * np.sin(ang)
    v[1::2, 2] = L
    facets = [[2 * i for i in range(step)], [2 * (step - 1 - k) + 1 for k in range(step)]]
    for i in range(step):
        if i < step - 1:
            facets.append([2 * i, 2 * i + 1, 2 * (i + 1) + 1, 2 * (i + 1)])
        else:
            facets.append([2 * i, 2 * i + 1, 1, 0])
    m = Model(v, facets, **kw)
    m.sticking[:] = wall_sticking
    m.sticking[0] = 1.0
    m.sticking[1] = 1.0
    m.desorb_type[0] = A.DES_COSINE
    m.outgassing[0] = 1.0
    return m


def config1_tube(texture_facet=2, tex=64):
    """Steady-state L/R=10 tube (R=1 cm, 64-gon), inlet cosine source, outlet
    sticking 1, walls sticking 0 diffuse, one 64x64 texture on a wall facet,
    Maxwell speeds at 28 g/mol and 293.15 K, constant flow."""
    m = build_pipe(L=10.0, R=1.0, step=64)
    if texture_facet is not None:
        m.tex_width[texture_facet] = float(tex)
        m.tex_height[texture_facet] = float(tex)
        m.count_flags[texture_facet] = A.COUNT_REFL | A.COUNT_ABS
    return m
