"""ctypes mirrors of the C structs declared in include/mfg.h."""
import ctypes as C

MFG_ABI_VERSION = 6
LOG_N = 8   # particle log record: u, v, theta, phi, oriRatio, decay moment, time, speed

MFG_OK = 0
MFG_ERR_INVALID_MODEL = 1
MFG_ERR_NO_SOURCE = 2
MFG_ERR_TIMEOUT = 3
MFG_ERR_ABORTED = 4
MFG_ERR_CUDA = 5
MFG_ERR_UNSUPPORTED_FEATURE = 6
MFG_ERR_INVALID_ARGUMENT = 7
MFG_ERR_BUSY = 8
MFG_ERR_NO_DEVICE = 9
MFG_ERR_LIMIT = 10
MFG_MAX_STRUCTURES = 65536

STATUS_NAMES = {
    0: "MFG_OK", 1: "MFG_ERR_INVALID_MODEL", 2: "MFG_ERR_NO_SOURCE", 3: "MFG_ERR_TIMEOUT",
    4: "MFG_ERR_ABORTED", 5: "MFG_ERR_CUDA", 6: "MFG_ERR_UNSUPPORTED_FEATURE",
    7: "MFG_ERR_INVALID_ARGUMENT", 8: "MFG_ERR_BUSY", 9: "MFG_ERR_NO_DEVICE", 10: "MFG_ERR_LIMIT",
}

DES_NONE, DES_UNIFORM, DES_COSINE, DES_COSINE_N, DES_ANGLEMAP = 0, 1, 2, 3, 4
PROFILE_NONE, PROFILE_U, PROFILE_V, PROFILE_ANGULAR = 0, 1, 2, 3
PROFILE_VELOCITY, PROFILE_ORT_VELOCITY, PROFILE_TAN_VELOCITY = 4, 5, 6
PROFILE_SIZE = 100
COUNT_DES, COUNT_ABS, COUNT_REFL, COUNT_TRANS, COUNT_DIR = 1, 2, 4, 8, 16

FC_NBMCHIT, FC_NBDESORBED, FC_NBABSORBED, FC_N = 0, 1, 2, 3
FS_NBHITEQUIV, FS_NBABSEQUIV, FS_SUM_1_PER_ORT_VEL, FS_SUM_V_ORT, FS_SUM_1_PER_VELOCITY, FS_N = 0, 1, 2, 3, 4, 5
G_NBMCHIT, G_NBHITEQUIV, G_NBDESORBED, G_NBABSEQUIV, G_NBLEAK, G_DIST_TOTAL, G_DIST_FULLHITS, G_N = 0, 1, 2, 3, 4, 5, 6, 8

PREC_FP64, PREC_FP32R = 0, 1

_d = C.POINTER(C.c_double)
_i32 = C.POINTER(C.c_int32)
_u8 = C.POINTER(C.c_uint8)
_u32 = C.POINTER(C.c_uint32)
_u64 = C.POINTER(C.c_uint64)

HIST_BOUNCE, HIST_DISTANCE, HIST_TIME = 1, 2, 4


class HistogramParams(C.Structure):
    _fields_ = [("record", C.c_uint32), ("pad", C.c_uint32), ("bounce_binsize", C.c_uint64),
                ("bounce_max", C.c_uint64), ("distance_binsize", C.c_double), ("distance_max", C.c_double),
                ("time_binsize", C.c_double), ("time_max", C.c_double)]


def histogram_sizes(h):
    """(bounce, distance, time) bin counts of a HistogramParams-like object, 0 when not recorded."""
    b = int(h.bounce_max) // max(int(h.bounce_binsize), 1) + 2 if h.record & HIST_BOUNCE else 0
    d = int(h.distance_max / h.distance_binsize) + 1 if h.record & HIST_DISTANCE else 0
    t = int(h.time_max / h.time_binsize) + 1 if h.record & HIST_TIME else 0
    return b, d, t


# (field name, ctypes type) in declaration order of mfg_model_desc
MODEL_DESC_FIELDS = [
    ("abi_version", C.c_uint32),
    ("n_vertices", C.c_int32),
    ("vertices", _d),
    ("n_facets", C.c_int32),
    ("facet_vertex_start", _i32),
    ("facet_vertex_index", _i32),
    ("sticking", _d),
    ("opacity", _d),
    ("outgassing", _d),
    ("temperature", _d),
    ("accommodation", _d),
    ("desorb_type", _i32),
    ("desorb_exponent", _d),
    ("refl_diffuse", _d),
    ("refl_specular", _d),
    ("refl_cos_exponent", _d),
    ("is_2sided", _u8),
    ("structure", _i32),
    ("link_dest", _i32),
    ("teleport_dest", _i32),
    ("tex_width", _d),
    ("tex_height", _d),
    ("count_flags", _u32),
    ("profile_type", _i32),
    ("max_speed", _d),
    ("anglemap_phi_width", _i32),
    ("anglemap_theta_limit", _d),
    ("anglemap_theta_lower_res", _i32),
    ("anglemap_theta_higher_res", _i32),
    ("anglemap_record", _u8),
    ("sticking_param", _i32),
    ("opacity_param", _i32),
    ("outgassing_param", _i32),
    ("temperature_param", _i32),
    ("enable_sojourn", _u8),
    ("sojourn_freq", _d),
    ("sojourn_e", _d),
    ("is_moving", _u8),
    ("gas_mass", C.c_double),
    ("use_maxwell", C.c_int32),
    ("constant_flow", C.c_int32),
    ("time_window", C.c_double),
    ("enable_decay", C.c_int32),
    ("half_life", C.c_double),
    ("low_flux_mode", C.c_int32),
    ("low_flux_cutoff", C.c_double),
    ("n_structures", C.c_int32),
    ("n_moments", C.c_int32),
    ("moment_time", _d),
    ("moment_window", _d),
    ("n_params", C.c_int32),
    ("param_start", _i32),
    ("param_t", _d),
    ("param_v", _d),
    ("param_log_x", _u8),
    ("param_log_y", _u8),
    ("global_histogram", HistogramParams),
    ("facet_histogram", C.POINTER(HistogramParams)),
    ("motion_type", C.c_int32),
    ("motion_vector1", C.c_double * 3),
    ("motion_vector2", C.c_double * 3),
    ("scatter_enabled", C.c_int32),
    ("scatter_cutoff_enabled", C.c_int32),
    ("scatter_mass_ratio", C.c_double),
    ("scatter_mean_free_path_cm", C.c_double),
    ("scatter_rho", C.c_double),
    ("scatter_cutoff_speed", C.c_double),
    ("desorb_anglemap", _u64),
    ("outgassing_map_width", _i32),
    ("outgassing_map_height", _i32),
    ("outgassing_map_ratio_u", _d),
    ("outgassing_map_ratio_v", _d),
    ("outgassing_map", _d),
    ("enable_force_measurement", C.c_int32),
    ("torque_ref_point", C.c_double * 3),
    ("bvh_facet_weight", _d),
    ("log_facet", C.c_int32),
    ("log_limit", C.c_int64),
]


class ModelDesc(C.Structure):
    _fields_ = MODEL_DESC_FIELDS


class StateLayout(C.Structure):
    _fields_ = [(n, C.c_int64) for n in (
        "n_facets", "n_moments", "texture_cells", "profile_facets", "direction_cells", "anglemap_cells",
        "n_global", "n_facet_counts", "n_facet_sums", "n_texture", "n_profile", "n_direction", "n_anglemap",
        "histogram_bins", "n_histogram", "n_force")]


class StateView(C.Structure):
    _fields_ = [
        ("global_", _d),
        ("facet_counts", _u64),
        ("facet_sums", _d),
        ("texture", _d),
        ("profile", _d),
        ("direction", _d),
        ("anglemap", _u64),
        ("histogram", _d),
        ("force", _d),
    ]


class RunOptions(C.Structure):
    _fields_ = [
        ("precision", C.c_int32),
        ("seed", C.c_uint64),
        ("block_size", C.c_int32),
        ("blocks_per_sm", C.c_int32),
        ("smem_bvh_levels", C.c_int32),
        ("time_limit_s", C.c_double),
        ("max_steps_per_particle", C.c_uint64),
        ("use_graph", C.c_int32),
        ("particles_per_request", C.c_int32),
    ]


class RunStats(C.Structure):
    _fields_ = [
        ("desorbed", C.c_uint64),
        ("hits", C.c_uint64),
        ("leaks", C.c_uint64),
        ("rechecks", C.c_uint64),
        ("dropped", C.c_uint64),
        ("kernel_ms", C.c_double),
        ("total_ms", C.c_double),
        ("status", C.c_int32),
        ("kernel_launches", C.c_int32),
    ]


def ptr(arr, ctype):
    """Pointer to a contiguous numpy array (None -> NULL)."""
    if arr is None:
        return C.POINTER(ctype)()
    return arr.ctypes.data_as(C.POINTER(ctype))
