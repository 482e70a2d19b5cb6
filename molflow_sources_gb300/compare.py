"""Comparison of two GlobalSimuState-shaped results with the rule of MolFlow+'s test suite:
GlobalSimuState::Compare (src/Simulation/MolflowSimGeom.cpp:559-1148), called by the test suite
with a 0.9 % global and a 7 % local threshold (tests/testsuite.cpp:460).

`compare_states(lhs, rhs, glob_threshold, loc_threshold)` returns the three error counts of the
reference, (global, facet, fine), and the messages.  A run passes the suite when the global and
facet counts are 0; "fine" differences (textures, profiles, directions, facet histograms) are
reported only.  The sample-size cut-offs (6400 counts for histogram bins and facet counters,
40000 Monte Carlo hits per facet and moment, 100 for a smoothed profile bin, 640 for a texture
cell), the per-moment threshold max(local, 1/sqrt(hits)), the 40x looser velocity thresholds and
the scales are the reference's, so that a result accepted here is accepted by the suite too.

Restated details of the reference:
* IsEqual(a, b, tol) lives in the absent shared MathTools; it is taken as a relative comparison,
  |a - b| < tol * max(|a|, |b|) (a zero pair is equal).
* The global velocity sums are compared as the reference does, but its tracer never adds into
  the global hit buffer's velocity sums (only facet buffers, Particle.cpp:1194-1230), so in both
  states they are zero; the result keeps no global velocity sums, and the three checks pass.
* The smoothed profile comparisons of sum_1_per_ort_velocity and sum_v_ort smooth countEquiv in
  the reference (MolflowSimGeom.cpp:865-903); this is kept, so the same bins are flagged.
"""
import math

import numpy as np

from . import _abi as A

VELOCITY_THRESHOLD_FACTOR = 40.0


def is_equal(a, b, tol):
    a = float(a)
    b = float(b)
    return abs(a - b) < max(1e-99, tol * max(abs(a), abs(b))) or a == b


def _too_few(a, b, cut):
    """The reference's `sqrt(max(1, min(a, b))) < 80` style skip, with the cut given as a count."""
    return max(1.0, min(float(a), float(b))) < cut


def compare_states(lhs, rhs, glob_threshold=0.009, loc_threshold=0.07):
    """Returns (global_errors, facet_errors, fine_errors, messages)."""
    msgs, fine_msgs = [], []
    g_err = f_err = fine_err = 0
    gl, gr = lhs.global_, rhs.global_
    des_l, des_r = float(gl[A.G_NBDESORBED]), float(gr[A.G_NBDESORBED])
    if des_l == 0 and des_r == 0:
        return 1, -1, -1, ["[Global][desorp] Neither state has recorded desorptions"]
    if des_l == 0:
        return 1, -1, -1, ["[Global][desorp] First state has no recorded desorptions"]
    if des_r == 0:
        return 1, -1, -1, ["[Global][desorp] Second state has no recorded desorptions"]
    a_l, a_r = gl[A.G_NBABSEQUIV] / des_l, gr[A.G_NBABSEQUIV] / des_r
    if not is_equal(a_l, a_r, glob_threshold):
        msgs.append("[Global][absRatio abs/des] has large difference: %r vs %r" % (a_l, a_r))
        g_err += 1
    h_l, h_r = gl[A.G_NBMCHIT] / des_l, gr[A.G_NBMCHIT] / des_r
    if not is_equal(h_l, h_r, glob_threshold):
        msgs.append("[Global][hits/des] has large difference: %r vs %r" % (h_l, h_r))
        g_err += 1
    hits_l, hits_r = float(gl[A.G_NBMCHIT]), float(gr[A.G_NBMCHIT])
    L = lhs.L
    # global histograms, every moment block
    nb_g = int(sum(L.get("global_hist_sizes", (0, 0, 0))))
    if nb_g:
        names = ("Bounces/global hits", "Dist", "Time")
        for m in range(lhs.histogram.shape[0]):
            o = 0
            for kind, n in enumerate(L["global_hist_sizes"]):
                for i in range(int(n)):
                    x, y = lhs.histogram[m, o + i], rhs.histogram[m, o + i]
                    if _too_few(x, y, 6400.0):
                        continue
                    if not is_equal(x / hits_l, y / hits_r, loc_threshold):
                        msgs.append("[Global][Hist][%s][%d] has large difference: %r vs %r"
                                    % (names[kind], i, x / hits_l, y / hits_r))
                        g_err += 1
                o += int(n)
    # facets
    if lhs.facet_counts.shape != rhs.facet_counts.shape:
        msgs.append("[FacetStates] Different number of facet states or moments")
        return g_err, f_err + 1, fine_err, msgs
    n_blocks, n_f = lhs.facet_counts.shape[0], lhs.facet_counts.shape[1]
    hitq_l, hitq_r = float(gl[A.G_NBHITEQUIV]), float(gr[A.G_NBHITEQUIV])
    scale_l, scale_r = 1.0 / hitq_l, 1.0 / hitq_r
    full_l = 1.0 / (hitq_l + float(gl[A.G_NBABSEQUIV]) + des_l)
    full_r = 1.0 / (hitq_r + float(gr[A.G_NBABSEQUIV]) + des_r)
    for f in range(n_f):
        for m in range(n_blocks):
            cl, cr = lhs.facet_counts[m, f], rhs.facet_counts[m, f]
            sl, sr = lhs.facet_sums[m, f], rhs.facet_sums[m, f]
            mc_l, mc_r = int(cl[A.FC_NBMCHIT]), int(cr[A.FC_NBMCHIT])
            if (mc_l == 0 and mc_r == 0) or mc_l < 40000 or mc_r < 40000:
                continue
            loc = max(loc_threshold, 1.0 / math.sqrt(min(mc_l, mc_r)))
            sum_hd_l = sl[A.FS_NBHITEQUIV] + float(cl[A.FC_NBDESORBED])
            sum_hd_r = sr[A.FS_NBHITEQUIV] + float(cr[A.FC_NBDESORBED])
            tag = "[Facet][%d]" % f
            if not _too_few(sl[A.FS_NBHITEQUIV], sr[A.FS_NBHITEQUIV], 6400.0):
                checks = (("facet_hits / global_hits", sl[A.FS_NBHITEQUIV] * scale_l, sr[A.FS_NBHITEQUIV] * scale_r, loc),
                          ("sum_v_ort", sl[A.FS_SUM_V_ORT] * scale_l, sr[A.FS_SUM_V_ORT] * scale_r, loc),
                          ("sum_1_per_velocity", sl[A.FS_SUM_1_PER_VELOCITY] * full_l, sr[A.FS_SUM_1_PER_VELOCITY] * full_r,
                           loc * VELOCITY_THRESHOLD_FACTOR),
                          ("sum_1_per_ort_velocity", sl[A.FS_SUM_1_PER_ORT_VEL] * full_l,
                           sr[A.FS_SUM_1_PER_ORT_VEL] * full_r, loc * VELOCITY_THRESHOLD_FACTOR))
                for name, x, y, t in checks:
                    if not is_equal(x, y, t):
                        msgs.append("%s[%s][moment%d] has large difference: %r vs %r" % (tag, name, m, x, y))
                        f_err += 1
            if not _too_few(sl[A.FS_NBABSEQUIV], sr[A.FS_NBABSEQUIV], 6400.0):
                x, y = sl[A.FS_NBABSEQUIV] / mc_l, sr[A.FS_NBABSEQUIV] / mc_r
                if not is_equal(x, y, loc):
                    msgs.append("%s[abs/hits ratio][moment%d] has large difference: %r vs %r" % (tag, m, x, y))
                    f_err += 1
            if not _too_few(cl[A.FC_NBDESORBED], cr[A.FC_NBDESORBED], 6400.0):
                x, y = float(cl[A.FC_NBDESORBED]) / mc_l, float(cr[A.FC_NBDESORBED]) / mc_r
                if not is_equal(x, y, loc):
                    msgs.append("%s[desRatio][moment%d] has large difference: %r vs %r" % (tag, m, x, y))
                    f_err += 1
            # profile: 1-4-6-4-1 smoothed counts
            k = int(L["prof_idx"][f])
            if k >= 0:
                pl, pr = lhs.profile[m, k, :, 0], rhs.profile[m, k, :, 0]
                for i in range(2, len(pl) - 2):
                    wl = (pl[i - 2] + 4 * pl[i - 1] + 6 * pl[i] + 4 * pl[i + 1] + pl[i + 2]) / 16.0
                    wr = (pr[i - 2] + 4 * pr[i - 1] + 6 * pr[i] + 4 * pr[i + 1] + pr[i + 2]) / 16.0
                    if max(1.0, min(wl, wr)) < 100:
                        continue
                    if not is_equal(wl / sum_hd_l, wr / sum_hd_r, loc):
                        fine_msgs.append("%s[Profile][%d][countEquiv][%d]" % (tag, i, m))
                        fine_err += 1
                    for name in ("sum_1_per_ort_velocity", "sum_v_ort"):
                        if not is_equal(wl * scale_l, wr * scale_r, loc * VELOCITY_THRESHOLD_FACTOR):
                            fine_msgs.append("%s[Profile][%d][%s][%d]" % (tag, i, name, m))
                            fine_err += 1
            # texture cells
            o = int(L["tex_off"][f])
            if o >= 0:
                n = int(L["tex_w"][f]) * int(L["tex_h"][f])
                tl, tr = lhs.texture[m, o:o + n], rhs.texture[m, o:o + n]
                for c in range(n):
                    if max(1.0, min(tl[c, 0], tr[c, 0])) < 640:
                        continue
                    if not is_equal(tl[c, 0] / sum_hd_l, tr[c, 0] / sum_hd_r, loc):
                        fine_msgs.append("%s[Texture][%d][countEquiv][%d]" % (tag, c, m))
                        fine_err += 1
                    if not is_equal(tl[c, 2] * full_l, tr[c, 2] * full_r, loc * VELOCITY_THRESHOLD_FACTOR):
                        fine_msgs.append("%s[Texture][%d][sum_1_per_ort_velocity][%d]" % (tag, c, m))
                        fine_err += 1
                    if not is_equal(tl[c, 1] * scale_l, tr[c, 1] * scale_r, loc * VELOCITY_THRESHOLD_FACTOR):
                        fine_msgs.append("%s[Texture][%d][sum_v_ort_per_area][%d]" % (tag, c, m))
                        fine_err += 1
            # direction cells
            o = int(L["dir_off"][f])
            if o >= 0:
                n = int(L["tex_w"][f]) * int(L["tex_h"][f])
                dl, dr = lhs.direction[m, o:o + n], rhs.direction[m, o:o + n]
                for c in range(n):
                    if _too_few(dl[c, 3], dr[c, 3], 6400.0):
                        continue
                    for j, name in ((3, "count"), (0, "dir.x"), (1, "dir.y"), (2, "dir.z")):
                        if not is_equal(dl[c, j], dr[c, j], loc):
                            fine_msgs.append("%s[dirs][%d][%s][%d]" % (tag, c, name, m))
                            fine_err += 1
            # facet histograms
            ho = int(L["hist_off"][f]) if "hist_off" in L else -1
            if ho >= 0:
                for n in L["hist_sizes"][f]:
                    for i in range(int(n)):
                        x, y = lhs.histogram[m, ho + i], rhs.histogram[m, ho + i]
                        if _too_few(x, y, 6400.0):
                            continue
                        if not is_equal(x / mc_l, y / mc_r, loc):
                            fine_msgs.append("%s[Hist][%d][%d]" % (tag, i, m))
                            fine_err += 1
                    ho += int(n)
    return g_err, f_err, fine_err, msgs + fine_msgs
