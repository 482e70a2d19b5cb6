"""MolFlow+ XML writer: a model and a GlobalSimuState-shaped result as a `<SimulationEnvironment
type="molflow">` file that MolFlow+ opens (the format of src/IO/WriterXML.cpp: SaveGeometry :72-365,
SaveFacet :684-903, SaveSimulationState :367-682) and that molflow_sources_gb300.xmlio reads back.

Written: vertices; facets with sticking, opacity, outgassing (constant, parameter or map), desorption
law, temperature, reflection mix, sojourn, structure and link, teleport, motion, profile, texture
and counting flags, angle-map settings and maps, histogram settings; the simulation settings (gas,
decay, scattering, low-flux mode, time settings with the moments, motion, forces, parameters,
global histograms); and per moment the global counters, facet hit buffers, forces, profiles,
textures, direction cells and histograms.  The GUI's interface settings (views, selections,
formulas) and the hit/leak display caches are not part of a result and are written empty.
Numbers are written in their shortest round-trip decimal form.
"""
import io
import zipfile
import xml.etree.ElementTree as ET

import numpy as np

from . import _abi as A
from .model import HIST_FIELDS

PROFILE_NAMES = {0: "none", 1: "pressure u", 2: "pressure v", 3: "angular", 4: "speed", 5: "ortho.v", 6: "tang.v."}


def _n(x):
    if isinstance(x, (bool, np.bool_)):
        return str(int(x))
    if isinstance(x, (int, np.integer)):
        return str(int(x))
    r = repr(float(x))
    return r[:-2] if r.endswith(".0") else r


def _sub(parent, tag, **attrs):
    e = ET.SubElement(parent, tag)
    for k, v in attrs.items():
        e.set(k, v if isinstance(v, str) else _n(v))
    return e


def _grid_text(vals, w, h, sep="\t"):
    rows = ["\n"]
    for y in range(h):
        rows.append(sep.join(_n(v) for v in vals[y * w:(y + 1) * w]) + sep + "\n")
    return "".join(rows)


def _hist_settings(node, p):
    if p["record"] & A.HIST_BOUNCE:
        _sub(node, "Bounces", binSize=int(p["bounce_binsize"]), max=int(p["bounce_max"]))
    if p["record"] & A.HIST_DISTANCE:
        _sub(node, "Distance", binSize=float(p["distance_binsize"]), max=float(p["distance_max"]))
    if p["record"] & A.HIST_TIME:
        _sub(node, "Time", binSize=float(p["time_binsize"]), max=float(p["time_max"]))


def _hist_results(node, p, sizes, values):
    o = 0
    for tag, rec, n, bs, mx in (("Bounces", A.HIST_BOUNCE, sizes[0], "bounce_binsize", "bounce_max"),
                                ("Distance", A.HIST_DISTANCE, sizes[1], "distance_binsize", "distance_max"),
                                ("Time", A.HIST_TIME, sizes[2], "time_binsize", "time_max")):
        if not (p["record"] & rec) or not n:
            continue
        h = _sub(node, tag, size=int(n), binSize=p[bs], max=p[mx])
        for k in range(int(n)):
            b = ET.SubElement(h, "Bin")
            b.set("start", "overRange" if k == n - 1 else _n(k * p[bs]))
            b.set("count", _n(values[o + k]))
        o += int(n)


def _facet_hist_params(model, i):
    return {k: (getattr(model, "hist_" + k)[i]) for k in HIST_FIELDS}


def build_tree(model, state=None, outgassing=None, facet_area=None, param_names=None, version="2.9.25"):
    """The document as an ElementTree root.  `outgassing`: GpuModel.outgassing() (written for
    external parsers, and used for molecules_per_TP); `facet_area`: cm^2 per facet."""
    nf = model.n_facets
    L = model.layout()
    root = ET.Element("SimulationEnvironment")
    root.set("type", "molflow")
    root.set("version", version)
    names = list(param_names) if param_names else ["param%d" % i for i in range(len(model.params))]

    # ---- geometry (SaveGeometry / SaveFacet) ----
    geom = _sub(root, "Geometry")
    vn = _sub(geom, "Vertices", nb=len(model.vertices))
    for i, v in enumerate(model.vertices):
        _sub(vn, "Vertex", id=i, x=float(v[0]), y=float(v[1]), z=float(v[2]))
    fn = _sub(geom, "Facets", nb=nf)
    for i in range(nf):
        f = _sub(fn, "Facet", id=i)

        def const_or_param(tag, pattr, value, p, default, extra=None):
            e = _sub(f, tag)
            if p >= 0:
                e.set(pattr, names[p])
                e.set("parameterId", _n(p))
                e.set("constValue", _n(default))
            else:
                e.set("constValue", _n(value))
                e.set("parameterId", "-1")
            for k, v in (extra or {}).items():
                e.set(k, _n(v))
            return e

        const_or_param("Sticking", "stickingParam", model.sticking[i], int(model.sticking_param[i]), 0.0)
        const_or_param("Opacity", "opacityParam", model.opacity[i], int(model.opacity_param[i]), 1.0,
                       {"is2sided": int(model.is_2sided[i])})
        has_map = i in model.outgassing_maps
        og = const_or_param("Outgassing", "outgassingParam", model.outgassing[i], int(model.outgassing_param[i]), 0.0,
                            {"is2sided": int(model.is_2sided[i])})
        og.set("desType", _n(int(model.desorb_type[i])))
        og.set("desExponent", _n(model.desorb_exponent[i]))
        og.set("hasOutgassingFile", _n(int(has_map)))
        og.set("useOutgassingFile", _n(int(has_map)))
        te = _sub(f, "Temperature")
        if int(model.temperature_param[i]) >= 0:
            te.set("tempParam", names[int(model.temperature_param[i])])
        else:
            te.set("value", _n(model.temperature[i]))
        te.set("accFactor", _n(model.accommodation[i]))
        if facet_area is not None:
            _sub(f, "Area", m2=float(facet_area[i]) * 1e-4)
        d, s = float(model.refl_diffuse[i]), float(model.refl_specular[i])
        _sub(f, "Reflection", diffusePart=d, specularPart=s, cosineExponent=float(model.refl_cos_exponent[i]),
             type=0 if d > 0.99 else (1 if s > 0.99 else 2), enableSojournTime=int(model.enable_sojourn[i]),
             sojournFreq=float(model.sojourn_freq[i]), sojournE=float(model.sojourn_e[i]))
        _sub(f, "Structure", inStructure=int(model.structure[i]), linksTo=int(model.link_dest[i]))
        _sub(f, "Teleport", target=int(model.teleport_dest[i]))
        _sub(f, "Motion", isMoving=int(model.is_moving[i]))
        rec = _sub(f, "Recordings")
        pt = int(model.profile_type[i])
        _sub(rec, "Profile", type=pt, name=PROFILE_NAMES.get(pt, "none"))
        cf = int(model.count_flags[i])
        _sub(rec, "Texture", hasMesh=int(bool(cf & (A.COUNT_DES | A.COUNT_ABS | A.COUNT_REFL | A.COUNT_TRANS))),
             texDimX=float(model.tex_width[i]), texDimY=float(model.tex_height[i]),
             countDes=int(bool(cf & A.COUNT_DES)), countAbs=int(bool(cf & A.COUNT_ABS)),
             countRefl=int(bool(cf & A.COUNT_REFL)), countTrans=int(bool(cf & A.COUNT_TRANS)),
             countDir=int(bool(cf & A.COUNT_DIR)), countAC=0)
        if model.anglemap_record[i]:
            _sub(rec, "IncidentAngleMap", record=int(model.anglemap_record[i]), phiWidth=int(model.anglemap_phi_width[i]),
                 thetaLimit=float(model.anglemap_theta_limit[i]), thetaLowerRes=int(model.anglemap_theta_lower_res[i]),
                 thetaHigherRes=int(model.anglemap_theta_higher_res[i]))
        ind = _sub(f, "Indices", nb=len(model.facets[i]))
        for k, v in enumerate(model.facets[i]):
            _sub(ind, "Indice", id=k, vertex=int(v))
        if has_map:
            mp = model.outgassing_maps[i]
            vals = np.asarray(mp["values"], np.float64)
            dn = _sub(f, "DynamicOutgassing", width=int(mp["width"]), height=int(mp["height"]),
                      ratioU=float(mp["ratio_u"]), ratioV=float(mp["ratio_v"]), totalDose=0.0,
                      totalOutgassing=float(vals.sum()), totalFlux=0.0)
            _sub(dn, "map").text = _grid_text(vals.ravel(), int(mp["width"]), int(mp["height"]))
        # angle map: the recorded one of the result, else the map a facet desorbs by
        w = int(model.anglemap_phi_width[i])
        rows = int(model.anglemap_theta_lower_res[i]) + int(model.anglemap_theta_higher_res[i])
        pdf = None
        if state is not None and L["ang_off"][i] >= 0 and state.anglemap.size:
            o = int(L["ang_off"][i])
            pdf = state.anglemap[o:o + w * rows]
        elif i in model.desorb_anglemaps:
            pdf = np.asarray(model.desorb_anglemaps[i], np.uint64)[:w * rows]
        if pdf is not None and w > 0 and rows > 0:
            am = _sub(f, "IncidentAngleMap", angleMapPhiWidth=w, angleMapThetaLimit=float(model.anglemap_theta_limit[i]),
                      angleMapThetaLowerRes=int(model.anglemap_theta_lower_res[i]),
                      angleMapThetaHigherRes=int(model.anglemap_theta_higher_res[i]))
            _sub(am, "map").text = _grid_text([int(x) for x in pdf], w, rows)
        _hist_settings(_sub(f, "Histograms"), _facet_hist_params(model, i))
    st = _sub(geom, "Structures", nb=int(model.n_structures))
    for s in range(int(model.n_structures)):
        _sub(st, "Structure", id=s, name="structure %d" % (s + 1))

    # ---- simulation settings ----
    sp = _sub(root, "MolflowSimuSettings")
    gas = _sub(sp, "Gas", mass=float(model.gas_mass), enableDecay=int(model.enable_decay), halfLife=float(model.half_life))
    sc = _sub(gas, "Scattering", enabled=int(model.scatter_enabled), massRatio=float(model.scatter_mass_ratio),
              meanFreePath_cm=float(model.scatter_mean_free_path_cm))
    _sub(sc, "LowSpeedCutoff", enabled=int(model.scatter_cutoff_enabled), speed=float(model.scatter_cutoff_speed))
    if outgassing is not None:
        _sub(gas, "Outgassing_info", final_rate_molecules_per_s=outgassing["final_outgassing_rate"],
             total_desorbed_molecules=outgassing["total_desorbed_molecules"])
    _sub(sp, "LowFluxMode", enabled=int(model.low_flux_mode), cutoff=float(model.low_flux_cutoff))
    ts = _sub(sp, "TimeSettings", timeWindow=float(model.time_window), useMaxwellDistr=int(model.use_maxwell),
              calcConstFlow=int(model.constant_flow))
    um = _sub(ts, "UserMoments", nb=len(model.moment_time))
    for k, (t, w) in enumerate(zip(model.moment_time, model.moment_window)):
        _sub(um, "UserEntry", id=k, content=_n(t), window=float(w))
    nm = len(model.moment_time)
    latest = (model.moment_time[-1] + 0.5 * model.moment_window[-1]) if nm else 0.5 * model.time_window
    _sub(ts, "Info", latest_moment_s=float(latest))
    mo = _sub(sp, "Motion", type=int(model.motion_type))
    if model.motion_type == 1:
        _sub(mo, "VelocityVector", vx=model.motion_vector2[0], vy=model.motion_vector2[1], vz=model.motion_vector2[2])
    elif model.motion_type == 2:
        _sub(mo, "AxisBasePoint", x=model.motion_vector1[0], y=model.motion_vector1[1], z=model.motion_vector1[2])
        _sub(mo, "RotationVector", x=model.motion_vector2[0], y=model.motion_vector2[1], z=model.motion_vector2[2])
    fm = _sub(sp, "MeasureForces", enabled=int(model.enable_force_measurement))
    _sub(_sub(fm, "Torque"), "refPoint", x=model.torque_ref_point[0], y=model.torque_ref_point[1], z=model.torque_ref_point[2])
    pn = _sub(sp, "Parameters", nb=len(model.params))
    for k, (t, v, lx, ly) in enumerate(model.params):
        p = _sub(pn, "Parameter", id=k, name=names[k], nbMoments=len(t), logXinterp=int(lx), logYinterp=int(ly))
        for j in range(len(t)):
            _sub(p, "Moment", id=j, t=float(t[j]), value=float(v[j]))
    _hist_settings(_sub(sp, "Global_histograms"), model.global_histogram)
    _sub(root, "Interface")

    # ---- results (SaveSimulationState) ----
    if state is not None:
        res = _sub(root, "MolflowResults")
        moms = _sub(res, "Moments", nb=nm + 1)
        ndes = float(state.global_[A.G_NBDESORBED])
        for m in range(nm + 1):
            mn = _sub(moms, "Moment", id=m)
            if m == 0:
                mn.set("time", "Constant flow")
                mn.set("timeWindow", "0")
            else:
                mn.set("time", _n(model.moment_time[m - 1]))
                mn.set("timeWindow", _n(model.moment_window[m - 1]))
            if outgassing is not None and ndes > 0:
                mpt = (outgassing["final_outgassing_rate"] / ndes if m == 0
                       else outgassing["total_desorbed_molecules"] / float(model.moment_window[m - 1]) / ndes)
                mn.set("molecules_per_TP", _n(mpt))
            if m == 0:
                g = state.global_
                gn = _sub(mn, "Global")
                _sub(gn, "Hits", totalHit=int(g[A.G_NBMCHIT]), totalHitEquiv=float(g[A.G_NBHITEQUIV]),
                     totalDes=int(g[A.G_NBDESORBED]), totalAbsEquiv=float(g[A.G_NBABSEQUIV]),
                     totalDist_total=float(g[A.G_DIST_TOTAL]), totalDist_fullHitsOnly=float(g[A.G_DIST_FULLHITS]),
                     totalLeak=int(g[A.G_NBLEAK]), maxDesorption=0)
                _sub(gn, "Hit_Cache", nb=0)
                _sub(gn, "Leak_Cache", nb=0)
            gh = model.global_histogram
            gsz = L["global_hist_sizes"]
            if gh["record"] and sum(gsz):
                _hist_results(_sub(mn, "Histograms"), gh, gsz, state.histogram[m, :sum(gsz)])
            fr = _sub(mn, "FacetResults")
            for i in range(nf):
                fnode = _sub(fr, "Facet", id=i)
                c, s_ = state.facet_counts[m, i], state.facet_sums[m, i]
                _sub(fnode, "Hits", nbHit=int(c[A.FC_NBMCHIT]), nbHitEquiv=float(s_[A.FS_NBHITEQUIV]),
                     nbDes=int(c[A.FC_NBDESORBED]), nbAbsEquiv=float(s_[A.FS_NBABSEQUIV]),
                     sum_v_ort=float(s_[A.FS_SUM_V_ORT]), sum_1_per_v=float(s_[A.FS_SUM_1_PER_ORT_VEL]),
                     sum_v=float(s_[A.FS_SUM_1_PER_VELOCITY]))
                if model.enable_force_measurement and state.force.shape[1]:
                    q = state.force[m, i]
                    fo = _sub(fnode, "Forces")
                    for tag, o in (("Impulse", 0), ("Impulse_square", 3), ("Impulse_momentum", 6)):
                        _sub(fo, tag, x=float(q[o]), y=float(q[o + 1]), z=float(q[o + 2]))
                k = int(L["prof_idx"][i])
                if k >= 0:
                    pr = _sub(fnode, "Profile", size=A.PROFILE_SIZE)
                    for j in range(A.PROFILE_SIZE):
                        p = state.profile[m, k, j]
                        _sub(pr, "Slice", id=j, countEquiv=float(p[0]), sum_1_per_v=float(p[2]), sum_v_ort=float(p[1]))
                o = int(L["tex_off"][i])
                if o >= 0:
                    w, h = int(L["tex_w"][i]), int(L["tex_h"][i])
                    t = state.texture[m, o:o + w * h]
                    tn = _sub(fnode, "Texture", width=w, height=h)
                    _sub(tn, "count").text = _grid_text(t[:, 0], w, h)
                    _sub(tn, "sum_1_per_v").text = _grid_text(t[:, 2], w, h)
                    _sub(tn, "sum_v_ort").text = _grid_text(t[:, 1], w, h)
                o = int(L["dir_off"][i])
                if o >= 0:
                    w, h = int(L["tex_w"][i]), int(L["tex_h"][i])
                    dv = state.direction[m, o:o + w * h]
                    dn = _sub(fnode, "Directions", width=w, height=h)
                    rows = ["\n"]
                    for y in range(h):
                        rows.append("".join("%s,%s,%s\t" % (_n(a[0]), _n(a[1]), _n(a[2])) for a in dv[y * w:(y + 1) * w]) + "\n")
                    _sub(dn, "vel.vectors").text = "".join(rows)
                    _sub(dn, "count").text = _grid_text([int(x) for x in dv[:, 3]], w, h)
                ho = int(L["hist_off"][i])
                if ho >= 0:
                    sz = L["hist_sizes"][i]
                    _hist_results(_sub(fnode, "Histograms"), _facet_hist_params(model, i), sz,
                                  state.histogram[m, ho:ho + int(sz.sum())])
    return root


def save(path, model, state=None, outgassing=None, facet_area=None, param_names=None):
    """Write the file (a .zip holding one .xml when the path ends in .zip)."""
    root = build_tree(model, state, outgassing, facet_area, param_names)
    buf = io.BytesIO()
    ET.ElementTree(root).write(buf, encoding="utf-8", xml_declaration=True)
    data = buf.getvalue()
    if str(path).lower().endswith(".zip"):
        import os
        inner = os.path.basename(str(path))[:-4] + ".xml"
        with zipfile.ZipFile(path, "w", compression=zipfile.ZIP_DEFLATED) as z:
            z.writestr(inner, data)
    else:
        with open(path, "wb") as f:
            f.write(data)
