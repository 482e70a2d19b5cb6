"""MolFlow+ XML reader: geometry, simulation settings and stored results.

Reads the `<SimulationEnvironment type="molflow">` files the reference writes
(src/IO/WriterXML.cpp:72-903) and reads (src/IO/LoaderXML.cpp:31-1130), plain
or inside a .zip, with the standard library only.  Produces a `Model` (the
facet fields used by the tracer, LoaderXML.cpp:831-1120) and a `SimuState`
with the stored GlobalSimuState (LoaderXML.cpp:366-760).
"""
import io
import zipfile
import xml.etree.ElementTree as ET

import numpy as np

from . import _abi as A
from .model import Model, SimuState


def _root(path_or_bytes):
    if isinstance(path_or_bytes, (bytes, bytearray)):
        data = bytes(path_or_bytes)
    elif str(path_or_bytes).lower().endswith(".zip"):
        with zipfile.ZipFile(path_or_bytes) as z:
            names = [n for n in z.namelist() if n.lower().endswith(".xml")]
            data = z.read(names[0])
    else:
        with open(path_or_bytes, "rb") as f:
            data = f.read()
    return ET.parse(io.BytesIO(data)).getroot()


def _f(node, attr, default=0.0):
    if node is None or node.get(attr) is None:
        return default
    return float(node.get(attr))


def _i(node, attr, default=0):
    if node is None or node.get(attr) is None:
        return default
    v = node.get(attr)
    if v in ("true", "false"):
        return int(v == "true")
    return int(float(v))


def _parse_user_moments(um_node):
    """UserMoments entries: 'begin,spacing,end' ranges or single times
    (TimeMoments::ParseUserMoment, TimeMoments.cpp:58-83): a range needs end > begin >= 0 and
    spacing < end - begin, is skipped when spacing < window, and is enumerated by repeated
    addition (time += spacing while time <= end), so the rounding of the sum decides whether
    the end point is included."""
    times, windows = [], []
    if um_node is None:
        return times, windows
    for u in um_node.findall("UserEntry"):
        content = u.get("content", "")
        win = float(u.get("window", "0"))
        parts = []
        for p in content.replace(" ", "").split(",")[:3]:
            try:
                parts.append(float(p))
            except ValueError:
                break
        if len(parts) == 1 and parts[0] >= 0.0:
            times.append(parts[0])
            windows.append(win)
        elif len(parts) == 3:
            b, sp, e = parts
            if b >= 0.0 and e > b and sp < e - b and not sp < win:
                t = b
                while t <= e:
                    times.append(t)
                    windows.append(win)
                    t += sp
    return times, windows


def _hist_params(node):
    """HistogramParams from a <Histograms>/<Global_histograms> settings node (LoaderXML.cpp:179-203,
    1080-1105): dict with record bits and bin sizes / limits."""
    h = dict(record=0, bounce_binsize=1, bounce_max=0, distance_binsize=1.0, distance_max=0.0,
             time_binsize=1.0, time_max=0.0)
    if node is None:
        return h
    b, d, t = node.find("Bounces"), node.find("Distance"), node.find("Time")
    if b is not None:
        h["record"] |= A.HIST_BOUNCE
        h["bounce_binsize"] = int(float(b.get("binSize", "1")))
        h["bounce_max"] = int(float(b.get("max", "0")))
    if d is not None:
        h["record"] |= A.HIST_DISTANCE
        h["distance_binsize"] = float(d.get("binSize"))
        h["distance_max"] = float(d.get("max"))
    if t is not None:
        h["record"] |= A.HIST_TIME
        h["time_binsize"] = float(t.get("binSize"))
        h["time_max"] = float(t.get("max"))
    return h


def _hist_values(node, sizes):
    """Stored histogram bins of a results <Histograms> node, concatenated bounce/distance/time."""
    out = []
    for tag, n in zip(("Bounces", "Distance", "Time"), sizes):
        if not n:
            continue
        vals = np.zeros(n)
        h = node.find(tag) if node is not None else None
        if h is not None and int(h.get("size", "0")) == n:
            for k, b in enumerate(h.findall("Bin")[:n]):
                vals[k] = float(b.get("count"))
        out.append(vals)
    return np.concatenate(out) if out else np.zeros(0)


def load_catalog(folder):
    """Parameters of a parameter-catalog folder: one parameter per .csv file of 't,value'
    rows, named "[catalog] <file name>", pairs kept sorted by t, linear interpolation
    (TimeDependentParameters::LoadParameterCatalog, MolflowSimGeom.cpp:1250-1319).
    Returns a list of (name, t, v)."""
    import os
    out = []
    if folder is None or not os.path.isdir(folder):
        return out
    for fn in sorted(os.listdir(folder)):
        if not fn.endswith(".csv"):
            continue
        pairs = []
        with open(os.path.join(folder, fn), encoding="utf-8-sig") as f:
            for line in f:
                row = [c.strip() for c in line.strip().split(",")]
                if row == [""]:
                    continue
                if len(row) != 2:
                    break
                pairs.append((float(row[0]), float(row[1])))
        pairs.sort(key=lambda p: p[0])
        out.append(("[catalog] " + fn, np.array([p[0] for p in pairs]), np.array([p[1] for p in pairs])))
    return out


def load(path_or_bytes, with_state=True, catalog=()):
    """Return (model, state or None, info dict).

    `catalog`: parameters of a parameter catalog (see load_catalog); they follow the file's
    own parameters, as in the reference (InsertParametersBeforeCatalog)."""
    r = _root(path_or_bytes)
    g = r.find("Geometry")
    vnode = g.find("Vertices")
    verts = np.array([[float(v.get("x")), float(v.get("y")), float(v.get("z"))] for v in vnode.findall("Vertex")])
    fnodes = g.find("Facets").findall("Facet")
    facets = [[int(i.get("vertex")) for i in f.find("Indices").findall("Indice")] for f in fnodes]
    m = Model(verts, facets)
    sims = r.find("MolflowSimuSettings")
    # time-dependent parameters (LoaderXML.cpp:69-100)
    names = []
    pnode = sims.find("Parameters") if sims is not None else None
    if pnode is not None:
        for p in pnode.findall("Parameter"):
            t = [float(x.get("t")) for x in p.findall("Moment")]
            v = [float(x.get("value")) for x in p.findall("Moment")]
            m.add_param(t, v, logx=_i(p, "logXinterp"), logy=_i(p, "logYinterp"))
            names.append(p.get("name"))
    for nm, t, v in catalog:
        m.add_param(t, v)
        names.append(nm)

    def param_ref(node, name_attr):
        # by name (2.9.15+ files), else by index into file + catalog parameters (LoaderXML.cpp:847-925)
        if node is None:
            return -1
        if node.get(name_attr):
            nm = node.get(name_attr)
            if nm not in names:
                raise ValueError("parameter %r not found" % nm)
            return names.index(nm)
        return _i(node, "parameterId", -1)

    for k, f in enumerate(fnodes):
        st = f.find("Sticking")
        op = f.find("Opacity")
        og = f.find("Outgassing")
        te = f.find("Temperature")
        rf = f.find("Reflection")
        su = f.find("Structure")
        rec = f.find("Recordings")
        tx = rec.find("Texture") if rec is not None else None
        m.sticking[k] = _f(st, "constValue")
        m.sticking_param[k] = param_ref(st, "stickingParam")
        m.opacity[k] = _f(op, "constValue", 1.0)
        m.opacity_param[k] = param_ref(op, "opacityParam")
        m.is_2sided[k] = _i(op, "is2sided")
        m.outgassing[k] = _f(og, "constValue")
        m.outgassing_param[k] = param_ref(og, "OutgassingParam")
        m.desorb_type[k] = _i(og, "desType")
        m.desorb_exponent[k] = _f(og, "desExponent")
        m.temperature[k] = _f(te, "value", 293.15)
        m.temperature_param[k] = param_ref(te, "tempParam")
        m.accommodation[k] = _f(te, "accFactor", 1.0)
        if rf is not None and rf.get("diffusePart") is not None:
            m.refl_diffuse[k] = _f(rf, "diffusePart", 1.0)
            m.refl_specular[k] = _f(rf, "specularPart", 0.0)
            m.refl_cos_exponent[k] = _f(rf, "cosineExponent", 0.0)
        elif rf is not None:
            t = _i(rf, "type")
            m.refl_diffuse[k], m.refl_specular[k] = (1.0, 0.0) if t == 0 else ((0.0, 1.0) if t == 1 else (0.0, 0.0))
        m.enable_sojourn[k] = _i(rf, "enableSojournTime")
        m.sojourn_freq[k] = _f(rf, "sojournFreq")
        m.sojourn_e[k] = _f(rf, "sojournE")
        m.structure[k] = _i(su, "inStructure")
        m.link_dest[k] = _i(su, "linksTo")
        m.teleport_dest[k] = _i(f.find("Teleport"), "target")
        m.is_moving[k] = _i(f.find("Motion"), "isMoving")
        if rec is not None:
            m.profile_type[k] = _i(rec.find("Profile"), "type")
            am = rec.find("IncidentAngleMap")
            if am is not None:
                m.anglemap_record[k] = _i(am, "record")
                m.anglemap_phi_width[k] = _i(am, "phiWidth")
                m.anglemap_theta_limit[k] = _f(am, "thetaLimit", 1.570796326)
                m.anglemap_theta_lower_res[k] = _i(am, "thetaLowerRes")
                m.anglemap_theta_higher_res[k] = _i(am, "thetaHigherRes")
        # a recorded angle map in the facet node sets the map parameters and is the source of
        # angle-map desorption; without one, angle-map desorption falls back to none
        # (LoaderXML.cpp:1043-1073)
        gam = f.find("IncidentAngleMap")
        if gam is not None and gam.find("map") is not None and gam.get("angleMapThetaLimit") is not None:
            m.anglemap_phi_width[k] = _i(gam, "angleMapPhiWidth")
            m.anglemap_theta_limit[k] = _f(gam, "angleMapThetaLimit")
            m.anglemap_theta_lower_res[k] = _i(gam, "angleMapThetaLowerRes")
            m.anglemap_theta_higher_res[k] = _i(gam, "angleMapThetaHigherRes")
            if m.desorb_type[k] == A.DES_ANGLEMAP:
                txt = gam.find("map").text or ""
                m.desorb_anglemaps[k] = np.array([int(float(x)) for x in txt.split()], np.uint64)
        elif m.desorb_type[k] == A.DES_ANGLEMAP:
            m.desorb_type[k] = A.DES_NONE
        # outgassing map (MolflowFacet.cpp:249-285): used only when the Outgassing node asks for it
        # and the DynamicOutgassing node has a map; the old format has one square ratio
        dyn = f.find("DynamicOutgassing")
        if _i(og, "useOutgassingFile") and dyn is not None and dyn.find("map") is not None:
            w, h = _i(dyn, "width"), _i(dyn, "height")
            ru = _f(dyn, "ratioU", _f(dyn, "ratio"))
            rv = _f(dyn, "ratioV", _f(dyn, "ratio"))
            vals = np.array([float(x) for x in (dyn.find("map").text or "").split()], np.float64)
            if w > 0 and h > 0 and vals.size >= w * h:
                m.outgassing_maps[k] = dict(width=w, height=h, ratio_u=ru, ratio_v=rv, values=vals[:w * h].reshape(h, w))
        hp = _hist_params(f.find("Histograms"))
        for key, val in hp.items():
            getattr(m, "hist_" + key)[k] = val
        if tx is not None:
            m.tex_width[k] = _f(tx, "texDimX")
            m.tex_height[k] = _f(tx, "texDimY")
            flags = 0
            for bit, attr in ((A.COUNT_DES, "countDes"), (A.COUNT_ABS, "countAbs"), (A.COUNT_REFL, "countRefl"),
                              (A.COUNT_TRANS, "countTrans"), (A.COUNT_DIR, "countDir")):
                if _i(tx, attr):
                    flags |= bit
            m.count_flags[k] = flags
    structs = g.find("Structures")
    m.n_structures = max(1, _i(structs, "nb", 1))
    if sims is not None:
        gas = sims.find("Gas")
        m.gas_mass = _f(gas, "mass", 28.0)
        sc = gas.find("Scattering") if gas is not None else None
        if sc is not None:   # LoaderXML.cpp:106-116 (the collision radius is not in the file)
            m.scatter_enabled = _i(sc, "enabled")
            m.scatter_mass_ratio = _f(sc, "massRatio", 1.0)
            m.scatter_mean_free_path_cm = _f(sc, "meanFreePath_cm", 1e30)
            co = sc.find("LowSpeedCutoff")
            if co is not None:
                m.scatter_cutoff_enabled = _i(co, "enabled")
                m.scatter_cutoff_speed = _f(co, "speed")
        mo = sims.find("Motion")   # LoaderXML.cpp:144-160
        if mo is not None:
            m.motion_type = _i(mo, "type")
            if m.motion_type == 1:
                v = mo.find("VelocityVector")
                m.motion_vector2 = (_f(v, "vx"), _f(v, "vy"), _f(v, "vz"))
            elif m.motion_type == 2:
                b, r = mo.find("AxisBasePoint"), mo.find("RotationVector")
                m.motion_vector1 = (_f(b, "x"), _f(b, "y"), _f(b, "z"))
                m.motion_vector2 = (_f(r, "x"), _f(r, "y"), _f(r, "z"))
        m.enable_decay = _i(gas, "enableDecay")
        m.half_life = _f(gas, "halfLife", 1.0)
        fm = sims.find("MeasureForces")   # LoaderXML.cpp:163-177
        if fm is not None:
            m.enable_force_measurement = _i(fm, "enabled")
            tq = fm.find("Torque")
            rp = tq.find("refPoint") if tq is not None else None
            if rp is not None:
                m.torque_ref_point = (_f(rp, "x"), _f(rp, "y"), _f(rp, "z"))
        lf = sims.find("LowFluxMode")
        m.low_flux_mode = _i(lf, "enabled")
        m.low_flux_cutoff = _f(lf, "cutoff", 1e-7)
        m.global_histogram = _hist_params(sims.find("Global_histograms"))
        ts = sims.find("TimeSettings")
        m.time_window = _f(ts, "timeWindow", 1e-10)
        m.use_maxwell = _i(ts, "useMaxwellDistr", 1)
        m.constant_flow = _i(ts, "calcConstFlow", 1)
        t, w = _parse_user_moments(ts.find("UserMoments") if ts is not None else None)
        if t:
            m.set_moments(t, w)
    info = {"n_structures": m.n_structures, "param_names": names}
    state = load_state(r, m) if with_state else None
    return m, state, info


def load_state(r, m):
    """Stored results (LoaderXML.cpp:366-760) into a SimuState; None if absent."""
    res = r.find("MolflowResults")
    if res is None:
        return None
    st = SimuState(m)
    L = st.L
    moments = res.find("Moments").findall("Moment")
    for mi, mom in enumerate(moments):
        if mi >= L["blocks"]:
            break
        if mi == 0:
            gh = mom.find("Global/Hits")
            st.global_[A.G_NBMCHIT] = _f(gh, "totalHit")
            st.global_[A.G_NBHITEQUIV] = _f(gh, "totalHitEquiv")
            st.global_[A.G_NBDESORBED] = _f(gh, "totalDes")
            st.global_[A.G_NBABSEQUIV] = _f(gh, "totalAbsEquiv")
            st.global_[A.G_NBLEAK] = _f(gh, "totalLeak")
            st.global_[A.G_DIST_TOTAL] = _f(gh, "totalDist_total")
            st.global_[A.G_DIST_FULLHITS] = _f(gh, "totalDist_fullHitsOnly")
        hb = L["histogram_bins"]
        if hb:
            gs = L["global_hist_sizes"]
            if sum(gs):
                st.histogram[mi, :sum(gs)] = _hist_values(mom.find("Histograms"), gs)
        for fr in mom.find("FacetResults").findall("Facet"):
            k = int(fr.get("id"))
            if hb and L["hist_off"][k] >= 0:
                o, sz = L["hist_off"][k], L["hist_sizes"][k]
                st.histogram[mi, o:o + sz.sum()] = _hist_values(fr.find("Histograms"), sz)
            h = fr.find("Hits")
            st.facet_counts[mi, k, A.FC_NBMCHIT] = int(float(h.get("nbHit")))
            st.facet_counts[mi, k, A.FC_NBDESORBED] = int(float(h.get("nbDes")))
            st.facet_counts[mi, k, A.FC_NBABSORBED] = int(round(float(h.get("nbAbsEquiv"))))
            st.facet_sums[mi, k, A.FS_NBHITEQUIV] = _f(h, "nbHitEquiv")
            st.facet_sums[mi, k, A.FS_NBABSEQUIV] = _f(h, "nbAbsEquiv")
            st.facet_sums[mi, k, A.FS_SUM_V_ORT] = _f(h, "sum_v_ort")
            st.facet_sums[mi, k, A.FS_SUM_1_PER_ORT_VEL] = _f(h, "sum_1_per_v")
            st.facet_sums[mi, k, A.FS_SUM_1_PER_VELOCITY] = _f(h, "sum_v")
            pr = fr.find("Profile")
            if pr is not None and L["prof_idx"][k] >= 0:
                p = st.profile[mi, L["prof_idx"][k]]
                for s in pr.findall("Slice"):
                    j = int(s.get("id"))
                    if j < A.PROFILE_SIZE:
                        p[j, 0] = _f(s, "countEquiv")
                        p[j, 1] = _f(s, "sum_v_ort")
                        p[j, 2] = _f(s, "sum_1_per_v")
            tx = fr.find("Texture")
            if tx is not None and L["tex_off"][k] >= 0:
                w, hh = int(L["tex_w"][k]), int(L["tex_h"][k])
                fw, fh = int(tx.get("width")), int(tx.get("height"))
                blocks = {}
                for c in tx:
                    vals = np.array(c.text.split(), dtype=np.float64) if c.text and c.text.strip() else np.zeros(0)
                    blocks[c.tag] = vals
                o = L["tex_off"][k]
                for field, tag in ((0, "count"), (1, "sum_v_ort"), (2, "sum_1_per_v")):
                    vals = blocks.get(tag)
                    if vals is None or vals.size < fw * fh:
                        continue
                    grid = vals[:fw * fh].reshape(fh, fw)[:hh, :w]
                    sub = np.zeros((hh, w))
                    sub[:grid.shape[0], :grid.shape[1]] = grid
                    st.texture[mi, o:o + w * hh, field] = sub.reshape(-1)
            dn = fr.find("Directions")
            if dn is not None and L["dir_off"][k] >= 0:   # direction cells (LoaderXML.cpp, "Directions")
                w, hh = int(L["tex_w"][k]), int(L["tex_h"][k])
                vv, cn = dn.find("vel.vectors"), dn.find("count")
                o = L["dir_off"][k]
                if vv is not None and vv.text:
                    vecs = [c for c in vv.text.replace("\n", "\t").split("\t") if c.strip()]
                    for c, item in enumerate(vecs[:w * hh]):
                        st.direction[mi, o + c, :3] = [float(x) for x in item.split(",")]
                if cn is not None and cn.text:
                    vals = np.array(cn.text.split(), dtype=np.float64)[:w * hh]
                    st.direction[mi, o:o + vals.size, 3] = vals
    # recorded incident-angle maps sit in the geometry's facet nodes (LoaderXML.cpp:1043-1070)
    for k, fnode in enumerate(r.find("Geometry").find("Facets").findall("Facet")):
        am = fnode.find("IncidentAngleMap")
        if am is None or am.find("map") is None or am.get("angleMapThetaLimit") is None or L["ang_off"][k] < 0:
            continue
        txt = am.find("map").text or ""
        vals = np.array(txt.split(), dtype=np.float64)
        o = L["ang_off"][k]
        n = min(vals.size, st.anglemap.size - o)
        st.anglemap[o:o + n] = vals[:n].astype(np.uint64)
    return st
