"""The C++ host's file reader (mfg_xml_*: LoaderXML.cpp:31-1130) against the Python reader on the
same files.

Files are written by the XML writer (plain .xml and .zip, with results) from the golden test-case
models and oracle runs; the model descriptor the library reads must equal the one the Python reader
builds, field by field, and the stored results it reads must equal the Python reader's.
"""
import ctypes as C
import zipfile

import numpy as np
import pytest

from molflow_sources_gb300 import _abi as A
from molflow_sources_gb300 import xmlio, xmlwriter
from molflow_sources_gb300.model import FACET_FIELDS, SimuState
from molflow_sources_gb300.simulation import GpuModel, MfgError, load_library
from oracle.oracle import Oracle
from tests import golden_util

CASES = ["01-quick_pipe_profiles_textures_2sided", "02-timedependent_with_two_parameters",
         "04-anglemap_desorb", "05-three_structures_nonsquare_textures", "09-histograms", "B04-lr10_pipe_trans"]
ARRAYS = ("global_", "facet_counts", "facet_sums", "texture", "profile", "direction", "anglemap", "histogram")


def _lib():
    L = load_library()
    L.mfg_xml_open.argtypes = [C.c_char_p, C.POINTER(C.c_void_p)]
    L.mfg_xml_desc.argtypes = [C.c_void_p]
    L.mfg_xml_desc.restype = C.POINTER(A.ModelDesc)
    L.mfg_xml_read_state.argtypes = [C.c_void_p, C.c_void_p, C.POINTER(A.StateView)]
    L.mfg_xml_close.argtypes = [C.c_void_p]
    L.mfg_model_create.argtypes = [C.POINTER(A.ModelDesc), C.POINTER(C.c_void_p)]
    return L


def _open(L, path):
    h = C.c_void_p()
    rc = L.mfg_xml_open(path.encode(), C.byref(h))
    if rc != A.MFG_OK:
        buf = C.create_string_buffer(4096)
        L.mfg_last_error(buf, 4096)
        raise MfgError(rc, buf.value.decode())
    return h


def _arr(ptr, n, dtype):
    if not ptr or n == 0:
        return None
    ct = np.ctypeslib.as_array(C.cast(ptr, C.POINTER({np.float64: C.c_double, np.int32: C.c_int32, np.uint8: C.c_uint8,
                                                      np.uint32: C.c_uint32, np.uint64: C.c_uint64}[dtype])), (n,))
    return np.array(ct, dtype=dtype)


def _assert_desc_equal(a, b):
    """Two mfg_model_desc structures describe the same model (every array and scalar)."""
    nf = a.n_facets
    assert (a.n_vertices, a.n_facets) == (b.n_vertices, b.n_facets)
    np.testing.assert_array_equal(_arr(a.vertices, 3 * a.n_vertices, np.float64), _arr(b.vertices, 3 * b.n_vertices, np.float64))
    np.testing.assert_array_equal(_arr(a.facet_vertex_start, nf + 1, np.int32), _arr(b.facet_vertex_start, nf + 1, np.int32))
    nv = int(_arr(a.facet_vertex_start, nf + 1, np.int32)[-1])
    np.testing.assert_array_equal(_arr(a.facet_vertex_index, nv, np.int32), _arr(b.facet_vertex_index, nv, np.int32))
    for name, (dt, _) in FACET_FIELDS.items():
        if name.startswith("hist_"):
            continue
        np.testing.assert_array_equal(_arr(getattr(a, name), nf, dt), _arr(getattr(b, name), nf, dt), err_msg=name)
    for f in ("gas_mass", "use_maxwell", "constant_flow", "time_window", "enable_decay", "half_life", "low_flux_mode",
              "low_flux_cutoff", "n_structures", "n_moments", "n_params", "motion_type", "scatter_enabled",
              "scatter_cutoff_enabled", "scatter_mass_ratio", "scatter_mean_free_path_cm", "scatter_rho",
              "scatter_cutoff_speed", "enable_force_measurement", "log_facet", "log_limit"):
        assert getattr(a, f) == getattr(b, f), f
    for f in ("motion_vector1", "motion_vector2", "torque_ref_point"):
        assert list(getattr(a, f)) == list(getattr(b, f)), f
    np.testing.assert_array_equal(_arr(a.moment_time, a.n_moments, np.float64), _arr(b.moment_time, b.n_moments, np.float64))
    np.testing.assert_array_equal(_arr(a.moment_window, a.n_moments, np.float64), _arr(b.moment_window, b.n_moments, np.float64))
    if a.n_params:
        st = _arr(a.param_start, a.n_params + 1, np.int32)
        np.testing.assert_array_equal(st, _arr(b.param_start, b.n_params + 1, np.int32))
        np.testing.assert_array_equal(_arr(a.param_t, st[-1], np.float64), _arr(b.param_t, st[-1], np.float64))
        np.testing.assert_array_equal(_arr(a.param_v, st[-1], np.float64), _arr(b.param_v, st[-1], np.float64))
        np.testing.assert_array_equal(_arr(a.param_log_x, a.n_params, np.uint8), _arr(b.param_log_x, b.n_params, np.uint8))
        np.testing.assert_array_equal(_arr(a.param_log_y, a.n_params, np.uint8), _arr(b.param_log_y, b.n_params, np.uint8))
    for f in ("record", "bounce_binsize", "bounce_max", "distance_binsize", "distance_max", "time_binsize", "time_max"):
        assert getattr(a.global_histogram, f) == getattr(b.global_histogram, f), f
    assert bool(a.facet_histogram) == bool(b.facet_histogram)
    if a.facet_histogram:
        for i in range(nf):
            for f in ("record", "bounce_binsize", "bounce_max", "distance_binsize", "distance_max", "time_binsize", "time_max"):
                assert getattr(a.facet_histogram[i], f) == getattr(b.facet_histogram[i], f), (i, f)
    dt = _arr(a.desorb_type, nf, np.int32)
    am = _arr(a.anglemap_phi_width, nf, np.int32) * (_arr(a.anglemap_theta_lower_res, nf, np.int32) +
                                                    _arr(a.anglemap_theta_higher_res, nf, np.int32))
    n_am = int(am[dt == A.DES_ANGLEMAP].sum())
    assert bool(a.desorb_anglemap) == bool(b.desorb_anglemap)
    if n_am:
        np.testing.assert_array_equal(_arr(a.desorb_anglemap, n_am, np.uint64), _arr(b.desorb_anglemap, n_am, np.uint64))
    assert bool(a.outgassing_map_width) == bool(b.outgassing_map_width)


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("ext", [".xml", ".zip"])
def test_native_reader_equals_python_reader(case, ext, tmp_path):
    L = _lib()
    m, _, _ = golden_util.load(case)
    st, _ = Oracle(m).run(3000, seed=5)
    gm = GpuModel(m)
    path = str(tmp_path / (case + ext))
    xmlwriter.save(path, m, st, gm.outgassing(), gm.facet_geometry()[1])
    m2, st2, _ = xmlio.load(path)
    pd = m2.desc()
    h = _open(L, path)
    try:
        cd = L.mfg_xml_desc(h).contents
        _assert_desc_equal(cd, pd)
        # the stored results through a model built from the library's own descriptor
        mh = C.c_void_p()
        assert L.mfg_model_create(C.byref(cd), C.byref(mh)) == A.MFG_OK
        try:
            got = SimuState(m2)
            for k in ARRAYS:   # prefill: the reader must clear what the file does not hold
                getattr(got, k)[...] = 7
            v = got.view()
            assert L.mfg_xml_read_state(h, mh, C.byref(v)) == A.MFG_OK
            for k in ARRAYS:
                np.testing.assert_array_equal(getattr(got, k), getattr(st2, k), err_msg=k)
        finally:
            L.mfg_model_destroy(mh)
    finally:
        L.mfg_xml_close(h)


def test_native_reader_user_moments_and_parameters(tmp_path):
    """Moment ranges ('begin,spacing,end') and parameters referenced by name, from a hand-written file."""
    L = _lib()
    m, _, _ = golden_util.load("02-timedependent_with_two_parameters")
    path = str(tmp_path / "m.xml")
    xmlwriter.save(path, m)
    text = open(path, encoding="utf-8").read()
    a = text.index("<UserMoments")
    b = text.index("</UserMoments>") + len("</UserMoments>")
    text = text[:a] + ('<UserMoments nb="3"><UserEntry content="0.001,0.0005,0.003" window="0.0001"/>'
                       '<UserEntry content="0.5" window="0.01"/><UserEntry content="0.1,0.2,0.05" window="0.0"/>'
                       '</UserMoments>') + text[b:]
    open(path, "w", encoding="utf-8").write(text)
    m2, _, _ = xmlio.load(path)
    h = _open(L, path)
    try:
        cd = L.mfg_xml_desc(h).contents
        _assert_desc_equal(cd, m2.desc())
        assert cd.n_moments == len(m2.moment_time) >= 5
    finally:
        L.mfg_xml_close(h)


def test_native_reader_errors(tmp_path):
    L = _lib()
    with pytest.raises(MfgError):
        _open(L, str(tmp_path / "missing.xml"))
    bad = tmp_path / "bad.xml"
    bad.write_text("<SimulationEnvironment><Geometry><Vertices></Geometry></SimulationEnvironment>")
    with pytest.raises(MfgError, match="end tag"):
        _open(L, str(bad))
    z = tmp_path / "noxml.zip"
    with zipfile.ZipFile(z, "w") as f:
        f.writestr("readme.txt", "no model here")
    with pytest.raises(MfgError, match="no .xml entry"):
        _open(L, str(z))
    # a file without results: the model loads, the results read is refused
    m, _, _ = golden_util.load("B02-lr10_pipe_tex")
    p = str(tmp_path / "geom.zip")
    xmlwriter.save(p, m)
    h = _open(L, p)
    try:
        cd = L.mfg_xml_desc(h).contents
        mh = C.c_void_p()
        assert L.mfg_model_create(C.byref(cd), C.byref(mh)) == A.MFG_OK
        st = SimuState(m)
        v = st.view()
        assert L.mfg_xml_read_state(h, mh, C.byref(v)) == A.MFG_ERR_INVALID_ARGUMENT
        L.mfg_model_destroy(mh)
    finally:
        L.mfg_xml_close(h)


def test_native_reader_parameter_catalog(tmp_path):
    """Catalog parameters (one .csv per parameter, LoadParameterCatalog) follow the file's own and
    can be referred to by name, as with the Python reader."""
    L = _lib()
    L.mfg_xml_open_catalog.argtypes = [C.c_char_p, C.c_char_p, C.POINTER(C.c_void_p)]
    cat = tmp_path / "catalog"
    cat.mkdir()
    (cat / "b_rate.csv").write_text("0.002, 0.5\n0.001,0.25\n\n0.003,0.75\n")
    (cat / "a_temp.csv").write_text("\ufeff0,300\n1,400\n")   # with a byte-order mark
    m, _, _ = golden_util.load("02-timedependent_with_two_parameters")
    path = str(tmp_path / "m.xml")
    xmlwriter.save(path, m)
    text = open(path, encoding="utf-8").read()
    i = text.index("<Sticking ", text.index('<Facet id="4"'))
    text = text[:i] + '<Sticking stickingParam="[catalog] b_rate.csv" ' + text[i + len("<Sticking "):]
    open(path, "w", encoding="utf-8").write(text)
    m2, _, info = xmlio.load(path, catalog=xmlio.load_catalog(str(cat)))
    h = C.c_void_p()
    assert L.mfg_xml_open_catalog(path.encode(), str(cat).encode(), C.byref(h)) == A.MFG_OK
    try:
        cd = L.mfg_xml_desc(h).contents
        _assert_desc_equal(cd, m2.desc())
        assert cd.n_params == 4
        assert _arr(cd.sticking_param, cd.n_facets, np.int32)[4] == 3   # after the file's two and a_temp.csv
        st = _arr(cd.param_start, 5, np.int32)
        np.testing.assert_array_equal(_arr(cd.param_t, st[-1], np.float64)[st[3]:st[4]], [0.001, 0.002, 0.003])
    finally:
        L.mfg_xml_close(h)
    with pytest.raises(MfgError, match="not found"):
        _open(L, path)


def test_cpp_adapter_reads_a_file(tmp_path):
    """mfg::XmlFile and mfg::ReadStoredResults from a C++ program (include/mfg_simulation.hpp)."""
    import os
    import subprocess
    from molflow_sources_gb300.simulation import library_path
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    load_library()
    lib = library_path()
    exe = str(tmp_path / "xml_check")
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(root, "include"),
                    os.path.join(root, "tests", "cpp", "xml_check.cpp"), "-o", exe,
                    "-L", os.path.dirname(lib), "-lmfg", "-Wl,-rpath," + os.path.dirname(lib)], check=True)
    m, _, _ = golden_util.load("09-histograms")
    st, _ = Oracle(m).run(2000, seed=5)
    gm = GpuModel(m)
    path = str(tmp_path / "r.zip")
    xmlwriter.save(path, m, st, gm.outgassing(), gm.facet_geometry()[1])
    out = subprocess.run([exe, path], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    lines = out.stdout.split("\n")
    assert lines[0] == "facets %d moments %d params %d results 1" % (m.n_facets, len(m.moment_time), len(m.params))
    g = lines[1].split()
    assert float(g[1]) == st.global_[A.G_NBMCHIT] and float(g[2]) == st.global_[A.G_NBDESORBED]
    assert int(g[5]) == int(st.facet_counts[..., A.FC_NBMCHIT].sum())
    assert int(g[7]) == int(st.facet_counts[..., A.FC_NBDESORBED].sum())
    # read and write back from C++: the copy holds the same model and results
    out2 = str(tmp_path / "copy.xml")
    again = subprocess.run([exe, path, "", out2], capture_output=True, text=True, timeout=120)
    assert again.returncode == 0 and "saved" in again.stdout, again.stdout + again.stderr
    m3, st3, _ = xmlio.load(out2)
    for k in ARRAYS:
        np.testing.assert_array_equal(getattr(st3, k), getattr(st, k), err_msg=k)
    _assert_desc_equal(m3.desc(), m.desc())
    bad = subprocess.run([exe, str(tmp_path / "none.zip")], capture_output=True, text=True, timeout=60)
    assert bad.returncode == 1 and "cannot open" in bad.stdout


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("ext", [".xml", ".zip"])
def test_native_writer_reads_back(case, ext, tmp_path):
    """mfg_xml_save (WriterXML.cpp:72-903 on the C++ host): the written file reads back, with the
    Python reader, as the same model and results, and the C++ reader gives the same descriptor."""
    L = _lib()
    L.mfg_xml_save.argtypes = [C.c_char_p, C.POINTER(A.ModelDesc), C.c_void_p, C.POINTER(A.StateView),
                               C.POINTER(C.c_char_p)]
    m, _, _ = golden_util.load(case)
    st, _ = Oracle(m).run(3000, seed=5)
    gm = GpuModel(m)
    path = str(tmp_path / (case + ext))
    v = st.view()
    names = (C.c_char_p * max(1, len(m.params)))(*[("p%d" % i).encode() for i in range(len(m.params))])
    assert L.mfg_xml_save(path.encode(), C.byref(gm._desc), gm.h, C.byref(v), names) == A.MFG_OK
    m2, st2, info = xmlio.load(path)
    for k in ARRAYS:
        np.testing.assert_array_equal(getattr(st2, k), getattr(st, k), err_msg=k)
    _assert_desc_equal(m2.desc(), gm._desc)
    assert info["param_names"] == ["p%d" % i for i in range(len(m.params))]
    h = _open(L, path)
    try:
        _assert_desc_equal(L.mfg_xml_desc(h).contents, gm._desc)
    finally:
        L.mfg_xml_close(h)
    # geometry and settings only
    p2 = str(tmp_path / ("geom" + ext))
    assert L.mfg_xml_save(p2.encode(), C.byref(gm._desc), gm.h, None, None) == A.MFG_OK
    m3, st3, _ = xmlio.load(p2)
    assert st3 is None
    _assert_desc_equal(m3.desc(), gm._desc)


def test_native_writer_and_reader_outgassing_map(tmp_path):
    """A facet desorbing from an outgassing map (DynamicOutgassing) goes through the C++ writer and
    the C++ reader unchanged: grid size, ratios and every cell."""
    from tests.og_model import og_tube
    L = _lib()
    L.mfg_xml_save.argtypes = [C.c_char_p, C.POINTER(A.ModelDesc), C.c_void_p, C.POINTER(A.StateView),
                               C.POINTER(C.c_char_p)]
    m, vals = og_tube()
    gm = GpuModel(m)
    path = str(tmp_path / "og.zip")
    assert L.mfg_xml_save(path.encode(), C.byref(gm._desc), gm.h, None, None) == A.MFG_OK
    m2, _, _ = xmlio.load(path)
    g, g2 = m.outgassing_maps[0], m2.outgassing_maps[0]
    assert (g["width"], g["height"], g["ratio_u"], g["ratio_v"]) == (g2["width"], g2["height"], g2["ratio_u"], g2["ratio_v"])
    np.testing.assert_array_equal(np.asarray(g["values"]).ravel(), np.asarray(g2["values"]).ravel())
    h = _open(L, path)
    try:
        cd = L.mfg_xml_desc(h).contents
        pd = gm._desc
        nf = cd.n_facets
        for f, dt in (("outgassing_map_width", np.int32), ("outgassing_map_height", np.int32),
                      ("outgassing_map_ratio_u", np.float64), ("outgassing_map_ratio_v", np.float64)):
            np.testing.assert_array_equal(_arr(getattr(cd, f), nf, dt), _arr(getattr(pd, f), nf, dt), err_msg=f)
        n = int((_arr(cd.outgassing_map_width, nf, np.int32) * _arr(cd.outgassing_map_height, nf, np.int32)).sum())
        np.testing.assert_array_equal(_arr(cd.outgassing_map, n, np.float64), _arr(pd.outgassing_map, n, np.float64))
    finally:
        L.mfg_xml_close(h)


def test_native_reader_old_formats(tmp_path):
    """Files of older versions: parameters referred to by index only (no names), the reflection
    given as a type (0 diffuse, 1 specular) instead of the diffuse/specular split, and a single
    outgassing-map ratio; the C++ reader takes them like the Python reader."""
    import re
    L = _lib()
    m, _, _ = golden_util.load("02-timedependent_with_two_parameters")
    path = str(tmp_path / "old.xml")
    xmlwriter.save(path, m)
    text = open(path, encoding="utf-8").read()
    text = re.sub(r' (stickingParam|opacityParam|outgassingParam|OutgassingParam)="[^"]*"', "", text)
    text = re.sub(r' diffusePart="[^"]*" specularPart="[^"]*" cosineExponent="[^"]*"', "", text)
    text = text.replace('<Reflection type="0"', '<Reflection type="1"', 3)   # three specular facets
    open(path, "w", encoding="utf-8").write(text)
    m2, _, _ = xmlio.load(path)
    assert (m2.refl_specular == 1.0).sum() == 3
    h = _open(L, path)
    try:
        _assert_desc_equal(L.mfg_xml_desc(h).contents, m2.desc())
    finally:
        L.mfg_xml_close(h)


def test_native_reader_xml_syntax(tmp_path):
    """The XML forms a file may use: a declaration, comments, CDATA text, character and entity
    references in attributes, single-quoted attributes, self-closing and empty elements."""
    L = _lib()
    m, _, _ = golden_util.load("B02-lr10_pipe_tex")
    path = str(tmp_path / "s.xml")
    xmlwriter.save(path, m)
    text = open(path, encoding="utf-8").read()
    text = text.replace("<Geometry>", "<!-- a comment <Geometry> -->\n<Geometry>", 1)
    text = text.replace('<Vertex id="0" x="', "<Vertex id='0' x=\"", 1)
    text = text.replace('<Structure id="0" name="structure 1" />',
                        '<Structure id="0" name="&lt;main&gt; &amp; &#233;&#x41;"></Structure>', 1)
    text = text.replace("<Interface />", "<Interface><![CDATA[ <not> parsed & kept ]]></Interface>", 1)
    for form in ("<!-- a comment", "<Vertex id='0'", "&#x41;", "<![CDATA["):
        assert form in text, form
    open(path, "w", encoding="utf-8").write(text)
    m2, _, _ = xmlio.load(path)
    h = _open(L, path)
    try:
        _assert_desc_equal(L.mfg_xml_desc(h).contents, m2.desc())
    finally:
        L.mfg_xml_close(h)
    bad = tmp_path / "bad2.xml"
    bad.write_text("<A><B x=1/></A>")
    with pytest.raises(MfgError, match="unquoted"):
        _open(L, str(bad))


def test_native_reader_extreme_values(tmp_path):
    """Out-of-range numbers in a file: counts that are not a number or negative read as 0, a stored
    texture whose declared size overflows is skipped, and a structure count past the limit is
    refused with MFG_ERR_LIMIT, not attempted."""
    L = _lib()
    m, _, _ = golden_util.load("B02-lr10_pipe_tex")
    st, _ = Oracle(m).run(3000, seed=5)
    gm = GpuModel(m)
    path = tmp_path / "b02.xml"
    xmlwriter.save(str(path), m, st, gm.outgassing(), gm.facet_geometry()[1])
    text = path.read_text()
    text = text.replace('nbAbsEquiv="', 'nbAbsEquiv="nan', 1)   # "nan<number>": not a number
    i = text.index("<MolflowResults")
    j = text.index('<Texture width="', i) + len('<Texture width="')
    text = text[:j] + "9.2e18" + text[text.index('"', j):]
    bad = tmp_path / "extreme.xml"
    bad.write_text(text)

    def read(p):
        h = _open(L, str(p))
        try:
            cd = L.mfg_xml_desc(h).contents
            mh = C.c_void_p()
            assert L.mfg_model_create(C.byref(cd), C.byref(mh)) == A.MFG_OK
            try:
                got = SimuState(m)
                v = got.view()
                assert L.mfg_xml_read_state(h, mh, C.byref(v)) == A.MFG_OK
                return got
            finally:
                L.mfg_model_destroy(mh)
        finally:
            L.mfg_xml_close(h)
    good, got = read(path), read(bad)
    fc_good = good.facet_counts.reshape(-1, A.FC_N)
    fc_got = got.facet_counts.reshape(-1, A.FC_N)
    changed = np.flatnonzero(fc_good[:, A.FC_NBABSORBED] != fc_got[:, A.FC_NBABSORBED])
    assert len(changed) == 1 and fc_got[changed[0], A.FC_NBABSORBED] == 0 and fc_good[changed[0], A.FC_NBABSORBED] > 0
    # the texture with the overflowing declared size is left empty, the others are read
    assert good.texture.any() and got.texture.sum() < good.texture.sum() and got.texture.any()
    many = tmp_path / "structures.xml"
    many.write_text(path.read_text().replace('<Structures nb="1"', '<Structures nb="2147483647"', 1))
    h = _open(L, str(many))
    try:
        cd = L.mfg_xml_desc(h).contents
        assert cd.n_structures == 2147483647
        mh = C.c_void_p()
        assert L.mfg_model_create(C.byref(cd), C.byref(mh)) == A.MFG_ERR_LIMIT
    finally:
        L.mfg_xml_close(h)


def test_model_size_limits():
    """Sizes past the device's 32-bit cell offsets and histogram settings that define no bins are
    refused before anything is allocated for them."""
    def code(m):
        with pytest.raises(MfgError) as e:
            GpuModel(m)
        return e.value.code
    m, _, _ = golden_util.load("B02-lr10_pipe_tex")
    k = int(np.flatnonzero(m.tex_width * m.tex_height > 0)[0])
    m.tex_width[k] = m.tex_height[k] = 50000.0   # 2.5e9 cells
    assert code(m) == A.MFG_ERR_LIMIT
    m, _, _ = golden_util.load("B02-lr10_pipe_tex")
    m.tex_width[0] = float("nan")
    assert code(m) == A.MFG_ERR_INVALID_MODEL
    m, _, _ = golden_util.load("B02-lr10_pipe_tex")
    m.n_structures = A.MFG_MAX_STRUCTURES + 1
    assert code(m) == A.MFG_ERR_LIMIT
    m, _, _ = golden_util.load("B02-lr10_pipe_tex")
    m.hist_record[0] = A.HIST_DISTANCE
    m.hist_distance_binsize[0] = 0.0
    m.hist_distance_max[0] = 10.0
    assert code(m) == A.MFG_ERR_INVALID_MODEL


def test_model_rejects_non_finite_vertex():
    m, _, _ = golden_util.load("B02-lr10_pipe_tex")
    m.vertices[3, 1] = float("inf")
    with pytest.raises(MfgError, match="not a finite point") as e:
        GpuModel(m)
    assert e.value.code == A.MFG_ERR_INVALID_MODEL


def test_native_writer_counts_out_of_range(tmp_path):
    """Counts held as doubles that are not a number or past the 64-bit range are written as 0 and
    as the clamped value, not converted with undefined results."""
    L = _lib()
    L.mfg_xml_save.argtypes = [C.c_char_p, C.POINTER(A.ModelDesc), C.c_void_p, C.POINTER(A.StateView),
                               C.POINTER(C.c_char_p)]
    m, _, _ = golden_util.load("B02-lr10_pipe_tex")
    st, _ = Oracle(m).run(3000, seed=5)
    gm = GpuModel(m)
    st.global_[A.G_NBMCHIT] = float("nan")
    st.global_[A.G_NBDESORBED] = -1e300
    st.global_[A.G_NBLEAK] = 1e300
    path = str(tmp_path / "counts.xml")
    v = st.view()
    assert L.mfg_xml_save(path.encode(), C.byref(gm._desc), gm.h, C.byref(v), None) == A.MFG_OK
    _, st2, _ = xmlio.load(path)
    assert st2.global_[A.G_NBMCHIT] == 0
    assert st2.global_[A.G_NBDESORBED] == -9.2e18
    assert st2.global_[A.G_NBLEAK] == 9.2e18


def test_native_reader_survives_mutated_files(tmp_path):
    """Seeded attribute mutations of a written file (extreme numbers, not a number, empty values):
    the C++ reader, the model build, the results read and the writer either succeed or return an
    error code; none of them crashes.  (The same mutations ran at scale under sanitizers.)"""
    import random
    L = _lib()
    L.mfg_xml_save.argtypes = [C.c_char_p, C.POINTER(A.ModelDesc), C.c_void_p, C.POINTER(A.StateView),
                               C.POINTER(C.c_char_p)]
    m, _, _ = golden_util.load("01-quick_pipe_profiles_textures_2sided")
    st, _ = Oracle(m).run(3000, seed=5)
    gm = GpuModel(m)
    base = str(tmp_path / "base.xml")
    xmlwriter.save(base, m, st, gm.outgassing(), gm.facet_geometry()[1])
    text = open(base).read()
    values = ["-1", "0", "2147483647", "-2147483648", "1e300", "-1e300", "nan", "inf", "", "x", "4294967296",
              "65536", "3", "-5", "0.5", "1e-300", "9223372036854775807"]
    r = random.Random(20261205)
    outcomes = {"read": 0, "model": 0, "results": 0, "refused": 0}
    for it in range(400):
        t = text
        for _ in range(1 + r.randrange(6)):
            q = t.find('="', r.randrange(len(t)))
            if q < 0:
                continue
            e = t.find('"', q + 2)
            t = t[:q + 2] + r.choice(values) + t[e:]
        p = str(tmp_path / "m.xml")
        open(p, "w").write(t)
        h = C.c_void_p()
        if L.mfg_xml_open(p.encode(), C.byref(h)) != A.MFG_OK:
            outcomes["refused"] += 1
            continue
        outcomes["read"] += 1
        try:
            cd = L.mfg_xml_desc(h).contents
            mh = C.c_void_p()
            if L.mfg_model_create(C.byref(cd), C.byref(mh)) != A.MFG_OK:
                continue
            outcomes["model"] += 1
            try:
                lay = A.StateLayout()
                assert L.mfg_state_layout_of(mh, C.byref(lay)) == A.MFG_OK
                if max(lay.n_texture, lay.n_facet_counts, lay.n_histogram, lay.n_direction, lay.n_profile) > 10 ** 7:
                    continue
                arrays = {f: np.zeros(max(1, getattr(lay, "n_" + f)), np.uint64 if f in ("facet_counts", "anglemap")
                                      else np.float64)
                          for f in ("global", "facet_counts", "facet_sums", "texture", "profile", "direction",
                                    "anglemap", "histogram", "force")}
                v = A.StateView(*[arrays[f].ctypes.data_as(C.POINTER(C.c_uint64 if arrays[f].dtype == np.uint64
                                                                      else C.c_double)) for f in
                                  ("global", "facet_counts", "facet_sums", "texture", "profile", "direction",
                                   "anglemap", "histogram", "force")])
                if L.mfg_xml_read_state(h, mh, C.byref(v)) == A.MFG_OK:
                    outcomes["results"] += 1
                    out = str(tmp_path / "w.zip")
                    if L.mfg_xml_save(out.encode(), C.byref(cd), mh, C.byref(v), None) == A.MFG_OK:
                        h2 = C.c_void_p()
                        assert L.mfg_xml_open(out.encode(), C.byref(h2)) == A.MFG_OK
                        L.mfg_xml_close(h2)
            finally:
                L.mfg_model_destroy(mh)
        finally:
            L.mfg_xml_close(h)
    assert outcomes["results"] > 10 and outcomes["model"] < outcomes["read"]
