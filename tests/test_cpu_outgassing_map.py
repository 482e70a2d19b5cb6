"""Outgassing maps (useOutgassingFile; StartFromSource, Particle.cpp:425-446 and 513-535) in the
oracle: a particle starts in a map cell chosen by its rate, uniformly inside the cell; the last
row and column of the grid are partial cells.  The map facet's weight among the sources is the
sum of its cells (MolflowSimGeom.cpp:303-310)."""
import numpy as np

from molflow_sources_gb300 import _abi as A
from molflow_sources_gb300 import xmlio
from oracle.oracle import Oracle
from tests.og_model import GRID, og_tube
from tests.stats import z_threshold

SEED = 0x4D6F6C66


def test_desorption_cells_follow_the_map():
    m, vals = og_tube()
    n = 400_000
    r, _ = Oracle(m).run(n, seed=SEED)
    assert r.global_[A.G_NBLEAK] == 0
    tex = r.texture_of(0)[..., 0].reshape(GRID, GRID)   # desorptions per cell (same grid as the map)
    assert tex.sum() == n
    p = vals / vals.sum()
    assert (tex[p == 0] == 0).all()
    z = (tex / n - p)[p > 0] / np.sqrt(p[p > 0] * (1 - p[p > 0]) / n)
    assert np.abs(z).max() < z_threshold(int((p > 0).sum())), np.abs(z).max()


def test_start_points_are_uniform_within_cells():
    """Half-cell last column: a finer texture (19 x 19 over the same extent) splits every map cell
    in four; inside a cell the four quarters get equal shares."""
    m, vals = og_tube()
    m.tex_width[0] = 19.0
    m.tex_height[0] = 19.0
    n = 400_000
    r, _ = Oracle(m).run(n, seed=SEED + 1)
    tex = r.texture_of(0)[..., 0].reshape(19, 19)
    for h in range(9):
        for w in range(9):
            if vals[h, w] == 0:
                continue
            q = tex[2 * h:2 * h + 2, 2 * w:2 * w + 2].astype(float)
            e = q.sum() / 4
            assert np.abs(q - e).max() < 5 * np.sqrt(e) + 1, (h, w, q)


def test_map_facet_weight_is_the_sum_of_its_cells():
    m, vals = og_tube()
    m.desorb_type[1] = A.DES_COSINE      # the outlet desorbs too, with a constant rate
    m.outgassing[1] = vals.sum()         # equal to the map's total
    n = 200_000
    r, _ = Oracle(m).run(n, seed=SEED + 2)
    d0, d1 = int(r.facet_counts[0, 0, A.FC_NBDESORBED]), int(r.facet_counts[0, 1, A.FC_NBDESORBED])
    assert abs(d0 - d1) < 5 * np.sqrt(n / 4)


def _xml_with_map(cells, w, h, ratio):
    """A one-facet square model in the reference's XML layout with a DynamicOutgassing map."""
    txt = " ".join("%g" % x for x in np.asarray(cells).ravel())
    return f"""<?xml version="1.0"?>
<SimulationEnvironment>
 <Geometry>
  <Vertices nb="4">
   <Vertex id="0" x="0" y="0" z="0"/><Vertex id="1" x="1" y="0" z="0"/>
   <Vertex id="2" x="1" y="1" z="0"/><Vertex id="3" x="0" y="1" z="0"/>
  </Vertices>
  <Facets nb="1">
   <Facet id="0">
    <Sticking constValue="1" parameterId="-1"/>
    <Opacity constValue="1" parameterId="-1" is2sided="0"/>
    <Outgassing constValue="0" parameterId="-1" desType="2" desExponent="0" hasOutgassingFile="1" useOutgassingFile="1"/>
    <Temperature value="293.15" accFactor="1"/>
    <Structure inStructure="0" linksTo="0"/>
    <DynamicOutgassing width="{w}" height="{h}" ratio="{ratio}" totalDose="0" totalOutgassing="{np.sum(cells)}" totalFlux="0"><map>{txt}</map></DynamicOutgassing>
    <Indices nb="4"><Indice i="0" vertex="0"/><Indice i="1" vertex="1"/><Indice i="2" vertex="2"/><Indice i="3" vertex="3"/></Indices>
   </Facet>
  </Facets>
  <Structures nb="1"><Structure name="s"/></Structures>
 </Geometry>
</SimulationEnvironment>"""


def test_xml_reader_takes_the_map():
    cells = np.arange(12, dtype=float).reshape(3, 4)
    m, _, _ = xmlio.load(_xml_with_map(cells, 4, 3, 2.5).encode(), with_state=False)
    g = m.outgassing_maps[0]
    assert (g["width"], g["height"], g["ratio_u"], g["ratio_v"]) == (4, 3, 2.5, 2.5)
    assert np.array_equal(g["values"], cells)
