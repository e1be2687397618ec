"""exnode / exelem reader and writer (iron_gb300/exfile.py).  Iron's own Cantilever and SimpleShear
outputs (linear Lagrange with grid-based element fields; cubic Hermite with derivatives and two
scale-factor sets; triquadratic Lagrange with one scale-factor set; tests/golden/exfile, copied by
tests/golden/make_golden.py) read and written again are byte-identical, which pins the writer to
Iron's FieldExport.c formats; the SimpleShear mesh pins the triquadratic generated-mesh numbering.  This package's Laplace and
Mooney-Rivlin exports round-trip exactly.  CPU only."""
from pathlib import Path

import numpy as np
import pytest

from iron_gb300 import exfile as X
from iron_gb300 import mesh as M

GOLD = Path(__file__).resolve().parent / "golden" / "exfile"
CASES = ["cantilever_linear_3x2x2", "cantilever_cubic_2x1x1", "simple_shear"]


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("ext", ["exnode", "exelem"])
def test_irons_files_round_trip_byte_identical(case, ext, tmp_path):
    text = (GOLD / f"{case}.{ext}").read_text()
    if ext == "exnode":
        ex = X.parse_exnode(text)
        X.write_exnode(tmp_path / "out", ex)
    else:
        ex = X.parse_exelem(text)
        X.write_exelem(tmp_path / "out", ex)
    assert (tmp_path / "out").read_text() == text


def test_linear_cantilever_content():
    nodes = X.read_exnode(GOLD / "cantilever_linear_3x2x2.exnode")
    assert nodes.group == "Region" and len(nodes.sections) == 1
    sec = nodes.sections[0]
    assert [f.name for f in sec.fields] == ["Geometry", "Fibre", "Dependent", "del U/del n"]
    assert len(sec.nodes) == 36  # 4 x 3 x 3 nodes of the 3 x 2 x 2 mesh
    x = X.node_values(nodes, "Geometry", 0)
    assert x[1] == 0.0 and x[2] == 20.0 and max(x.values()) == 60.0  # 60 x 40 x 40 beam
    elems = X.read_exelem(GOLD / "cantilever_linear_3x2x2.exelem")
    es = elems.sections[0]
    assert es.header.n_nodes == 8 and len(es.elements) == 12
    assert es.elements[0].nodes == [1, 2, 5, 6, 13, 14, 17, 18]
    # the pressure component of the dependent field is grid based (element constant)
    assert es.header.fields[2].components[3].grid == "#xi1=1, #xi2=1, #xi3=1"


def test_triquadratic_mesh_matches_irons_generated_mesh():
    """Iron's SimpleShear output (a 2x2x2 triquadratic generated mesh of the unit cube) has the
    element node lists and node positions of mesh.RegularMesh(order=2), the mesh the Q2/Q1
    Mooney-Rivlin path builds its element DOF lists from."""
    elems = X.read_exelem(GOLD / "simple_shear.exelem")
    es = elems.sections[0]
    assert es.header.n_nodes == 27 and len(es.elements) == 8
    assert es.header.scale_sets == [("q.Lagrange*q.Lagrange*q.Lagrange", 27)]
    m = M.RegularMesh((2, 2, 2), order=2)
    assert np.array_equal(np.array([e.nodes for e in es.elements]) - 1, m.elem_nodes)
    nodes = X.read_exnode(GOLD / "simple_shear.exnode")
    assert [f.name for f in nodes.sections[0].fields] == ["Geometry", "Fibre", "Dependent", "del U/del n",
                                                          "Material"]
    xyz = [X.node_values(nodes, "Geometry", c) for c in range(3)]
    coords = np.array([[xyz[c][k] for k in sorted(xyz[c])] for c in range(3)])
    assert np.array_equal(coords, m.coords)


def test_trilinear_mesh_matches_irons_generated_mesh():
    """The linear Cantilever output (a 3x2x2 trilinear generated mesh of a 60 x 40 x 40 beam) has
    the element node lists and node positions of mesh.RegularMesh(order=1), the mesh of the
    regular-mesh Laplace kernels."""
    es = X.read_exelem(GOLD / "cantilever_linear_3x2x2.exelem").sections[0]
    m = M.RegularMesh((3, 2, 2), order=1, extent=(60.0, 40.0, 40.0))
    assert np.array_equal(np.array([e.nodes for e in es.elements]) - 1, m.elem_nodes)
    nodes = X.read_exnode(GOLD / "cantilever_linear_3x2x2.exnode")
    xyz = [X.node_values(nodes, "Geometry", c) for c in range(3)]
    assert np.array_equal(np.array([[xyz[c][k] for k in sorted(xyz[c])] for c in range(3)]), m.coords)


def test_cubic_hermite_mesh_matches_irons_generated_mesh():
    """The cubic Cantilever output (a 2x1x1 tricubic Hermite generated mesh of a 60 x 40 x 40
    beam, arc-length scaling) has the geometric parameters (value and 7 derivatives a node and
    component), element node lists and Hermite scale factors of mesh.HermiteMesh(scaling=
    "arc_length"), whose element parameter lists run node by node, 8 derivatives each."""
    hm = M.HermiteMesh((2, 1, 1), extent=(60.0, 40.0, 40.0), scaling="arc_length")
    sec = X.read_exnode(GOLD / "cantilever_cubic_2x1x1.exnode").sections[0]
    geo = np.array([[sec.nodes[i][1][c] for i in range(len(sec.nodes))] for c in range(3)])
    assert np.array_equal(geo.reshape(3, -1), hm.params)
    els = X.read_exelem(GOLD / "cantilever_cubic_2x1x1.exelem").sections[0].elements
    nodes = np.array([e.nodes for e in els]) - 1
    assert np.array_equal(hm.elem_params.reshape(len(els), 8, 8), nodes[:, :, None] * 8 + np.arange(8))
    assert np.array_equal(np.array([e.scale_factors[0] for e in els]), hm.scale)


def test_cubic_hermite_derivatives_and_scale_factors():
    nodes = X.read_exnode(GOLD / "cantilever_cubic_2x1x1.exnode")
    comp = nodes.sections[0].fields[0].components[0]
    assert comp.n_derivatives == 7 and comp.derivative_labels.startswith("(d/ds1,d/ds2,")
    assert len(nodes.sections[0].nodes[0][1][0]) == 8  # value + 7 derivatives on one line
    elems = X.read_exelem(GOLD / "cantilever_cubic_2x1x1.exelem")
    h = elems.sections[0].header
    assert h.scale_sets == [("c.Hermite*c.Hermite*c.Hermite", 64), ("l.Lagrange*l.Lagrange*l.Lagrange", 8)]
    assert h.fields[0].components[0].nodes[1] == (2, list(range(1, 9)), list(range(9, 17)))
    assert [len(r) for r in elems.sections[0].elements[0].scale_factors] == [64, 8]


def test_laplace_export_round_trips(tmp_path):
    m = M.RegularMesh((3, 2, 2))
    m.jitter_interior(1)
    u = np.random.default_rng(2).standard_normal(m.n_nodes)
    exn, exe = X.laplace_exfiles(m.coords, m.elem_nodes, u)
    X.write_exnode(tmp_path / "a.exnode", exn)
    X.write_exelem(tmp_path / "a.exelem", exe)
    back = X.read_exnode(tmp_path / "a.exnode")
    for c in range(3):
        got = X.node_values(back, "Geometry", c)
        assert np.array_equal(np.array([got[k + 1] for k in range(m.n_nodes)]), m.coords[c])
    got = X.node_values(back, "Phi", 0)
    assert np.array_equal(np.array([got[k + 1] for k in range(m.n_nodes)]), u)
    e = X.read_exelem(tmp_path / "a.exelem")
    assert [el.nodes for el in e.sections[0].elements] == (m.elem_nodes + 1).tolist()
    assert X.format_exelem(e) == (tmp_path / "a.exelem").read_text()


def test_mooney_rivlin_export_round_trips(tmp_path):
    ne = (2, 2, 1)
    eq2 = M.regular_elements(ne, 2)
    xg = M.regular_coords(ne, 2)
    elin, lin2g = M.linear_component(eq2, 2)
    n_q2, n_lin = xg.shape[1], len(lin2g)
    rng = np.random.default_rng(3)
    dep = np.r_[(xg * 1.1).ravel(), rng.standard_normal(n_lin)]
    exn, exe = X.mr_exfiles(xg, eq2, elin, dep)
    X.write_exnode(tmp_path / "mr.exnode", exn)
    X.write_exelem(tmp_path / "mr.exelem", exe)
    back = X.read_exnode(tmp_path / "mr.exnode")
    assert [len(s.fields[1].components) for s in back.sections] == [3, 4]  # pressure only on corner nodes
    p = X.node_values(back, "Dependent", 3)
    assert sorted(p) == sorted((lin2g + 1).tolist())
    assert np.array_equal(np.array([p[g + 1] for g in lin2g]), dep[3 * n_q2:])
    z = X.node_values(back, "Dependent", 1)
    assert np.array_equal(np.array([z[k + 1] for k in range(n_q2)]), dep[n_q2:2 * n_q2])
    e = X.read_exelem(tmp_path / "mr.exelem")
    pcomp = e.sections[0].header.fields[1].components[3]
    assert pcomp.basis == "l.Lagrange*l.Lagrange*l.Lagrange" and [n[0] for n in pcomp.nodes] == [1, 3, 7, 9, 19, 21, 25, 27]
    assert X.format_exelem(e) == (tmp_path / "mr.exelem").read_text()


def test_malformed_input_is_rejected():
    with pytest.raises(X.ExFormatError):
        X.parse_exnode(" Group name: g\n Node:            1\n  1.0E+00\n")
    with pytest.raises(X.ExFormatError):
        X.parse_exelem(" Group name: g\n Element:            1 0 0\n")
