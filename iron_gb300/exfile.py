"""exnode / exelem files: Iron's field export format (CMISS ex-format), read and written.

Iron exports fields through src/field_IO_routines.F90 (FIELD_IO_NODES_EXPORT / FIELD_IO_ELEMENTS_EXPORT)
and the formatting layer src/FieldExport.c.  The writer here reproduces that layer's lines:
  " Group name: %s"                                   FieldExport_File_Group
  " #Fields=%d",  " %d) %s, %s, #Components=%d"       FieldExport_File_FieldCount / _Variable
  "   %s.  Value index= %d, #Derivatives= %d(...)"    FieldExport_File_(Coordinate)DerivativeIndices
  " Node:            %d",  then per component "  %.16E" x values     FieldExport_File_NodeValues
  " Shape.  Dimension=%d",  " #Scale factor sets= %d",  " <basis>, #Scale factors=%d"
  " #Nodes=           %d"                             FieldExport_File_NodeCount
  "   %s.   <basis>, no modify, standard node based." / "grid based."  (InterpolationHeader)
  "     #Nodes= %d",  " %5d.  #Values=%d",  "      Value indices:  " + " %3d" x n,
  "      Scale factor indices: " + (" %3d" x n | " 0" x n)           FieldExport_File_NodeScaleIndexes
  "     #xi1=%d, #xi2=%d, #xi3=%d"                    FieldExport_File_ElementGridSize
  " Element:            %d 0 0"                       FieldExport_File_ElementIndex
  "   Values:" + "  " + "   %.16E" x n per grid-based component        _ElementGridValues
  "   Nodes:" + "  %10d" x n                          FieldExport_File_ElementNodeIndices
  "   Scale factors:" + "  " + "   %.16E" x n per scale-factor set     _ElementNodeScales
so a file read from Iron and written again is byte-identical (tests/test_exfile.py, on Iron's own
Cantilever outputs).  Builders export this package's Laplace and Mooney-Rivlin results in the same
format, readable by Iron's tools and cmgui.
"""
from __future__ import annotations

import re
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

# ------------------------------------------------------------------------------------------------
# data model
# ------------------------------------------------------------------------------------------------


@dataclass
class NodeComponent:
    name: str
    value_index: int
    n_derivatives: int = 0
    derivative_labels: str = ""  # "(d/ds1,d/ds2,...)" as written after the count, or ""


@dataclass
class NodeField:
    name: str
    label: str  # e.g. "coordinate, rectangular cartesian", "field,  rectangular cartesian"
    components: list[NodeComponent]


@dataclass
class NodeSection:
    fields: list[NodeField]
    nodes: list[tuple[int, list[list[float]]]] = field(default_factory=list)  # (number, one list per component)


@dataclass
class ExNode:
    group: str
    sections: list[NodeSection]


@dataclass
class ElemComponent:
    name: str
    basis: str                      # e.g. "l.Lagrange*l.Lagrange*l.Lagrange"
    grid: str | None = None         # grid-based: "#xi1=1, #xi2=1, #xi3=1"
    # node-based: (local node index, value indices, scale-factor indices or None when unscaled)
    nodes: list[tuple[int, list[int], list[int] | None]] = field(default_factory=list)


@dataclass
class ElemField:
    name: str
    label: str
    components: list[ElemComponent]


@dataclass
class ElemHeader:
    shape: str                                 # text after " Shape.  ", e.g. "Dimension=3"
    scale_sets: list[tuple[str, int]]          # (basis, number of scale factors)
    n_nodes: int
    fields: list[ElemField]


@dataclass
class Element:
    number: int
    values: list[list[float]]                  # one list per grid-based component
    nodes: list[int]
    scale_factors: list[list[float]]           # one list per scale-factor set


@dataclass
class ElemSection:
    header: ElemHeader
    elements: list[Element] = field(default_factory=list)


@dataclass
class ExElem:
    group: str
    sections: list[ElemSection]


# ------------------------------------------------------------------------------------------------
# writers
# ------------------------------------------------------------------------------------------------


def _e16(v: float) -> str:
    return f"{float(v):.16E}"


def _field_line(i: int, name: str, label: str, n: int) -> str:
    return f" {i}) {name}, {label}, #Components={n}\n"


def format_exnode(ex: ExNode) -> str:
    out = [f" Group name: {ex.group}\n"]
    for sec in ex.sections:
        out.append(f" #Fields={len(sec.fields)}\n")
        for i, f in enumerate(sec.fields, 1):
            out.append(_field_line(i, f.name, f.label, len(f.components)))
            for c in f.components:
                out.append(f"   {c.name}.  Value index= {c.value_index}, #Derivatives= {c.n_derivatives}"
                           f"{c.derivative_labels}\n")
        for number, comps in sec.nodes:
            out.append(f" Node:            {number}\n")
            for vals in comps:
                out.append("".join("  " + _e16(v) for v in vals) + "\n")
    return "".join(out)


def format_exelem(ex: ExElem) -> str:
    out = [f" Group name: {ex.group}\n"]
    for sec in ex.sections:
        h = sec.header
        out.append(f" Shape.  {h.shape}\n")
        out.append(f" #Scale factor sets= {len(h.scale_sets)}\n")
        for basis, count in h.scale_sets:
            out.append(f" {basis}, #Scale factors={count}\n")
        out.append(f" #Nodes=           {h.n_nodes}\n")
        out.append(f" #Fields={len(h.fields)}\n")
        for i, f in enumerate(h.fields, 1):
            out.append(_field_line(i, f.name, f.label, len(f.components)))
            for c in f.components:
                kind = "grid based" if c.grid is not None else "standard node based"
                out.append(f"   {c.name}.   {c.basis}, no modify, {kind}.\n")
                if c.grid is not None:
                    out.append(f"     {c.grid}\n")
                    continue
                out.append(f"     #Nodes= {len(c.nodes)}\n")
                for local, vidx, sidx in c.nodes:
                    out.append(f" {local:5d}.  #Values={len(vidx)}\n")
                    out.append("      Value indices:  " + "".join(f" {v:3d}" for v in vidx) + "\n")
                    scale = "".join(f" {s:3d}" for s in sidx) if sidx is not None else " 0" * len(vidx)
                    out.append("      Scale factor indices: " + scale + "\n")
        for e in sec.elements:
            out.append(f" Element:            {e.number} 0 0\n")
            if e.values:
                out.append("   Values:\n")
                for row in e.values:
                    out.append("  " + "".join("   " + _e16(v) for v in row) + "\n")
            out.append("   Nodes:\n")
            out.append("".join(f"  {n:10d}" for n in e.nodes) + "\n")
            if e.scale_factors:
                out.append("   Scale factors:\n")
                for row in e.scale_factors:
                    out.append("  " + "".join("   " + _e16(v) for v in row) + "\n")
    return "".join(out)


def write_exnode(path, ex: ExNode) -> None:
    Path(path).write_text(format_exnode(ex))


def write_exelem(path, ex: ExElem) -> None:
    Path(path).write_text(format_exelem(ex))


# ------------------------------------------------------------------------------------------------
# readers
# ------------------------------------------------------------------------------------------------

_RE_FIELD = re.compile(r"^ (\d+)\) (.*?), (.*), #Components=(\d+)$")
_RE_NODE_COMP = re.compile(r"^   (\S+)\.  Value index= (\d+), #Derivatives= (\d+)(.*)$")
_RE_ELEM_COMP = re.compile(r"^   (\S+)\.   (.*), no modify, (standard node based|grid based)\.$")


class ExFormatError(ValueError):
    pass


def _floats(line: str) -> list[float]:
    return [float(t) for t in line.split()]


def _is_number_row(line: str) -> bool:
    toks = line.split()
    if not toks:
        return False
    try:
        float(toks[0])
    except ValueError:
        return False
    return True


def parse_exnode(text: str) -> ExNode:
    lines = text.splitlines()
    group, sections, i = "", [], 0
    cur_node = None
    while i < len(lines):
        ln = lines[i]
        if ln.startswith(" Group name: "):
            group = ln[len(" Group name: "):]
            i += 1
        elif ln.startswith(" #Fields="):
            nf = int(ln.split("=")[1])
            fields, i = [], i + 1
            for _ in range(nf):
                m = _RE_FIELD.match(lines[i])
                if not m:
                    raise ExFormatError(f"line {i + 1}: expected a field header, got {lines[i]!r}")
                comps, i = [], i + 1
                for _ in range(int(m.group(4))):
                    mc = _RE_NODE_COMP.match(lines[i])
                    if not mc:
                        raise ExFormatError(f"line {i + 1}: expected a component header, got {lines[i]!r}")
                    comps.append(NodeComponent(mc.group(1), int(mc.group(2)), int(mc.group(3)), mc.group(4)))
                    i += 1
                fields.append(NodeField(m.group(2), m.group(3), comps))
            sections.append(NodeSection(fields))
            cur_node = None
        elif ln.startswith(" Node:"):
            if not sections:
                raise ExFormatError(f"line {i + 1}: node before any field header")
            cur_node = (int(ln.split(":")[1]), [])
            sections[-1].nodes.append(cur_node)
            i += 1
        elif ln.strip() == "":
            i += 1
        else:
            if cur_node is None:
                raise ExFormatError(f"line {i + 1}: values outside a node: {ln!r}")
            cur_node[1].append(_floats(ln))
            i += 1
    return ExNode(group, sections)


def parse_exelem(text: str) -> ExElem:
    lines = text.splitlines()
    group, sections, i = "", [], 0
    n = len(lines)
    while i < n:
        ln = lines[i]
        if ln.startswith(" Group name: "):
            group = ln[len(" Group name: "):]
            i += 1
        elif ln.startswith(" Shape.  "):
            shape = ln[len(" Shape.  "):]
            i += 1
            if not lines[i].startswith(" #Scale factor sets= "):
                raise ExFormatError(f"line {i + 1}: expected the scale-factor sets")
            ns = int(lines[i].split("=")[1])
            i += 1
            sets = []
            for _ in range(ns):
                basis, cnt = lines[i].strip().rsplit(", #Scale factors=", 1)
                sets.append((basis, int(cnt)))
                i += 1
            if not lines[i].startswith(" #Nodes="):
                raise ExFormatError(f"line {i + 1}: expected the element node count")
            n_nodes = int(lines[i].split("=")[1])
            i += 1
            nf = int(lines[i].split("=")[1])
            i += 1
            fields = []
            for _ in range(nf):
                m = _RE_FIELD.match(lines[i])
                if not m:
                    raise ExFormatError(f"line {i + 1}: expected a field header, got {lines[i]!r}")
                comps, i = [], i + 1
                for _ in range(int(m.group(4))):
                    mc = _RE_ELEM_COMP.match(lines[i])
                    if not mc:
                        raise ExFormatError(f"line {i + 1}: expected a component header, got {lines[i]!r}")
                    i += 1
                    if mc.group(3) == "grid based":
                        comps.append(ElemComponent(mc.group(1), mc.group(2), grid=lines[i].strip()))
                        i += 1
                        continue
                    nn = int(lines[i].split("=")[1])
                    i += 1
                    cnodes = []
                    for _ in range(nn):
                        local = int(lines[i].split(".")[0])
                        vidx = [int(t) for t in lines[i + 1].split(":")[1].split()]
                        stext = lines[i + 2].split(":", 1)[1][1:]  # after "Scale factor indices: "
                        scaled = stext != " 0" * len(vidx)
                        sidx = [int(t) for t in stext.split()] if scaled else None
                        cnodes.append((local, vidx, sidx))
                        i += 3
                    comps.append(ElemComponent(mc.group(1), mc.group(2), nodes=cnodes))
                fields.append(ElemField(m.group(2), m.group(3), comps))
            sections.append(ElemSection(ElemHeader(shape, sets, n_nodes, fields)))
        elif ln.startswith(" Element:"):
            if not sections:
                raise ExFormatError(f"line {i + 1}: element before any header")
            e = Element(int(ln.split(":")[1].split()[0]), [], [], [])
            i += 1
            while i < n and lines[i].strip() in ("Values:", "Nodes:", "Scale factors:"):
                tag = lines[i].strip()
                i += 1
                rows = []
                while i < n and _is_number_row(lines[i]):
                    rows.append(lines[i])
                    i += 1
                if tag == "Values:":
                    e.values = [_floats(r) for r in rows]
                elif tag == "Nodes:":
                    e.nodes = [int(t) for r in rows for t in r.split()]
                else:
                    e.scale_factors = [_floats(r) for r in rows]
            sections[-1].elements.append(e)
        elif ln.strip() == "":
            i += 1
        else:
            raise ExFormatError(f"line {i + 1}: unexpected {ln!r}")
    return ExElem(group, sections)


def read_exnode(path) -> ExNode:
    return parse_exnode(Path(path).read_text())


def read_exelem(path) -> ExElem:
    return parse_exelem(Path(path).read_text())


def node_values(ex: ExNode, field_name: str, component: int = 0, derivative: int = 0) -> dict[int, float]:
    """{node number: value} of one component (0-based) and derivative slot of a field, over all
    sections that carry the field."""
    out = {}
    for sec in ex.sections:
        for fi, f in enumerate(sec.fields):
            if f.name != field_name or component >= len(f.components):
                continue
            # component lines are written in field order, one line per component
            line = sum(len(g.components) for g in sec.fields[:fi]) + component
            for number, comps in sec.nodes:
                out[number] = comps[line][derivative]
    return out


# ------------------------------------------------------------------------------------------------
# builders for this package's meshes
# ------------------------------------------------------------------------------------------------

_XYZ = ("x", "y", "z")
_LIN3 = "l.Lagrange*l.Lagrange*l.Lagrange"
_QUAD3 = "q.Lagrange*q.Lagrange*q.Lagrange"


def _geometry_node_field(first_index: int = 1) -> NodeField:
    return NodeField("Geometry", "coordinate, rectangular cartesian",
                     [NodeComponent(_XYZ[c], first_index + c) for c in range(3)])


def _node_based(name: str, basis: str, locals_: list[int]) -> ElemComponent:
    return ElemComponent(name, basis, nodes=[(k, [1], None) for k in locals_])


def laplace_exfiles(coords: np.ndarray, elem_nodes: np.ndarray, u: np.ndarray, group: str = "LaplaceEquation",
                    name: str = "Phi") -> tuple[ExNode, ExElem]:
    """Trilinear mesh (coords [3][N], elem_nodes [E][8] 0-based, Iron's local node order) with the
    nodal solution u [N] as Iron exports a Laplace problem: Geometry (x, y, z) and the dependent
    field, node based, one l.Lagrange scale-factor set of unit factors per element."""
    coords = np.asarray(coords, dtype=np.float64)
    u = np.asarray(u, dtype=np.float64)
    sec = NodeSection([_geometry_node_field(), NodeField(name, "field,  real", [NodeComponent("1", 4)])])
    for k in range(coords.shape[1]):
        sec.nodes.append((k + 1, [[coords[0, k]], [coords[1, k]], [coords[2, k]], [u[k]]]))
    locals8 = list(range(1, 9))
    hdr = ElemHeader("Dimension=3", [(_LIN3, 8)], 8, [
        ElemField("Geometry", "coordinate, rectangular cartesian", [_node_based(c, _LIN3, locals8) for c in _XYZ]),
        ElemField(name, "field,  real", [_node_based("1", _LIN3, locals8)]),
    ])
    esec = ElemSection(hdr)
    for e, nd in enumerate(np.asarray(elem_nodes)):
        esec.elements.append(Element(e + 1, [], [int(v) + 1 for v in nd], [[1.0] * 8]))
    return ExNode(group, [sec]), ExElem(group, [esec])


_CORNERS27 = [1, 3, 7, 9, 19, 21, 25, 27]  # xi1 fastest: the 8 vertices of the 3x3x3 node grid


def mr_exfiles(xg: np.ndarray, eq2: np.ndarray, elin: np.ndarray, dep: np.ndarray,
               group: str = "FiniteElasticity") -> tuple[ExNode, ExElem]:
    """Triquadratic geometry xg [3][n_q2] with the mixed dependent field of the Mooney-Rivlin
    problem (deformed positions on the n_q2 quadratic nodes, pressure on the n_lin linear nodes;
    dep in Iron's separated order) and elements eq2 [E][27], elin [E][8] (0-based; linear node j
    of an element sits at its j-th corner).  Nodes with a pressure value form a second
    node-header section (4 dependent components), the others carry 3; in the elements the
    pressure component is trilinear over the 8 corner nodes of the 27."""
    xg = np.asarray(xg, dtype=np.float64)
    n_q2 = xg.shape[1]
    eq2, elin = np.asarray(eq2), np.asarray(elin)
    dep = np.asarray(dep, dtype=np.float64)
    z = dep[: 3 * n_q2].reshape(3, n_q2)
    p = dep[3 * n_q2:]
    p_at = np.full(n_q2, np.nan)
    corner_q2 = eq2[:, [k - 1 for k in _CORNERS27]]
    p_at[corner_q2.ravel()] = p[elin.ravel()]
    dep3 = NodeField("Dependent", "field,  rectangular cartesian", [NodeComponent(str(c + 1), 4 + c) for c in range(3)])
    dep4 = NodeField("Dependent", "field,  rectangular cartesian", [NodeComponent(str(c + 1), 4 + c) for c in range(4)])
    s3, s4 = NodeSection([_geometry_node_field(), dep3]), NodeSection([_geometry_node_field(), dep4])
    for k in range(n_q2):
        vals = [[xg[0, k]], [xg[1, k]], [xg[2, k]], [z[0, k]], [z[1, k]], [z[2, k]]]
        if np.isnan(p_at[k]):
            s3.nodes.append((k + 1, vals))
        else:
            s4.nodes.append((k + 1, vals + [[p_at[k]]]))
    locals27 = list(range(1, 28))
    corners = _CORNERS27
    hdr = ElemHeader("Dimension=3", [(_QUAD3, 27), (_LIN3, 8)], 27, [
        ElemField("Geometry", "coordinate, rectangular cartesian", [_node_based(c, _QUAD3, locals27) for c in _XYZ]),
        ElemField("Dependent", "field,  rectangular cartesian",
                  [_node_based(str(c + 1), _QUAD3, locals27) for c in range(3)] + [_node_based("4", _LIN3, corners)]),
    ])
    esec = ElemSection(hdr)
    for e, nd in enumerate(np.asarray(eq2)):
        esec.elements.append(Element(e + 1, [], [int(v) + 1 for v in nd], [[1.0] * 27, [1.0] * 8]))
    return ExNode(group, [s for s in (s3, s4) if s.nodes]), ExElem(group, [esec])
