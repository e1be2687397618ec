"""Regular generated hexahedral meshes with Iron's numbering, plus the element colouring the
deterministic scatter needs.

Numbering follows Iron's generated regular mesh (src/generated_mesh_routines.F90:1568-1640):
nodes are numbered xi1 fastest over the grid of the first basis; elements are numbered xi1
fastest; the element's local nodes are xi1 fastest.  A second, linear mesh component of a
quadratic mesh takes the corner nodes of each quadratic element
(src/generated_mesh_routines.F90:4941-5100) and numbers its own nodes by ascending global node
number (src/mesh_routines.F90:9159-9272).  Geometry: origin + index * extent / (nodes_xi - 1)
(src/generated_mesh_routines.F90:3217-3383).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


def _grid_nodes(nelem, order):
    return [order * n + 1 for n in nelem]


def regular_elements(nelem, order: int) -> np.ndarray:
    """elem_nodes[E][(order+1)^3] (0-based) of a 3D regular mesh of Lagrange order 1, 2 or 3."""
    nx, ny, nz = nelem
    tx, ty, _ = _grid_nodes(nelem, order)
    e1, e2, e3 = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    # element numbering xi1 fastest -> flatten with e1 fastest
    e1 = e1.transpose(2, 1, 0).reshape(-1)
    e2 = e2.transpose(2, 1, 0).reshape(-1)
    e3 = e3.transpose(2, 1, 0).reshape(-1)
    first = e1 * order + e2 * order * tx + e3 * order * tx * ty
    a = np.arange(order + 1)
    a1, a2, a3 = np.meshgrid(a, a, a, indexing="ij")
    off = (a1 + a2 * tx + a3 * tx * ty).transpose(2, 1, 0).reshape(-1)  # local nodes xi1 fastest
    return (first[:, None] + off[None, :]).astype(np.int32)


def regular_coords(nelem, order: int, origin=(0.0, 0.0, 0.0), extent=(1.0, 1.0, 1.0)) -> np.ndarray:
    """coords[3][N] in separated component order."""
    tx, ty, tz = _grid_nodes(nelem, order)
    i = np.arange(tx, dtype=np.float64)
    j = np.arange(ty, dtype=np.float64)
    k = np.arange(tz, dtype=np.float64)
    out = np.empty((3, tx * ty * tz))
    K, J, I = np.meshgrid(k, j, i, indexing="ij")
    out[0] = (origin[0] + I * (extent[0] / (tx - 1))).reshape(-1)
    out[1] = (origin[1] + J * (extent[1] / (ty - 1))).reshape(-1)
    out[2] = (origin[2] + K * (extent[2] / (tz - 1))).reshape(-1)
    return out


def linear_component(elem_first: np.ndarray, order_first: int):
    """Corner (trilinear) component of a higher-order mesh.

    Returns (elem_lin[E][8] in component-local numbers, lin_to_global[n_lin])."""
    n = order_first
    corners = [a1 + (n + 1) * (a2 + (n + 1) * a3) for a3 in (0, n) for a2 in (0, n) for a1 in (0, n)]
    c = elem_first[:, corners]
    glob, inv = np.unique(c.reshape(-1), return_inverse=True)
    return inv.reshape(c.shape).astype(np.int32), glob.astype(np.int32)


def boundary_node_mask(nelem, order: int) -> np.ndarray:
    tx, ty, tz = _grid_nodes(nelem, order)
    K, J, I = np.meshgrid(np.arange(tz), np.arange(ty), np.arange(tx), indexing="ij")
    b = (I == 0) | (I == tx - 1) | (J == 0) | (J == ty - 1) | (K == 0) | (K == tz - 1)
    return b.reshape(-1)


def parity_colouring(nelem):
    """8-colour element colouring of a regular hex mesh: colour = parity of (e1, e2, e3).

    Elements of one colour share no node.  Returns (colour_elems[E], colour_ptr[9])."""
    nx, ny, nz = nelem
    e = np.arange(nx * ny * nz)
    e1, e2, e3 = e % nx, (e // nx) % ny, e // (nx * ny)
    col = (e1 & 1) + 2 * (e2 & 1) + 4 * (e3 & 1)
    order = np.argsort(col, kind="stable").astype(np.int32)
    ptr = np.zeros(9, np.int32)
    np.cumsum(np.bincount(col, minlength=8), out=ptr[1:])
    return order, ptr


def greedy_colouring(elem_nodes: np.ndarray, n_nodes: int, max_colours: int = 64):
    """Greedy element colouring for an arbitrary mesh (elements in order, lowest free colour).

    Elements of one colour share no node.  Returns (colour_elems, colour_ptr)."""
    used = np.zeros(n_nodes, np.uint64)
    E = elem_nodes.shape[0]
    col = np.empty(E, np.int64)
    for e in range(E):
        nodes = elem_nodes[e]
        mask = np.bitwise_or.reduce(used[nodes])
        c = 0
        while (int(mask) >> c) & 1:
            c += 1
        if c >= max_colours:
            raise ValueError("mesh needs more than 64 colours")
        col[e] = c
        used[nodes] |= np.uint64(1 << c)
    nc = int(col.max()) + 1 if E else 1
    order = np.argsort(col, kind="stable").astype(np.int32)
    ptr = np.zeros(nc + 1, np.int32)
    np.cumsum(np.bincount(col, minlength=nc), out=ptr[1:])
    return order, ptr


@dataclass
class RegularMesh:
    """A generated regular hex mesh on a box (Iron's GENERATED_MESH_REGULAR_TYPE)."""

    nelem: tuple
    order: int = 1
    origin: tuple = (0.0, 0.0, 0.0)
    extent: tuple = (1.0, 1.0, 1.0)
    elem_nodes: np.ndarray = field(init=False)
    coords: np.ndarray = field(init=False)

    def __post_init__(self):
        self.nelem = tuple(int(n) for n in self.nelem)
        self.elem_nodes = regular_elements(self.nelem, self.order)
        self.coords = regular_coords(self.nelem, self.order, self.origin, self.extent)

    @property
    def n_elements(self) -> int:
        return int(np.prod(self.nelem))

    @property
    def n_nodes(self) -> int:
        return self.coords.shape[1]

    @property
    def nodes_xi(self):
        return _grid_nodes(self.nelem, self.order)

    def h(self):
        return np.array(self.extent, dtype=np.float64) / np.array(self.nelem)

    def jitter_interior(self, seed: int, fraction: float = 0.1) -> None:
        """Move every interior node uniformly within +-fraction*h per coordinate (seeded)."""
        rng = np.random.default_rng(seed)
        hh = self.h() / self.order if self.order > 1 else self.h()
        d = rng.uniform(-1.0, 1.0, size=self.coords.shape) * (fraction * hh)[:, None]
        d[:, boundary_node_mask(self.nelem, self.order)] = 0.0
        self.coords = self.coords + d

    def colouring(self):
        return parity_colouring(self.nelem)

    def node_index(self, i, j, k):
        tx, ty, _ = self.nodes_xi
        return i + tx * (j + ty * k)

    def face_nodes(self, axis: int, side: int) -> np.ndarray:
        """Nodes on the face axis = 0 (side 0) or axis = max (side 1)."""
        tx, ty, tz = self.nodes_xi
        K, J, I = np.meshgrid(np.arange(tz), np.arange(ty), np.arange(tx), indexing="ij")
        idx = (I, J, K)[axis]
        lim = (tx, ty, tz)[axis] - 1
        return np.nonzero((idx == (0 if side == 0 else lim)).reshape(-1))[0].astype(np.int64)


@dataclass
class HermiteMesh:
    """Iron's regular generated mesh of tricubic Hermite hexahedra on a box: 8 parameters per node
    (value, d/ds1, d/ds2, d2/ds1ds2, d/ds3, d2/ds1ds3, d2/ds2ds3, d3/ds1ds2ds3), DOF = 8 node + k,
    nodes and elements numbered xi1 fastest.

    scaling "unit": derivative parameters are derivatives with respect to xi, no scale factors.
    scaling "arc_length": derivative parameters are with respect to arc length, and each element
    carries scale factors h1^d1 h2^d2 h3^d3 for the parameter with derivative bits (d1, d2, d3),
    as Iron's arc-length scaling stores them.
    elem_params [E][64], params [3][8N] (geometric parameters per DOF), scale [E][64] or None."""

    nelem: tuple
    extent: tuple = (1.0, 1.0, 1.0)
    scaling: str = "unit"
    elem_params: np.ndarray = field(init=False)
    params: np.ndarray = field(init=False)
    scale: np.ndarray | None = field(init=False)

    def __post_init__(self):
        nx, ny, nz = self.nelem
        tx, ty, tz = nx + 1, ny + 1, nz + 1
        h = np.array(self.extent, dtype=np.float64) / np.array(self.nelem, dtype=np.float64)
        N = tx * ty * tz
        K, J, I = np.meshgrid(np.arange(tz), np.arange(ty), np.arange(tx), indexing="ij")
        pos = np.stack([I.reshape(-1) * h[0], J.reshape(-1) * h[1], K.reshape(-1) * h[2]])
        p = np.zeros((3, 8 * N))
        for c in range(3):
            p[c, 0::8] = pos[c]
            # d/ds_c of coordinate c: 1 per unit arc length, h_c per unit xi
            p[c, (1 << c)::8] = 1.0 if self.scaling == "arc_length" else h[c]
        self.params = p
        lin = regular_elements(self.nelem, 1)  # [E][8] local nodes xi1 fastest
        self.elem_params = (8 * lin[:, :, None] + np.arange(8)[None, None, :]).reshape(len(lin), 64).astype(np.int32)
        if self.scaling == "arc_length":
            k = np.arange(8)
            sf = h[0] ** (k & 1) * h[1] ** ((k >> 1) & 1) * h[2] ** ((k >> 2) & 1)
            self.scale = np.tile(np.tile(sf, 8), (len(lin), 1))
        elif self.scaling == "unit":
            self.scale = None
        else:
            raise ValueError(self.scaling)

    @property
    def n_nodes(self) -> int:
        return int(np.prod([n + 1 for n in self.nelem]))

    @property
    def n_dofs(self) -> int:
        return 8 * self.n_nodes

    @property
    def n_elements(self) -> int:
        return int(np.prod(self.nelem))

    def jitter_interior(self, seed: int, fraction: float = 0.05) -> None:
        """Move interior nodes and perturb their first and cross derivatives (seeded), so that
        elements are curved but keep a positive Jacobian."""
        rng = np.random.default_rng(seed)
        interior = ~boundary_node_mask(self.nelem, 1)
        h = np.array(self.extent) / np.array(self.nelem)
        for c in range(3):
            for k in range(8):
                d = self.params[c, k::8]
                scale = h[c] if k == 0 else (self.params[c, (1 << c)::8].max() if k in (1, 2, 4) else 0.2 * h[c])
                d[interior] += rng.uniform(-1, 1, interior.sum()) * fraction * scale

    def colouring(self):
        return parity_colouring(self.nelem)

    def face_dofs(self, axis: int, side: int) -> np.ndarray:
        """All parameter DOFs of the nodes on the face xi_axis = side (0 or 1)."""
        tx, ty, tz = [n + 1 for n in self.nelem]
        K, J, I = np.meshgrid(np.arange(tz), np.arange(ty), np.arange(tx), indexing="ij")
        idx = (I, J, K)[axis].reshape(-1)
        nodes = np.flatnonzero(idx == (0 if side == 0 else (tx, ty, tz)[axis] - 1))
        return (8 * nodes[:, None] + np.arange(8)[None, :]).reshape(-1)


# Iron's cubic-simplex node position indices per area coordinate (1..4), local nodes 1..20
CUBIC_TET_POSITIONS = [(4, 1, 1, 1), (1, 4, 1, 1), (1, 1, 4, 1), (1, 1, 1, 4), (3, 2, 1, 1), (2, 3, 1, 1),
                       (3, 1, 2, 1), (2, 1, 3, 1), (3, 1, 1, 2), (2, 1, 1, 3), (1, 3, 2, 1), (1, 2, 3, 1),
                       (1, 1, 3, 2), (1, 1, 2, 3), (1, 3, 1, 2), (1, 2, 1, 3), (2, 2, 2, 1), (2, 2, 1, 2),
                       (2, 1, 2, 2), (1, 2, 2, 2)]


@dataclass
class TetMesh:
    """Tetrahedral mesh of a box: every cell of a regular grid split into six tetrahedra along its
    main diagonal (conforming across cells), order 1 (4 vertices), 2 (plus 6 edge nodes in
    Iron's quadratic-simplex order: edges 1-2, 1-3, 1-4, 2-3, 3-4, 2-4) or 3 (Iron's 20-node cubic
    simplex: vertices, two nodes on each edge, one on each face, in the order of the node
    position indices of src/basis_routines.F90:5236-5353).  coords [3][N], elem_nodes
    [E][4, 10 or 20] (0-based); vertices are nodes 0..n_vertices-1."""

    nelem: tuple
    order: int = 1
    extent: tuple = (1.0, 1.0, 1.0)
    elem_nodes: np.ndarray = field(init=False)
    coords: np.ndarray = field(init=False)

    def __post_init__(self):
        nx, ny, nz = self.nelem
        tx, ty, tz = nx + 1, ny + 1, nz + 1
        vid = lambda i, j, k: i + tx * (j + ty * k)  # noqa: E731
        tets = []
        perms = [(0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)]
        for k in range(nz):
            for j in range(ny):
                for i in range(nx):
                    for p in perms:
                        cur = [i, j, k]
                        t = [vid(*cur)]
                        for d in p:
                            cur[d] += 1
                            t.append(vid(*cur))
                        tets.append(t)
        tets = np.array(tets, dtype=np.int64)
        K, J, I = np.meshgrid(np.arange(tz), np.arange(ty), np.arange(tx), indexing="ij")
        h = np.array(self.extent) / np.array(self.nelem)
        verts = np.stack([I.reshape(-1) * h[0], J.reshape(-1) * h[1], K.reshape(-1) * h[2]])
        self.n_vertices = verts.shape[1]
        if self.order == 1:
            self.elem_nodes, self.coords = tets.astype(np.int32), verts
        elif self.order == 2:
            pairs = [(0, 1), (0, 2), (0, 3), (1, 2), (2, 3), (1, 3)]
            e = np.stack([np.sort(tets[:, [a, b]], axis=1) for a, b in pairs], axis=1)  # [E][6][2]
            uniq, inv = np.unique(e.reshape(-1, 2), axis=0, return_inverse=True)
            mid = (verts[:, uniq[:, 0]] + verts[:, uniq[:, 1]]) / 2.0
            self.coords = np.concatenate([verts, mid], axis=1)
            self.elem_nodes = np.concatenate([tets, self.n_vertices + inv.reshape(-1, 6)], axis=1).astype(np.int32)
            self.edges = uniq
        elif self.order == 3:
            # a node is the point sum_i (p_i - 1)/3 V_i of its position indices p_i: keyed by the
            # (vertex, weight) pairs with non-zero weight, so neighbouring elements share it
            pos = np.array(CUBIC_TET_POSITIONS) - 1  # [20][4] weights in thirds
            E = tets.shape[0]
            vid4 = np.broadcast_to(tets[:, None, :], (E, 20, 4))
            wt = np.broadcast_to(pos[None, :, :], (E, 20, 4))
            key_v = np.where(wt > 0, vid4, -1)
            order = np.argsort(key_v, axis=2, kind="stable")
            kv = np.take_along_axis(key_v, order, axis=2)
            kw = np.take_along_axis(np.where(wt > 0, wt, 0), order, axis=2)
            keys = np.concatenate([kv, kw], axis=2).reshape(-1, 8)
            higher = (pos.max(axis=1) < 3)[None, :].repeat(E, axis=0).reshape(-1)
            uniq, inv = np.unique(keys[higher], axis=0, return_inverse=True)
            nodes = np.empty(E * 20, dtype=np.int64)
            nodes[~higher] = tets[:, pos.argmax(axis=1)[pos.max(axis=1) == 3]].reshape(-1)
            nodes[higher] = self.n_vertices + inv.reshape(-1)
            self.elem_nodes = nodes.reshape(E, 20).astype(np.int32)
            self.node_vertices = uniq[:, :4]
            self.node_weights = uniq[:, 4:] / 3.0
            self.coords = np.concatenate([verts, self._higher_coords(verts)], axis=1)
        else:
            raise ValueError("tetrahedra of order 1, 2 or 3")

    def _higher_coords(self, verts):
        """Coordinates of the cubic edge and face nodes from their vertices and weights."""
        out = np.zeros((3, self.node_vertices.shape[0]))
        for k in range(4):
            v = self.node_vertices[:, k]
            on = v >= 0
            out[:, on] += self.node_weights[on, k] * verts[:, v[on]]
        return out

    @property
    def n_nodes(self) -> int:
        return self.coords.shape[1]

    @property
    def n_elements(self) -> int:
        return self.elem_nodes.shape[0]

    def boundary_mask(self) -> np.ndarray:
        x = self.coords
        ext = np.array(self.extent)[:, None]
        return np.any(np.isclose(x, 0.0) | np.isclose(x, ext), axis=0)

    def jitter_interior(self, seed: int, fraction: float = 0.1) -> None:
        """Move interior vertices (seeded) and keep edge nodes at their edges' midpoints, so that
        elements stay straight-sided."""
        rng = np.random.default_rng(seed)
        h = np.array(self.extent) / np.array(self.nelem)
        interior = ~self.boundary_mask()[: self.n_vertices]
        d = rng.uniform(-1, 1, (3, self.n_vertices)) * (fraction * h)[:, None]
        d[:, ~interior] = 0.0
        self.coords[:, : self.n_vertices] += d
        if self.order == 2:
            self.coords[:, self.n_vertices:] = (self.coords[:, self.edges[:, 0]] + self.coords[:, self.edges[:, 1]]) / 2
        elif self.order == 3:
            self.coords[:, self.n_vertices:] = self._higher_coords(self.coords[:, : self.n_vertices])

    def face_nodes(self, axis: int, side: int) -> np.ndarray:
        target = 0.0 if side == 0 else self.extent[axis]
        return np.flatnonzero(np.isclose(self.coords[axis], target))
