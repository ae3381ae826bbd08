"""Mesh files in and results out, without meshio: Gmsh MSH 2.2 / 4.1 (ASCII) and legacy VTK.

AutoPDEx's examples read their meshes through pygmsh/meshio and use two things of the
result: ``mesh.points`` (n x 3, sliced to the space dimension) and ``mesh.cells_dict``
(element name -> connectivity), e.g. examples/cooks_membrane/quadrilaterals_autopdex_and_acegen.py:62-65
and examples/heat_conduction/maze_backward_euler.py:293-294; they write results with
``meshio.Mesh(points, cells, point_data=...).write(...)``.  ``read`` returns an object with
those attributes (meshio's element names, node ordering as in the file, which for Gmsh is
the ordering pygmsh/meshio hand to AutoPDEx); ``write_vtk`` writes a legacy ASCII file that
ParaView and meshio open.

Both set-up steps run once per mesh on the host; the connectivity then goes to
``settings['connectivity']`` as for any other mesh (the general, unstructured pattern path).
"""
import numpy as np

# Gmsh element type -> (meshio name, nodes per element)
GMSH_TYPES = {
    1: ("line", 2), 2: ("triangle", 3), 3: ("quad", 4), 4: ("tetra", 4), 5: ("hexahedron", 8),
    6: ("wedge", 6), 7: ("pyramid", 5), 8: ("line3", 3), 9: ("triangle6", 6), 10: ("quad9", 9),
    11: ("tetra10", 10), 12: ("hexahedron27", 27), 15: ("vertex", 1), 16: ("quad8", 8),
    17: ("hexahedron20", 20),
}
# VTK cell type <-> meshio name
VTK_TYPES = {
    1: "vertex", 3: "line", 5: "triangle", 9: "quad", 10: "tetra", 12: "hexahedron", 13: "wedge",
    14: "pyramid", 21: "line3", 22: "triangle6", 23: "quad8", 24: "tetra10", 25: "hexahedron20",
    28: "quad9", 29: "hexahedron27",
}
VTK_IDS = {v: k for k, v in VTK_TYPES.items()}


class Mesh:
    """Points, cells by element name and per-cell data, in meshio's layout.

    ``cells_dict[name]`` is an int64 (n_cells, nodes) array of 0-based point indices (all
    blocks of one element type concatenated in file order); ``cell_data_dict[key][name]``
    the matching per-cell values ('gmsh:physical', 'gmsh:geometrical' for Gmsh files);
    ``point_data`` per-point arrays (VTK files)."""

    def __init__(self, points, cells, cell_data=None, point_data=None, field_data=None):
        self.points = np.asarray(points, dtype=np.float64)
        self.cells = [(name, np.asarray(c, dtype=np.int64)) for name, c in cells]
        self.cell_data = cell_data or {}
        self.point_data = point_data or {}
        self.field_data = field_data or {}

    @property
    def cells_dict(self):
        out = {}
        for name, c in self.cells:
            out.setdefault(name, []).append(c)
        return {k: np.concatenate(v) if len(v) > 1 else v[0] for k, v in out.items()}

    @property
    def cell_data_dict(self):
        out = {}
        for key, blocks in self.cell_data.items():
            per = {}
            for (name, _), vals in zip(self.cells, blocks):
                per.setdefault(name, []).append(np.asarray(vals))
            out[key] = {k: np.concatenate(v) if len(v) > 1 else v[0] for k, v in per.items()}
        return out


def read(path):
    """Read a Gmsh ``.msh`` (format 2.2 or 4.1, ASCII) or legacy ``.vtk`` (ASCII) file."""
    with open(path, "rb") as fh:
        head = fh.read(64)
    if head.startswith(b"$MeshFormat"):
        return _read_gmsh(path)
    if head.lstrip().startswith(b"# vtk DataFile"):
        return _read_vtk(path)
    raise ValueError(f"{path}: neither a Gmsh MSH nor a legacy VTK file")


# ---- Gmsh ---------------------------------------------------------------------------------
def _sections(lines):
    """{name: [lines between $name and $Endname]} (the last of repeated sections)."""
    out, i = {}, 0
    while i < len(lines):
        ln = lines[i].strip()
        if ln.startswith("$") and not ln.startswith("$End"):
            name = ln[1:]
            j = i + 1
            while j < len(lines) and lines[j].strip() != "$End" + name:
                j += 1
            out[name] = lines[i + 1:j]
            i = j + 1
        else:
            i += 1
    return out


def _read_gmsh(path):
    with open(path, "r", errors="replace") as fh:
        lines = fh.read().splitlines()
    sec = _sections(lines)
    version, ftype = sec["MeshFormat"][0].split()[:2]
    if ftype != "0":
        raise NotImplementedError("binary Gmsh files are not supported: save the mesh as ASCII")
    field = {}
    for ln in sec.get("PhysicalNames", [])[1:]:
        dim, tag, name = ln.split(maxsplit=2)
        field[name.strip().strip('"')] = np.array([int(tag), int(dim)])
    if version.startswith("2"):
        return _gmsh2(sec, field)
    if version.startswith("4"):
        return _gmsh4(sec, field)
    raise NotImplementedError(f"Gmsh format {version} is not supported (2.2 and 4.1 are)")


def _index_map(tags):
    m = np.full(int(tags.max()) + 1, -1, dtype=np.int64)
    m[tags] = np.arange(tags.size)
    return m


def _group(types, conns, phys, geom):
    """Consecutive elements of one type become one cell block (meshio's blocks)."""
    cells, cphys, cgeom = [], [], []
    start = 0
    for k in range(1, len(types) + 1):
        if k == len(types) or types[k] != types[start]:
            name, nn = GMSH_TYPES[types[start]]
            cells.append((name, np.array(conns[start:k], dtype=np.int64).reshape(-1, nn)))
            cphys.append(np.array(phys[start:k], dtype=np.int64))
            cgeom.append(np.array(geom[start:k], dtype=np.int64))
            start = k
    return cells, {"gmsh:physical": cphys, "gmsh:geometrical": cgeom}


def _gmsh2(sec, field):
    nl = sec["Nodes"]
    n = int(nl[0])
    raw = np.array(" ".join(nl[1:n + 1]).split(), dtype=np.float64).reshape(n, 4)
    tags = raw[:, 0].astype(np.int64)
    points = raw[:, 1:4]
    imap = _index_map(tags)
    el = sec["Elements"]
    m = int(el[0])
    types, conns, phys, geom = [], [], [], []
    for ln in el[1:m + 1]:
        v = [int(t) for t in ln.split()]
        et, ntag = v[1], v[2]
        if et not in GMSH_TYPES:
            raise NotImplementedError(f"Gmsh element type {et} is not supported")
        nn = GMSH_TYPES[et][1]
        nodes = v[3 + ntag:3 + ntag + nn]
        types.append(et)
        conns.append(imap[np.array(nodes)])
        phys.append(v[3] if ntag > 0 else 0)
        geom.append(v[4] if ntag > 1 else 0)
    cells, cdata = _group(types, conns, phys, geom)
    return Mesh(points, cells, cdata, field_data=field)


def _gmsh4(sec, field):
    # physical tag of every entity (dimension, tag) from $Entities
    ent_phys = {}
    if "Entities" in sec:
        tok = " ".join(sec["Entities"]).split()
        counts = [int(t) for t in tok[:4]]
        pos = 4
        for dim, cnt in enumerate(counts):
            for _ in range(cnt):
                tag = int(tok[pos])
                pos += 4 if dim == 0 else 7  # tag + x y z, or tag + bounding box
                nphys = int(tok[pos])
                ph = [int(t) for t in tok[pos + 1:pos + 1 + nphys]]
                pos += 1 + nphys
                if dim > 0:
                    pos += 1 + int(tok[pos])  # bounding entities
                ent_phys[(dim, tag)] = ph[0] if ph else 0
    tok = " ".join(sec["Nodes"]).split()
    nblocks, nnodes = int(tok[0]), int(tok[1])
    pos = 4
    tags = np.empty(nnodes, dtype=np.int64)
    points = np.empty((nnodes, 3))
    k = 0
    for _ in range(nblocks):
        parametric, nin = int(tok[pos + 2]), int(tok[pos + 3])
        if parametric:
            raise NotImplementedError("parametric node coordinates are not supported")
        pos += 4
        tags[k:k + nin] = np.array(tok[pos:pos + nin], dtype=np.int64)
        pos += nin
        points[k:k + nin] = np.array(tok[pos:pos + 3 * nin], dtype=np.float64).reshape(nin, 3)
        pos += 3 * nin
        k += nin
    imap = _index_map(tags)
    tok = " ".join(sec["Elements"]).split()
    nblocks = int(tok[0])
    pos = 4
    cells, cphys, cgeom = [], [], []
    for _ in range(nblocks):
        dim, etag, et, nin = (int(t) for t in tok[pos:pos + 4])
        pos += 4
        if et not in GMSH_TYPES:
            raise NotImplementedError(f"Gmsh element type {et} is not supported")
        name, nn = GMSH_TYPES[et]
        blk = np.array(tok[pos:pos + nin * (nn + 1)], dtype=np.int64).reshape(nin, nn + 1)
        pos += nin * (nn + 1)
        cells.append((name, imap[blk[:, 1:]]))
        cphys.append(np.full(nin, ent_phys.get((dim, etag), 0), dtype=np.int64))
        cgeom.append(np.full(nin, etag, dtype=np.int64))
    return Mesh(points, cells, {"gmsh:physical": cphys, "gmsh:geometrical": cgeom}, field_data=field)


# ---- legacy VTK ---------------------------------------------------------------------------
def _read_vtk(path):
    with open(path, "r", errors="replace") as fh:
        lines = fh.read().splitlines()
    if lines[2].strip().upper() != "ASCII":
        raise NotImplementedError("binary VTK files are not supported: write them as ASCII")
    if "UNSTRUCTURED_GRID" not in lines[3].upper():
        raise NotImplementedError("only legacy VTK UNSTRUCTURED_GRID files are supported")
    tok = " ".join(lines[4:]).split()
    pos = 0
    points, cells_flat, offsets, conn, ctypes = None, None, None, None, None
    point_data, cell_data, mode, npts, ncells = {}, {}, None, 0, 0

    def take(k, dtype):
        nonlocal pos
        out = np.array(tok[pos:pos + k], dtype=dtype)
        pos += k
        return out

    while pos < len(tok):
        key = tok[pos].upper()
        if key == "POINTS":
            npts = int(tok[pos + 1])
            pos += 3
            points = take(3 * npts, np.float64).reshape(npts, 3)
        elif key == "CELLS":
            a, b = int(tok[pos + 1]), int(tok[pos + 2])
            pos += 3
            if pos < len(tok) and tok[pos].upper() == "OFFSETS":  # format 5.1
                pos += 2
                offsets = take(a, np.int64)
                pos += 2  # CONNECTIVITY <type>
                conn = take(b, np.int64)
                ncells = a - 1
            else:
                cells_flat = take(b, np.int64)
                ncells = a
        elif key == "CELL_TYPES":
            pos += 2
            ctypes = take(ncells, np.int64)
        elif key in ("POINT_DATA", "CELL_DATA"):
            mode = key
            pos += 2
        elif key in ("SCALARS", "VECTORS"):
            name = tok[pos + 1]
            if key == "SCALARS":
                ncomp = 1
                pos += 3
                if pos < len(tok) and tok[pos].lstrip("-").isdigit():
                    ncomp = int(tok[pos])
                    pos += 1
                if pos < len(tok) and tok[pos].upper() == "LOOKUP_TABLE":
                    pos += 2
            else:
                ncomp = 3
                pos += 3
            count = npts if mode == "POINT_DATA" else ncells
            arr = take(count * ncomp, np.float64)
            arr = arr.reshape(count, ncomp) if ncomp > 1 else arr
            (point_data if mode == "POINT_DATA" else cell_data)[name] = arr
        else:
            raise NotImplementedError(f"VTK section {tok[pos]} is not supported")
    if offsets is not None:
        groups = [conn[offsets[i]:offsets[i + 1]] for i in range(ncells)]
    else:
        groups, p = [], 0
        for _ in range(ncells):
            k = int(cells_flat[p])
            groups.append(cells_flat[p + 1:p + 1 + k])
            p += 1 + k
    cells, start = [], 0
    for k in range(1, ncells + 1):
        if k == ncells or ctypes[k] != ctypes[start]:
            if int(ctypes[start]) not in VTK_TYPES:
                raise NotImplementedError(f"VTK cell type {int(ctypes[start])} is not supported")
            cells.append((VTK_TYPES[int(ctypes[start])], np.array(groups[start:k], dtype=np.int64)))
            start = k
    cdata = {}
    for name, arr in cell_data.items():
        blocks, s = [], 0
        for _, c in cells:
            blocks.append(arr[s:s + len(c)])
            s += len(c)
        cdata[name] = blocks
    return Mesh(points, cells, cdata, point_data)


def write_vtk(path, points, cells, point_data=None, cell_data=None, title="autopdex_gb300"):
    """Legacy ASCII VTK (version 4.2) of an unstructured grid.

    ``cells``: a dict {meshio name: connectivity} or a list of (name, connectivity);
    ``point_data`` / ``cell_data``: {name: array with one row per point / cell} (numbers or
    vectors of 1-3 components; 2-component vectors are padded with a zero z)."""
    pts = np.asarray(points, dtype=np.float64)
    if pts.shape[1] < 3:
        pts = np.hstack([pts, np.zeros((pts.shape[0], 3 - pts.shape[1]))])
    blocks = list(cells.items()) if isinstance(cells, dict) else list(cells)
    blocks = [(name, np.asarray(c, dtype=np.int64)) for name, c in blocks]
    ncell = sum(len(c) for _, c in blocks)
    size = sum(c.size + len(c) for _, c in blocks)
    out = [f"# vtk DataFile Version 4.2", title, "ASCII", "DATASET UNSTRUCTURED_GRID",
           f"POINTS {len(pts)} double"]
    out += [" ".join(repr(float(v)) for v in row) for row in pts]
    out.append(f"CELLS {ncell} {size}")
    for _, c in blocks:
        out += [f"{c.shape[1]} " + " ".join(str(int(i)) for i in row) for row in c]
    out.append(f"CELL_TYPES {ncell}")
    for name, c in blocks:
        if name not in VTK_IDS:
            raise NotImplementedError(f"element {name} has no VTK cell type")
        out += [str(VTK_IDS[name])] * len(c)

    def data(kind, count, arrays):
        if not arrays:
            return
        out.append(f"{kind} {count}")
        for name, a in arrays.items():
            a = np.asarray(a, dtype=np.float64)
            if a.ndim == 1 or a.shape[1] == 1:
                out.append(f"SCALARS {name} double 1")
                out.append("LOOKUP_TABLE default")
                out.extend(repr(float(v)) for v in a.reshape(-1))
            else:
                if a.shape[1] == 2:
                    a = np.hstack([a, np.zeros((a.shape[0], 1))])
                out.append(f"VECTORS {name} double")
                out.extend(" ".join(repr(float(v)) for v in row) for row in a)

    data("POINT_DATA", len(pts), point_data)
    data("CELL_DATA", ncell, cell_data)
    with open(path, "w") as fh:
        fh.write("\n".join(out) + "\n")


def write_gmsh(path, points, cells):
    """Gmsh MSH 4.1 ASCII: all points in one node block (tags 1..n), one element block per
    entry of ``cells`` ({meshio name: connectivity} or a list of (name, connectivity)), each
    on its own entity of the element's dimension, without physical groups."""
    pts = np.asarray(points, dtype=np.float64)
    if pts.shape[1] < 3:
        pts = np.hstack([pts, np.zeros((pts.shape[0], 3 - pts.shape[1]))])
    blocks = list(cells.items()) if isinstance(cells, dict) else list(cells)
    gid = {name: t for t, (name, _) in GMSH_TYPES.items()}
    dims = {"vertex": 0, "line": 1, "line3": 1, "triangle": 2, "triangle6": 2, "quad": 2, "quad8": 2, "quad9": 2}
    n = len(pts)
    ne = sum(len(c) for _, c in blocks)
    out = ["$MeshFormat", "4.1 0 8", "$EndMeshFormat", "$Nodes", f"1 {n} 1 {n}", f"2 1 0 {n}"]
    out += [str(i + 1) for i in range(n)]
    out += [" ".join(repr(float(v)) for v in row) for row in pts]
    out += ["$EndNodes", "$Elements", f"{len(blocks)} {ne} 1 {ne}"]
    tag = 1
    for k, (name, c) in enumerate(blocks):
        c = np.asarray(c, dtype=np.int64)
        out.append(f"{dims.get(name, 3)} {k + 1} {gid[name]} {len(c)}")
        for row in c:
            out.append(f"{tag} " + " ".join(str(int(i) + 1) for i in row))
            tag += 1
    out.append("$EndElements")
    with open(path, "w") as fh:
        fh.write("\n".join(out) + "\n")
