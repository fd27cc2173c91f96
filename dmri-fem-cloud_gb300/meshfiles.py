"""Mesh input: the file formats the reference's meshes come in.

* gmsh ``.msh`` (ASCII 2.2 — the format of the meshes shipped with the
  reference, ``comri/meshes/*.msh.zip`` — and ASCII 4.1), plain or zipped.  The
  cell marker of a tetrahedron is its first tag (the physical group), as
  ``GetPartitionMarkers`` (``DmriFemLib.py:689-752``) extracts it; the
  reference then takes ``phase = marker % 2`` (``CreatePhaseFunc``,
  ``DmriFemLib.py:754-764``).
* DOLFIN ``.xml`` meshes (``Mesh("file.xml")``, what ``dolfin-convert`` writes,
  ``PreprocessingMultiCompt.py:52-57``), with cell markers from a ``<domains>``
  mesh value collection when present, and DOLFIN ``.xml`` mesh functions (the
  ``pmk_*.xml`` partition-marker files ``GetPartitionMarkers`` writes).
* Compartments given as sub-meshes (``CreatePhaseFunc`` with ``evengroup`` /
  ``oddgroup``, ``DmriFemLib.py:765-798``): a cell belongs to sub-mesh i when its
  midpoint lies in one of that sub-mesh's tetrahedra; markers 2i+2 (even group,
  phase 0) and 2i+1 (odd group, phase 1), 0 elsewhere.

Everything returns 0-based ``int32`` tetrahedra and ``float64`` coordinates in
file order (``dolfin-convert`` keeps the node and element order), ready for
``bt_mesh_upload``.
"""

import io
import os
import xml.etree.ElementTree as ET
import zipfile

import numpy as np

GMSH_TET = 4          # gmsh element type of the 4-node tetrahedron


def _open_text(path):
    """Text stream of a file, or of the single matching member of a .zip."""
    if str(path).endswith(".zip"):
        z = zipfile.ZipFile(path)
        base = os.path.basename(str(path))[:-4]
        names = [n for n in z.namelist() if not n.startswith("__MACOSX")]
        name = base if base in names else names[0]
        return io.TextIOWrapper(z.open(name), encoding="utf-8", errors="replace")
    return open(path, "r", encoding="utf-8", errors="replace")


def _sections(stream):
    """Yield (name, lines) for every $Name ... $EndName section."""
    name, buf = None, []
    for line in stream:
        s = line.strip()
        if s.startswith("$"):
            if name is None:
                name, buf = s[1:], []
            elif s == "$End" + name:
                yield name, buf
                name = None
            else:
                raise ValueError("malformed .msh: %s inside $%s" % (s, name))
        elif name is not None:
            buf.append(s)
    if name is not None:
        raise ValueError("malformed .msh: $%s is not closed" % name)


def read_msh(path):
    """gmsh ASCII mesh (2.2 or 4.1, optionally zipped).

    Returns dict(xyz[n,3] f64, tets[m,4] i32, markers[m] i32 (physical tag, 0
    when the element has none), node_ids[n] (the file's node numbers)).
    Elements other than 4-node tetrahedra (boundary triangles, lines) are
    skipped; nodes that no tetrahedron uses are dropped."""
    with _open_text(path) as f:
        secs = dict(_sections(f))
    if "MeshFormat" not in secs:
        raise ValueError("%s: no $MeshFormat section" % path)
    fmt = secs["MeshFormat"][0].split()
    version, binary = fmt[0], int(fmt[1])
    if binary:
        raise ValueError("%s: binary .msh is not supported (save as ASCII)" % path)
    if version.startswith("2"):
        ids, xyz, tet_nodes, tags = _msh2(secs)
    elif version.startswith("4"):
        ids, xyz, tet_nodes, tags = _msh4(secs)
    else:
        raise ValueError("%s: .msh version %s is not supported" % (path, version))
    if len(tet_nodes) == 0:
        raise ValueError("%s: no tetrahedra" % path)
    # map node numbers to 0-based indices, keeping only used nodes (in file order)
    order = np.argsort(ids, kind="stable")
    pos = np.searchsorted(ids, tet_nodes, sorter=order)
    if np.any(pos >= len(ids)) or np.any(ids[order[np.minimum(pos, len(ids) - 1)]] != tet_nodes):
        raise ValueError("%s: a tetrahedron refers to a node that is not defined" % path)
    local = order[pos]
    used = np.zeros(len(ids), bool)
    used[local.ravel()] = True
    new_index = np.cumsum(used) - 1
    return {"xyz": np.ascontiguousarray(xyz[used]), "tets": new_index[local].astype(np.int32),
            "markers": np.asarray(tags, np.int32), "node_ids": ids[used]}


def _msh2(secs):
    nodes = secs["Nodes"]
    n = int(nodes[0])
    arr = np.array([ln.split() for ln in nodes[1:n + 1]], dtype=np.float64)
    ids = arr[:, 0].astype(np.int64)
    xyz = arr[:, 1:4]
    els = secs["Elements"]
    m = int(els[0])
    tets, tags = [], []
    for ln in els[1:m + 1]:
        p = ln.split()
        if int(p[1]) != GMSH_TET:
            continue
        nt = int(p[2])
        tags.append(int(p[3]) if nt > 0 else 0)
        tets.append([int(v) for v in p[3 + nt:7 + nt]])
    return ids, xyz, np.array(tets, np.int64).reshape(-1, 4), tags


def _msh4(secs):
    # physical tag of each volume entity ($Entities, 4.1 layout)
    phys = {}
    if "Entities" in secs:
        e = secs["Entities"]
        npt, ncu, nsu, nvo = (int(x) for x in e[0].split()[:4])
        for ln in e[1 + npt + ncu + nsu:1 + npt + ncu + nsu + nvo]:
            p = ln.split()
            tag = int(p[0])
            nph = int(p[7])
            phys[tag] = int(p[8]) if nph > 0 else 0
    nodes = secs["Nodes"]
    nblocks = int(nodes[0].split()[0])
    ids, xyz, i = [], [], 1
    for _ in range(nblocks):
        _, _, _, cnt = (int(x) for x in nodes[i].split())
        i += 1
        ids.extend(int(x) for x in nodes[i:i + cnt])
        xyz.extend([float(v) for v in ln.split()[:3]] for ln in nodes[i + cnt:i + 2 * cnt])
        i += 2 * cnt
    els = secs["Elements"]
    nblocks = int(els[0].split()[0])
    tets, tags, i = [], [], 1
    for _ in range(nblocks):
        edim, etag, etype, cnt = (int(x) for x in els[i].split())
        i += 1
        if etype == GMSH_TET:
            for ln in els[i:i + cnt]:
                p = ln.split()
                tets.append([int(v) for v in p[1:5]])
            tags.extend([phys.get(etag, 0)] * cnt)
        i += cnt
    return np.array(ids, np.int64), np.array(xyz, np.float64).reshape(-1, 3), \
        np.array(tets, np.int64).reshape(-1, 4), tags


def read_dolfin_xml(path):
    """DOLFIN XML mesh: dict(xyz, tets, markers or None).  Markers come from a
    dim-3 ``<mesh_value_collection>`` inside ``<domains>`` when the file has one."""
    with _open_text(path) as f:
        root = ET.parse(f).getroot()
    mesh = root.find("mesh")
    if mesh is None:
        raise ValueError("%s: no <mesh> element" % path)
    if mesh.get("celltype", "tetrahedron") != "tetrahedron":
        raise ValueError("%s: only tetrahedral meshes are supported" % path)
    verts = mesh.find("vertices")
    nv = int(verts.get("size"))
    xyz = np.zeros((nv, 3))
    for v in verts:
        xyz[int(v.get("index"))] = (float(v.get("x")), float(v.get("y", 0.0)), float(v.get("z", 0.0)))
    cells = mesh.find("cells")
    nc = int(cells.get("size"))
    tets = np.zeros((nc, 4), np.int32)
    for c in cells:
        tets[int(c.get("index"))] = (int(c.get("v0")), int(c.get("v1")), int(c.get("v2")), int(c.get("v3")))
    markers = None
    dom = mesh.find("domains")
    if dom is not None:
        for mvc in dom.findall("mesh_value_collection"):
            if int(mvc.get("dim", -1)) == 3:
                markers = _collection_values(mvc, nc)
    return {"xyz": xyz, "tets": tets, "markers": markers}


def _collection_values(mvc, n):
    out = np.zeros(n, np.int32)
    for v in mvc.findall("value"):
        out[int(v.get("cell_index"))] = int(v.get("value"))
    return out


def read_mesh_function(path, n_cells=None):
    """DOLFIN XML cell function (``<mesh_function>``: a ``<mesh_value_collection>``
    or a plain list of ``<entity index value>``), e.g. the ``pmk_*.xml`` partition
    markers.  Returns int32 values per cell."""
    with _open_text(path) as f:
        root = ET.parse(f).getroot()
    mf = root.find("mesh_function")
    if mf is None:
        raise ValueError("%s: no <mesh_function> element" % path)
    mvc = mf.find("mesh_value_collection")
    if mvc is not None:
        n = n_cells if n_cells is not None else int(mvc.get("size"))
        return _collection_values(mvc, n)
    ents = mf.findall("entity")
    n = n_cells if n_cells is not None else int(mf.get("size", len(ents)))
    out = np.zeros(n, np.int32)
    for e in ents:
        out[int(e.get("index"))] = int(e.get("value"))
    return out


def write_msh2(path, xyz, tets, markers=None):
    """Write an ASCII 2.2 gmsh file (tetrahedra, two tags: physical = marker,
    elementary = marker); used to hand meshes to gmsh-based tools and in tests."""
    xyz = np.asarray(xyz, np.float64)
    tets = np.asarray(tets)
    mk = np.zeros(len(tets), np.int64) if markers is None else np.asarray(markers)
    with open(path, "w") as f:
        f.write("$MeshFormat\n2.2 0 8\n$EndMeshFormat\n$Nodes\n%d\n" % len(xyz))
        for i, (x, y, z) in enumerate(xyz):
            f.write("%d %.17g %.17g %.17g\n" % (i + 1, x, y, z))
        f.write("$EndNodes\n$Elements\n%d\n" % len(tets))
        for i, (t, m) in enumerate(zip(tets, mk)):
            f.write("%d 4 2 %d %d %d %d %d %d\n" % (i + 1, m, m, t[0] + 1, t[1] + 1, t[2] + 1, t[3] + 1))
        f.write("$EndElements\n")


def _locate(points, xyz, tets, eps=1e-12):
    """For each point, whether it lies in (or on) some tetrahedron of the mesh.
    Uniform-grid binning of the tetrahedra's bounding boxes, then barycentric
    tests of the candidates."""
    P = np.asarray(points, np.float64)
    V = np.asarray(xyz, np.float64)[np.asarray(tets)]          # [m,4,3]
    lo, hi = V.min(axis=1), V.max(axis=1)
    glo, ghi = lo.min(axis=0), hi.max(axis=0)
    m = len(V)
    nb = max(1, int(round(m ** (1.0 / 3.0))))
    h = np.maximum((ghi - glo) / nb, 1e-300)
    i0 = np.clip(((lo - glo) / h).astype(np.int64), 0, nb - 1)
    i1 = np.clip(((hi - glo) / h).astype(np.int64), 0, nb - 1)
    buckets = {}
    for t in range(m):
        for a in range(i0[t, 0], i1[t, 0] + 1):
            for b in range(i0[t, 1], i1[t, 1] + 1):
                for c in range(i0[t, 2], i1[t, 2] + 1):
                    buckets.setdefault((a, b, c), []).append(t)
    # barycentric solve per tetrahedron: [v1-v0, v2-v0, v3-v0] lam = p - v0
    T = np.transpose(V[:, 1:] - V[:, :1], (0, 2, 1))
    Tinv = np.linalg.inv(T)
    inside = np.zeros(len(P), bool)
    cell = ((P - glo) / h).astype(np.int64)
    for k, p in enumerate(P):
        if np.any(p < glo - eps) or np.any(p > ghi + eps):
            continue
        key = tuple(np.clip(cell[k], 0, nb - 1))
        cand = buckets.get(key)
        if not cand:
            continue
        cand = np.asarray(cand)
        lam = np.einsum("tij,tj->ti", Tinv[cand], p - V[cand, 0])
        ok = (lam >= -eps).all(axis=1) & (lam.sum(axis=1) <= 1 + eps)
        inside[k] = bool(ok.any())
    return inside


def markers_from_submeshes(xyz, tets, evengroup=(), oddgroup=()):
    """``CreatePhaseFunc`` with sub-meshes (``DmriFemLib.py:765-798``): every
    cell whose midpoint lies in even sub-mesh i gets marker 2i+2 (phase 0), in odd
    sub-mesh i marker 2i+1 (phase 1); the odd groups are tested after the even
    ones and win, as in the reference's loop order; other cells get 0.  Each
    sub-mesh is a (xyz, tets) pair.  Cells outside every sub-mesh keep the
    reference's initial phase (0, or 1 when only even groups are given).
    Returns (markers, phase)."""
    xyz = np.asarray(xyz, np.float64)
    tets = np.asarray(tets)
    mid = xyz[tets].mean(axis=1)
    mk = np.zeros(len(tets), np.int32)
    # the reference's initial phase: 0 with no even group, 1 with only even groups
    phase = np.full(len(tets), 1 if (len(evengroup) and not len(oddgroup)) else 0, np.int32)
    for i, (sx, st) in enumerate(evengroup):
        hit = _locate(mid, sx, st)
        mk[hit], phase[hit] = 2 * i + 2, 0
    for i, (sx, st) in enumerate(oddgroup):
        hit = _locate(mid, sx, st)
        mk[hit], phase[hit] = 2 * i + 1, 1
    return mk, phase
