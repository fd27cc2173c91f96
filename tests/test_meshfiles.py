"""Mesh input formats (no GPU): gmsh 2.2 / 4.1 ASCII, DOLFIN XML meshes and
mesh functions, compartments from sub-meshes, and the meshes the reference
ships (read from the reference tree when it is present)."""

import os
import zipfile

import numpy as np
import pytest

# the reference checkout's root, when present (DMRI_REFERENCE); the tests on its
# shipped meshes are skipped without it
REF_MESHES = os.path.join(os.environ.get("DMRI_REFERENCE", ""), "comri", "meshes") \
    if os.environ.get("DMRI_REFERENCE") else ""


def tet_volumes(xyz, tets):
    X = xyz[tets]
    return np.einsum("ij,ij->i", np.cross(X[:, 1] - X[:, 0], X[:, 2] - X[:, 0]), X[:, 3] - X[:, 0]) / 6.0


def test_msh2_round_trip_and_zip(pkg, tmp_path):
    mf = pkg.meshfiles
    xyz, tets = pkg.meshgen.kuhn_box(-2.0, 2.0, 4)
    mk = pkg.meshgen.cylinder_regions(xyz, tets, [(0.0, 0.0)], [1.1]) * 3 + 1     # tags 1 and 4
    p = tmp_path / "box.msh"
    mf.write_msh2(p, xyz, tets, mk)
    d = mf.read_msh(p)
    assert np.array_equal(d["xyz"], xyz) and np.array_equal(d["tets"], tets) and np.array_equal(d["markers"], mk)
    z = tmp_path / "box.msh.zip"
    with zipfile.ZipFile(z, "w") as zf:
        zf.write(p, "box.msh")
    dz = mf.read_msh(z)
    assert np.array_equal(dz["tets"], tets) and np.array_equal(dz["markers"], mk)
    m = pkg.Mesh.read(z, compact_markers=True)
    assert set(np.unique(m.markers)) == {0, 1} and np.array_equal(m.markers % 2, mk % 2)


def test_msh2_skips_boundary_elements_and_unused_nodes(pkg, tmp_path):
    txt = """$MeshFormat
2.2 0 8
$EndMeshFormat
$PhysicalNames
1
3 7 "cell"
$EndPhysicalNames
$Nodes
6
10 0 0 0
11 1 0 0
12 0 1 0
13 0 0 1
14 5 5 5
15 1 1 1
$EndNodes
$Elements
4
1 2 2 3 3 10 11 12
2 4 2 7 1 10 11 12 13
3 15 2 3 3 14
4 4 2 8 2 11 12 13 15
$EndElements
"""
    p = tmp_path / "t.msh"
    p.write_text(txt)
    d = pkg.meshfiles.read_msh(p)
    assert d["tets"].tolist() == [[0, 1, 2, 3], [1, 2, 3, 4]]
    assert d["markers"].tolist() == [7, 8]
    assert d["node_ids"].tolist() == [10, 11, 12, 13, 15]          # node 14 is used by no tetrahedron
    assert np.allclose(d["xyz"][4], [1, 1, 1])


def test_msh41(pkg, tmp_path):
    txt = """$MeshFormat
4.1 0 8
$EndMeshFormat
$Entities
0 0 0 2
1 0 0 0 1 1 1 1 5 0
2 0 0 0 1 1 1 1 6 0
$EndEntities
$Nodes
1 5 1 5
3 1 0 5
1
2
3
4
5
0 0 0
1 0 0
0 1 0
0 0 1
1 1 1
$EndNodes
$Elements
2 2 1 2
3 1 4 1
1 1 2 3 4
3 2 4 1
2 2 3 4 5
$EndElements
"""
    p = tmp_path / "t4.msh"
    p.write_text(txt)
    d = pkg.meshfiles.read_msh(p)
    assert d["tets"].tolist() == [[0, 1, 2, 3], [1, 2, 3, 4]]
    assert d["markers"].tolist() == [5, 6]


def test_dolfin_xml_and_mesh_function(pkg, tmp_path):
    mesh_xml = """<?xml version="1.0"?>
<dolfin xmlns:dolfin="http://fenicsproject.org">
  <mesh celltype="tetrahedron" dim="3">
    <vertices size="5">
      <vertex index="0" x="0" y="0" z="0" />
      <vertex index="1" x="1" y="0" z="0" />
      <vertex index="2" x="0" y="1" z="0" />
      <vertex index="3" x="0" y="0" z="1" />
      <vertex index="4" x="1" y="1" z="1" />
    </vertices>
    <cells size="2">
      <tetrahedron index="0" v0="0" v1="1" v2="2" v3="3" />
      <tetrahedron index="1" v0="1" v1="2" v2="3" v3="4" />
    </cells>
    <domains>
      <mesh_value_collection type="uint" dim="3" size="2">
        <value cell_index="0" local_entity="0" value="2" />
        <value cell_index="1" local_entity="0" value="3" />
      </mesh_value_collection>
    </domains>
  </mesh>
</dolfin>
"""
    pmk_xml = """<?xml version="1.0"?>
<dolfin xmlns:dolfin="http://fenicsproject.org">
  <mesh_function>
    <mesh_value_collection type="uint" dim="3" size="2">
      <value cell_index="0" local_entity="0" value="1" />
      <value cell_index="1" local_entity="0" value="0" />
    </mesh_value_collection>
  </mesh_function>
</dolfin>
"""
    pm = tmp_path / "m.xml"
    pm.write_text(mesh_xml)
    pp = tmp_path / "pmk_m.xml"
    pp.write_text(pmk_xml)
    d = pkg.meshfiles.read_dolfin_xml(pm)
    assert d["tets"].tolist() == [[0, 1, 2, 3], [1, 2, 3, 4]] and d["markers"].tolist() == [2, 3]
    assert pkg.meshfiles.read_mesh_function(pp).tolist() == [1, 0]
    m = pkg.Mesh.read(pm, markers=pp)
    assert m.markers.tolist() == [1, 0] and m.num_vertices() == 5


def test_markers_from_submeshes(pkg):
    """CreatePhaseFunc with sub-meshes: cells whose midpoint lies in the inner
    box get the odd-group marker 1 and phase 1 (an even group: marker 2, phase 0)."""
    xyz, tets = pkg.meshgen.kuhn_box(-3.0, 3.0, 6)
    sx, st = pkg.meshgen.kuhn_box(-1.0, 1.0, 2)
    mid = xyz[tets].mean(axis=1)
    inside = np.all(np.abs(mid) < 1.0, axis=1)
    mk, ph = pkg.meshfiles.markers_from_submeshes(xyz, tets, oddgroup=[(sx, st)])
    assert np.array_equal(mk == 1, inside) and np.array_equal(ph == 1, inside)
    mk2, ph2 = pkg.meshfiles.markers_from_submeshes(xyz, tets, evengroup=[(sx, st)])
    assert np.array_equal(mk2 == 2, inside) and np.array_equal(ph2 == 0, inside) and np.all(ph2[~inside] == 1)


@pytest.mark.skipif(not REF_MESHES or not os.path.isdir(REF_MESHES),
                    reason="reference checkout not given (DMRI_REFERENCE)")
@pytest.mark.parametrize("name", ["cyl6_r_3E_6_vol.msh.zip", "undyAxon_Ax_1E_6_vol.msh.zip"])
def test_reference_shipped_meshes(pkg, name):
    """The meshes shipped with the reference parse: every declared node is used,
    no tetrahedron is degenerate, and the physical tags give the compartments."""
    path = os.path.join(REF_MESHES, name)
    with zipfile.ZipFile(path) as z:
        head = z.open(z.namelist()[0]).read(4096).decode()
    n_declared = int(head.split("$Nodes")[1].split()[0])
    m = pkg.Mesh.read(path)
    assert m.num_vertices() == n_declared
    vol = np.abs(tet_volumes(m.xyz, m.tets))
    assert vol.min() > 1e-12 * vol.max()
    assert m.markers is not None and len(np.unique(m.markers)) >= 1
