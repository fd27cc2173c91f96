"""Box meshes for the oracle -- TEST INFRASTRUCTURE ONLY.

``box_mesh`` reproduces DOLFIN's ``BoxMesh(Point(x0,y0,z0), Point(x1,y1,z1),
nx, ny, nz)`` as used in the reference's ``ConvergenceTest.ipynb:245``: vertices
numbered x-fastest, every cube cut into the 6 tetrahedra that share the diagonal
from its (0,0,0) corner to its (1,1,1) corner (the Kuhn / Freudenthal split).
The 216-vertex / 750-tet count of the reference's n=5 box
(``ConvergenceTest.ipynb:261-263``) is checked in the tests.
"""

import numpy as np


def box_mesh(lo, hi, n):
    """Return (xyz[n_v,3] float64, tets[n_t,4] int32) for a Kuhn-split box.

    ``lo``/``hi`` are 3-sequences of corner coordinates and ``n`` a 3-sequence
    (or an int) of cube counts per axis.
    """
    if np.isscalar(n):
        n = (int(n),) * 3
    nx, ny, nz = (int(v) for v in n)
    lo = np.asarray(lo, dtype=np.float64)
    hi = np.asarray(hi, dtype=np.float64)
    ix = np.arange(nx + 1)
    iy = np.arange(ny + 1)
    iz = np.arange(nz + 1)
    x = lo[0] + ix * (hi[0] - lo[0]) / nx
    y = lo[1] + iy * (hi[1] - lo[1]) / ny
    z = lo[2] + iz * (hi[2] - lo[2]) / nz
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    xyz = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)

    cz, cy, cx = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    v0 = (cz * (ny + 1) * (nx + 1) + cy * (nx + 1) + cx).ravel()
    sx, sy, sz = 1, nx + 1, (nx + 1) * (ny + 1)
    c = {  # cube corners by (dx,dy,dz)
        (0, 0, 0): v0, (1, 0, 0): v0 + sx, (0, 1, 0): v0 + sy, (1, 1, 0): v0 + sx + sy,
        (0, 0, 1): v0 + sz, (1, 0, 1): v0 + sx + sz, (0, 1, 1): v0 + sy + sz,
        (1, 1, 1): v0 + sx + sy + sz,
    }
    # the 6 monotone lattice paths (0,0,0) -> (1,1,1), one tet each
    tets = []
    for order in ((0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)):
        p = [0, 0, 0]
        verts = [c[tuple(p)]]
        for axis in order:
            p[axis] = 1
            verts.append(c[tuple(p)])
        tets.append(np.stack(verts, axis=1))
    # cube-major order: the 6 tets of a cube are consecutive
    tets = np.stack(tets, axis=1).reshape(-1, 4).astype(np.int32)
    return xyz, tets


def region_from_centroids(xyz, tets, predicate_list):
    """Region id per tet: 0 unless the centroid satisfies predicate k (first
    match wins), which gives region k+1."""
    cen = xyz[tets].mean(axis=1)
    region = np.zeros(len(tets), dtype=np.int32)
    assigned = np.zeros(len(tets), dtype=bool)
    for k, pred in enumerate(predicate_list):
        m = pred(cen) & ~assigned
        region[m] = k + 1
        assigned |= m
    return region
