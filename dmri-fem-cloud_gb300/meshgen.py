"""Synthetic geometries for the benchmark workloads (all seeded, host-side numpy).

* ``kuhn_box``: [lo, hi] box cut into n^3 cubes, each split into the 6
  tetrahedra around its (0,0,0) -> (1,1,1) diagonal; vertices numbered
  x-fastest.  This is DOLFIN's ``BoxMesh`` layout, which the reference uses in
  ``ConvergenceTest.ipynb:245``.
* region markers from cell centroids: z-aligned cylinders (staircase), nested
  spherical layers;
* ``fibonacci_directions``: golden-angle spiral on the unit sphere;
* ``workload(name)``: the five benchmark configurations (mesh, coefficients,
  sequences, q and directions), deterministic for a given seed.
"""

import math

import numpy as np

from . import sequences as seqs


def kuhn_box(lo, hi, n):
    n = (int(n),) * 3 if np.isscalar(n) else tuple(int(v) for v in n)
    nx, ny, nz = n
    lo = np.asarray(lo, np.float64) * np.ones(3)
    hi = np.asarray(hi, np.float64) * np.ones(3)
    axes = [lo[a] + np.arange(n[a] + 1) * (hi[a] - lo[a]) / n[a] for a in range(3)]
    xyz = np.empty(((nx + 1) * (ny + 1) * (nz + 1), 3))
    xyz[:, 0] = np.tile(axes[0], (ny + 1) * (nz + 1))
    xyz[:, 1] = np.tile(np.repeat(axes[1], nx + 1), nz + 1)
    xyz[:, 2] = np.repeat(axes[2], (nx + 1) * (ny + 1))
    ix, iy, iz = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    base = (iz * (ny + 1) + iy) * (nx + 1) + ix
    base = np.transpose(base, (2, 1, 0)).ravel()       # cube order: x fastest
    step = np.array([1, nx + 1, (nx + 1) * (ny + 1)])
    perms = [(0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)]
    cells = np.empty((len(base), 6, 4), np.int64)
    for j, perm in enumerate(perms):
        off = 0
        cells[:, j, 0] = base
        for k, axis in enumerate(perm):
            off = off + step[axis]
            cells[:, j, k + 1] = base + off
    return xyz, cells.reshape(-1, 4).astype(np.int32)


def centroids(xyz, tets):
    return xyz[tets].mean(axis=1)


def cylinder_regions(xyz, tets, centres, radii):
    """Region 1 for cells whose centroid lies inside any z-cylinder, else 0."""
    c = centroids(xyz, tets)
    inside = np.zeros(len(tets), bool)
    for (cx, cy), r in zip(centres, radii):
        inside |= (c[:, 0] - cx) ** 2 + (c[:, 1] - cy) ** 2 < r * r
    return inside.astype(np.int32)


def layered_sphere_regions(xyz, tets, radii):
    """Region i for the i-th shell r_{i-1} <= |c| < r_i, len(radii) outside."""
    c = centroids(xyz, tets)
    r2 = (c ** 2).sum(axis=1)
    reg = np.full(len(tets), len(radii), np.int32)
    for i in reversed(range(len(radii))):
        reg[r2 < radii[i] ** 2] = i
    return reg


def fibonacci_directions(n):
    """Golden-angle spiral: z_i = 1 - (2i+1)/n, phi_i = i * pi (3 - sqrt 5)."""
    i = np.arange(n)
    z = 1.0 - (2.0 * i + 1.0) / n
    r = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    phi = i * math.pi * (3.0 - math.sqrt(5.0))
    return np.stack([r * np.cos(phi), r * np.sin(phi), z], axis=1)


def random_cylinders(rng, half, rmin, rmax, count=None, volume_fraction=None, max_tries=20000):
    """Non-overlapping z-cylinders inside the square [-half, half]^2 (rejection
    sampling on centre distance > r1 + r2), either ``count`` of them or until
    their area fraction reaches ``volume_fraction``.  Radii are capped at
    0.9 half so that a cylinder always fits (small test boxes)."""
    rmax = min(rmax, 0.9 * half)
    rmin = min(rmin, rmax)
    cs, rs = [], []
    area = 0.0
    tries = 0
    while tries < max_tries:
        if count is not None and len(cs) >= count:
            break
        if volume_fraction is not None and area / (2 * half) ** 2 >= volume_fraction:
            break
        tries += 1
        r = rng.uniform(rmin, rmax)
        c = rng.uniform(-half + r, half - r, size=2)
        if all(np.hypot(*(c - c2)) > r + r2 for c2, r2 in zip(cs, rs)):
            cs.append(c)
            rs.append(r)
            area += math.pi * r * r
    return np.array(cs), np.array(rs)


def workload(name, seed=0, n=None):
    """Benchmark configurations (synthetic, deterministic for ``seed``).

    Returns a dict with mesh arrays, per-region coefficients, a list of time
    profiles and per-signal (q, gdir, profile index, b).
    """
    rng = np.random.default_rng(seed)
    pg = seqs.pgse(10600, 43100)
    if name == "cfg1":      # one compartment, 20^3 box
        n = n or 20
        xyz, tets = kuhn_box(-10, 10, n)
        reg = np.zeros(len(tets), np.int32)
        sig = [(1000.0, (1.0, 0.0, 0.0), 0)]
        return dict(name=name, xyz=xyz, tets=tets, region=reg, n_regions=1, D=[3e-3], invT2=None,
                    kappa=None, profiles=[pg], signals=sig, dt=200.0, multiple=False)
    if name == "cfg2":      # two compartments: staircase cylinder x^2 + y^2 < 36
        n = n or 40
        xyz, tets = kuhn_box(-10, 10, n)
        reg = cylinder_regions(xyz, tets, [(0.0, 0.0)], [6.0])
        sig = [(1000.0, (0.0, 1.0, 0.0), 0), (3000.0, (0.0, 1.0, 0.0), 0)]
        return dict(name=name, xyz=xyz, tets=tets, region=reg, n_regions=2, D=[3e-3, 3e-3], invT2=None,
                    kappa=1e-5, profiles=[pg], signals=sig, dt=200.0, multiple=True)
    if name == "cfg3":      # 8 cylinders, 64 directions x 8 b, PGSE / cos-OGSE
        n = n or 64
        xyz, tets = kuhn_box(-15, 15, n)
        cs, rs = random_cylinders(rng, 15.0, 2.0, 5.0, count=8)
        reg = cylinder_regions(xyz, tets, cs, rs)
        dirs = fibonacci_directions(64)
        bvals = np.linspace(500, 4000, 8)
        og = seqs.cos_ogse(10600, 43100)
        sig = []
        for i, g in enumerate(dirs):
            for b in bvals:
                sig.append((float(b), tuple(g), 0 if i < 32 else 1))
        return dict(name=name, xyz=xyz, tets=tets, region=reg, n_regions=2, D=[3e-3, 3e-3], invT2=None,
                    kappa=5e-5, profiles=[pg, og], signals=sig, dt=200.0, multiple=True,
                    cylinders=(cs, rs))
    if name == "cfg4":      # layered sphere, per-layer D and T2, per-interface kappa
        n = n or 48
        xyz, tets = kuhn_box(-12, 12, n)
        reg = layered_sphere_regions(xyz, tets, [4.0, 7.0, 10.0])
        kp = np.zeros((4, 4))
        for (i, j), v in {(0, 1): 1e-5, (1, 2): 3e-5, (2, 3): 5e-5}.items():
            kp[i, j] = kp[j, i] = v
        T2 = np.array([50e3, 80e3, 100e3, np.inf])
        dirs = fibonacci_directions(30)
        sig = [(float(b), tuple(g), 0) for g in dirs for b in (1000, 2000, 3000, 4000)]
        return dict(name=name, xyz=xyz, tets=tets, region=reg, n_regions=4, D=[1e-3, 2e-3, 3e-3, 3e-3],
                    invT2=1.0 / T2, kappa=kp, profiles=[pg], signals=sig, dt=200.0, multiple=True)
    raise ValueError("unknown workload %r" % name)


def uneven_meshes(count=16, seed=0, nmin=24, nmax=96, cube=0.5):
    """Meshes of the uneven batch: edge counts stepped evenly from nmin to nmax
    (cubes of edge ``cube`` um), random non-overlapping z-cylinders (radii
    U[1.5,5]) up to an area fraction drawn from U[0.1,0.4], kappa ~
    U[1e-5,1e-4], D_in = 2e-3, D_out = 3e-3."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        n = int(round(nmin + (nmax - nmin) * i / max(1, count - 1)))
        half = 0.5 * cube * n
        xyz, tets = kuhn_box(-half, half, n)
        vf = rng.uniform(0.1, 0.4)
        cs, rs = random_cylinders(rng, half, 1.5, 5.0, volume_fraction=vf)
        reg = cylinder_regions(xyz, tets, cs, rs)
        out.append(dict(n=n, xyz=xyz, tets=tets, region=reg, kappa=float(rng.uniform(1e-5, 1e-4)),
                        D=[3e-3, 2e-3], volume_fraction=vf))
    return out
