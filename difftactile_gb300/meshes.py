"""Object meshes to MPM particles, as the reference's ObjLoader.generate_particles
(object_model/obj_loader.py:22-60): the mesh is centred and scaled so that its largest extent is 1
(normalize_mesh), the cube [-0.5, 0.5]^3 is sampled on the regular grid linspace(-0.5, 0.5, d + 1)^3
(sample_cube, d = the particle density), and the samples inside the mesh are kept.

The reference reads the mesh with trimesh and keeps the samples whose cell of a filled 1/128-pitch
voxelisation is occupied; here OBJ and STL files are parsed directly and a sample is inside when a ray
from it along +x crosses the closed surface an odd number of times.  The two agree except for samples
within one voxel (1/128 of the object's size) of its surface.
"""
from __future__ import annotations

import os
import struct

import numpy as np


def read_mesh(path: str) -> tuple[np.ndarray, np.ndarray]:
    """Vertices [n, 3] (float64) and triangles [m, 3] (int) of an OBJ (polygons fanned into triangles)
    or STL (ASCII or binary) file."""
    ext = os.path.splitext(path)[1].lower()
    if ext == ".obj":
        verts, faces = [], []
        with open(path) as fh:
            for line in fh:
                parts = line.split()
                if not parts:
                    continue
                if parts[0] == "v":
                    verts.append([float(c) for c in parts[1:4]])
                elif parts[0] == "f":
                    idx = [int(p.split("/")[0]) for p in parts[1:]]
                    idx = [i - 1 if i > 0 else len(verts) + i for i in idx]
                    for k in range(1, len(idx) - 1):
                        faces.append([idx[0], idx[k], idx[k + 1]])
        return np.asarray(verts, np.float64), np.asarray(faces, np.int64).reshape(-1, 3)
    if ext == ".stl":
        with open(path, "rb") as fh:
            data = fh.read()
        if data[:5].lower() == b"solid" and b"facet" in data[:1024]:
            pts = [[float(c) for c in ln.split()[1:4]] for ln in data.decode(errors="ignore").splitlines()
                   if ln.strip().startswith("vertex")]
            tri = np.asarray(pts, np.float64).reshape(-1, 3, 3)
        else:
            n = struct.unpack("<I", data[80:84])[0]
            rec = np.frombuffer(data[84:84 + 50 * n], dtype=np.dtype([("n", "<f4", 3), ("v", "<f4", (3, 3)),
                                                                      ("a", "<u2")]))
            tri = rec["v"].astype(np.float64)
        verts, inv = np.unique(tri.reshape(-1, 3), axis=0, return_inverse=True)
        return verts, inv.reshape(-1, 3)
    raise ValueError(f"{path}: mesh files are read as .obj or .stl")


def normalize(verts: np.ndarray) -> np.ndarray:
    """Centre the bounding box at the origin and scale its largest extent to 1 (normalize_mesh)."""
    lo, hi = verts.min(0), verts.max(0)
    return (verts - (lo + hi) / 2.0) / (hi - lo).max()


def inside_grid(verts: np.ndarray, faces: np.ndarray, coords: np.ndarray) -> np.ndarray:
    """[n, n, n] mask of the grid points (coords[i], coords[j], coords[k]) inside the closed mesh, by the
    parity of a ray's crossings along +x through each (y, z) column."""
    n = len(coords)
    tri = verts[faces]                                    # [m, 3, 3]
    # the rays pass a hair off the grid so that none runs exactly through an edge or a vertex
    span = max(float(np.ptp(verts[:, 1])), float(np.ptp(verts[:, 2])), 1e-12)
    oy, oz = 1.3e-9 * span, 2.9e-9 * span
    a, b, c = tri[:, 0], tri[:, 1], tri[:, 2]
    ylo, yhi = tri[:, :, 1].min(1), tri[:, :, 1].max(1)
    zlo, zhi = tri[:, :, 2].min(1), tri[:, :, 2].max(1)
    mask = np.zeros((n, n, n), bool)
    for j, y in enumerate(coords + oy):
        rows = np.nonzero((ylo <= y) & (yhi >= y))[0]
        if len(rows) == 0:
            continue
        ta, tb, tc = a[rows], b[rows], c[rows]
        zl, zh = zlo[rows], zhi[rows]
        for k, z in enumerate(coords + oz):
            sel = np.nonzero((zl <= z) & (zh >= z))[0]
            if len(sel) == 0:
                continue
            p0, p1, p2 = ta[sel], tb[sel], tc[sel]
            # barycentric coordinates of (y, z) in the triangle's projection on the yz plane
            d1y, d1z = p1[:, 1] - p0[:, 1], p1[:, 2] - p0[:, 2]
            d2y, d2z = p2[:, 1] - p0[:, 1], p2[:, 2] - p0[:, 2]
            det = d1y * d2z - d2y * d1z
            ok = np.abs(det) > 1e-300
            ry, rz = y - p0[:, 1], z - p0[:, 2]
            with np.errstate(divide="ignore", invalid="ignore"):
                u = (ry * d2z - d2y * rz) / det
                v = (d1y * rz - ry * d1z) / det
            hit = ok & (u >= 0) & (v >= 0) & (u + v <= 1)
            if not hit.any():
                continue
            xs = np.sort(p0[hit, 0] + u[hit] * (p1[hit, 0] - p0[hit, 0]) + v[hit] * (p2[hit, 0] - p0[hit, 0]))
            crossings_beyond = len(xs) - np.searchsorted(xs, coords, side="right")
            mask[:, j, k] = (crossings_beyond & 1).astype(bool)
    return mask


def generate_particles(path: str, particle_density: int) -> np.ndarray:
    """Particles of the mesh at ``path`` in its normalised frame ([-0.5, 0.5], centred), sampled on the
    (particle_density + 1)^3 grid (ObjLoader.generate_particles)."""
    verts, faces = read_mesh(path)
    verts = normalize(verts)
    x = np.linspace(-0.5, 0.5, int(particle_density) + 1)
    m = inside_grid(verts, faces, x)
    I, J, K = np.nonzero(m)
    return np.stack([x[I], x[J], x[K]], 1).astype(np.float32)


def object_particles(obj, particle_density: int) -> np.ndarray:
    """The object's particles in its own frame: an [N, 3] array as given, a .npy file of one, or an OBJ /
    STL mesh sampled as ObjLoader.generate_particles."""
    if obj is None:
        raise ValueError("no object: give a mesh file (.obj, .stl), a .npy particle file or an [N, 3] array")
    if isinstance(obj, np.ndarray):
        return np.asarray(obj, np.float32).reshape(-1, 3)
    path = os.fspath(obj)
    if path.lower().endswith(".npy"):
        return np.load(path).astype(np.float32).reshape(-1, 3)
    return generate_particles(path, particle_density)
