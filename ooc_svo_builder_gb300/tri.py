"""The .tri / .tridata triangle-soup format and seeded synthetic meshes.

Format (libtri, src/libs/libtri/include/tri_tools.h:75-128 and tri_util.h:7-55):

* ``<base>.tri`` is a text header::

      #tri 1
      ntriangles <T>
      geo_only <0|1>
      bbox  <minx> <miny> <minz> <maxx> <maxy> <maxz>
      END

* ``<base>.tridata`` holds T packed little-endian FP32 records: 9 floats
  (v0, v1, v2) when ``geo_only`` is 1, or 21 floats (v0, v1, v2, normal,
  c0, c1, c2) when it is 0 (tri_util.h:7-11, 29-55).

The generators follow tri_convert's conventions (src/tri_convert/tri_convert.cpp:98-99,
tri_convert_util.h:168-189): the bounding box starts at the origin and is a cube,
and a face normal is ``normalize(cross(v0 - v1, v1 - v2))`` in FP32.
"""
from __future__ import annotations

import os
from dataclasses import dataclass

import numpy as np

BINARY_FLOATS = 9
PAYLOAD_FLOATS = 21


@dataclass
class TriHeader:
    version: int
    n_triangles: int
    geo_only: int
    bbox_min: tuple
    bbox_max: tuple
    base: str


def _fmt(v: float) -> str:
    # Nine significant digits round-trip any FP32 value exactly.
    return "%.9g" % float(np.float32(v))


def write_tri(base: str, tris: np.ndarray, bbox_min=(0.0, 0.0, 0.0), bbox_max=(1.0, 1.0, 1.0)) -> str:
    """Write ``<base>.tri`` + ``<base>.tridata``; returns the header path."""
    tris = np.ascontiguousarray(tris, dtype=np.float32)
    if tris.ndim != 2 or tris.shape[1] not in (BINARY_FLOATS, PAYLOAD_FLOATS):
        raise ValueError("triangles must be [T, 9] or [T, 21] float32")
    geo_only = 1 if tris.shape[1] == BINARY_FLOATS else 0
    d = os.path.dirname(base)
    if d:
        os.makedirs(d, exist_ok=True)
    with open(base + ".tri", "w") as f:
        f.write("#tri 1\n")
        f.write("ntriangles %d\n" % tris.shape[0])
        f.write("geo_only %d\n" % geo_only)
        f.write("bbox  " + " ".join(_fmt(v) for v in (*bbox_min, *bbox_max)) + "\n")
        f.write("END\n")
    tris.astype("<f4").tofile(base + ".tridata")
    return base + ".tri"


def read_tri_header(path: str) -> TriHeader:
    """Parse a .tri header like parseTriHeader (tri_tools.h:75-115): whitespace-separated
    words after ``#tri <version>``; ``ntriangles``, ``geo_only`` and ``bbox`` take their
    values, ``END`` ends the header, and any other word skips the rest of its line."""
    with open(path) as f:
        text = f.read()
    pos = 0

    def word():
        nonlocal pos
        while pos < len(text) and text[pos].isspace():
            pos += 1
        start = pos
        while pos < len(text) and not text[pos].isspace():
            pos += 1
        return text[start:pos] if pos > start else None

    if word() != "#tri":
        raise ValueError("first word is not #tri")
    version = int(word())
    n, geo = 0, 0
    bmin = bmax = (0.0, 0.0, 0.0)
    while True:
        t = word()
        if t is None:
            raise ValueError("error reading header")
        if t == "END":
            break
        if t == "ntriangles":
            n = int(word())
        elif t == "geo_only":
            geo = int(word())
        elif t == "bbox":
            vals = [float(np.float32(word())) for _ in range(6)]
            bmin, bmax = tuple(vals[:3]), tuple(vals[3:])
        else:
            nl = text.find("\n", pos)
            pos = len(text) if nl < 0 else nl + 1
    return TriHeader(version, n, geo, bmin, bmax, path[: path.rfind(".")])


def read_tri(path: str):
    """Return (header, triangles[T, 9|21] float32)."""
    h = read_tri_header(path)
    w = BINARY_FLOATS if h.geo_only else PAYLOAD_FLOATS
    data = np.fromfile(h.base + ".tridata", dtype="<f4", count=h.n_triangles * w)
    return h, data.reshape(h.n_triangles, w)


# --------------------------------------------------------------------------
# FP32 helpers that follow tri_convert's normal convention
# --------------------------------------------------------------------------

def face_normals(v0: np.ndarray, v1: np.ndarray, v2: np.ndarray) -> np.ndarray:
    """normalize(cross(v0 - v1, v1 - v2)) in FP32 (tri_convert_util.h:183-189)."""
    a = (v0 - v1).astype(np.float32)
    b = (v1 - v2).astype(np.float32)
    c = np.empty_like(a)
    c[:, 0] = a[:, 1] * b[:, 2] - a[:, 2] * b[:, 1]
    c[:, 1] = a[:, 2] * b[:, 0] - a[:, 0] * b[:, 2]
    c[:, 2] = a[:, 0] * b[:, 1] - a[:, 1] * b[:, 0]
    sq = (c[:, 0] * c[:, 0] + c[:, 1] * c[:, 1]) + c[:, 2] * c[:, 2]
    with np.errstate(divide="ignore", invalid="ignore"):
        r = np.float32(1.0) / np.sqrt(sq)
        return (c * r[:, None]).astype(np.float32)


def pack(v0, v1, v2, normals=None, colors=None) -> np.ndarray:
    """Assemble [T, 9] (no colours) or [T, 21] (with colours) records."""
    v0 = np.asarray(v0, np.float32)
    v1 = np.asarray(v1, np.float32)
    v2 = np.asarray(v2, np.float32)
    if colors is None:
        return np.ascontiguousarray(np.concatenate([v0, v1, v2], axis=1), dtype=np.float32)
    if normals is None:
        normals = face_normals(v0, v1, v2)
    c0, c1, c2 = colors
    return np.ascontiguousarray(
        np.concatenate([v0, v1, v2, normals, c0, c1, c2], axis=1), dtype=np.float32)


# --------------------------------------------------------------------------
# Seeded synthetic meshes
# --------------------------------------------------------------------------

_UNIT_ICOSPHERES: dict = {}


def _unit_icosphere(subdiv: int):
    """Vertices on the unit sphere and faces of the subdivided icosahedron (cached per level)."""
    if subdiv in _UNIT_ICOSPHERES:
        return _UNIT_ICOSPHERES[subdiv]
    t = (1.0 + 5.0 ** 0.5) / 2.0
    verts = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t),
             (0, -1, -t), (0, 1, -t), (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4),
             (11, 10, 2), (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8),
             (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    V = np.array(verts, dtype=np.float64)
    V /= np.linalg.norm(V, axis=1, keepdims=True)
    F = np.array(faces, dtype=np.int64)
    for _ in range(subdiv):
        e = np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]], axis=0)
        e.sort(axis=1)
        uniq, inv = np.unique(e, axis=0, return_inverse=True)
        inv = inv.reshape(-1)
        mid = V[uniq[:, 0]] + V[uniq[:, 1]]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        base = V.shape[0]
        V = np.concatenate([V, mid], axis=0)
        nf = F.shape[0]
        m01 = base + inv[0:nf]
        m12 = base + inv[nf:2 * nf]
        m20 = base + inv[2 * nf:3 * nf]
        F = np.concatenate([
            np.stack([F[:, 0], m01, m20], 1), np.stack([F[:, 1], m12, m01], 1),
            np.stack([F[:, 2], m20, m12], 1), np.stack([m01, m12, m20], 1)], axis=0)
    _UNIT_ICOSPHERES[subdiv] = (V, F)
    return V, F


def icosphere(subdiv: int, radius: float = 0.4, center=(0.5, 0.5, 0.5), jitter: float = 0.002,
              seed: int = 1):
    """Icosphere with 20 * 4**subdiv faces; every unique vertex moves radially by N(0, jitter).

    Returns (vertices[V, 3] float64 on the unit sphere scaled and jittered, faces[F, 3]).
    """
    V, F = _unit_icosphere(subdiv)
    rng = np.random.default_rng(seed)
    r = radius + rng.normal(0.0, jitter, size=V.shape[0])
    P = np.asarray(center, np.float64)[None, :] + V * r[:, None]
    return P, F


def icosphere_tris(subdiv: int = 5, radius: float = 0.4, jitter: float = 0.002, seed: int = 1,
                   payload: bool = False) -> np.ndarray:
    """Configuration 1's mesh: an icosphere in the unit cube as [T, 9] (or [T, 21])."""
    P, F = icosphere(subdiv, radius, (0.5, 0.5, 0.5), jitter, seed)
    P = P.astype(np.float32)
    v0, v1, v2 = P[F[:, 0]], P[F[:, 1]], P[F[:, 2]]
    if not payload:
        return pack(v0, v1, v2)
    rng = np.random.default_rng(seed + 1000)
    col = rng.random((P.shape[0], 3), dtype=np.float32)
    return pack(v0, v1, v2, colors=(col[F[:, 0]], col[F[:, 1]], col[F[:, 2]]))


def _value_noise(x: np.ndarray, y: np.ndarray, freq: int, rng: np.random.Generator) -> np.ndarray:
    """Bilinear value noise on a (freq+1)^2 lattice of uniform values, smoothstep-blended."""
    lat = rng.random((freq + 1, freq + 1))
    fx = x * freq
    fy = y * freq
    ix = np.minimum(np.floor(fx).astype(np.int64), freq - 1)
    iy = np.minimum(np.floor(fy).astype(np.int64), freq - 1)
    tx = fx - ix
    ty = fy - iy
    sx = tx * tx * (3 - 2 * tx)
    sy = ty * ty * (3 - 2 * ty)
    a = lat[ix, iy]
    b = lat[ix + 1, iy]
    c = lat[ix, iy + 1]
    d = lat[ix + 1, iy + 1]
    return (a * (1 - sx) + b * sx) * (1 - sy) + (c * (1 - sx) + d * sx) * sy


def heightfield_tris(n: int = 1024, seed: int = 2, payload: bool = True) -> np.ndarray:
    """Configuration 2's mesh: an n x n vertex heightfield over [0,1]^2.

    h = 0.3 + 0.15 * sum_{o=0..3} 0.5^o * valuenoise(f_o * (x, y)), f = 4, 8, 16, 32;
    two triangles per cell (2 (n-1)^2 triangles), per-vertex RGB uniform in [0, 1].
    """
    rng = np.random.default_rng(seed)
    g = np.linspace(0.0, 1.0, n)
    X, Y = np.meshgrid(g, g, indexing="ij")
    H = np.zeros_like(X)
    for o, f in enumerate((4, 8, 16, 32)):
        H += 0.5 ** o * _value_noise(X, Y, f, rng)
    H = 0.3 + 0.15 * H
    P = np.stack([X, Y, H], axis=-1).reshape(-1, 3).astype(np.float32)
    col = rng.random((P.shape[0], 3), dtype=np.float32)
    idx = np.arange(n * n).reshape(n, n)
    a = idx[:-1, :-1].reshape(-1)
    b = idx[1:, :-1].reshape(-1)
    c = idx[:-1, 1:].reshape(-1)
    d = idx[1:, 1:].reshape(-1)
    F = np.concatenate([np.stack([a, b, d], 1), np.stack([a, d, c], 1)], axis=0)
    v0, v1, v2 = P[F[:, 0]], P[F[:, 1]], P[F[:, 2]]
    if not payload:
        return pack(v0, v1, v2)
    return pack(v0, v1, v2, colors=(col[F[:, 0]], col[F[:, 1]], col[F[:, 2]]))


def _unit_vectors(rng: np.random.Generator, k: int) -> np.ndarray:
    u = rng.normal(size=(k, 3))
    return u / np.linalg.norm(u, axis=1, keepdims=True)


def soup_tris(n_tris: int, gridsize: int, seed: int = 3, sigma: float = 1.0, n_spheres: int = 200,
              payload: bool = False, median_voxels: float = 4.0, clip_voxels: float = 512.0) -> np.ndarray:
    """Configuration 3's triangle soup (skewed per-triangle work).

    Half the triangles are small (edge <= 1 voxel) and lie tangent to the surfaces of
    ``n_spheres`` seeded spheres (centres U[0.2, 0.8]^3, radii U[0.01, 0.2]); the other half have
    centres U[0, 1]^3 and edge length LogNormal(median ``median_voxels`` voxels, ``sigma``) clipped at
    ``clip_voxels`` voxels.  Vertices are clamped to [-0.5, 1.5].
    """
    rng = np.random.default_rng(seed)
    u = 1.0 / gridsize
    n_small = n_tris // 2
    n_big = n_tris - n_small
    centres = rng.uniform(0.2, 0.8, size=(n_spheres, 3))
    radii = rng.uniform(0.01, 0.2, size=n_spheres)
    which = rng.integers(0, n_spheres, size=n_small)
    dirs = _unit_vectors(rng, n_small)
    pos = centres[which] + dirs * radii[which, None]
    # Two tangent directions to build a small triangle in the tangent plane.
    helper = np.where(np.abs(dirs[:, :1]) < 0.9, np.array([[1.0, 0, 0]]), np.array([[0, 1.0, 0]]))
    t1 = np.cross(dirs, helper)
    t1 /= np.linalg.norm(t1, axis=1, keepdims=True)
    t2 = np.cross(dirs, t1)
    edge = rng.uniform(0.2, 1.0, size=n_small) * u
    ang = rng.uniform(0, 2 * np.pi, size=n_small)
    sv = []
    for k in range(3):
        a = ang + k * 2 * np.pi / 3
        sv.append(pos + (np.cos(a)[:, None] * t1 + np.sin(a)[:, None] * t2) * (edge / np.sqrt(3))[:, None])
    c = rng.uniform(0.0, 1.0, size=(n_big, 3))
    L = np.minimum(median_voxels * np.exp(rng.normal(0.0, sigma, size=n_big)), clip_voxels) * u
    bv = [c + _unit_vectors(rng, n_big) * (L / 2)[:, None] for _ in range(3)]
    V = [np.clip(np.concatenate([sv[k], bv[k]], 0), -0.5, 1.5).astype(np.float32) for k in range(3)]
    perm = rng.permutation(n_tris)
    v0, v1, v2 = V[0][perm], V[1][perm], V[2][perm]
    if not payload:
        return pack(v0, v1, v2)
    col = [rng.random((n_tris, 3), dtype=np.float32) for _ in range(3)]
    return pack(v0, v1, v2, colors=col)


def random_tris(n_tris: int, seed: int, payload: bool, lo: float = 0.0, hi: float = 1.0,
                max_edge: float = 0.2) -> np.ndarray:
    """Small random soup for parity tests: centres U[lo, hi]^3, edges up to ``max_edge``."""
    rng = np.random.default_rng(seed)
    c = rng.uniform(lo, hi, size=(n_tris, 3))
    L = rng.uniform(0.0, max_edge, size=n_tris)
    V = [(c + _unit_vectors(rng, n_tris) * L[:, None] / 2).astype(np.float32) for _ in range(3)]
    if not payload:
        return pack(*V)
    col = [rng.random((n_tris, 3), dtype=np.float32) for _ in range(3)]
    return pack(*V, colors=col)


def to_binary(tris: np.ndarray) -> np.ndarray:
    """Drop normals and colours: [T, 21] -> [T, 9]."""
    return np.ascontiguousarray(tris[:, :9])


def batch_meshes(n_meshes: int = 4096, seed: int = 4, tri_min: int = 64, tri_max: int = 200_000,
                 gridsizes=(64, 128, 256, 512)):
    """Configuration 4's mesh set: (triangles, gridsize, payload) per mesh.

    Triangle counts are log-uniform in [tri_min, tri_max]; half the meshes are
    icospheres (subdivision 1..7, the one closest below the drawn count), half
    soups as in configuration 3 at that count; gridsize uniform in `gridsizes`;
    binary or payload mode at 50/50.
    """
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n_meshes):
        T = int(round(float(np.exp(rng.uniform(np.log(tri_min), np.log(tri_max))))))
        N = int(rng.choice(gridsizes))
        payload = bool(rng.integers(0, 2))
        sub_seed = int(rng.integers(0, 2**31 - 1))
        if rng.random() < 0.5:
            s = int(np.clip(np.floor(np.log(max(T, 80) / 20.0) / np.log(4.0)), 1, 7))
            tris = icosphere_tris(s, radius=float(rng.uniform(0.2, 0.45)), jitter=0.002, seed=sub_seed,
                                  payload=payload)
        else:
            tris = soup_tris(T, N, seed=sub_seed, sigma=1.0, n_spheres=max(1, min(200, T // 500)),
                             payload=payload)
        out.append((tris, N, payload))
    return out
