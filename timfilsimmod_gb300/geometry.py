"""Seeded synthetic swimmer geometries for the RPY mobility path.

A swimmer is a rigid sphere of radius R discretised by blobs at the vertices
of an icosahedron subdivided k times and projected to the sphere (k = 3, 4, 5
give 642, 2562, 10242 blobs), carrying `nfil` filaments of `nseg` segments
rooted at Fibonacci-lattice points. The reference reads the same kind of
geometry from its `.seed` files (rigid_body.cpp:325-365, swimmer.cpp:312-391):
blob references on the body surface and filament bases at
R + RBLOB + 0.5 DL along the surface normal (config.hpp:341
BASE_HEIGHT_ABOVE_SURFACE).

Everything is float64 in the reference's AoS layouts:
x_segs (Ns, 3), f_segs (Ns, 6), x_blobs (Nb, 3), f_blobs (Nb, 3).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


def icosphere(subdivisions: int) -> np.ndarray:
    """Unit-sphere vertices of an icosahedron subdivided `subdivisions` times
    (10 * 4**k + 2 points), in a deterministic order."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    verts = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t),
             (0, -1, -t), (0, 1, -t), (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4),
             (11, 10, 2), (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8),
             (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    pts = [np.array(v, dtype=np.float64) / np.linalg.norm(v) for v in verts]
    for _ in range(subdivisions):
        cache: dict[tuple[int, int], int] = {}

        def mid(a: int, b: int) -> int:
            key = (a, b) if a < b else (b, a)
            if key not in cache:
                m = pts[a] + pts[b]
                pts.append(m / np.linalg.norm(m))
                cache[key] = len(pts) - 1
            return cache[key]

        new_faces = []
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            new_faces += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = new_faces
    return np.stack(pts)


def fibonacci_sphere(n: int) -> np.ndarray:
    """n nearly uniform unit vectors on the Fibonacci (golden-angle) lattice."""
    i = np.arange(n, dtype=np.float64)
    z = 1.0 - (2.0 * i + 1.0) / n
    rho = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    phi = i * np.pi * (3.0 - 5.0 ** 0.5)
    return np.stack([rho * np.cos(phi), rho * np.sin(phi), z], axis=1)


def _tangent_frames(normals: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """Two unit vectors orthogonal to each normal (and to each other)."""
    helper = np.where(np.abs(normals[:, 2:3]) < 0.9, [[0.0, 0.0, 1.0]], [[1.0, 0.0, 0.0]])
    t1 = np.cross(normals, helper)
    t1 /= np.linalg.norm(t1, axis=1, keepdims=True)
    t2 = np.cross(normals, t1)
    return t1, t2


@dataclass
class Swimmer:
    x_segs: np.ndarray    # (Ns, 3)
    f_segs: np.ndarray    # (Ns, 6)
    x_blobs: np.ndarray   # (Nb, 3)
    f_blobs: np.ndarray   # (Nb, 3)
    blob_references: np.ndarray  # (Nb, 3) body-frame blob offsets
    body_x: np.ndarray    # (3,)
    nfil: int
    nseg: int
    radius: float
    seg_sep: float

    @property
    def num_segs(self) -> int:
        return self.x_segs.shape[0]

    @property
    def num_blobs(self) -> int:
        return self.x_blobs.shape[0]


def make_swimmer(radius: float, subdivisions: int, nfil: int, nseg: int = 20,
                 seg_sep: float = 2.2, a_seg: float = 1.0, a_blob: float = 1.0,
                 jitter: float = 1e-3, shape: str = "straight", seed: int = 0,
                 centre=(0.0, 0.0, 0.0)) -> Swimmer:
    """Seeded swimmer geometry plus N(0,1) forces/torques on every particle.

    shape "straight": filaments along the surface normal with N(0, jitter)
    tangential jitter per segment. shape "beat": each filament bends in the
    plane of its normal and a tangent direction, as a planar beat at a phase
    drawn uniformly per filament; consecutive segments stay seg_sep apart.
    """
    rng = np.random.default_rng(seed)
    centre = np.asarray(centre, dtype=np.float64)
    blob_refs = radius * icosphere(subdivisions)
    x_blobs = centre + blob_refs
    normals = fibonacci_sphere(nfil)
    t1, t2 = _tangent_frames(normals)
    base = centre + (radius + a_blob + 0.5 * seg_sep) * normals
    s = np.arange(nseg, dtype=np.float64)
    if shape == "straight":
        x = base[:, None, :] + seg_sep * s[None, :, None] * normals[:, None, :]
        jit = rng.normal(0.0, jitter, size=(nfil, nseg, 2))
        jit[:, 0, :] = 0.0  # the base segment sits on its root
        x = x + jit[..., 0:1] * t1[:, None, :] + jit[..., 1:2] * t2[:, None, :]
    elif shape == "beat":
        phase = rng.uniform(0.0, 2.0 * np.pi, size=nfil)
        # tangent angle from the normal: grows along the filament, swings with phase
        frac = (s + 0.5) / nseg
        theta = 0.9 * np.sin(phase[:, None] - 2.0 * frac[None, :]) * frac[None, :]
        tang = (np.cos(theta)[..., None] * normals[:, None, :]
                + np.sin(theta)[..., None] * t1[:, None, :])
        steps = np.concatenate([np.zeros((nfil, 1, 3)), seg_sep * tang[:, :-1, :]], axis=1)
        x = base[:, None, :] + np.cumsum(steps, axis=1)
    else:
        raise ValueError(f"unknown shape {shape!r}")
    x_segs = x.reshape(-1, 3)
    f_segs = rng.normal(size=(x_segs.shape[0], 6))
    f_blobs = rng.normal(size=(x_blobs.shape[0], 3))
    return Swimmer(x_segs=np.ascontiguousarray(x_segs), f_segs=f_segs, x_blobs=x_blobs,
                   f_blobs=f_blobs, blob_references=blob_refs, body_x=centre.copy(), nfil=nfil,
                   nseg=nseg, radius=radius, seg_sep=seg_sep)


# The synthetic configurations of the reference's RPY path, by name.
CONFIGS = {
    # one sphere R = 20a, 642 blobs, 32 x 20 segments
    "small": dict(radius=20.0, subdivisions=3, nfil=32, nseg=20),
    # one sphere R = 60a, 2562 blobs, 640 x 20 segments
    "medium": dict(radius=60.0, subdivisions=4, nfil=640, nseg=20),
    # one sphere R = 150a, 10242 blobs, 4000 x 20 segments, planar-beat shapes
    "large": dict(radius=150.0, subdivisions=5, nfil=4000, nseg=20, shape="beat"),
}


def make_config(name: str, seed: int = 0, **overrides) -> Swimmer:
    kw = dict(CONFIGS[name])
    kw.update(overrides)
    return make_swimmer(seed=seed, **kw)


def flow_grid(n: int, half_width: float, centre=(0.0, 0.0, 0.0)) -> np.ndarray:
    """n^3 evaluation points at the cell centres of a uniform grid over the
    cube centre +- half_width, x fastest, as an (n^3, 3) float64 array."""
    c = (np.arange(n, dtype=np.float64) + 0.5) / n * (2.0 * half_width) - half_width
    z, y, x = np.meshgrid(c, c, c, indexing="ij")
    pts = np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1)
    return np.ascontiguousarray(pts + np.asarray(centre, dtype=np.float64))


def elastic_swimmer(nfil: int, nseg: int = 20, seg_sep: float = 2.2, a_blob: float = 1.0):
    """A swimmer for the implicit step: a sphere of 642 blobs (R = 20a) when
    nfil < 128, else 2562 blobs (R = 60a), with nfil straight filaments
    rooted on a Fibonacci lattice one blob radius plus half a segment gap
    above the surface, along the normals. Returns (blob_refs (Nb, 3),
    fil_refs (nfil, 3), fil_dirs (nfil, 3), radius)."""
    radius, subdiv = (20.0, 3) if nfil < 128 else (60.0, 4)
    blob_refs = radius * icosphere(subdiv)
    normals = fibonacci_sphere(nfil)
    fil_refs = (radius + a_blob + 0.5 * seg_sep) * normals
    return blob_refs, fil_refs, normals, radius


def quat_rot(q) -> np.ndarray:
    """Rotation matrix of the unit quaternion q = (q0, q1, q2, q3), scalar
    first (quaternion.cpp rot_mat)."""
    q0, q1, q2, q3 = (float(v) for v in q)
    return np.array([
        [1 - 2 * (q2 * q2 + q3 * q3), 2 * (q1 * q2 - q0 * q3), 2 * (q1 * q3 + q0 * q2)],
        [2 * (q1 * q2 + q0 * q3), 1 - 2 * (q1 * q1 + q3 * q3), 2 * (q2 * q3 - q0 * q1)],
        [2 * (q1 * q3 - q0 * q2), 2 * (q2 * q3 + q0 * q1), 1 - 2 * (q1 * q1 + q2 * q2)]])


@dataclass
class PrescribedSwimmer:
    """A sphere of blobs carrying filaments whose shapes follow a prescribed
    beat: link j of a filament at phase phi makes the angle
    theta_j = A sin(phi - k s_j) s_j (s_j = (j + 1/2) / nseg) with the surface
    normal n, in the plane of n and a tangent t1, and the whole shape is
    tilted by the shape-rotation angle psi about t2 = n x t1 (the axis the
    reference's DYNAMIC_SHAPE_ROTATION turns the beat plane's vertical about).
    Synthetic kinematics of the reference's prescribed-cilia solve, whose
    shape sequences (filament.cpp:680-860) need its fitted s-value files."""
    blob_references: np.ndarray  # (Nb, 3) body frame
    normals: np.ndarray          # (nfil, 3) body frame
    t1: np.ndarray
    t2: np.ndarray
    base: np.ndarray             # (nfil, 3) body frame: filament roots
    nfil: int
    nseg: int
    seg_sep: float
    amplitude: float = 0.9
    wavenumber: float = 2.0

    def kinematics(self, phase, angle, body_x=(0.0, 0.0, 0.0), body_q=(1.0, 0.0, 0.0, 0.0)):
        """Segment positions x (Ns, 3) and the velocity directions d x / d phase
        and d x / d psi (Ns, 3 each) at the filaments' phases and shape-rotation
        angles, in the lab frame of the body pose (body_x, body_q)."""
        phase = np.asarray(phase, dtype=np.float64)[:, None]
        psi = np.asarray(angle, dtype=np.float64)[:, None, None]
        s = (np.arange(self.nseg, dtype=np.float64) + 0.5) / self.nseg
        th = self.amplitude * np.sin(phase - self.wavenumber * s[None, :]) * s[None, :]
        dth = self.amplitude * np.cos(phase - self.wavenumber * s[None, :]) * s[None, :]
        n, t1, t2 = self.normals[:, None, :], self.t1[:, None, :], self.t2[:, None, :]
        # the beat in the (n, t1) plane tilted by psi about t2: n -> n cos psi - t1 sin psi
        nt = n * np.cos(psi) - t1 * np.sin(psi)
        tt = t1 * np.cos(psi) + n * np.sin(psi)
        tang = np.cos(th)[..., None] * nt + np.sin(th)[..., None] * tt
        dtang = (-np.sin(th) * dth)[..., None] * nt + (np.cos(th) * dth)[..., None] * tt
        zero = np.zeros((self.nfil, 1, 3))
        rel = np.cumsum(np.concatenate([zero, self.seg_sep * tang[:, :-1, :]], axis=1), axis=1)
        vphi = np.cumsum(np.concatenate([zero, self.seg_sep * dtang[:, :-1, :]], axis=1), axis=1)
        vpsi = np.cross(rel, np.broadcast_to(t2, rel.shape))  # d rel / d psi
        R = quat_rot(body_q)
        bx = np.asarray(body_x, dtype=np.float64)
        x = bx + (self.base[:, None, :] + rel).reshape(-1, 3) @ R.T
        return (np.ascontiguousarray(x), np.ascontiguousarray(vphi.reshape(-1, 3) @ R.T),
                np.ascontiguousarray(vpsi.reshape(-1, 3) @ R.T))


def prescribed_swimmer(nfil: int, nseg: int = 10, radius: float = 10.0, subdivisions: int = 2,
                       seg_sep: float = 2.6, a_blob: float = 1.0) -> PrescribedSwimmer:
    """Blobs on an icosphere of the given radius, filaments rooted on a
    Fibonacci lattice one blob radius plus half a segment gap above it."""
    normals = fibonacci_sphere(nfil)
    t1, t2 = _tangent_frames(normals)
    return PrescribedSwimmer(blob_references=radius * icosphere(subdivisions), normals=normals,
                             t1=t1, t2=t2, base=(radius + a_blob + 0.5 * seg_sep) * normals,
                             nfil=nfil, nseg=nseg, seg_sep=seg_sep)
