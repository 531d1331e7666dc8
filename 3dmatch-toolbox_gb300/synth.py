"""Seeded synthetic scenes: the stand-in for the 3DMatch fragments.

A room 4 x 4 x 3 m (6 wall planes) with 8 boxes (sides U[0.2, 0.8] m) and 5
spheres (radii U[0.1, 0.4] m) is ray cast analytically into a 640 x 480 depth
map with the intrinsics of the reference's sample data (fx = fy = 585,
cx = 320, cy = 240), Gaussian depth noise (sigma 2 mm) is added, and the map is
back-projected as core/demo.m:84-90 does (camera frame, z forward, depth in
(0, 6) m).  Fragment B is seen from camera A moved by a random rigid transform
(angle <= 30 deg about a random axis, |t| <= 0.5 m); the returned Rt maps B's
points into A's frame.  No graphics API is involved.
"""
from __future__ import annotations

import numpy as np

W, H = 640, 480
K = np.array([[585.0, 0.0, 320.0], [0.0, 585.0, 240.0], [0.0, 0.0, 1.0]])
ROOM = np.array([4.0, 4.0, 3.0])


class Room:
    def __init__(self, seed: int):
        rng = np.random.default_rng(seed)
        self.boxes = []
        for _ in range(8):
            size = rng.uniform(0.2, 0.8, 3)
            lo = np.array([rng.uniform(0.2, ROOM[0] - 0.2 - size[0]), rng.uniform(0.2, ROOM[1] - 0.2 - size[1]),
                           rng.choice([0.0, rng.uniform(0.0, 1.5)])])
            self.boxes.append((lo, lo + size))
        self.spheres = []
        for _ in range(5):
            r = rng.uniform(0.1, 0.4)
            c = rng.uniform([r + 0.1, r + 0.1, r], [ROOM[0] - r - 0.1, ROOM[1] - r - 0.1, ROOM[2] - r - 0.1])
            self.spheres.append((c, r))

    def cast(self, origin: np.ndarray, dirs: np.ndarray) -> np.ndarray:
        """Ray parameter t of the first hit for unit-less directions dirs [N,3]."""
        n = dirs.shape[0]
        best = np.full(n, np.inf)
        with np.errstate(divide="ignore", invalid="ignore"):
            # walls: inside of the box [0, ROOM]
            for a in range(3):
                for wall in (0.0, ROOM[a]):
                    t = (wall - origin[a]) / dirs[:, a]
                    t = np.where(t > 1e-6, t, np.inf)
                    best = np.minimum(best, t)
            for lo, hi in self.boxes:
                t0 = (lo - origin) / dirs
                t1 = (hi - origin) / dirs
                tmin = np.nanmax(np.minimum(t0, t1), axis=1)
                tmax = np.nanmin(np.maximum(t0, t1), axis=1)
                hit = (tmax >= tmin) & (tmax > 1e-6)
                t = np.where(tmin > 1e-6, tmin, tmax)
                best = np.where(hit & (t < best), t, best)
            for c, r in self.spheres:
                oc = origin - c
                b = dirs @ oc
                a = np.einsum("ij,ij->i", dirs, dirs)
                cc = oc @ oc - r * r
                disc = b * b - a * cc
                sq = np.sqrt(np.maximum(disc, 0.0))
                t = (-b - sq) / a
                t = np.where(t > 1e-6, t, (-b + sq) / a)
                hit = (disc >= 0) & (t > 1e-6)
                best = np.where(hit & (t < best), t, best)
        return best


def look_at(eye, target, up=(0.0, 0.0, 1.0)) -> np.ndarray:
    """camera-to-world 4x4 for a camera at eye looking at target (x right, y down, z forward)."""
    eye = np.asarray(eye, float)
    z = np.asarray(target, float) - eye
    z /= np.linalg.norm(z)
    x = np.cross(z, up)
    x /= np.linalg.norm(x)
    y = np.cross(z, x)
    T = np.eye(4)
    T[:3, 0], T[:3, 1], T[:3, 2], T[:3, 3] = x, y, z, eye
    return T


def render_depth(room: Room, cam2world: np.ndarray, rng, noise=0.002) -> np.ndarray:
    """Depth map (metres, z in the camera frame) with Gaussian noise."""
    u, v = np.meshgrid(np.arange(W, dtype=np.float64), np.arange(H, dtype=np.float64))
    dc = np.stack([(u - K[0, 2]) / K[0, 0], (v - K[1, 2]) / K[1, 1], np.ones_like(u)], -1).reshape(-1, 3)
    dw = dc @ cam2world[:3, :3].T
    t = room.cast(cam2world[:3, 3], dw)
    depth = t  # dc has unit z, so t is the camera-frame depth
    depth = depth + rng.normal(0.0, noise, depth.shape)
    depth[~np.isfinite(depth)] = 0.0
    return depth.reshape(H, W)


def backproject(depth: np.ndarray) -> np.ndarray:
    """core/demo.m:84-90: camera-frame points of the pixels with 0 < z < 6."""
    u, v = np.meshgrid(np.arange(W, dtype=np.float64), np.arange(H, dtype=np.float64))
    z = depth
    ok = (z > 0) & (z < 6)
    x = (u - K[0, 2]) * z / K[0, 0]
    y = (v - K[1, 2]) * z / K[1, 1]
    return np.stack([x[ok], y[ok], z[ok]], 1)


def random_rotation(rng, max_deg: float) -> np.ndarray:
    axis = rng.normal(size=3)
    axis /= np.linalg.norm(axis)
    ang = np.deg2rad(rng.uniform(0.0, max_deg))
    Kx = np.array([[0, -axis[2], axis[1]], [axis[2], 0, -axis[0]], [-axis[1], axis[0], 0]])
    return np.eye(3) + np.sin(ang) * Kx + (1 - np.cos(ang)) * Kx @ Kx


def fragment_pair(seed: int, n_points=150_000, max_deg=30.0, max_t=0.5):
    """Two fragments of one room.  Returns (pts_a, pts_b, Rt) with
    pts_a ~= R @ pts_b + t for the overlapping surface (float32 points)."""
    rng = np.random.default_rng(seed)
    room = Room(seed)
    eye = np.array([rng.uniform(1.5, 2.5), rng.uniform(0.4, 0.8), rng.uniform(1.2, 1.8)])
    target = np.array([rng.uniform(1.0, 3.0), 4.0, rng.uniform(0.6, 1.4)])
    cam_a = look_at(eye, target)
    D = np.eye(4)
    D[:3, :3] = random_rotation(rng, max_deg)
    tv = rng.normal(size=3)
    D[:3, 3] = tv / np.linalg.norm(tv) * rng.uniform(0.0, max_t)
    cam_b = cam_a @ D  # camera B = camera A moved in its own frame
    out = []
    for cam in (cam_a, cam_b):
        p = backproject(render_depth(room, cam, rng))
        if n_points is not None and p.shape[0] > n_points:
            p = p[np.sort(rng.choice(p.shape[0], n_points, replace=False))]
        out.append(p.astype(np.float32))
    Rt = np.linalg.inv(cam_a) @ cam_b  # B frame -> A frame
    return out[0], out[1], Rt


def scene_fragments(seed: int, n_views=8, n_points=150_000):
    """Fragments of one room seen from cameras along a sweep (x from 1 to 3 m,
    looking towards the far wall with a slowly turning yaw).  Returns
    [(points float32 in the camera frame, camera-to-world 4x4)]; the
    ground-truth transform of fragment j into fragment i's frame is
    inv(cam_i) @ cam_j (getGtInfoLog.m's relExt)."""
    rng = np.random.default_rng(seed)
    room = Room(seed)
    out = []
    for v in range(n_views):
        s = v / max(n_views - 1, 1)
        eye = np.array([1.0 + 2.0 * s, rng.uniform(0.4, 0.7), rng.uniform(1.3, 1.6)])
        target = np.array([1.0 + 2.0 * s + 1.2 * np.sin(2.5 * s - 1.2), 4.0, rng.uniform(0.7, 1.2)])
        cam = look_at(eye, target)
        p = backproject(render_depth(room, cam, rng))
        if n_points is not None and p.shape[0] > n_points:
            p = p[np.sort(rng.choice(p.shape[0], n_points, replace=False))]
        out.append((p.astype(np.float32), cam))
    return out


def fragment(seed: int, n_points=150_000):
    return fragment_pair(seed, n_points)[0]


def depth_sequence(seed: int, n_frames=50, max_deg=2.0, max_t=0.02, dropout=0.01):
    """n_frames uint16 millimetre depth maps along a smooth seeded trajectory
    and their camera-to-base poses (base = first frame)."""
    rng = np.random.default_rng(seed)
    room = Room(seed)
    eye = np.array([2.0, 0.6, 1.5])
    cam = look_at(eye, np.array([2.0, 4.0, 1.0]))
    base = cam.copy()
    frames, poses = [], []
    for _ in range(n_frames):
        d = render_depth(room, cam, rng)
        mm = np.clip(np.round(d * 1000.0), 0, 65535).astype(np.uint16)
        mm[rng.random(mm.shape) < dropout] = 0
        frames.append(mm)
        poses.append(np.linalg.inv(base) @ cam)
        step = np.eye(4)
        step[:3, :3] = random_rotation(rng, max_deg)
        tv = rng.normal(size=3)
        step[:3, 3] = tv / np.linalg.norm(tv) * rng.uniform(0.0, max_t)
        cam = cam @ step
    return np.stack(frames), np.stack(poses).astype(np.float32)
