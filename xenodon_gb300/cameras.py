"""Camera scripts in the reference's format (src/camera/ScriptCameraController.cpp:17-40).

Each line holds nine floats: forward xyz, up xyz, position xyz.  The volume
occupies [0, dim/max_dim] in these units (resources/dda.comp:65-66; an octree
spans [0, 1]^3 with the grid in its low corner).  The reference has no field
of view parameter: the horizontal half-angle satisfies tan = 0.5/|forward|
(resources/common.glsl:45-56), so a field of view is encoded by the length of
`forward`.
"""
from __future__ import annotations

import math
from pathlib import Path

import numpy as np


def forward_length_for_vfov(vfov_deg: float, width: int, height: int) -> float:
    """|forward| giving vertical field of view `vfov_deg` at width x height."""
    return 0.5 * (height / width) / math.tan(math.radians(vfov_deg) / 2)


def look_at(pos, target, fwd_len=1.0, up=(0.0, 1.0, 0.0)):
    pos, target = np.asarray(pos, np.float64), np.asarray(target, np.float64)
    f = target - pos
    f /= np.linalg.norm(f)
    u = np.asarray(up, np.float64)
    u = u - f * np.dot(u, f)  # the reference wants up perpendicular to forward
    nu = np.linalg.norm(u)
    if nu < 1e-9:
        u = np.array([0.0, 0.0, 1.0]) - f * f[2]
        nu = np.linalg.norm(u)
    return (f * fwd_len, u / nu, pos)


def volume_centre(dims) -> np.ndarray:
    m = float(max(dims))
    return np.array([d / m for d in dims]) * 0.5


def orbit(centre, distance, frames, fwd_len=1.0, start_angle=0.0):
    out = []
    for i in range(frames):
        a = start_angle + 2 * math.pi * i / frames
        pos = centre + distance * np.array([math.sin(a), 0.0, -math.cos(a)])
        out.append(look_at(pos, centre, fwd_len))
    return out


def ct_path(dims=(512, 361, 512), frames_per_leg=150, fwd_len=1.0):
    """450-frame benchmark path: an orbit at 2x the extent, a dolly to 0.3x
    the extent (inside the volume), and a rotation about an interior point;
    the shape of the reference's camera.txt (orbit, zoom in, rotate inside)."""
    c = volume_centre(dims)
    path = orbit(c, 2.0, frames_per_leg, fwd_len)
    d0 = np.array([0.0, 0.0, -1.0])
    for i in range(frames_per_leg):
        s = i / max(1, frames_per_leg - 1)
        dist = 2.0 + (0.3 - 2.0) * s
        path.append(look_at(c + dist * d0, c, fwd_len))
    pivot = c + np.array([0.05, 0.02, -0.1])
    for i in range(frames_per_leg):
        a = 2 * math.pi * i / frames_per_leg
        target = pivot + np.array([math.sin(a), 0.0, math.cos(a)])
        path.append(look_at(pivot, target, fwd_len))
    return path


def fibonacci_sphere(n: int, centre, distance, fwd_len):
    out = []
    golden = math.pi * (3.0 - math.sqrt(5.0))
    for i in range(n):
        y = 1 - 2 * (i + 0.5) / n
        r = math.sqrt(max(0.0, 1 - y * y))
        a = golden * i
        d = np.array([r * math.cos(a), y, r * math.sin(a)])
        out.append(look_at(centre + distance * d, centre, fwd_len))
    return out


def format_line(cam) -> str:
    f, u, p = cam
    return " ".join(f"{v:.9g}" for v in (*f, *u, *p))


def write_script(path, cams) -> None:
    Path(path).write_text("\n".join(format_line(c) for c in cams) + "\n")


def read_script(path):
    cams = []
    for line in Path(path).read_text().split("\n"):
        if not line.strip():
            continue
        v = [float(x) for x in line.split()]
        if len(v) != 9:
            raise ValueError("Syntax error in camera input file")
        cams.append((tuple(v[0:3]), tuple(v[3:6]), tuple(v[6:9])))
    return cams
