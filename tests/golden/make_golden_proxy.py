"""Generate golden vectors of the reference's proxy-plane geometry (host build, oracle/_ref).

Run here, where the reference checkout (project/boundingBox.cpp and its vendored glm) exists:
    python tests/golden/make_golden_proxy.py
Writes tests/golden/proxy_planes.npz: for each case (view origin, view direction, box centre,
box dimensions, plane count) the output of the reference's own
BoundingBox::generateProxyGeometry (project/boundingBox.cpp:133-181) in smk_proxy_planes'
layout.  The GPU machine has no reference checkout; the proxy-plane tests there check against
this file.

Cases: the reference application's proxy planes (view origin 0, direction -halfView for its
default camera and light, main.cpp:686, 100 planes, an 80^3 box of unit cells at the origin),
axis-aligned and diagonal directions, a box with unequal sides seen from off the origin, and
seeded random directions.  The box is centred at the origin in every case, as in the
application: the reference places the planes between the extreme projections of a box at the
origin (boundingBox.cpp:139-152), so for a box centred elsewhere a plane can miss it, and the
reference's teselate then runs past the end of its point list (points.size() - 2 on an unsigned
size) until its allocation fails.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from smoke_simulation_gb300 import scenes as S  # noqa: E402


def app_half_view() -> tuple:
    """halfView of the reference application's default camera and light (main.cpp): the unit
    half vector between the camera's view direction and the light's."""
    cam_pos = np.array([1.0, 20.0, 100.0], np.float32)
    light_pos = np.array([120.0, 80.0, 0.0], np.float32)
    view = -cam_pos / np.linalg.norm(cam_pos)
    light = -light_pos / np.linalg.norm(light_pos)
    if np.dot(view, light) > 0:
        h = view + light
    else:
        h = -view + light
    return tuple(float(x) for x in (h / np.linalg.norm(h)))


def cases() -> list:
    hv = app_half_view()
    out = [((0.0, 0.0, 0.0), tuple(-x for x in hv), (0.0, 0.0, 0.0), (80.0, 80.0, 80.0), 100),
           ((0.0, 0.0, 0.0), (0.0, 0.0, 1.0), (0.0, 0.0, 0.0), (80.0, 80.0, 80.0), 50),
           ((0.0, 0.0, 0.0), (1.0, 1.0, 0.0), (0.0, 0.0, 0.0), (80.0, 80.0, 80.0), 50),
           ((0.0, 0.0, 0.0), (-0.3, -0.2, 0.93), (0.0, 0.0, 0.0), (80.0, 80.0, 80.0), 50),
           ((0.0, 0.0, 0.0), (-0.51, 0.67, -0.2), (0.0, 0.0, 0.0), (80.0, 80.0, 80.0), 50),
           ((5.0, -3.0, 40.0), (0.2, -0.7, 0.4), (0.0, 0.0, 0.0), (64.0, 32.0, 48.0), 64),
           ((-10.0, 20.0, 100.0), (0.57, 0.57, 0.59), (0.0, 0.0, 0.0), (128.0, 128.0, 128.0), 37)]
    rng = S.SplitMix64(7, lane=9)
    for _ in range(12):
        d = rng.uniform(3, -1.0, 1.0)
        out.append(((0.0, 0.0, 0.0), tuple(float(x) for x in d), (0.0, 0.0, 0.0), (80.0, 80.0, 80.0), 40))
    return out


def main():
    data = {}
    for k, (vo, vd, bp, dm, planes) in enumerate(cases()):
        v, c, t = O.reference_proxy_planes(vo, vd, bp, dm, planes)
        data["case%02d_args" % k] = np.array(list(vo) + list(vd) + list(bp) + list(dm) + [planes], np.float64)
        data["case%02d_vertices" % k] = v
        data["case%02d_counts" % k] = c
        data["case%02d_triangles" % k] = t
    path = os.path.join(HERE, "proxy_planes.npz")
    np.savez_compressed(path, **data)
    print("wrote", path)


if __name__ == "__main__":
    main()
