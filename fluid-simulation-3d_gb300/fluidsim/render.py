"""Views for the headless render (sph_render): the camera matrices the
reference's RenderUtils::Camera builds (engine/render/camera.cc:66-95), in
glm's column-major layout, and the sph_view they fill.

`look_at` and `perspective` follow glm::lookAt and glm::perspective
(right-handed, clip depth -1..1): the Camera's projection is
glm::perspective(radians(90), width / height, 0.01, 1000) (camera.cc:69,
gameApp.cc:120) and its ViewProjection is Projection * View (camera.cc:92).
"""
from __future__ import annotations

import math

import numpy as np

from ._lib import View

SCALE = 0.34  # OutPositions.w, the billboard size (physicsWorld.cc:107)


def look_at(eye, center, up=(0.0, 1.0, 0.0)) -> np.ndarray:
    """glm::lookAt as a 4x4 float32 matrix, indexed m[column][row]."""
    eye, center, up = (np.asarray(v, np.float64) for v in (eye, center, up))
    f = center - eye
    f /= np.linalg.norm(f)
    s = np.cross(f, up)
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    m = np.eye(4)
    m[0][0], m[1][0], m[2][0] = s
    m[0][1], m[1][1], m[2][1] = u
    m[0][2], m[1][2], m[2][2] = -f
    m[3][0], m[3][1], m[3][2] = -s @ eye, -u @ eye, f @ eye
    return m.astype(np.float32)


def perspective(fovy_deg=90.0, aspect=16.0 / 9.0, near=0.01, far=1000.0) -> np.ndarray:
    """glm::perspective as a 4x4 float32 matrix, indexed m[column][row]."""
    t = math.tan(math.radians(fovy_deg) / 2.0)
    m = np.zeros((4, 4))
    m[0][0] = 1.0 / (aspect * t)
    m[1][1] = 1.0 / t
    m[2][2] = -(far + near) / (far - near)
    m[2][3] = -1.0
    m[3][2] = -(2.0 * far * near) / (far - near)
    return m.astype(np.float32)


def view(eye, center, width, height, fovy_deg=90.0, near=0.01, far=1000.0,
         up=(0.0, 1.0, 0.0), scale=SCALE, clear=(0.0, 0.0, 0.0, 1.0)) -> View:
    """The sph_view of a camera at `eye` looking at `center`."""
    p = perspective(fovy_deg, width / height, near, far)
    # Projection * View (both stored m[column][row], so transpose to multiply)
    vp = (p.T.astype(np.float64) @ look_at(eye, center, up).T.astype(np.float64)).T
    vp = vp.astype(np.float32)
    v = View()
    v.view_proj[:] = [float(x) for x in vp.reshape(-1)]
    v.proj[:] = [float(x) for x in p.reshape(-1)]
    v.width, v.height = int(width), int(height)
    v.scale = float(scale)
    v.clear[:] = [float(x) for x in clear]
    return v
