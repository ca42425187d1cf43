"""The render restatement (oracle/sph_render_oracle.cc) against closed forms
of what the reference's frame shows: the speed gradient of
FluidSimCPU::updateColors (fluidSimCPU.cc:100-124, colours fluidSimCPU.h:26-29),
the splat's size from the billboard and discard shaders
(particleRender.vs:32-43, particleRender.fs:12-13), its depth, and GL_LESS
depth testing with draw order breaking ties (gameApp.cc:158)."""
import math

import numpy as np
import pytest

W, H = 200, 150


def cam(eye=(0.0, 0.0, 5.0), center=(0.0, 0.0, 0.0)):
    from fluidsim import render
    return render.view(eye, center, W, H)


def draw(oracle_mod, pos, vel, view):
    return oracle_mod.render(np.asarray(pos, np.float32), np.asarray(vel, np.float32), view)


@pytest.mark.parametrize("speed,rgba", [
    (0.0, (0, 191, 255, 255)),     # Color1 (0, 0.75, 1)
    (0.495, (0, 255, 0, 255)),     # breakpoint 0.33 -> Color2
    (0.99, (255, 255, 0, 255)),    # breakpoint 0.66 -> Color3
    (1.5, (255, 0, 0, 255)),       # clamp at 1.5 -> Color4
    (9.0, (255, 0, 0, 255)),
])
def test_speed_gradient_endpoints(oracle_mod, speed, rgba):
    img, _ = draw(oracle_mod, [[0, 0, 0]], [[speed, 0, 0]], cam())
    covered = np.any(img[..., :3] != 0, axis=-1)
    assert covered.any()
    assert tuple(img[covered][0]) == rgba


def test_gradient_midpoint_blend(oracle_mod):
    # |v| = 0.2475 -> normalized 0.165 = half way from Color1 to Color2
    img, _ = draw(oracle_mod, [[0, 0, 0]], [[0.2475, 0, 0]], cam())
    px = img[np.any(img[..., :3] != 0, axis=-1)][0]
    want = np.array([0.0, 0.5 * 0.75 + 0.5 * 1.0, 0.5 * 1.0 + 0.0, 1.0]) * 255.0
    assert np.all(np.abs(px.astype(np.float64) - want) <= 1.0)


def test_splat_is_the_discard_ellipse(oracle_mod):
    """Centre on the axis: the covered pixels are those within s/4 of the
    offset ellipse, i.e. semi-axes (s/4) * (W/2) / w and (s/4) * (H/2) / w in
    pixels, and the splat's depth is the centre's window depth."""
    v = cam()
    img, depth = draw(oracle_mod, [[0, 0, 0]], [[0, 0, 0]], v)
    covered = depth < 1.0
    vp = np.array(list(v.view_proj), np.float64).reshape(4, 4).T
    c = vp @ np.array([0.0, 0.0, 0.0, 1.0])
    rx = (0.34 / 4) * (W / 2) / c[3]
    ry = (0.34 / 4) * (H / 2) / c[3]
    area = math.pi * rx * ry
    assert abs(covered.sum() - area) <= 2 * math.pi * max(rx, ry)  # one-pixel rim
    ys, xs = np.nonzero(covered)
    assert abs(xs.mean() + 0.5 - W / 2) < 1.0 and abs(ys.mean() + 0.5 - H / 2) < 1.0
    assert np.allclose(depth[covered], 0.5 * c[2] / c[3] + 0.5, rtol=1e-6)
    assert np.all(img[~covered] == np.array([0, 0, 0, 255], np.uint8))


def test_nearer_particle_wins_and_ties_go_to_the_first(oracle_mod):
    v = cam()
    # same screen centre, the second nearer the camera: its colour shows
    img, _ = draw(oracle_mod, [[0, 0, 0], [0, 0, 1]], [[0, 0, 0], [2, 0, 0]], v)
    assert tuple(img[H // 2, W // 2]) == (255, 0, 0, 255)
    # identical positions: the lower index (drawn first under GL_LESS) wins
    img2, _ = draw(oracle_mod, [[0, 0, 0], [0, 0, 0]], [[0, 0, 0], [2, 0, 0]], v)
    assert tuple(img2[H // 2, W // 2]) == (0, 191, 255, 255)


def test_particles_behind_or_beyond_the_clip_range_are_not_drawn(oracle_mod):
    v = cam()
    img, depth = draw(oracle_mod, [[0, 0, 9], [0, 0, -2000]], [[0, 0, 0], [0, 0, 0]], v)
    assert np.all(depth == 1.0)
    assert np.all(img == np.array([0, 0, 0, 255], np.uint8))
