"""Headless impostor render (mb_render_topdown) against the oracle's CPU
restatement of the same per-pixel arithmetic.  Floating point: the sphere that
wins a pixel must agree (integer), colours within 2/255 and heights within 1e-4
on all but a handful of pixels where exp2/log2 rounding moves a march step
across its 0.001 stopping threshold."""

import numpy as np
import pytest

import oracle
from bevy_millions_ball_gb300 import World, save_png, scenes

pytestmark = pytest.mark.gpu


def compare_render(w, window, width, height):
    img, hmap = w.render_topdown(width, height, window)
    p, _ = w.get_state()
    rgba, rh, win = oracle.render_topdown(p, width, height, *window)
    ref = rgba.view(np.uint8).reshape(height, width, 4)
    diff = np.abs(img.astype(np.int32) - ref.astype(np.int32)).max(axis=2)
    bad = (diff > 2) | (np.abs(hmap - rh) > 1e-4)
    assert bad.mean() <= 1e-3, f"{bad.sum()} of {bad.size} pixels differ"
    assert np.all(img[..., 3] == 255)
    return img, win


def test_render_matches_oracle(built_lib, cuda, tmp_path):
    sc = scenes.plain_uniform(3000, 64, seed=5)
    with World(sc.plugin) as w:
        w.set_state(sc.pos_scale, sc.vfme)
        w.step(12)
        img, win = compare_render(w, (-32.0, -32.0, 32.0, 32.0), 192, 160)
        assert (win > 0).mean() > 0.1  # spheres are visible
        save_png(tmp_path / "render.png", img)
        assert (tmp_path / "render.png").stat().st_size > 100


def test_render_reference_lattice_zoomed(built_lib, cuda):
    """Spheres much larger than a pixel (radius 1 over 24 pixels)."""
    sc = scenes.reference_default()
    with World(sc.plugin) as w:
        w.set_state(sc.pos_scale, sc.vfme)
        w.step(3)
        compare_render(w, (-20.0, -20.0, 20.0, 20.0), 480, 480)


def test_render_rejects_bad_windows(built_lib, cuda):
    from bevy_millions_ball_gb300 import MbError
    sc = scenes.plain_uniform(100, 16, seed=1)
    with World(sc.plugin) as w:
        with pytest.raises(MbError):
            w.render_topdown(8, 8, (0, 0, 1, 1))  # no state yet
        w.set_state(sc.pos_scale, sc.vfme)
        with pytest.raises(MbError):
            w.render_topdown(8, 8, (1, 0, 0, 1))
        with pytest.raises(MbError):
            w.render_topdown(0, 8, (0, 0, 1, 1))


def compare_view(w, width, height, eye=None, target=None, fov=0.0):
    """mb_render_view against the oracle's restatement: the winning sphere per
    pixel (integer) on all but a handful of pixels, colours within 2/255 and depth
    within 1e-5 relative elsewhere (exp2 / log2 / pow rounding differs)."""
    img, depth = w.render_view(width, height, eye, target, fov)
    p, _ = w.get_state()
    s = w.settings
    hs = s.number_of_grids_one_dimension * s.grid_size / 2.0
    rgba, rd, win = oracle.render_view(p, width, height, hs, 2.0 * s.half_map_height, eye, target, fov)
    ref = rgba.view(np.uint8).reshape(height, width, 4)
    diff = np.abs(img.astype(np.int32) - ref.astype(np.int32)).max(axis=2)
    bad = (diff > 2) | (np.abs(depth - rd) > 1e-5 * np.maximum(np.abs(rd), 1.0))
    assert bad.mean() <= 1e-3, f"{bad.sum()} of {bad.size} pixels differ"
    assert np.all(img[..., 3] == 255)
    return img, depth, win


def test_render_view_reference_camera(built_lib, cuda, tmp_path):
    """The reference's own view (eye (0, 64, 64) onto the origin, 45 degrees) of its
    start-up lattice after a few frames, and of a settled uniform scene."""
    sc = scenes.reference_default()
    with World(sc.plugin) as w:
        w.set_state(sc.pos_scale, sc.vfme)
        w.step(3)
        img, depth, win = compare_view(w, 320, 180)
        assert (win > 0).mean() > 0.2  # spheres fill a good part of the view
        assert (depth > 0).all()  # the box fills the rest: no clear colour from this camera
        save_png(tmp_path / "view.png", img)
    sc = scenes.plain_uniform(20_000, 64, seed=7)
    with World(sc.plugin) as w:
        w.set_state(sc.pos_scale, sc.vfme)
        w.step(40)
        compare_view(w, 256, 256)


def test_render_view_custom_cameras(built_lib, cuda):
    """Other eyes, targets and fields of view: low over the floor, inside the box,
    wide and narrow; pixels off the box show the clear colour."""
    sc = scenes.plain_uniform(5_000, 32, seed=8)
    with World(sc.plugin) as w:
        w.set_state(sc.pos_scale, sc.vfme)
        w.step(25)
        _, depth, _ = compare_view(w, 200, 150, eye=(40.0, 6.0, 0.0), target=(0.0, 1.0, 0.0), fov=60.0)
        compare_view(w, 160, 160, eye=(0.0, 8.0, 12.0), target=(1.0, 0.0, -3.0), fov=90.0)
        compare_view(w, 96, 64, eye=(-5.0, 30.0, 30.0), target=(0.0, 0.0, 0.0), fov=15.0)
        _, depth, win = compare_view(w, 128, 128, eye=(0.0, 200.0, 400.0), target=(0.0, 0.0, 0.0), fov=30.0)
        assert (depth == 0).any() and (win > 0).any()  # far away: the box sits in the clear colour


def test_render_view_rejects_bad_cameras(built_lib, cuda):
    from bevy_millions_ball_gb300 import MbError
    sc = scenes.plain_uniform(100, 16, seed=1)
    with World(sc.plugin) as w:
        with pytest.raises(MbError):
            w.render_view(8, 8)  # no state yet
        w.set_state(sc.pos_scale, sc.vfme)
        with pytest.raises(MbError):
            w.render_view(8, 8, eye=(0.0, 10.0, 0.0), target=(0.0, 0.0, 0.0))  # vertical
        with pytest.raises(MbError):
            w.render_view(8, 8, eye=(1.0, 1.0, 1.0), target=(1.0, 1.0, 1.0))  # no direction
        with pytest.raises(MbError):
            w.render_view(8, 8, fov_y_degrees=180.0)
        with pytest.raises(MbError):
            w.render_view(0, 8)
