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
