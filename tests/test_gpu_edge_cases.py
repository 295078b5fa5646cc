"""Edge cases of the render against the oracle: a scene without lights (ambient and background
only), a DEM with holes (posts at +inf leave no triangles, cpu: image_utils.ipp:371-404), frames
of one pixel, one row and one column, and a camera that sees nothing but sky.  Direct lighting
with deterministic light sampling: triangle ids bit-exact, planes within 1e-4 relative."""
from __future__ import annotations

import numpy as np
import pytest

from helpers import gpu_render_host, oracle_render, rel_err
from vira_gb300 import FOUR_BAND, Mesh, Scene, capi, synthetic

pytestmark = pytest.mark.gpu

PLANES = ("total_radiance", "direct_radiance", "indirect_radiance", "albedo", "normal_global", "depth", "alpha")


def _scene(holes=False, sun=True, res=(48, 40)):
    h = synthetic.fbm_heights(65, 0.8, seed=12, lo=-60.0, hi=60.0)
    if holes:
        h = h.copy()
        h[10:20, 30:45] = np.inf
        h[40, 5] = np.inf
    s = Scene(FOUR_BAND)
    s.add_mesh(Mesh.from_dem(h, 20.0, albedo=0.14, nbands=4))
    s.new_instance(("mesh", 0))
    if sun:
        sid = s.new_sun(5778.0)
        s.set_sun_direction(sid, 20.0, 40.0)
    cid = s.new_camera()
    c = s[cid]
    c.set_resolution(*res)
    c.set_sensor_size(0.036)
    c.set_field_of_view(50.0)
    c.set_local_position(640.0, -900.0, 1500.0)
    c.look_at((640.0, 640.0, 0.0))
    pt = s.pathtracer
    pt.options.samples = 2
    pt.options.deterministic_light = True
    pt.render_passes.simulate_lighting = True
    return s, cid


def _compare(s, cid):
    g = gpu_render_host(s, cid)
    o, counts = oracle_render(s, cid)
    assert np.array_equal(g["triangle_id"], o["triangle_id"])
    for k in PLANES:
        assert float(rel_err(g[k], o[k]).max()) <= 1e-4, k
    st = s.pathtracer.last_stats
    assert st.rays_closest == counts[0] and st.rays_shadow == counts[1]
    return g, o


def test_no_lights_ambient_and_background(gpu):
    s, cid = _scene(sun=False)
    s.set_ambient(0.05)
    s.set_background_emission(0.2)
    s.pathtracer.options.show_background = True
    g, _ = _compare(s, cid)
    assert s.pathtracer.last_stats.rays_shadow == 0
    hit = g["triangle_id"] != capi.NO_HIT
    assert hit.any() and (~hit).any()
    assert (g["total_radiance"][:, hit] > 0).all() and (g["total_radiance"][:, ~hit] > 0).all()
    s.close()


def test_dem_with_holes(gpu):
    s, cid = _scene(holes=True)
    g, _ = _compare(s, cid)
    assert (g["triangle_id"] == capi.NO_HIT).any()
    s.close()


@pytest.mark.parametrize("res", [(1, 1), (57, 1), (1, 43)], ids=["1x1", "row", "column"])
def test_degenerate_frame_shapes(gpu, res):
    s, cid = _scene(res=res)
    _compare(s, cid)
    s.close()


def test_camera_sees_only_sky(gpu):
    s, cid = _scene()
    s[cid].look_at((640.0, -5000.0, 6000.0))   # up and away from the terrain
    g, _ = _compare(s, cid)
    assert np.all(g["triangle_id"] == capi.NO_HIT)
    assert np.all(np.isinf(g["depth"])) and np.all(g["alpha"] == 0)
    assert s.pathtracer.last_stats.rays_shadow == 0
    s.close()
