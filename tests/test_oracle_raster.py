"""The oracle's restatement of CPURasterizer::render on the CPU: a known-answer square facing the
camera (coverage of the integer pixel corners, interpolated distance, face normal, the shared
edge going to the earlier triangle, the sun's radiance through the Lambertian BSDF), and the
camera's forward intrinsic matrix against its inverse."""
from __future__ import annotations

import math

import numpy as np

from oracle import oracle
from vira_gb300 import Camera, capi


def _square_camera(W=100, f=100.0):
    cam = capi.Camera()
    cam.width = cam.height = W
    rot = np.eye(3, dtype=np.float32)
    for k in range(9):
        cam.rotation[k] = float(rot.T.ravel()[k])
    cam.z_dir = 1.0
    for b in range(4):
        cam.power_scale[b] = 1.0
    K = np.array([f, 0.0, W / 2, 0.0, f, W / 2], np.float32)
    return cam, K


def test_square_known_answers():
    pos = np.array([[-1, -1, 10], [1, -1, 10], [1, 1, 10], [-1, 1, 10]], np.float32)
    idx = np.array([[0, 1, 2], [0, 2, 3]], np.uint32)
    alb = np.full((4, 4), 0.25, np.float32)
    osc = oracle.OracleScene(pos, idx, 4, albedo=alb)
    cam, K = _square_camera()
    L = (capi.Light * 1)()
    L[0].position[:] = [0.0, 0.0, 1.0e11]
    L[0].radius = 6.96e8
    for b in range(4):
        L[0].radiance[b] = 2.0e7
    out = osc.rasterize(cam, K, L, 1, True, False, np.ones((100, 100), np.float32))
    osc.close()
    cov = np.isfinite(out["depth"])
    ys, xs = np.nonzero(cov)
    assert cov.sum() == 400 and xs.min() == 40 and xs.max() == 59 and ys.min() == 40 and ys.max() == 59
    assert np.allclose(out["depth"][cov], math.sqrt(102.0), rtol=1e-6)
    assert np.all(np.isinf(out["alpha"][cov])) and np.all(out["alpha"][~cov] == 0)
    assert np.all(out["normal_global"][2][cov] == 1.0) and np.all(out["normal_global"][:2][:, cov] == 0.0)
    tid = out["triangle_id"]
    diag = cov & (np.arange(100)[None, :] == np.arange(100)[:, None])
    assert np.all(tid[diag] == 1)                       # the shared edge: the earlier triangle
    assert set(np.unique(tid[cov])) == {1, 2} and np.all(tid[~cov] == 0xFFFFFFFF)
    assert np.allclose(out["albedo"][:, cov], 0.25, rtol=1e-6)
    d = 1.0e11 - 10.0
    omega = 2 * math.pi * (1 - math.sqrt(d * d - 6.96e8 ** 2) / d)
    want = 2.0e7 * 0.25 / math.pi * omega
    # the pdf is 1/omega with omega in FP32, which loses ~0.3 % to cancellation for the sun's
    # tiny cap (the reference's arithmetic); every fragment sees the same distance here
    tr = out["total_radiance"][:, cov]
    assert float(np.ptp(tr)) <= 1e-5 * float(tr.mean())   # albedo interpolation rounds per fragment
    assert abs(float(tr[0, 0]) / want - 1.0) < 1e-2
    assert np.array_equal(out["received_power"], out["total_radiance"])   # power scale 1, omega 1


def test_triangles_behind_the_camera_are_culled():
    pos = np.array([[-1, -1, 10], [1, -1, 10], [1, 1, -1]], np.float32)   # one corner behind
    idx = np.array([[0, 1, 2]], np.uint32)
    osc = oracle.OracleScene(pos, idx, 4)
    cam, K = _square_camera()
    out = osc.rasterize(cam, K, None, 0, False, False)
    osc.close()
    assert not np.isfinite(out["depth"]).any()


def test_intrinsic_matrix_is_the_inverse_of_kinv():
    c = Camera()
    c.set_resolution(640, 480)
    c.set_sensor_size(0.036)
    c.set_field_of_view(35.0)
    for blender in (False, True):
        c.blender_frame = blender
        K = c.intrinsic_matrix().astype(np.float64)
        Ki = c.kinv().astype(np.float64)
        M = np.array([[K[0], K[1], K[2]], [K[3], K[4], K[5]], [0, 0, 1]])
        Mi = np.array([[Ki[0], Ki[2], Ki[4]], [Ki[1], Ki[3], Ki[5]], [0, 0, 1]])
        assert np.allclose(M @ Mi, np.eye(3), atol=1e-4)   # FP32 entries, principal point ~300 px


def test_square_triangle_size_and_velocity_passes():
    """The square's triangles project to right triangles with legs of 20 pixels: the triangle-size
    pass is the hypotenuse sqrt(800) (the longest projected edge, cpu_rasterizer.ipp:123-129);
    a static scene under a camera moving at v reads 0 global velocity and -v in the camera frame
    (identity rotation)."""
    pos = np.array([[-1, -1, 10], [1, -1, 10], [1, 1, 10], [-1, 1, 10]], np.float32)
    idx = np.array([[0, 1, 2], [0, 2, 3]], np.uint32)
    osc = oracle.OracleScene(pos, idx, 4)
    cam, K = _square_camera()
    cam.velocity[:] = [1.0, 2.0, 3.0]
    out = osc.rasterize(cam, K, None, 0, False, False, passes=True)
    osc.close()
    cov = np.isfinite(out["depth"])
    assert cov.sum() == 400
    assert np.all(out["triangle_size"][cov] == np.float32(math.sqrt(800.0)))
    assert np.all(np.isinf(out["triangle_size"][~cov]))
    assert np.all(out["velocity_global"] == 0.0)
    for k, v in enumerate((-1.0, -2.0, -3.0)):
        assert np.all(out["velocity_camera"][k][cov] == v) and np.all(out["velocity_camera"][k][~cov] == 0.0)
