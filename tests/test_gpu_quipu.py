"""DEM Quipu LoDs read into device meshes (vgb_quipu_read_mesh) against the oracle.

For every LoD of the committed fixtures: positions (DEM::makeVertexBuffer through the non-OGR
DEMProjection, tile offsets and dx included), indices (imageToIndexBuffer), per-vertex albedo
(constant / grey x profile / per band, Vertex's default 1 on no-data posts) and vertex normals
(Mesh::calculateNormals) are bit-identical to the oracle's restatement.  A 2049^2 pyramid written
by the product and read on the GPU matches the host triangulation of its decoded heights.
"""
from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

from oracle import oracle
from oracle import quipu as Q
from vira_gb300 import capi, synthetic
from vira_gb300 import quipu as VQ

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"
MESH_FIXTURES = ["quipu_u16_lz4_color", "quipu_u8_raw_grey", "quipu_f32_lz4_constant", "quipu_noalbedo"]


def _eq(a, b):
    return np.array_equal(np.asarray(a), np.asarray(b), equal_nan=True)


@pytest.mark.parametrize("name", MESH_FIXTURES)
def test_lod_meshes_match_the_oracle(gpu, name):
    path = GOLDEN / f"{name}.qld"
    o = Q.read(path)
    q = VQ.DEMQuipu(path, nbands=4)
    for i, L in enumerate(o.lods):
        pos, idx, alb, nrm = q.read_lod_mesh(i, gpu=0)
        h = Q.heights(L)
        opos = Q.vertex_positions(h, L.projection)
        oidx = Q.index_buffer(h)
        oalb = Q.vertex_albedo(L, h, 4)
        onrm = oracle.compute_normals(opos, oidx)
        assert _eq(pos, opos), (name, i, "positions")
        assert _eq(idx, oidx), (name, i, "indices")
        assert _eq(alb, oalb), (name, i, "albedo")
        assert _eq(nrm, onrm), (name, i, "normals")
        dpos, didx, dalb, dnrm = q.read_lod_mesh(i, gpu=0, device_arrays=True)
        assert _eq(dpos.cpu().numpy(), pos) and _eq(didx.cpu().numpy().astype(np.uint32), idx)
        assert _eq(dalb.cpu().numpy(), alb) and _eq(dnrm.cpu().numpy(), nrm)
    q.close()


def test_reader_options(gpu):
    # grey albedo times a per-band profile
    path = GOLDEN / "quipu_u8_raw_grey.qld"
    o = Q.read(path)
    prof = np.array([0.5, 1.0, 1.5, 2.0], np.float32)
    q = VQ.DEMQuipu(path, VQ.DEMQuipuReaderOptions(albedo_profile=prof), nbands=4)
    _, _, alb, _ = q.read_lod_mesh(0)
    h = Q.heights(o.lods[0])
    assert _eq(alb, Q.vertex_albedo(o.lods[0], h, 4, profile=prof))
    q.close()
    # albedo not read: the default for every finite post
    q = VQ.DEMQuipu(path, VQ.DEMQuipuReaderOptions(read_albedos=False, default_albedo=0.3), nbands=3)
    _, _, alb, _ = q.read_lod_mesh(1)
    assert _eq(alb, Q.vertex_albedo(o.lods[1], Q.heights(o.lods[1]), 3, read_albedos=False, default_albedo=0.3))
    q.close()
    # per-band albedo with the wrong band count
    q = VQ.DEMQuipu(GOLDEN / "quipu_u16_lz4_color.qld", nbands=3)
    with pytest.raises(capi.VgbError, match="channels"):
        q.read_lod_mesh(0)
    q.close()
    # map-projected LoDs need GDAL
    q = VQ.DEMQuipu(GOLDEN / "quipu_ogr.qld", nbands=1)
    with pytest.raises(capi.VgbError, match="GDAL"):
        q.read_lod_mesh(0)
    q.close()


def test_lod_beyond_32_bit_triangle_ids_is_refused(gpu, tmp_path):
    # 50000^2 posts (9.8 MB on disk at LZ4's largest expansion): the C entry refuses it before it
    # reads a pixel or writes the (here one-element) output arrays
    import ctypes as C

    from helpers import quipu_with_claimed_lod
    from vira_gb300.scene import _mesh_context

    q = VQ.DEMQuipu(quipu_with_claimed_lod(tmp_path / "big.qld", 50000, 50000), nbands=1)
    lib = capi.load()
    ctx = _mesh_context(0)
    one = [np.zeros(4, np.float32) for _ in range(3)]
    idx = np.zeros(4, np.uint32)
    nt = C.c_uint32(7)
    st = lib.vgb_quipu_read_mesh(ctx, q._h, 0, C.byref(q._read_options(1)), capi.ptr(one[0]), capi.ptr(one[1]),
                                 capi.ptr(one[2]), capi.ptr(idx), C.byref(nt), 0)
    assert st == 1 and b"2^31" in lib.vgb_last_error(ctx)
    assert nt.value == 7 and not idx.any() and not any(a.any() for a in one)
    q.close()


def test_read_buffers_picks_the_lod_once(gpu):
    q = VQ.DEMQuipu(GOLDEN / "quipu_u16_lz4_color.qld", nbands=4)
    m = q.read_buffers(25.0)
    assert m is not None and m.positions.shape == (33 * 25, 3) and q.current_gsd == 20.0
    assert q.read_buffers(30.0) is None          # same LoD: no update (dem_quipu.ipp:154-159)
    m = q.read_buffers(100.0)
    assert m.positions.shape == (17 * 13, 3) and q.current_gsd == 40.0
    assert q.default_gsd == 20.0
    q.close()


def test_large_pyramid_round_trip(gpu, tmp_path):
    n = 2049
    z = synthetic.fbm_heights(n, 0.8, seed=8, lo=-150.0, hi=150.0)
    z = synthetic.add_crater_field(z, 2.0, seed=9, dmin=20, dmax=600)
    z = np.ascontiguousarray(z, np.float32)
    z[100:140, 200:260] = np.inf
    dem = VQ.DEM(z, VQ.DEMProjection(n, n, (2.0, 2.0)), np.array([0.12], np.float32), VQ.CONSTANT_ALBEDO)
    pyr = [dem, dem.downsample(4)]
    VQ.DEMQuipu.write(tmp_path / "big", pyr, options=VQ.DEMQuipuWriterOptions(compress=True))
    q = VQ.DEMQuipu(tmp_path / "big.qld", nbands=1)
    assert q.lods[0].precision == 4 and q.lods[0].compressed
    h = q.read_heights(0)
    pos, idx, alb, nrm = q.read_lod_mesh(0)
    lib = capi.load()
    hp = np.empty((n * n, 3), np.float32)
    hi = np.empty((2 * (n - 1) ** 2, 3), np.uint32)
    import ctypes as C

    nt = C.c_uint32(0)
    capi.check(lib.vgb_dem_triangulate(capi.ptr(h), n, n, 2.0, 2.0, capi.ptr(hp), capi.ptr(hi), C.byref(nt)))
    assert _eq(pos, hp) and _eq(idx, hi[: nt.value])
    hn = np.empty_like(hp)
    capi.check(lib.vgb_compute_vertex_normals(capi.ptr(hp), n * n, capi.ptr(hi), nt.value, capi.ptr(hn)))
    assert _eq(nrm, hn)
    fin = np.isfinite(h.ravel())
    assert np.all(alb[fin] == np.float32(0.12)) and np.all(alb[~fin] == 1.0)
    q.close()


def test_level_of_detail_manager_swaps_quipu_lods(gpu):
    import torch

    from vira_gb300 import FOUR_BAND, Mesh, Scene

    path = GOLDEN / "quipu_u16_lz4_color.qld"
    s = Scene(FOUR_BAND)
    m = Mesh.from_quipu(path, nbands=4)
    assert m.gsd() == 40.0 and m.positions.shape[0] == 17 * 13      # the default: the coarsest LoD
    s.add_mesh(m)
    s.new_instance(("mesh", 0))
    sun = s.new_sun(5778.0)
    s.set_sun_direction(sun, 20.0, 40.0)
    cid = s.new_camera()
    c = s[cid]
    c.set_resolution(256, 256)
    c.set_sensor_size(0.036)
    c.set_field_of_view(30.0)
    c.set_local_position(100.0, -150.0, 1500.0)
    c.look_at((0.0, 0.0, 0.0))
    s.pathtracer.options.samples = 2
    s.pathtracer.render_passes.simulate_lighting = True
    s.pathtracer.render(c, s)
    assert s.update_level_of_detail(cid) == 1
    assert m.gsd() == 10.0 and m.positions.shape[0] == 65 * 49
    q = VQ.DEMQuipu(path, nbands=4)
    pos, idx, alb, nrm = q.read_lod_mesh(0)
    q.close()
    assert _eq(m.positions, pos) and _eq(m.indices, idx) and _eq(m.normals, nrm)
    rp = s.pathtracer.render(c, s)
    torch.cuda.synchronize()
    tid = rp.triangle_id.cpu().numpy()
    assert (tid >= 0).mean() > 0.3 and tid.max() < idx.shape[0]   # the fine LoD's triangles
    c.set_local_position(100.0, -150.0, 40000.0)
    assert s.update_level_of_detail(cid) == 1 and m.gsd() == 40.0
    s.close()
