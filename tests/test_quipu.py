"""DEM Quipu files on the CPU: the LZ4 block codec, the reader's index, heights and albedo, the
LoD choice and the writer, against the oracle's restatement of the format (oracle/quipu.py) and
against liblz4 1.9.4 (the reference's pinned LZ4), on the committed fixtures of tests/golden/
(written with liblz4's LZ4_compress_default by tests/golden/make_quipu.py).  No kernel runs here.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np
import pytest

from helpers import lz4_zero_run, quipu_with_claimed_lod
from oracle import quipu as Q
from vira_gb300 import capi
from vira_gb300 import quipu as VQ

GOLDEN = Path(__file__).resolve().parent / "golden"
FIXTURES = ["quipu_u16_lz4_color", "quipu_u8_raw_grey", "quipu_f32_lz4_constant", "quipu_noalbedo", "quipu_ogr"]


def _lz4_cases():
    rng = np.random.default_rng(0)
    walk = np.cumsum(rng.integers(-3, 4, 60000)).astype(np.uint16).tobytes()
    return [b"a", b"abc" * 3, bytes(rng.integers(0, 256, 3000, dtype=np.uint8)), bytes(70000),
            (b"abcd" * 5000) + bytes(rng.integers(0, 4, 20000, dtype=np.uint8)), walk,
            bytes(range(256)) * 300]


def _ours_decode(block: bytes, n: int):
    lib = capi.load()
    out = np.empty(max(n, 1), np.uint8)
    src = np.frombuffer(block, np.uint8) if block else np.zeros(1, np.uint8)
    got = lib.vgb_lz4_decompress(src.ctypes.data, len(block), out.ctypes.data, n)
    return got, out[:n].tobytes()


def _ours_encode(data: bytes) -> bytes:
    lib = capi.load()
    n = len(data)
    cap = lib.vgb_lz4_bound(n)
    dst = np.empty(cap, np.uint8)
    src = np.frombuffer(data, np.uint8) if n else np.zeros(1, np.uint8)
    cs = lib.vgb_lz4_compress(src.ctypes.data, n, dst.ctypes.data, cap)
    assert cs > 0
    return dst[:cs].tobytes()


def test_lz4_decoders_match_liblz4():
    if Q.liblz4() is None:
        pytest.skip("liblz4 is not installed")
    assert Q.liblz4().LZ4_versionNumber() == 10904   # 1.9.4, the version the reference pins
    for data in _lz4_cases():
        blk = Q.lz4_compress_reference(data)
        got, out = _ours_decode(blk, len(data))
        assert got == len(data) and out == data
        assert Q.lz4_decompress(blk, len(data)) == data


def test_lz4_encoder_blocks_decode_with_liblz4():
    lib = Q.liblz4()
    for data in _lz4_cases() + [b""]:
        blk = _ours_encode(data)
        got, out = _ours_decode(blk, len(data))
        assert got == len(data) and out == data
        if lib is not None:
            back = C.create_string_buffer(max(len(data), 1))
            src = C.create_string_buffer(blk, len(blk))
            assert lib.LZ4_decompress_safe(src, back, len(blk), len(data)) == len(data)
            assert back.raw[: len(data)] == data


def test_lz4_rejects_malformed_blocks():
    data = (b"quipu heights " * 400)
    blk = _ours_encode(data)
    n = len(data)
    assert _ours_decode(blk, n)[0] == n
    assert _ours_decode(blk, n - 1)[0] == -1            # output would overrun
    assert _ours_decode(blk[:-3], n)[0] == -1           # truncated
    assert _ours_decode(b"", n)[0] == -1
    assert _ours_decode(bytes([0x04, 0x00, 0x00, 0x00]), 64)[0] == -1   # offset 0
    assert _ours_decode(bytes([0x14, ord("a"), 0x05, 0x00, 0x00]), 64)[0] == -1  # offset past the start
    for bad in (blk[:-3], bytes([0x04, 0x00, 0x00, 0x00])):
        with pytest.raises(ValueError):
            Q.lz4_decompress(bad, n)


def test_fixture_index_matches_the_oracle():
    for name in FIXTURES:
        path = GOLDEN / f"{name}.qld"
        o = Q.read(path)
        q = VQ.DEMQuipu(path)
        assert q.class_id == o.class_id == 2002
        assert q.number_of_lods == o.num_lods and q.has_albedos() == o.has_albedos
        assert np.array_equal(q.position, np.array(o.position))
        assert np.array_equal(q.rotation.T.ravel(), np.array(o.rotation))
        assert np.array_equal(q.scale, np.array(o.scale))
        assert np.array_equal(q.normal, np.array(o.normal, np.float32)) and q.cone_angle == np.float32(o.cone_angle)
        for L, OL in zip(q.lods, o.lods):
            pr, opr = L.projection, OL.projection
            assert (L.gsd, L.offset) == (OL.gsd, OL.offset)
            assert (L.width, L.height) == (OL.heights.w, OL.heights.h)
            assert (pr.width, pr.height, tuple(pr.pixel_scale)) == (opr["width"], opr["height"], opr["pixel_scale"])
            assert (pr.xoff, pr.yoff, pr.dx, pr.dy, bool(pr.is_ogr)) == (opr["xoff"], opr["yoff"], opr["dx"], opr["dy"],
                                                                        opr["is_ogr"])
            assert (tuple(pr.tile_definitions), pr.tile_row, pr.tile_col) == (opr["tile_definitions"], opr["tile_row"],
                                                                              opr["tile_col"])
            if opr["is_ogr"]:
                assert tuple(pr.model_tie_point) == opr["model_tie_point"]
            assert (L.height_min, L.height_max) == (OL.hmin, OL.hmax)
            assert L.precision == OL.precision and bool(L.compressed) == OL.heights.compressed
            at = capi.QUIPU_NO_ALBEDO if OL.albedo_type is None else OL.albedo_type
            assert L.albedo_type == at
            if at == Q.COLOR_IMAGE_ALBEDO:
                assert L.albedo_channels == len(OL.planes)
        q.close()


def test_fixture_heights_and_albedo_match_the_oracle():
    for name in FIXTURES:
        path = GOLDEN / f"{name}.qld"
        o = Q.read(path)
        q = VQ.DEMQuipu(path, nbands=4)
        for i, OL in enumerate(o.lods):
            h = q.read_heights(i)
            assert np.array_equal(h, Q.heights(OL), equal_nan=True), (name, i)
            a = q.read_albedo(i)
            if OL.albedo_type is None:
                assert a is None
            elif OL.albedo_type == Q.CONSTANT_ALBEDO:
                assert np.array_equal(a, np.frombuffer(OL.constant_bytes[:16], np.float32))
            else:
                ref = np.stack([Q.fixed_to_float(img.pixels, mn, mx) for mn, mx, img in OL.planes], 2)
                assert np.array_equal(a.reshape(ref.shape[0], ref.shape[1], -1), ref)
        q.close()


def test_fixture_decode_follows_the_fixed_point_rule():
    """Decoded heights sit within one quantum above the source DEM (the reference's code is
    trunc((m-1) v + 1), decoded as code/(m-1)); non-finite posts decode to +inf."""
    src = np.load(GOLDEN / "quipu_sources.npz")
    for name, key in (("quipu_u16_lz4_color", "u16_heights"), ("quipu_u8_raw_grey", "u8_heights"),
                      ("quipu_f32_lz4_constant", "f32_heights"), ("quipu_noalbedo", "noalb_heights")):
        o = Q.read(GOLDEN / f"{name}.qld")
        L = o.lods[0]
        z = src[key]
        h = Q.heights(L)
        fin = np.isfinite(z)
        if L.precision == Q.CLS_FLOAT:
            assert np.array_equal(h, z, equal_nan=True)
            continue
        m = 255.0 if L.precision == Q.CLS_U8 else 65535.0
        q = (float(L.hmax) - float(L.hmin)) / (m - 1.0)
        d = h[fin].astype(np.float64) - z[fin]
        assert d.min() >= -1e-3 * q - 1e-4 and d.max() <= 1.001 * q + 1e-4, (name, d.min(), d.max(), q)
        assert np.all(np.isinf(h[~fin]))


def test_select_lod_follows_read_buffers():
    path = GOLDEN / "quipu_u16_lz4_color.qld"
    q = VQ.DEMQuipu(path)
    o = Q.read(path)
    assert q.gsds == [10.0, 20.0, 40.0]
    for g, want in ((1.0, 0), (10.0, 0), (15.0, 0), (20.0, 1), (39.9, 1), (40.0, 2), (1e9, 2), (float("inf"), 2)):
        assert q.select_lod(g) == want == Q.select_lod(o, g), g
    q.close()


def _dems(kind):
    from vira_gb300 import synthetic

    z = np.ascontiguousarray(synthetic.fbm_heights(37, 0.8, seed=5, lo=-50.0, hi=80.0)[:29, :37], np.float32)
    z[4, 5] = np.inf
    z[9, 20] = np.nan
    if kind == "u8":
        ps = (200.0, 200.0)
    elif kind == "u16":
        ps = (10.0, 10.0)
    else:
        ps = (0.01, 0.01)
    g = np.ascontiguousarray(synthetic.lognormal_albedo(37, 0.12, 0.3, seed=6)[:29, :37], np.float32)
    col = np.ascontiguousarray(np.stack([g, 0.5 * g, np.full_like(g, 0.2), g * g], 2))  # one flat channel
    out = []
    for f in (1, 2):
        zz = np.ascontiguousarray(z[::f, ::f])
        proj = VQ.DEMProjection(zz.shape[1], zz.shape[0], ps, (2, 3), 1, 0, 5.0, 7.0, float(f), float(f))
        out.append((zz, proj, np.ascontiguousarray(g[::f, ::f]), np.ascontiguousarray(col[::f, ::f])))
    return out


def _oracle_lods(dems, atype):
    lods = []
    for zz, proj, g, col in dems:
        a = {Q.CONSTANT_ALBEDO: np.array([0.1, 0.2, 0.3, 0.4], np.float32), Q.FLOAT_IMAGE_ALBEDO: g,
             Q.COLOR_IMAGE_ALBEDO: col}[atype]
        pr = Q.projection(proj.width, proj.height, proj.pixel_scale, proj.dx, proj.dy, proj.xoff, proj.yoff,
                          (proj.tile_definitions[0], proj.tile_definitions[1], proj.tile_row, proj.tile_col))
        lods.append(dict(heights=zz, projection=pr, albedo_type=atype, albedo=a))
    return lods


@pytest.mark.parametrize("kind", ["u8", "u16", "f32"])
@pytest.mark.parametrize("atype", [Q.CONSTANT_ALBEDO, Q.FLOAT_IMAGE_ALBEDO, Q.COLOR_IMAGE_ALBEDO])
def test_writer_bytes_equal_the_oracle_writer(tmp_path, kind, atype):
    """Raw payloads: the product's file is byte-identical to the oracle's restatement of
    DEMQuipu::write (header, normal cone, table, projections, fixed point, column order; a
    flat albedo channel goes through the reference's 0/0 and is stored as code 0)."""
    dems = _dems(kind)
    olods = _oracle_lods(dems, atype)
    Q.write(tmp_path / "oracle", olods, position=(1.0, 2.0, 3.0), scale=(1.0, 1.0, 2.0), compress=False)
    pyr = [VQ.DEM(L["heights"], VQ.DEMProjection(**{k: v for k, v in L["projection"].items() if k != "is_ogr"}),
                  L["albedo"], atype) for L in olods]
    VQ.DEMQuipu.write(tmp_path / "ours.bin", pyr, position=(1.0, 2.0, 3.0), scale=(1.0, 1.0, 2.0),
                      options=VQ.DEMQuipuWriterOptions(compress=False))
    a = (tmp_path / "oracle.qld").read_bytes()
    b = (tmp_path / "ours.qld").read_bytes()    # the .qld extension is forced, as in the reference
    assert len(a) == len(b)
    assert a == b
    o = Q.read(tmp_path / "ours.qld")
    assert o.lods[0].precision == {"u8": Q.CLS_U8, "u16": Q.CLS_U16, "f32": Q.CLS_FLOAT}[kind]


def test_compressed_writer_round_trips(tmp_path):
    dems = _dems("u16")
    pyr = [VQ.DEM(zz, proj, col, Q.COLOR_IMAGE_ALBEDO) for zz, proj, g, col in dems]
    VQ.DEMQuipu.write(tmp_path / "c", pyr, options=VQ.DEMQuipuWriterOptions(compress=True))
    VQ.DEMQuipu.write(tmp_path / "r", pyr, options=VQ.DEMQuipuWriterOptions(compress=False))
    oc, orr = Q.read(tmp_path / "c.qld"), Q.read(tmp_path / "r.qld")
    assert all(L.heights.compressed for L in oc.lods)
    for Lc, Lr in zip(oc.lods, orr.lods):
        assert np.array_equal(Lc.heights.pixels, Lr.heights.pixels)
        for (a, b, ia), (c, d, ib) in zip(Lc.planes, Lr.planes):
            assert (a, b) == (c, d) and np.array_equal(ia.pixels, ib.pixels)
    q = VQ.DEMQuipu(tmp_path / "c.qld", nbands=4)
    assert np.array_equal(q.read_heights(1), Q.heights(oc.lods[1]))
    q.close()



def test_product_blocks_decode_with_liblz4(tmp_path, monkeypatch):
    """Every LZ4 block the product writes decodes with liblz4's LZ4_decompress_safe to the
    pixels the oracle's own decoder gives."""
    lib = Q.liblz4()
    if lib is None:
        pytest.skip("liblz4 is not installed")
    dems = _dems("u16")
    pyr = [VQ.DEM(zz, proj, col, Q.COLOR_IMAGE_ALBEDO) for zz, proj, g, col in dems]
    VQ.DEMQuipu.write(tmp_path / "c", pyr, options=VQ.DEMQuipuWriterOptions(compress=True))
    want = Q.read(tmp_path / "c.qld")
    calls = []

    def via_liblz4(block, raw_size):
        out = C.create_string_buffer(max(raw_size, 1))
        src = C.create_string_buffer(block, len(block))
        assert lib.LZ4_decompress_safe(src, out, len(block), raw_size) == raw_size
        calls.append(raw_size)
        return out.raw[:raw_size]

    monkeypatch.setattr(Q, "lz4_decompress", via_liblz4)
    got = Q.read(tmp_path / "c.qld")
    assert len(calls) == 2 * (1 + 4)
    for a, b in zip(got.lods, want.lods):
        assert np.array_equal(a.heights.pixels, b.heights.pixels)
        assert all(np.array_equal(x[2].pixels, y[2].pixels) for x, y in zip(a.planes, b.planes))


def test_reader_errors(tmp_path):
    bad = tmp_path / "bad.qld"
    bad.write_bytes(b"QUIPX" + bytes(200))
    with pytest.raises(capi.VgbError, match="not a valid Quipu"):
        VQ.DEMQuipu(bad)
    with pytest.raises(capi.VgbError, match="no file"):
        VQ.DEMQuipu(tmp_path / "missing.qld")
    data = (GOLDEN / "quipu_u16_lz4_color.qld").read_bytes()
    for cut in (7, 60, 200, 260, 400, len(data) // 2, len(data) - 10):
        t = tmp_path / f"cut{cut}.qld"
        t.write_bytes(data[:cut])
        with pytest.raises(capi.VgbError):
            q = VQ.DEMQuipu(t, nbands=4)
            for i in range(q.number_of_lods):
                q.read_heights(i)
                q.read_albedo(i)
    # a corrupted LZ4 block: the stored block size grows past the file
    o = Q.read(GOLDEN / "quipu_noalbedo.qld")
    q = VQ.DEMQuipu(GOLDEN / "quipu_noalbedo.qld")
    assert q.lods[0].compressed
    q.close()
    raw = bytearray((GOLDEN / "quipu_noalbedo.qld").read_bytes())
    pos = o.lods[0].offset + 73 + 8 + 2 + 2 + 8 + 1 + 8      # projection, min/max, class, image head, raw size
    raw[pos:pos + 8] = (10 ** 6).to_bytes(8, "little")
    t = tmp_path / "blk.qld"
    t.write_bytes(bytes(raw))
    with pytest.raises(capi.VgbError):
        VQ.DEMQuipu(t)
    # a block whose bytes are flipped decodes to an error or to some pixels, never past the buffer
    raw = bytearray((GOLDEN / "quipu_noalbedo.qld").read_bytes())
    for k in range(pos + 8, len(raw), 7):
        raw[k] ^= 0x5A
    t.write_bytes(bytes(raw))
    q = VQ.DEMQuipu(t)
    try:
        q.read_heights(0)
    except capi.VgbError as e:
        assert "LZ4" in str(e)
    q.close()
    # channel count of a per-band albedo must match the reader's bands
    q = VQ.DEMQuipu(GOLDEN / "quipu_u16_lz4_color.qld")
    out = np.empty((49, 65, 3), np.float32)
    assert capi.load().vgb_quipu_read_albedo(q._h, 0, 3, capi.ptr(out)) != 0
    assert b"channels" in capi.load().vgb_quipu_last_error()
    q.close()


def test_claimed_sizes_are_bounded_before_allocation(tmp_path):
    """An LZ4 block expands at most 255-fold, so a height image claiming more is refused when the
    file opens, before a buffer of the claimed size exists; a block at the largest expansion is a
    valid file (all codes 0: no-data, +inf).  A LoD of 2^31 posts or more is refused before its
    mesh arrays are allocated (triangle ids are 32-bit)."""
    t = quipu_with_claimed_lod(tmp_path / "claim.qld", 4000, 4000, block=lz4_zero_run(1000))
    with pytest.raises(capi.VgbError, match="bad or truncated height image"):
        VQ.DEMQuipu(t)
    q = VQ.DEMQuipu(quipu_with_claimed_lod(tmp_path / "run.qld", 300, 200))
    h = q.read_heights(0)
    assert h.shape == (200, 300) and np.isposinf(h).all()
    q.close()
    q = VQ.DEMQuipu(quipu_with_claimed_lod(tmp_path / "big.qld", 50000, 50000))
    assert (q.lods[0].width, q.lods[0].height) == (50000, 50000)
    with pytest.raises(capi.VgbError, match="2\\^31"):
        q.read_lod_mesh(0)
    q.close()


def test_writer_rejects_bad_pyramids(tmp_path):
    z = np.zeros((4, 4), np.float32)
    p = VQ.DEMProjection(4, 4)
    with pytest.raises(capi.VgbError, match="albedo type"):
        VQ.DEMQuipu.write(tmp_path / "x", [VQ.DEM(z, p, np.ones(4, np.float32), 0),
                                           VQ.DEM(z, p, np.ones((4, 4), np.float32), 1)])
    ogr = VQ.DEMProjection(4, 4, is_ogr=True)
    with pytest.raises(capi.VgbError, match="GDAL"):
        VQ.DEMQuipu.write(tmp_path / "y", [VQ.DEM(z, ogr, None)])
    with pytest.raises(capi.VgbError):
        VQ.DEMQuipu.write(tmp_path / "z", [VQ.DEM(np.zeros((1, 4), np.float32), VQ.DEMProjection(4, 1), None)])


def test_read_pyramid_and_transformation():
    q = VQ.DEMQuipu(GOLDEN / "quipu_u16_lz4_color.qld", nbands=4)
    pyr = q.read_pyramid()
    assert [d.heights.shape for d in pyr] == [(49, 65), (25, 33), (13, 17)]
    assert [d.get_gsd() for d in pyr] == [(10.0, 10.0), (20.0, 20.0), (40.0, 40.0)]
    T = q.get_transformation()
    assert np.allclose(T[:3, 3], [1.0e3, -2.0e3, 3.5e2])
    assert np.allclose(T[:3, :3], [[0.0, -1.0, 0.0], [1.0, 0.0, 0.0], [0.0, 0.0, 1.0]])
    q.close()
    q = VQ.DEMQuipu(GOLDEN / "quipu_noalbedo.qld", VQ.DEMQuipuReaderOptions(default_albedo=0.2), nbands=2)
    d = q.read_pyramid()[0]
    assert d.albedo_type == VQ.CONSTANT_ALBEDO and np.array_equal(d.albedo, np.full(2, 0.2, np.float32))
    q.close()
