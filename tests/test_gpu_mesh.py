"""DEM triangulation and vertex normals on the GPU against the host functions: bit-identical
positions, index buffers (with infinite posts skipped) and normals."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from vira_gb300 import capi, synthetic

pytestmark = pytest.mark.gpu


def _ctx():
    lib = capi.load()
    ctx = C.c_void_p()
    capi.check(lib.vgb_context_create(C.byref(ctx), 0), None, "context_create")
    return lib, ctx


def _host_dem(lib, h, posting):
    H, W = h.shape
    pos = np.empty((H * W, 3), np.float32)
    idx = np.empty((2 * (W - 1) * (H - 1), 3), np.uint32)
    nt = C.c_uint32(0)
    capi.check(lib.vgb_dem_triangulate(capi.ptr(h), W, H, posting, posting, capi.ptr(pos), capi.ptr(idx), C.byref(nt)))
    return pos, idx[: nt.value]


@pytest.mark.parametrize("holes", [False, True])
def test_dem_triangulation_and_normals_equal_host(gpu, holes):
    lib, ctx = _ctx()
    h = synthetic.fbm_heights(257, 0.8, seed=3, lo=-50.0, hi=50.0).astype(np.float32)
    W = h.shape[1]
    if holes:
        rng = np.random.default_rng(1)
        h.ravel()[rng.choice(h.size, 300, replace=False)] = np.inf
    hp, hi_ = _host_dem(lib, h, 7.5)
    H = h.shape[0]
    gpos = np.empty_like(hp)
    gidx = np.empty((2 * (W - 1) * (H - 1), 3), np.uint32)
    nt = C.c_uint32(0)
    capi.check(lib.vgb_dem_triangulate_gpu(ctx, capi.ptr(h), W, H, 7.5, 7.5, capi.ptr(gpos), capi.ptr(gidx),
                                           C.byref(nt), 0), ctx, "dem_gpu")
    assert nt.value == hi_.shape[0]
    assert np.array_equal(gpos.view(np.uint32), hp.view(np.uint32))
    assert np.array_equal(gidx[: nt.value], hi_)
    hn = np.empty_like(hp)
    capi.check(lib.vgb_compute_vertex_normals(capi.ptr(hp), hp.shape[0], capi.ptr(hi_), hi_.shape[0], capi.ptr(hn)))
    gn = np.empty_like(hp)
    capi.check(lib.vgb_compute_vertex_normals_gpu(ctx, capi.ptr(hp), hp.shape[0], capi.ptr(hi_), hi_.shape[0],
                                                  capi.ptr(gn), 0), ctx, "normals_gpu")
    assert np.array_equal(np.isnan(gn), np.isnan(hn))
    ok = ~np.isnan(hn)
    assert np.array_equal(gn[ok].view(np.uint32), hn[ok].view(np.uint32))
    lib.vgb_context_destroy(ctx)


def test_icosphere_normals_equal_host_and_bad_indices_are_rejected(gpu):
    lib, ctx = _ctx()
    v, f = synthetic.icosphere(5)
    p = (v * (250.0 + 5.0 * synthetic.real_sh_noise(v, 8, seed=2))[:, None]).astype(np.float32)
    f = np.ascontiguousarray(f, np.uint32)
    hn = np.empty_like(p)
    capi.check(lib.vgb_compute_vertex_normals(capi.ptr(p), p.shape[0], capi.ptr(f), f.shape[0], capi.ptr(hn)))
    gn = np.empty_like(p)
    capi.check(lib.vgb_compute_vertex_normals_gpu(ctx, capi.ptr(p), p.shape[0], capi.ptr(f), f.shape[0], capi.ptr(gn), 0),
               ctx, "normals_gpu")
    assert np.array_equal(gn.view(np.uint32), hn.view(np.uint32))
    bad = f.copy()
    bad[7, 1] = p.shape[0]
    assert lib.vgb_compute_vertex_normals_gpu(ctx, capi.ptr(p), p.shape[0], capi.ptr(bad), bad.shape[0], capi.ptr(gn), 0) != 0
    lib.vgb_context_destroy(ctx)
