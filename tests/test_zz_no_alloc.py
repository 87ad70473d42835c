"""The render without device allocation (mypbr_gpu_render_noalloc), on the GPU.

Some callers may not allocate device memory while they render: a host
application that hands this library a fixed device-memory budget up front and
forbids allocation afterwards, or a per-frame callback of an interactive
viewer, where the device-wide synchronisation an allocation can cause would
stall the frame. For them the library keeps its render scratch in one static
18 MiB device array (at most 65,536 pixels per render).

This checks, through the C ABI, that two calls in a row give the frame the
allocating entry point (mypbr_gpu_render) gives for the same scene, camera and
seed. Both draw the same samples (the random numbers are keyed by pixel and
pass), so they differ only in the order FP64 film additions land: the bound is
1e-9 relative, far inside the Monte Carlo tolerances of the parity tests. It
also checks that a second call leaves the device's free memory unchanged, that
a smaller frame after a larger one carries nothing over, and that the pixel
limit applies to the rendered rows (a band of a wide frame renders). The file
is named so that pytest collects it last.
"""
import ctypes
import os

import numpy as np
import pytest

import mypbr_gb300 as mp
from conftest import scene_path

pytestmark = pytest.mark.gpu


def _bind():
    L = mp.lib()
    L.mypbr_gpu_render_noalloc.argtypes = [ctypes.c_void_p, ctypes.POINTER(mp.CameraStruct),
                                           ctypes.POINTER(mp.RenderOptsStruct), ctypes.c_void_p, ctypes.c_void_p,
                                           ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    L.mypbr_gpu_render_noalloc.restype = ctypes.c_int
    return L


def test_render_without_allocation_matches_render_twice():
    torch = pytest.importorskip("torch")
    L = _bind()
    scene = mp.load_scene(scene_path("cornell_c1.scene"))
    gpu = mp.GpuScene(scene)
    cam = scene.camera
    cam.image_width = 64
    cam.samples_per_pixel = 16
    cam.collect_features = 1
    cam.seed = 5
    ref = cam.render(gpu)  # the allocating entry point
    c, o = cam.structs()
    h, w = c.image_height, c.image_width
    dev = torch.device("cuda", 0)
    for call in range(2):
        # outputs prefilled with NaN: every pixel must be written
        rad = torch.full((h, w, 3), float("nan"), dtype=torch.float64, device=dev)
        alb = torch.full((h, w, 3), float("nan"), dtype=torch.float64, device=dev)
        nrm = torch.full((h, w, 3), float("nan"), dtype=torch.float64, device=dev)
        var = torch.full((h, w), float("nan"), dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        mp.check(L.mypbr_gpu_render_noalloc(gpu.handle, ctypes.byref(c), ctypes.byref(o), rad.data_ptr(),
                                            alb.data_ptr(), nrm.data_ptr(), var.data_ptr(), None))
        for got, want in ((rad, ref.radiance), (alb, ref.albedo), (nrm, ref.normal), (var, ref.variance)):
            np.testing.assert_allclose(got.cpu().numpy(), want, rtol=1e-9, atol=1e-12,
                                       err_msg=f"call {call + 1} differs from mypbr_gpu_render")


def _noalloc(L, gpu, cam, torch, rad=None):
    c, o = cam.structs()
    h, w = c.image_height, c.image_width
    if rad is None:
        rad = torch.full((h, w, 3), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    mp.check(L.mypbr_gpu_render_noalloc(gpu.handle, ctypes.byref(c), ctypes.byref(o), rad.data_ptr(), None, None,
                                        None, None))
    return rad.cpu().numpy()


def test_render_without_allocation_allocates_nothing_and_keeps_nothing():
    torch = pytest.importorskip("torch")
    L = _bind()
    scene = mp.load_scene(scene_path("cornell_c1.scene"))
    gpu = mp.GpuScene(scene)
    cam = scene.camera
    cam.samples_per_pixel = 8
    cam.seed = 9
    cam.image_width = 48
    big = _noalloc(L, gpu, cam, torch)  # warm-up: the first call looks up the array
    assert np.isfinite(big).all()
    cam.image_width = 24
    out = torch.full((cam.height(), 24, 3), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    free_before, _ = torch.cuda.mem_get_info()
    c, o = cam.structs()
    mp.check(L.mypbr_gpu_render_noalloc(gpu.handle, ctypes.byref(c), ctypes.byref(o), out.data_ptr(), None, None,
                                        None, None))
    torch.cuda.synchronize()
    free_after, _ = torch.cuda.mem_get_info()
    assert free_after == free_before, (free_before, free_after)
    # a smaller frame after a larger one: nothing of the first is left in it
    want = cam.render(gpu).radiance
    np.testing.assert_allclose(out.cpu().numpy(), want, rtol=1e-9, atol=1e-12)


def test_render_without_allocation_renders_a_band_of_a_wide_frame():
    """The limit is on the rendered rows: 12 rows of a 1920-wide frame
    (23,040 pixels of a 2,073,600-pixel image). Only the band is written."""
    torch = pytest.importorskip("torch")
    L = _bind()
    scene = mp.load_scene(scene_path("cornell_c1.scene"))
    gpu = mp.GpuScene(scene)
    cam = scene.camera
    cam.image_width = 1920
    cam.samples_per_pixel = 2
    cam.seed = 4
    cam.first_row = 700
    cam.row_count = 12
    got = _noalloc(L, gpu, cam, torch)
    want = cam.render(gpu).radiance
    band = slice(700, 712)
    np.testing.assert_allclose(got[band], want[band], rtol=1e-9, atol=1e-12)
    assert np.isnan(got[:700]).all() and np.isnan(got[712:]).all()
    cam.first_row = 0
    cam.row_count = 0


def test_render_without_allocation_rejects_large_images():
    torch = pytest.importorskip("torch")
    L = _bind()
    scene = mp.load_scene(scene_path("cornell_c1.scene"))
    gpu = mp.GpuScene(scene)
    cam = scene.camera
    cam.image_width = 257  # 257 x 257 > 65,536 pixels
    cam.samples_per_pixel = 1
    c, o = cam.structs()
    rad = torch.zeros((c.image_height, c.image_width, 3), dtype=torch.float64, device="cuda")
    status = L.mypbr_gpu_render_noalloc(gpu.handle, ctypes.byref(c), ctypes.byref(o), rad.data_ptr(), None, None,
                                        None, None)
    assert status == 5  # MYPBR_ERR_INVALID_ARGUMENT
    assert b"65536-pixel limit" in L.mypbr_last_error()
    cam.image_width = 1920  # 35 rows of 1920 = 67,200 pixels
    cam.row_count = 35
    c, o = cam.structs()
    status = L.mypbr_gpu_render_noalloc(gpu.handle, ctypes.byref(c), ctypes.byref(o), rad.data_ptr(), None, None,
                                        None, None)
    assert status == 5
    o.row_count = 0
    o.guided = 1
    cam.image_width = 64
    c, o = cam.structs()
    o.guided = 1
    status = L.mypbr_gpu_render_noalloc(gpu.handle, ctypes.byref(c), ctypes.byref(o), rad.data_ptr(), None, None,
                                        None, None)
    assert status == 2  # MYPBR_ERR_UNSUPPORTED
    assert b"guided rendering is not supported" in L.mypbr_last_error()
