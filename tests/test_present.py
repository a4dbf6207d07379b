"""Headless presentation: VK_EXT_headless_surface + VK_KHR_swapchain.

The reference presents with GDI (wsi.cpp); here a swapchain's images stay in
device memory and vkQueuePresentKHR copies the presented image to a pinned host
copy in queue order.  With VSD_PRESENT the harness renders target 0 into an
acquired swapchain image, presents after every submit and reads the frame back
from the present, which must equal the oracle's frame.
"""
import os

import numpy as np
import pytest

import visor_gb300 as vg
from oracle import loader
import scenes_edge

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def device():
    d = vg.Device()
    yield d
    d.close()


@pytest.mark.parametrize("name", ["cfg1_sphere", "blend_overlap", "load_pass", "cfg4_small"])
def test_presented_frame_equals_oracle(device, name):
    h = scenes_edge.build(device.lib, name)
    cols, deps, _ = loader.Oracle().render(h)
    up = device.upload(h, vg.PRESENT)
    try:
        for _ in range(3):  # the second and third submits replay a CUDA graph
            up.submit()
            got_c, got_d = up.read()
            for a, b in zip(got_c, cols):
                assert np.array_equal(a, b)
            for a, b in zip(got_d, deps):
                assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    finally:
        up.release()


def test_present_writes_ppm_frames(device, tmp_path, monkeypatch):
    monkeypatch.setenv("VISOR_GB300_PRESENT_DIR", str(tmp_path))
    h = scenes_edge.build(device.lib, "cfg1_sphere")
    cols, _, _ = loader.Oracle().render(h)
    up = device.upload(h, vg.PRESENT)
    try:
        up.submit()
        up.submit()
    finally:
        up.release()
    frames = sorted(os.listdir(tmp_path))
    assert frames == ["frame_000000.ppm", "frame_000001.ppm"]
    data = open(tmp_path / frames[-1], "rb").read()
    w, hgt = h.targets()[0]
    header = f"P6\n{w} {hgt}\n255\n".encode()
    assert data.startswith(header)
    rgb = np.frombuffer(data[len(header):], np.uint8).reshape(hgt, w, 3)
    bgra = cols[0].reshape(hgt, w, 4)
    assert np.array_equal(rgb, bgra[..., [2, 1, 0]])


def test_surface_queries(device):
    """Extension lists and surface capabilities a headless client relies on."""
    import ctypes as C
    L = device.lib
    gpa = L.vk_icdGetInstanceProcAddr
    gpa.restype = C.c_void_p
    gpa.argtypes = [C.c_void_p, C.c_char_p]
    for name in (b"vkCreateHeadlessSurfaceEXT", b"vkDestroySurfaceKHR", b"vkCreateSwapchainKHR",
                 b"vkQueuePresentKHR", b"vkAcquireNextImageKHR", b"vkGetSwapchainImagesKHR",
                 b"vkGetPhysicalDeviceSurfaceCapabilitiesKHR"):
        assert gpa(None, name), name
