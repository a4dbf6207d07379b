"""Mip chains built on the GPU with vkCmdBlitImage.

The scene generator box-filters every RGBA8 mip on the host ((a + b + c + d + 2)
>> 2 per channel).  Uploaded with VSD_GPU_MIPS, a texture sends only mip 0 and
the upload command buffer blits each level from the one above (2:1, linear),
which the blit kernel computes with the same rounding.  Trilinear rendering
reads every level, so frames must equal the oracle's bit for bit.
"""
import numpy as np
import pytest

import visor_gb300 as vg
from oracle import loader
import scenes_edge

pytestmark = pytest.mark.gpu

VSD_GPU_MIPS = 4


@pytest.fixture(scope="module")
def device():
    d = vg.Device()
    yield d
    d.close()


@pytest.mark.parametrize("name", ["cfg3_small_trilinear", "cfg5_request_trilinear"])
@pytest.mark.parametrize("mode", [vg.MODE_BATCHED, vg.MODE_PER_DRAW])
def test_blitted_mips_render_like_host_mips(device, name, mode):
    vg.set_mode(mode)
    try:
        h = scenes_edge.build(device.lib, name)
        cols, deps, counters = loader.Oracle().render(h)
        up = device.upload(h, VSD_GPU_MIPS)
        try:
            device.reset_stats()
            up.submit()
            got_c, got_d = up.read()
            st = device.stats()
            assert st["shaded"] == counters["shaded"]
            for a, b in zip(got_c, cols):
                assert np.array_equal(a, b)
            for a, b in zip(got_d, deps):
                assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
        finally:
            up.release()
    finally:
        vg.set_mode(vg.MODE_BATCHED)
