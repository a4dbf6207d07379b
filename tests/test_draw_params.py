"""Vulkan draw parameters: vertexOffset, instanceCount, firstInstance and per-instance
vertex input rate.

The reference ignores all four (cmd_exec.cpp:129-142 passes only the count and the
first index/vertex to DrawTriangles; rasterizer.cpp:100-119 fetches every attribute
by vertex index), and so does this library by default.  With the switch on, each
instanced or offset draw must render exactly what an equivalent scene without draw
parameters renders: the draw repeated once per instance, the offset folded into the
indices, per-instance attributes copied into per-vertex ones.  The oracle renders the
equivalent scene; the GPU renders the original.  Counters are compared except
`draws`, which counts an instanced draw once.
"""
import struct

import numpy as np
import pytest

import visor_gb300 as vg
from visor_gb300 import scene as vs
from oracle import loader
import scenes_edge

W, H = 48, 40
HALF_BLEND = {"blend_enable": 1, "src_factor": vs.BLEND_SRC_ALPHA, "dst_factor": vs.BLEND_ONE_MINUS_SRC_ALPHA,
              "depth_op": vs.CMP_LEQUAL}


def _vertex(px, py, z, rgba, w=W, h=H):
    return scenes_edge._color_vertex(px, py, z, rgba, w, h)


def _mesh(seed, ntris, w=W, h=H):
    """Seeded triangles (pixel positions, depth, translucent colours) as 3*ntris vertices."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(ntris):
        cx, cy = rng.uniform(2, w - 2), rng.uniform(2, h - 2)
        z = float(rng.uniform(0.1, 0.9))
        col = tuple(int(c) for c in rng.integers(0, 256, 3)) + (int(rng.integers(60, 200)),)
        for _ in range(3):
            out.append((float(np.clip(cx + rng.uniform(-12, 12), -4, w + 4)),
                        float(np.clip(cy + rng.uniform(-12, 12), -4, h + 4)), z, col))
    return out


FILLER = [(1.0, 1.0, 0.05, (255, 255, 255, 255)), (W - 2.0, 3.0, 0.05, (255, 255, 255, 255)),
          (5.0, H - 2.0, 0.05, (255, 255, 255, 255))] * 3


def _scene(lib, draws, pipe_kw, topology=vs.TOPOLOGY_TRIANGLE_LIST, w=W, h=H):
    """draws: list of dicts with 'verts' (vertex tuples), optional 'idx' (indices into
    verts), 'lead' (filler vertices stored before verts), 'vertex_offset', 'instances',
    'first_instance', 'inst_colors' (per-instance RGBA8, pipeline reads colour per instance),
    'shader' (default COLOR) and 'xshift' (instance index whose clip-x move the stored
    vertices already carry, as the instanced shader computes it in binary32)."""
    sh = vs.new_scene(lib)
    s = sh.ptr
    t = lib.vsc_add_target(s, w, h)
    first_draw = None
    for d in draws:
        kw = dict(pipe_kw)
        if d.get("inst_colors") is not None:
            kw["instance_attr"] = 2  # location 1 (colour) + 1
        pi = lib.vsc_add_pipeline(s, vs.make_pipeline(d.get("shader", vs.SHADER_COLOR), topology=topology, **kw))
        verts = d.get("lead", []) + d["verts"]
        data = b"".join(_vertex(*v, w=w, h=h) for v in verts)
        if d.get("xshift") is not None:
            v = np.frombuffer(data, np.uint8).reshape(-1, 20).copy()
            x = v[:, 0:4].copy().view(np.float32).reshape(-1)
            x = x + np.float32(np.float32(d["xshift"]) * np.float32(0.25))
            v[:, 0:4] = x.astype(np.float32).view(np.uint8).reshape(-1, 4)
            data = v.tobytes()
        off = lib.vsc_add_vertices(s, data, len(data))
        inst_off = 0
        if d.get("inst_colors") is not None:
            cb = bytes(c for col in d["inst_colors"] for c in col)
            inst_off = lib.vsc_add_vertices(s, cb, len(cb))
        extra = dict(vertex_offset=d.get("vertex_offset", 0), instances=d.get("instances", 0),
                     first_instance=d.get("first_instance", 0), inst_vb_offset=inst_off)
        if d.get("idx") is not None:
            ia = np.array(d["idx"], np.uint32)
            first = lib.vsc_add_indices(s, ia.ctypes.data, len(ia))
            dr = vs.make_draw(pi, len(ia), int(first), indexed=True, vb_offset=off, **extra)
        else:
            dr = vs.make_draw(pi, len(verts), 0, vb_offset=off, **extra)
        di = lib.vsc_add_draw(s, dr)
        first_draw = di if first_draw is None else first_draw
    lib.vsc_add_pass(s, t, 1, first_draw if first_draw is not None else 0, len(draws))
    return sh


def _recolor(verts, col):
    return [(x, y, z, col) for (x, y, z, _) in verts]


def _cases():
    """(name, vulkan-scene draws, equivalent draws, pipeline state, topology)"""
    m = _mesh(11, 6)
    m2 = _mesh(12, 5)
    idx = list(range(len(m)))[::-1]
    idx2 = list(range(len(m2)))[::-1]
    lead = FILLER
    K = len(lead)
    strip = [(4 + i * 4.0, 8.0 if i % 2 == 0 else 34.0, 0.2 + 0.05 * i, (30 * i % 256, 90, 200, 150))
             for i in range(10)]
    cols = [(250, 30, 30, 120), (30, 250, 30, 140), (30, 30, 250, 160), (200, 200, 30, 180),
            (30, 200, 200, 100), (200, 30, 200, 90), (120, 120, 120, 200), (10, 10, 10, 255)]
    many = _mesh(13, 40, 8, 8)
    return [
        ("vertex_offset",
         [dict(verts=m, lead=lead, idx=idx, vertex_offset=K)],
         [dict(verts=m, lead=lead, idx=[i + K for i in idx])], HALF_BLEND, vs.TOPOLOGY_TRIANGLE_LIST),
        ("instances_blend",
         [dict(verts=m, instances=3, first_instance=5)],
         [dict(verts=m)] * 3, HALF_BLEND, vs.TOPOLOGY_TRIANGLE_LIST),
        ("instances_indexed_offset",
         [dict(verts=m2, lead=lead, idx=idx2, vertex_offset=K, instances=2), dict(verts=m, instances=2)],
         [dict(verts=m2, lead=lead, idx=[i + K for i in idx2])] * 2 + [dict(verts=m)] * 2,
         HALF_BLEND, vs.TOPOLOGY_TRIANGLE_LIST),
        ("instances_zero",
         [dict(verts=m, instances=vs.NONE), dict(verts=m2)],
         [dict(verts=m2)], HALF_BLEND, vs.TOPOLOGY_TRIANGLE_LIST),
        ("instance_rate_colors",
         [dict(verts=m, instances=4, first_instance=2, inst_colors=cols)],
         [dict(verts=_recolor(m, cols[2 + i])) for i in range(4)], HALF_BLEND, vs.TOPOLOGY_TRIANGLE_LIST),
        ("instance_rate_strip_offset",
         [dict(verts=strip, lead=lead, idx=list(range(10)), vertex_offset=K, instances=3, first_instance=4,
               inst_colors=cols)],
         [dict(verts=_recolor(strip, cols[4 + i]), lead=lead, idx=[j + K for j in range(10)]) for i in range(3)],
         HALF_BLEND, vs.TOPOLOGY_TRIANGLE_STRIP),
        ("instance_index_shader",
         # gl_InstanceIndex (first_instance included) moves each instance right
         [dict(verts=m, instances=3, first_instance=1, shader=vs.SHADER_COLOR_INSTANCED)],
         [dict(verts=m, xshift=1 + i) for i in range(3)], HALF_BLEND, vs.TOPOLOGY_TRIANGLE_LIST),
        ("instance_rate_opaque_deep",
         # more triangles than pixels in an opaque job: the raster runs the vertex
         # shader again for the shaded triangles, with their instance index (LEQUAL:
         # the last instance wins the ties)
         [dict(verts=many, instances=3, first_instance=1, inst_colors=cols)],
         [dict(verts=_recolor(many, cols[1 + i])) for i in range(3)],
         {"depth_op": vs.CMP_LEQUAL}, vs.TOPOLOGY_TRIANGLE_LIST),
    ]


CASES = {c[0]: c for c in _cases()}
MODES = {"batched": vg.MODE_BATCHED, "per_draw": vg.MODE_PER_DRAW}


def _build(lib, name, which):
    _, vk, eq, pipe, topo = CASES[name]
    w, h = (8, 8) if name == "instance_rate_opaque_deep" else (W, H)
    return _scene(lib, vk if which == "vulkan" else eq, pipe, topology=topo, w=w, h=h)


def _no_draws(k):
    return {n: v for n, v in k.items() if n != "draws"}


def test_scene_struct_layouts_match_header(tmp_path):
    """The ctypes mirrors of the scene's draw and pipeline have the layout of include/visor_scene.h."""
    import ctypes
    import os
    import subprocess
    from conftest import REPO
    checks = {"vsc_draw": vs.Draw, "vsc_pipeline": vs.Pipeline}
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "visor_scene.h"', "int main(void) {"]
    for cname, py in checks.items():
        lines.append(f'printf("{cname} sizeof %zu\\n", sizeof({cname}));')
        for f, _ in py._fields_:
            lines.append(f'printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.check_call(["gcc", "-I", os.path.join(REPO, "include"), str(src), "-o", str(exe)])
    got = {}
    for line in subprocess.check_output([str(exe)], text=True).splitlines():
        name, field, value = line.split()
        got[(name, field)] = int(value)
    for cname, py in checks.items():
        assert got[(cname, "sizeof")] == ctypes.sizeof(py), cname
        for f, _ in py._fields_:
            assert got[(cname, f)] == getattr(py, f).offset, (cname, f)


def test_switch_round_trip():
    was = vg.draw_parameters()
    try:
        vg.set_draw_parameters(True)
        assert vg.draw_parameters()
        vg.set_draw_parameters(False)
        assert not vg.draw_parameters()
    finally:
        vg.set_draw_parameters(was)


def test_oracle_refuses_per_instance_attributes():
    o = loader.Oracle()
    h = _build(o.lib, "instance_rate_colors", "vulkan")
    cols, deps = vs.target_buffers(h)
    cp, dp = vs.pointer_arrays(cols, deps)
    assert o.lib.vor_render(h.ptr, cp, dp, None) == -2


@pytest.mark.parametrize("name", [n for n in CASES if "instance_rate" not in n])
def test_oracle_ignores_draw_parameters(name):
    """The oracle follows the reference: the parameters change nothing it renders, so
    the vulkan scene without them renders the same as with them."""
    o = loader.Oracle()
    a = o.render(_build(o.lib, name, "vulkan"))
    hb = _build(o.lib, name, "vulkan")
    for i in range(hb.s.num_draws):
        d = hb.s.draws[i]
        d.vertex_offset, d.instances, d.first_instance = 0, 0, 0
    b = o.render(hb)
    for x, y in zip(a[0] + a[1], b[0] + b[1]):
        assert np.array_equal(x, y)
    assert a[2] == b[2]


@pytest.mark.parametrize("name", [n for n in CASES if "instance_rate" not in n])
def test_cases_depend_on_draw_parameters(name):
    """Each case renders differently when its parameters are ignored, so the GPU test
    below fails for an implementation that drops them."""
    o = loader.Oracle()
    a = o.render(_build(o.lib, name, "vulkan"))
    b = o.render(_build(o.lib, name, "expanded"))
    assert any(not np.array_equal(x, y) for x, y in zip(a[0] + a[1], b[0] + b[1]))


@pytest.mark.parametrize("name", list(CASES))
def test_expanded_scenes_pinned_to_reference(name):
    """The equivalent scenes the GPU output is compared with render the same in the
    reference build as in the oracle, so each Vulkan-semantics image is pinned to the
    reference's own rasterizer too."""
    try:
        ref = loader.Reference()
    except OSError:
        pytest.skip("reference build not present")
    o = loader.Oracle()
    oc, od, ok = o.render(_build(o.lib, name, "expanded"))
    rc, rd, rk, _ = ref.render(_build(ref.lib, name, "expanded"), threaded=False)
    assert ok == rk
    for a, b in zip(oc + od, rc + rd):
        assert np.array_equal(a, b)


@pytest.fixture(scope="module")
def device():
    d = vg.Device()
    yield d
    d.close()


@pytest.fixture
def vulkan_params():
    was = vg.draw_parameters()
    vg.set_draw_parameters(True)
    yield
    vg.set_draw_parameters(was)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", list(MODES))
@pytest.mark.parametrize("name", list(CASES))
def test_vulkan_draw_parameters_match_expanded_scene(device, vulkan_params, name, mode):
    o = loader.Oracle()
    gc, gd, gk = vg.render(_build(vg.lib(), name, "vulkan"), MODES[mode], device)
    oc, od, ok = o.render(_build(o.lib, name, "expanded"))
    scenes_edge_compare(gc, gd, oc, od)
    assert _no_draws(gk) == _no_draws(ok)


@pytest.mark.gpu
@pytest.mark.parametrize("name", [n for n in CASES if "instance_rate" not in n])
def test_reference_behaviour_by_default(device, name):
    """Without the switch the parameters are ignored, as in the reference."""
    assert not vg.draw_parameters()
    o = loader.Oracle()
    gc, gd, gk = vg.render(_build(vg.lib(), name, "vulkan"), vg.MODE_BATCHED, device)
    oc, od, ok = o.render(_build(o.lib, name, "vulkan"))
    scenes_edge_compare(gc, gd, oc, od)
    assert gk == ok


def scenes_edge_compare(gc, gd, oc, od):
    for t, (a, b) in enumerate(zip(gc, oc)):
        bad = np.argwhere(np.any(a != b, axis=-1))
        assert len(bad) == 0, f"target {t}: {len(bad)} colour pixels differ, first {bad[:4].tolist()}"
    for t, (a, b) in enumerate(zip(gd, od)):
        bad = np.argwhere(a.view(np.uint32) != b.view(np.uint32))
        assert len(bad) == 0, f"target {t}: {len(bad)} depth values differ, first {bad[:4].tolist()}"
