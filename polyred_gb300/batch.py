"""Batched rendering: many views of several scenes as one GPU job.

The reference renders one view per Renderer. Batch uploads each scene once
(pr_batch_add_scene) and renders a list of views (scene, camera, lights,
outputs) with pr_batch_render: per-view results equal pr_render's on a fresh
context, bit for bit, while the work of all views and all their shadow maps
runs in a few multi-view launches (one persistent raster launch over a
global work queue) captured in a CUDA graph. Batch.tune() runs the
library's autotuner over the raster task size and persistent grid.
"""
import ctypes as C
import json
import math

import numpy as np

from . import _abi, native, pmath, procedural, render, scene as sc


class Batch:
    def __init__(self, ordinal=0):
        import torch
        self.torch = torch
        self.lib = native.load()
        h = C.c_void_p()
        native.check(self.lib.pr_batch_create(int(ordinal), C.byref(h)))
        self.handle = h
        self.scenes = []

    def close(self):
        if self.handle:
            self.lib.pr_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_scene(self, scene):
        flat = render.FlatScene(scene)
        d = flat.desc()
        idx = C.c_uint32()
        native.check(self.lib.pr_batch_add_scene(self.handle, C.byref(d), C.byref(idx)))
        self.scenes.append(scene)
        return idx.value

    def views(self, specs, outputs=("rgba", "tri_id", "depth")):
        """pr_batch_view array for specs [(scene_index, opts, shadow_cams)],
        with device output tensors; returns (array, outputs per view, keep)."""
        t = self.torch
        arr = (_abi.pr_batch_view * len(specs))()
        outs, keep = [], []
        for k, (si, opts, cams) in enumerate(specs):
            fd = render.FrameDesc(opts, cams)
            W, H = opts["width"], opts["height"]
            o = {}
            od = _abi.pr_outputs()
            od.size = C.sizeof(_abi.pr_outputs)
            od.flags = _abi.PR_OUT_DEVICE_PTRS
            for name in outputs:
                ch, dt = render.Outputs.FIELDS[name]
                tdt = {np.uint8: t.uint8, np.uint32: t.int32, np.float32: t.float32, np.int32: t.int32}[dt]
                shape = (H, W, ch) if ch > 1 else (H, W)
                o[name] = t.empty(shape, dtype=tdt, device="cuda")
                setattr(od, name, o[name].data_ptr())
            arr[k].scene = si
            arr[k].frame = C.pointer(fd.desc)
            arr[k].out = C.pointer(od)
            keep += [fd, od]
            outs.append(o)
        return arr, outs, keep

    def render(self, arr):
        self.torch.cuda.synchronize()
        native.check(self.lib.pr_batch_render(self.handle, len(arr), arr))

    def tune(self, arr):
        buf = C.create_string_buffer(8192)
        self.torch.cuda.synchronize()
        native.check(self.lib.pr_batch_tune(self.handle, len(arr), arr, buf, len(buf)))
        return json.loads(buf.value.decode())

    def stats(self):
        st = _abi.pr_batch_stats()
        st.size = C.sizeof(_abi.pr_batch_stats)
        native.check(self.lib.pr_batch_get_stats(self.handle, C.byref(st)))
        return {k: getattr(st, k) for k, _ in _abi.pr_batch_stats._fields_ if k not in ("size", "reserved")}


def sphere_scene(n_tris, seed, n_lights=16, ao=True):
    """A config-2-style sphere field of about n_tris triangles: between 4 and
    256 UV spheres (centres U[-10,10]^3, radii U[0.2,1.5], the config-2
    materials), tessellated to reach the count, lit by n_lights casting
    point lights on a sphere of radius 20 (seeded)."""
    rng = procedural.Xoshiro128(seed)
    n_sph = max(4, min(256, int(round(n_tris / 2000))))
    per = max(8, n_tris / n_sph)
    lon = max(4, int(round(math.sqrt(per))))
    lat = max(3, lon // 2 + 1)
    mats = procedural.sphere_materials(ao)
    mesh = procedural.uv_sphere(lon, lat, 1.0)
    objs = []
    for _ in range(n_sph):
        c = [rng.uniform(-10, 10) for _ in range(3)]
        r = rng.uniform(0.2, 1.5)
        g = sc.Geometry(mesh, mats[rng.integer(4)])
        g.scale(r, r, r).translate(*c)
        objs.append(g)
    s = sc.Scene(*objs)
    for k in range(n_lights):
        z = rng.uniform(-1, 1)
        a = rng.uniform(0, 2 * math.pi)
        rr = math.sqrt(max(0.0, 1 - z * z))
        s.add(sc.Point(position=(20 * rr * math.cos(a), 20 * z, 20 * rr * math.sin(a)), intensity=2.0 / n_lights,
                       cast_shadow=True))
    s.add(sc.Ambient(intensity=0.1))
    return s


def ring_cameras(n, width, height, radius=6.0, height_y=2.0, fov=60.0):
    return [sc.Perspective(position=(radius * math.cos(2 * math.pi * k / n), height_y,
                                     radius * math.sin(2 * math.pi * k / n)), target=(0, 0, 0), up=(0, 1, 0),
                           fov=fov, aspect=width / height, near=0.1, far=100) for k in range(n)]


def shadow_cams(opts):
    cams = {}
    if not opts["shadow_map"]:
        return cams
    src, _ = opts["scene"].lights()
    center = opts["scene"].center()
    cv, cp = opts["camera"].view_matrix(), opts["camera"].proj_matrix()
    for k, l in enumerate(src):
        if l.cast_shadow:
            pos = l.position if isinstance(l, sc.Point) else (center - l.direction).astype(np.float32)
            cams[k] = pmath.shadow_camera(pos, center, cv, cp)
    return cams


def view_opts(scene, cam, width, height, shadow):
    return dict(width=width, height=height, camera=cam, scene=scene, perspective=True, shadow_map=True, gamma=True,
                background=(0, 0, 0, 255), shadow_size=(shadow, shadow))


def config4(n_scenes=32, views_per_scene=8, n_lights=16, width=1280, height=720, shadow=1024, lo=1_000, hi=500_000,
            seed=0x5EED0004, ao=True):
    """The batched workload: scenes with triangle counts log-uniform in
    [lo, hi] (scene s seeded seed + s), views_per_scene ring cameras each.
    Returns (scenes, [(scene_index, opts, shadow_cams)])."""
    g = np.random.default_rng(seed)
    counts = np.exp(g.uniform(math.log(lo), math.log(hi), n_scenes))
    scenes = [sphere_scene(int(n), seed + s, n_lights, ao) for s, n in enumerate(counts)]
    specs = []
    for si, s in enumerate(scenes):
        for cam in ring_cameras(views_per_scene, width, height):
            o = view_opts(s, cam, width, height, shadow)
            specs.append((si, o, shadow_cams(o)))
    return scenes, specs
