"""polyred's render API on the CUDA path.

Mirrors render.NewRenderer(opts...).Render() (render/raster.go:84-199) and
its options (render/options.go:38-120), with CUDA(dev) beside the
reference's GPU(dev): every pass of the frame (shadow maps, forward raster,
deferred shading, gamma) runs in libpolyred_cuda.so. There is no CPU
fallback; a failure raises native.RenderError.

Usage::

    r = NewRenderer(Size(800, 500), Camera(cam), Scene(s), GammaCorrection(True))
    img = r.Render()          # (H, W, 4) uint8, top-down rows like *image.RGBA
    ids, depth = r.tri_id(), r.depth()
"""
import ctypes as C
import weakref

import numpy as np

from . import _abi, native, scene as sc

F32 = np.float32


# ---------------------------------------------------------------- device

class Device:
    """A CUDA context on one GPU (pr_create). The caller owns it: a renderer
    given a device through CUDA(dev) never destroys it (the ownership rule of
    render.GPU, render/raster.go:57-60)."""

    def __init__(self, ordinal=0):
        self._lib = native.load()
        h = C.c_void_p()
        native.check(self._lib.pr_create(int(ordinal), C.byref(h)))
        self.handle = h
        self.ordinal = ordinal
        self._fin = weakref.finalize(self, Device._destroy, self._lib, h)

    @staticmethod
    def _destroy(lib, h):
        if h and h.value:
            lib.pr_destroy(h)

    def close(self):
        self._fin()

    def stream(self):
        s = C.c_void_p()
        native.check(self._lib.pr_stream(self.handle, C.byref(s)))
        return s.value


# ---------------------------------------------------------------- options

class _Option:
    def __init__(self, fn):
        self.fn = fn


def Size(width, height):
    return _Option(lambda o: o.update(width=int(width), height=int(height)))


def Camera(cam):
    def f(o):
        o["camera"] = cam
        o["perspective"] = isinstance(cam, sc.Perspective)  # render/options.go:49-56
    return _Option(f)


def Scene(s):
    return _Option(lambda o: o.update(scene=s))


def Background(rgba):
    return _Option(lambda o: o.update(background=tuple(int(c) for c in rgba)))


def MSAA(n):
    return _Option(lambda o: o.update(msaa=int(n)))


def ShadowMap(enable):
    return _Option(lambda o: o.update(shadow_map=bool(enable)))


def GammaCorrection(enable):
    return _Option(lambda o: o.update(gamma=bool(enable)))


def Workers(n):
    """Accepted for API compatibility; results always equal the reference's
    render.Workers(1) order."""
    return _Option(lambda o: o.update(workers=int(n)))


def BatchSize(n):
    """Accepted for API compatibility (no effect on the CUDA path)."""
    return _Option(lambda o: o.update(batch_size=int(n)))


def Debug(enable):
    return _Option(lambda o: o.update(debug=bool(enable)))


def CUDA(dev):
    """Render on the given Device (or CUDA ordinal)."""
    return _Option(lambda o: o.update(device=dev))


def ShadowMapSize(width, height):
    """Extension: shadow maps of their own size (the reference always uses the
    framebuffer size, render/shadow.go:87)."""
    return _Option(lambda o: o.update(shadow_size=(int(width), int(height))))


def DirectionalShadows(enable):
    """Extension: shadow maps for casting directional lights (the reference
    builds no camera for them and fails, render/shadow.go:66-85)."""
    return _Option(lambda o: o.update(directional_shadows=bool(enable)))


# ---------------------------------------------------------------- flattening

class FlatScene:
    """The scene as the C ABI consumes it: triangles in IterObjects order
    (scene/core.go:86-111), per-geometry model matrices and material bases,
    the flat material table (render/raster.go:240-262)."""

    def __init__(self, scene):
        items = [(o, mm) for o, mm in scene.iter_objects() if isinstance(o, sc.Geometry)]
        from . import pmath
        pos, nor, uv, col, mid = [], [], [], [], []
        self.objects = (_abi.pr_object * max(len(items), 1))()
        mats = []
        first = 0
        for k, (g, mm) in enumerate(items):
            m = g.mesh
            ob = self.objects[k]
            ob.first_tri = first
            ob.n_tris = m.n_tris
            ob.mat_base = len(mats)
            model = pmath.mat4_mul(mm, g.model_matrix())
            for i in range(16):
                ob.model[i] = float(model[i])
            for mt in g.materials:
                mats.append(mt)
            pos.append(m.pos)
            nor.append(m.nor)
            uv.append(m.uv)
            col.append(m.col)
            mid.append(m.mat_id)
            first += m.n_tris
        self.n_objects = len(items)
        self.n_tris = first
        cat = lambda xs, shape, dt: (np.ascontiguousarray(np.concatenate(xs), dt) if xs else np.zeros(shape, dt))
        self.pos = cat(pos, (0, 3, 4), F32)
        self.nor = cat(nor, (0, 3, 4), F32)
        self.uv = cat(uv, (0, 3, 2), F32)
        self.col = cat(col, (0, 3, 4), np.uint8)
        self.mat_id = cat(mid, (0,), np.int32)
        self.materials = (_abi.pr_material * max(len(mats), 1))()
        images = [mt.texture if isinstance(mt.texture, sc.ImageTexture) else None for mt in mats]
        self.textures = None  # pr_texture per material when any material has an image
        if any(t is not None for t in images):
            self.textures = (_abi.pr_texture * len(mats))()
            for k, t in enumerate(images):
                if t is not None:
                    self.textures[k].width = t.rgba.shape[1]
                    self.textures[k].height = t.rgba.shape[0]
                    self.textures[k].rgba = t.rgba.ctypes.data
        self._images = images  # keep the pixel arrays alive with the descriptor
        for k, mt in enumerate(mats):
            dst = self.materials[k]
            dst.diffuse[:] = mt.diffuse
            dst.specular[:] = mt.specular
            dst.texture[:] = (255, 255, 255, 255) if images[k] is not None else mt.texture
            dst.shininess = float(mt.shininess)
            dst.flags = ((_abi.PR_MAT_FLAT_SHADING if mt.flat_shading else 0)
                         | (_abi.PR_MAT_AO if mt.ambient_occlusion else 0)
                         | (_abi.PR_MAT_RECEIVE_SHADOW if mt.receive_shadow else 0)
                         | (_abi.PR_MAT_MIPMAP if mt.mipmap else 0))
            dst.texture_size = 1
        self.n_materials = len(mats)

    def desc(self):
        d = _abi.pr_scene_desc()
        d.size = C.sizeof(_abi.pr_scene_desc)
        d.flags = 0
        d.n_tris = self.n_tris
        d.n_objects = self.n_objects
        d.n_materials = self.n_materials
        d.pos = self.pos.ctypes.data
        d.nor = self.nor.ctypes.data
        d.uv = self.uv.ctypes.data
        d.col = self.col.ctypes.data
        d.mat_id = self.mat_id.ctypes.data
        d.objects = self.objects
        d.materials = self.materials
        d.textures = C.cast(self.textures, C.c_void_p) if self.textures is not None else None
        return d


class FrameDesc:
    """pr_frame_desc for one Render(): camera matrices, lights in
    scene.Lights() order with the shadow cameras of initShadowMaps."""

    def __init__(self, opts, shadow_cams):
        cam = opts["camera"]
        s = opts["scene"]
        src, env = s.lights()
        f = _abi.pr_frame_desc()
        f.size = C.sizeof(_abi.pr_frame_desc)
        f.flags = ((_abi.PR_FRAME_PERSPECTIVE if opts["perspective"] else 0)
                   | (_abi.PR_FRAME_SHADOWMAP if opts["shadow_map"] else 0)
                   | (_abi.PR_FRAME_GAMMA if opts["gamma"] else 0))
        f.width = opts["width"]
        f.height = opts["height"]
        f.msaa = int(opts.get("msaa", 1))
        v, p = cam.view_matrix(), cam.proj_matrix()
        for i in range(16):
            f.view[i] = float(v[i])
            f.proj[i] = float(p[i])
        f.cam_pos[:] = [float(c) for c in cam.position]
        f.background[:] = opts["background"]
        self.lights = (_abi.pr_light * max(len(src), 1))()
        for k, l in enumerate(src):
            d = self.lights[k]
            d.type = _abi.PR_LIGHT_POINT if isinstance(l, sc.Point) else _abi.PR_LIGHT_DIRECTIONAL
            d.cast_shadow = 1 if l.cast_shadow else 0
            d.pos[:] = [float(c) for c in l.position]
            if isinstance(l, sc.Directional):
                d.dir[:] = [float(c) for c in l.direction]
            d.intensity = float(l.intensity)
            d.color[:] = l.color
            if k in shadow_cams:
                sv, sp = shadow_cams[k]
                for i in range(16):
                    d.shadow_view[i] = float(sv[i])
                    d.shadow_proj[i] = float(sp[i])
        self.ambient = (C.c_float * max(len(env), 1))(*[float(e.intensity) for e in env])
        f.n_lights = len(src)
        f.n_ambient = len(env)
        f.lights = self.lights
        f.ambient = self.ambient
        sw, sh = opts.get("shadow_size") or (0, 0)
        f.shadow_width = sw
        f.shadow_height = sh
        self.desc = f


def _free_host(lib, ptrs):
    for p in ptrs:
        lib.pr_host_free(p)


def host_array(shape, dtype):
    """A zeroed numpy array in page-locked memory from pr_host_alloc (freed
    with the array's last reference)."""
    lib = native.load()
    n = int(np.prod(shape)) * np.dtype(dtype).itemsize
    ptr = C.c_void_p()
    native.check(lib.pr_host_alloc(max(n, 1), C.byref(ptr)))
    buf = (C.c_uint8 * max(n, 1)).from_address(ptr.value)
    a = np.frombuffer(buf, np.uint8, n).view(dtype).reshape(shape)
    a[...] = 0
    weakref.finalize(buf, _free_host, lib, [ptr.value])
    return a


class Outputs:
    """Host arrays a frame writes (pr_outputs); pinned=True places them in
    page-locked memory (pr_host_alloc), which the device writes at full link
    speed."""

    FIELDS = {"rgba": (4, np.uint8), "tri_id": (1, np.uint32), "depth": (1, F32), "nor": (4, F32),
              "face_nor": (4, F32), "world_pos": (4, F32), "uvd": (4, F32), "vcol": (4, np.uint8),
              "mat_id": (1, np.int32)}

    def __init__(self, width, height, want=("rgba",), n_shadow=0, shadow_size=None, pinned=False, msaa=1):
        """rgba is (height, width, 4); with msaa > 1 every other field has
        the framebuffer's msaa*height x msaa*width pixels."""
        self.arrays = {}
        o = _abi.pr_outputs()
        o.size = C.sizeof(_abi.pr_outputs)
        o.flags = 0
        alloc = host_array if pinned else np.zeros
        for name in want:
            if name == "shadow_maps":
                sw, sh = shadow_size
                a = alloc((max(n_shadow, 1), sh, sw), F32)
            else:
                k, dt = self.FIELDS[name]
                h, w = (height, width) if name == "rgba" else (height * msaa, width * msaa)
                a = alloc((h, w, k) if k > 1 else (h, w), dt)
            self.arrays[name] = a
            setattr(o, name, a.ctypes.data)
        self.desc = o


# ---------------------------------------------------------------- renderer

class Renderer:
    """render.Renderer on the CUDA path."""

    def __init__(self, *opts):
        self._opts = dict(width=800, height=600, msaa=1, shadow_map=False, gamma=False, debug=False, scene=None,
                          camera=None, perspective=False, background=(0, 0, 0, 0), workers=1, batch_size=32,
                          device=None, shadow_size=None, directional_shadows=False,
                          outputs=("rgba", "tri_id", "depth"))
        self._own_device = None
        self._lib = native.load()
        self._apply(opts)
        self._last = None
        self.stats = None

    # NewRenderer / Options (render/raster.go:84-143, render/options.go:125-141)
    def _apply(self, opts):
        for o in opts:
            o.fn(self._opts)
        if not 1 <= self._opts["msaa"] <= 16:
            raise native.RenderError(_abi.PR_ERR_INVALID_ARG, f"MSAA {self._opts['msaa']} outside 1..16")
        dev = self._opts["device"]
        if dev is None:
            if self._own_device is None:
                self._own_device = Device(0)
            self.device = self._own_device
        elif isinstance(dev, Device):
            self.device = dev
        else:
            self.device = Device(int(dev))
            self._own_device = self.device
        self._flat = None
        if self._opts["scene"] is not None:
            self._upload()
            self._init_shadow_maps()

    def Options(self, *opts):
        self._apply(opts)

    def _upload(self):
        self._flat = FlatScene(self._opts["scene"])
        d = self._flat.desc()
        native.check(self._lib.pr_scene_upload(self.device.handle, C.byref(d)))

    def _init_shadow_maps(self):
        """initShadowMaps (render/shadow.go:33-90): a light camera per casting
        light, fitted with the camera of this moment; maps start zeroed."""
        self._shadow_cams = {}
        o = self._opts
        if not o["shadow_map"] or o["camera"] is None:
            return
        src, _ = o["scene"].lights()
        center = o["scene"].center()
        cv, cp = o["camera"].view_matrix(), o["camera"].proj_matrix()
        from . import pmath
        for k, l in enumerate(src):
            if not l.cast_shadow:
                continue
            if isinstance(l, sc.Point):
                self._shadow_cams[k] = pmath.shadow_camera(l.position, center, cv, cp)
            elif o["directional_shadows"]:
                pos = (center - l.direction).astype(F32)
                self._shadow_cams[k] = pmath.shadow_camera(pos, center, cv, cp)
            else:
                raise native.RenderError(_abi.PR_ERR_UNSUPPORTED,
                                         "a shadow-casting directional light needs DirectionalShadows(True)")
        native.check(self._lib.pr_shadow_reset(self.device.handle))

    def Render(self):
        """Render one frame and return the (H, W, 4) RGBA image."""
        o = self._opts
        if o["scene"] is None or o["camera"] is None:
            raise native.RenderError(_abi.PR_ERR_NO_SCENE, "renderer needs Scene and Camera options")
        if self._flat is None:
            self._upload()
            self._init_shadow_maps()
        fd = FrameDesc(o, getattr(self, "_shadow_cams", {}))
        src, _ = o["scene"].lights()
        m = o["msaa"]
        sw, sh = o["shadow_size"] or (o["width"] * m, o["height"] * m)
        out = Outputs(o["width"], o["height"], o["outputs"], n_shadow=len(src), shadow_size=(sw, sh), msaa=m)
        native.check(self._lib.pr_render(self.device.handle, C.byref(fd.desc), C.byref(out.desc)))
        st = _abi.pr_stats()
        st.size = C.sizeof(_abi.pr_stats)
        native.check(self._lib.pr_frame_stats(self.device.handle, C.byref(st)))
        self.stats = {k: getattr(st, k) for k, _ in _abi.pr_stats._fields_ if k not in ("size", "reserved")}
        self._last = out.arrays
        return out.arrays.get("rgba")

    def outputs(self):
        return self._last

    def tri_id(self):
        return None if self._last is None else self._last.get("tri_id")

    def depth(self):
        return None if self._last is None else self._last.get("depth")

    def close(self):
        if self._own_device is not None:
            self._own_device.close()
            self._own_device = None


def NewRenderer(*opts):
    return Renderer(*opts)


def Outputs_(*names):
    """Choose which per-pixel arrays Render() fetches (rgba, tri_id, depth,
    nor, face_nor, world_pos, uvd, vcol, mat_id, shadow_maps)."""
    return _Option(lambda o: o.update(outputs=tuple(names)))
