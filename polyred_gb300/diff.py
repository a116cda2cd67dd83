"""Differentiable deferred shading on the CUDA path.

The reference has no gradients; this module adds a Forward/Backward pair
over pr_diff_forward / pr_diff_backward following torch.autograd.Function's
contract: ShadeFunction.apply(vertex_color, vertex_normal, kd, ks,
shininess, light_pos, light_intensity, ambient, renderer, view) renders view
`view` and returns its float radiance (H, W, 4); its backward returns the
gradient of each tensor input. Visibility (triangle IDs, shadow and AO
factors) is held fixed by the differentiation G-buffer each forward call
saves; the backward kernel recomputes every interpolated attribute and
per-light term from it.

Parameters, as torch tensors:
  vertex_color     (n_tris, 3, 4) float32 on the device, RGBA in [0, 1]
  vertex_normal    (n_tris, 3, 4) float32 on the device, object space
  kd, ks           (n_materials, 3) float32, Diffuse/255 and Specular/255
  shininess        (n_materials,)
  light_pos        (n_lights, 3) point-light positions (directional: unused)
  light_intensity  (n_lights,)
  ambient          (n_ambient,) light.Environment intensities
"""
import copy
import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _abi, native, pmath, render, scene as sc

PARAM_NAMES = ("vertex_color", "vertex_normal", "kd", "ks", "shininess", "light_pos", "light_intensity", "ambient")


@dataclass
class View:
    camera: object
    width: int
    height: int


class DiffRenderer:
    """One scene on one device, rendered from several views (one
    NewRenderer per view in reference terms: each frame starts from zeroed
    shadow maps, as the first Render() of a new renderer)."""

    def __init__(self, scene, views, device=None, shadow_map=True, shadow_size=None, background=(0, 0, 0, 255)):
        import torch
        self.torch = torch
        self.scene = scene
        self.views = list(views)
        self.device = device or render.Device(0)
        self.lib = native.load()
        self.flat = render.FlatScene(scene)
        d = self.flat.desc()
        native.check(self.lib.pr_scene_upload(self.device.handle, C.byref(d)))
        self.src, self.env = scene.lights()
        self.shadow_map = shadow_map
        self.shadow_size = shadow_size
        self.background = tuple(background)
        self.center = scene.center()

    # ---- parameters --------------------------------------------------------
    def initial_params(self):
        """The scene's own parameters as tensors (vertex data on the device)."""
        t = self.torch
        f = self.flat
        mats = [f.materials[k] for k in range(f.n_materials)]
        p = {
            "vertex_color": t.from_numpy(f.col.astype(np.float32) / 255.0).cuda(),
            "vertex_normal": t.from_numpy(np.ascontiguousarray(f.nor)).cuda(),
            "kd": t.tensor([[m.diffuse[k] / 255.0 for k in range(3)] for m in mats], dtype=t.float32).reshape(-1, 3),
            "ks": t.tensor([[m.specular[k] / 255.0 for k in range(3)] for m in mats], dtype=t.float32).reshape(-1, 3),
            "shininess": t.tensor([m.shininess for m in mats], dtype=t.float32),
            "light_pos": t.tensor([[float(c) for c in l.position] for l in self.src], dtype=t.float32).reshape(-1, 3),
            "light_intensity": t.tensor([float(l.intensity) for l in self.src], dtype=t.float32),
            "ambient": t.tensor([float(e.intensity) for e in self.env], dtype=t.float32),
        }
        return p

    # ---- C ABI plumbing ----------------------------------------------------
    def frame(self, view, light_pos, light_intensity, ambient):
        """pr_frame_desc for a view with the given light parameters (shadow
        cameras follow the light positions, render/shadow.go:41-85)."""
        v = self.views[view]
        src = []
        lp = np.asarray(light_pos, np.float32).reshape(-1, 3)
        li = np.asarray(light_intensity, np.float32).reshape(-1)
        for k, l in enumerate(self.src):
            q = copy.copy(l)
            if isinstance(l, sc.Point):
                q.position = lp[k].copy()
            q.intensity = np.float32(li[k])
            src.append(q)
        env = [sc.Ambient(intensity=float(a)) for a in np.asarray(ambient, np.float32).reshape(-1)]
        view_scene = _LightsOnly(src, env, self.center)
        opts = dict(width=v.width, height=v.height, camera=v.camera, scene=view_scene,
                    perspective=isinstance(v.camera, sc.Perspective), shadow_map=self.shadow_map, gamma=False,
                    background=self.background, shadow_size=self.shadow_size)
        cams = {}
        if self.shadow_map:
            cv, cp = v.camera.view_matrix(), v.camera.proj_matrix()
            for k, l in enumerate(src):
                if l.cast_shadow:
                    pos = l.position if isinstance(l, sc.Point) else (self.center - l.direction).astype(np.float32)
                    cams[k] = pmath.shadow_camera(pos, self.center, cv, cp)
        return render.FrameDesc(opts, cams)

    def _params_struct(self, p):
        keep = []
        d = _abi.pr_diff_params()
        d.size = C.sizeof(_abi.pr_diff_params)
        d.n_materials = self.flat.n_materials
        vc = p["vertex_color"].detach().contiguous()
        vn = p["vertex_normal"].detach().contiguous()
        keep += [vc, vn]
        d.vertex_color = vc.data_ptr()
        d.vertex_normal = vn.data_ptr()
        for name in ("kd", "ks", "shininess"):
            a = np.ascontiguousarray(p[name].detach().cpu().numpy(), np.float32)
            keep.append(a)
            setattr(d, name, a.ctypes.data_as(_abi.FP))
        return d, keep

    def forward_raw(self, view, p):
        """(radiance, gbuf) device tensors of one view."""
        t = self.torch
        v = self.views[view]
        fd = self.frame(view, p["light_pos"].detach().cpu().numpy(), p["light_intensity"].detach().cpu().numpy(),
                        p["ambient"].detach().cpu().numpy())
        d, keep = self._params_struct(p)
        rad = t.empty((v.height, v.width, 4), dtype=t.float32, device="cuda")
        gbuf = t.empty((v.height, v.width, _abi.PR_DGB_FLOATS), dtype=t.float32, device="cuda")
        t.cuda.synchronize()
        native.check(self.lib.pr_shadow_reset(self.device.handle))
        native.check(self.lib.pr_diff_forward(self.device.handle, C.byref(fd.desc), C.byref(d), rad.data_ptr(),
                                              gbuf.data_ptr(), None))
        return rad, gbuf

    def backward_raw(self, view, p, gbuf, grad):
        """Gradients (dict of tensors shaped like the parameters)."""
        t = self.torch
        f = self.flat
        fd = self.frame(view, p["light_pos"].detach().cpu().numpy(), p["light_intensity"].detach().cpu().numpy(),
                        p["ambient"].detach().cpu().numpy())
        d, keep = self._params_struct(p)
        g_vc = t.empty_like(p["vertex_color"], device="cuda")
        g_vn = t.empty_like(p["vertex_normal"], device="cuda")
        nm, nl, na = f.n_materials, len(self.src), len(self.env)
        host = {k: np.zeros(n, np.float64) for k, n in
                (("kd", 3 * nm), ("ks", 3 * nm), ("shininess", nm), ("light_pos", 3 * nl),
                 ("light_intensity", nl), ("ambient", na))}
        g = _abi.pr_diff_grads()
        g.size = C.sizeof(_abi.pr_diff_grads)
        g.vertex_color = g_vc.data_ptr()
        g.vertex_normal = g_vn.data_ptr()
        for k, a in host.items():
            setattr(g, k, a.ctypes.data_as(_abi.DP) if a.size else None)
        gr = grad.detach().contiguous()
        t.cuda.synchronize()
        native.check(self.lib.pr_diff_backward(self.device.handle, C.byref(fd.desc), C.byref(d), gbuf.data_ptr(),
                                               gr.data_ptr(), C.byref(g)))
        out = {"vertex_color": g_vc, "vertex_normal": g_vn}
        for k, a in host.items():
            out[k] = t.from_numpy(a.astype(np.float32)).reshape(p[k].shape).to(p[k].device)
        return out


class _LightsOnly:
    """The light list a FrameDesc needs, with parameters substituted."""

    def __init__(self, src, env, center):
        self._src, self._env, self._center = src, env, center

    def lights(self):
        return self._src, self._env

    def center(self):
        return self._center


def _function():
    import torch

    class ShadeFunction(torch.autograd.Function):
        """Radiance of one view; gradients for the eight parameter tensors."""

        @staticmethod
        def forward(ctx, vertex_color, vertex_normal, kd, ks, shininess, light_pos, light_intensity, ambient,
                    renderer, view):
            p = dict(zip(PARAM_NAMES, (vertex_color, vertex_normal, kd, ks, shininess, light_pos, light_intensity,
                                       ambient)))
            rad, gbuf = renderer.forward_raw(view, p)
            ctx.renderer = renderer
            ctx.view = view
            ctx.save_for_backward(gbuf, vertex_color, vertex_normal, kd, ks, shininess, light_pos, light_intensity,
                                  ambient)
            return rad

        @staticmethod
        def backward(ctx, grad):
            gbuf, *vals = ctx.saved_tensors
            p = dict(zip(PARAM_NAMES, vals))
            g = ctx.renderer.backward_raw(ctx.view, p, gbuf, grad)
            outs = tuple(g[k] if ctx.needs_input_grad[i] else None for i, k in enumerate(PARAM_NAMES))
            return outs + (None, None)

    return ShadeFunction


_SHADE = None


def shade(params, renderer, view):
    """Radiance (H, W, 4) of `view` as a differentiable function of params."""
    global _SHADE
    if _SHADE is None:
        _SHADE = _function()
    return _SHADE.apply(*[params[k] for k in PARAM_NAMES], renderer, view)


def inverse_render(renderer, targets, params, trainable, steps=200, lr=0.01, log=None):
    """Adam over the `trainable` parameters to match `targets` (one radiance
    image per view, L2 loss over RGB); returns the per-step losses."""
    import torch
    opt = torch.optim.Adam([params[k] for k in trainable], lr=lr)
    losses = []
    for it in range(steps):
        opt.zero_grad()
        loss = 0.0
        for v in range(len(renderer.views)):
            r = shade(params, renderer, v)
            loss = loss + ((r[..., :3] - targets[v][..., :3]) ** 2).mean()
        loss.backward()
        opt.step()
        losses.append(float(loss.detach()))
        if log:
            log(it, losses[-1])
    return losses
