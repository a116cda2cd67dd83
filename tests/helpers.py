"""Shared test helpers: run the CUDA path (through the C ABI) and the CPU
oracle on the same descriptors and compare."""
import ctypes as C
import os

import numpy as np

from polyred_gb300 import _abi, native, render, scene as sc

# The reference checkout whose own test assets also pin the oracle and the
# loaders (tests that read it skip where it is absent, as on a GPU host).
REFERENCE_ROOT = os.environ.get("POLYRED_REFERENCE_ROOT", "/root/reference")


def reference_testdata():
    return os.path.join(REFERENCE_ROOT, "internal", "testdata")


ALL_OUTPUTS = ("rgba", "tri_id", "depth", "nor", "face_nor", "world_pos", "uvd", "vcol", "mat_id")
THREADS = max(1, min(16, os.cpu_count() or 1))


def options(scene, cam, W, H, shadow_map=False, gamma=True, background=(0, 0, 0, 0), shadow_size=None,
            directional_shadows=False, msaa=1):
    return dict(width=W, height=H, camera=cam, scene=scene, perspective=isinstance(cam, sc.Perspective),
                shadow_map=shadow_map, gamma=gamma, background=tuple(background), shadow_size=shadow_size,
                directional_shadows=directional_shadows, msaa=msaa)


def shadow_cams(opts):
    from polyred_gb300 import pmath
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


class Pair:
    """One scene rendered by both sides, frame after frame (shadow maps
    persist on both sides, as in the reference)."""

    def __init__(self, device, opts, outputs=ALL_OUTPUTS, threads=THREADS, cams=None):
        self.device = device
        self.opts = opts
        self.outputs = tuple(outputs)
        self.threads = threads
        self.flat = render.FlatScene(opts["scene"])
        self.cams = shadow_cams(opts) if cams is None else cams
        lib = native.load()
        d = self.flat.desc()
        native.check(lib.pr_scene_upload(device.handle, C.byref(d)))
        native.check(lib.pr_shadow_reset(device.handle))
        src, _ = opts["scene"].lights()
        self.n_lights = len(src)
        self.msaa = opts.get("msaa", 1)
        sw, sh = opts["shadow_size"] or (opts["width"] * self.msaa, opts["height"] * self.msaa)
        self.sshape = (max(self.n_lights, 1), sh, sw)
        self.shadow_state = np.zeros(self.sshape, np.float32)
        self.stats = None

    def frame(self, with_shadow_maps=False):
        import oracle
        fd = render.FrameDesc(self.opts, self.cams)
        want = self.outputs + (("shadow_maps",) if with_shadow_maps else ())
        W, H = self.opts["width"], self.opts["height"]
        sw, sh = self.sshape[2], self.sshape[1]
        gpu = render.Outputs(W, H, want, n_shadow=self.n_lights, shadow_size=(sw, sh), msaa=self.msaa)
        lib = native.load()
        native.check(lib.pr_render(self.device.handle, C.byref(fd.desc), C.byref(gpu.desc)))
        st = _abi.pr_stats()
        st.size = C.sizeof(_abi.pr_stats)
        native.check(lib.pr_frame_stats(self.device.handle, C.byref(st)))
        self.stats = {k: getattr(st, k) for k, _ in _abi.pr_stats._fields_}
        cpu = render.Outputs(W, H, want, n_shadow=self.n_lights, shadow_size=(sw, sh), msaa=self.msaa)
        oracle.render(self.flat.desc(), fd.desc, cpu.desc, shadow_state=self.shadow_state, threads=self.threads)
        return gpu.arrays, cpu.arrays


def same_bits(a, b):
    """Elementwise equality of bit patterns; any NaN equals any NaN."""
    a = np.asarray(a)
    b = np.asarray(b)
    if a.dtype.kind == "f":
        ua = a.view(np.uint32 if a.dtype == np.float32 else np.uint64)
        ub = b.view(ua.dtype)
        return (ua == ub) | (np.isnan(a) & np.isnan(b))
    return a == b


def assert_bitexact(gpu, cpu, names=None):
    names = names or sorted(set(gpu) & set(cpu))
    for n in names:
        eq = same_bits(gpu[n], cpu[n])
        if not eq.all():
            bad = np.argwhere(~eq)
            first = tuple(bad[0])
            raise AssertionError(f"{n}: {len(bad)} mismatching elements, first at {first}: "
                                 f"gpu={np.asarray(gpu[n])[first]} cpu={np.asarray(cpu[n])[first]}")
