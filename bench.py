"""Benchmark of the render path on GB300.

Workload (one step = one frame): the 1M-triangle sphere field at 1920x1080 —
256 UV spheres of 3,906 triangles (999,936 in all), 4 Blinn-Phong materials,
one point and one directional light both casting 2048^2 shadow maps, AO on,
sRGB gamma. Metric: Mtri/s = input triangles per second of frame time.

  value  frames rendered with the scene resident in HBM (pr_render_async into
         device outputs), CUDA events on the library's stream
  e2e    the same through the public C ABI with host buffers: every step
         uploads the triangle soup from pinned host memory and reads back
         RGBA8 + triangle IDs + depth into page-locked buffers from
         pr_host_alloc (pr_frame_submit: the next step's upload overlaps the
         current frame), timed from before the first upload to after the
         last readback
  --impl reference  the CPU restatement of the reference renderer (oracle/),
         all host threads, single-worker draw order

Further legs in the same line (each skippable): small_800x500 (the small
UV-sphere workload), diff (the adjoint and its 200-step Adam loop, --no-diff),
soup_4k (10M triangles at 3840x2160, --no-soup), batched (many views in one
job, --no-batch), msaa_2x and textured_1080p (--no-msaa), obj_ingest
(loading a 41 MB Wavefront OBJ, --no-obj), cpu_baseline (--no-cpu-baseline).

Multi-GPU: frames do not shard (one view); N ranks render N independent
replicas (weak scaling), the value is the total over ranks.
"""
import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_TRIS = 999_936
W, H = 1920, 1080
SHADOW = (2048, 2048)


def workload():
    from polyred_gb300 import procedural
    return procedural.sphere_field(width=W, height=H)


def frame_opts(scene, cam):
    return dict(width=W, height=H, camera=cam, scene=scene, perspective=True, shadow_map=True, gamma=True,
                background=(0, 0, 0, 0), shadow_size=SHADOW, directional_shadows=True)


def shadow_cams(opts):
    from polyred_gb300 import pmath, scene as sc
    import numpy as np
    src, _ = opts["scene"].lights()
    center = opts["scene"].center()
    cv, cp = opts["camera"].view_matrix(), opts["camera"].proj_matrix()
    cams = {}
    for k, l in enumerate(src):
        if l.cast_shadow:
            pos = l.position if isinstance(l, sc.Point) else (center - l.direction).astype(np.float32)
            cams[k] = pmath.shadow_camera(pos, center, cv, cp)
    return cams


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "20"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic():
    """DRAM bytes per launch of the AO kernel from the committed ncu summary
    (profiles/ao_kernel_sphere_field_1080p.txt), or None."""
    p = os.path.join(ROOT, "profiles", "ao_kernel_sphere_field_1080p.txt")
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith("dram_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].strip().split()[0])
            except ValueError:
                return None
    return None


def bench_config(world):
    """The workload's config dict; both arms print this same dict."""
    return {"workload": "sphere_field_1M_1080p", "n_tris": N_TRIS, "width": W, "height": H,
            "shadow_maps": "2 x 2048^2 (point + directional)", "ao": True, "gamma": True,
            "l2": "inputs larger than L2 (136 MB triangle soup per frame)",
            "parallelism": f"replicas x{world}"}


def oracle_frame(threads, want=("rgba", "tri_id", "depth")):
    """Scene, frame and outputs of the workload built without the product
    library: pmath's matrix helpers run on the oracle's host math, so the
    process maps liboracle.so alone. Returns a callable rendering one frame
    with the oracle."""
    import numpy as np
    import oracle
    from oracle import hostmath
    from polyred_gb300 import pmath, render
    prev = pmath._backend
    pmath.set_backend(hostmath)
    try:
        s, cam = workload()
        opts = frame_opts(s, cam)
        flat = render.FlatScene(s)
        fd = render.FrameDesc(opts, shadow_cams(opts))
    finally:
        pmath.set_backend(prev)
    state = np.zeros((3, SHADOW[1], SHADOW[0]), np.float32)
    out = render.Outputs(W, H, want)
    sd = flat.desc()

    def frame():
        oracle.render(sd, fd.desc, out.desc, shadow_state=state, threads=threads)
    frame.keep = (flat, fd, out, state)
    return frame


def ncu_instructions(kernel="ao_kernel", name="ao_kernel_sphere_field_1080p.txt"):
    """Warp instructions one launch of kernel executes (sm__inst_executed),
    from its committed ncu summary under profiles/, or None."""
    p = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith("instructions executed"):
            try:
                return float(line.split()[2]) * 1e6
            except (IndexError, ValueError):
                return None
    return None


def run_reference(args, rank):
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    world = int(os.environ.get("WORLD_SIZE", "1"))
    frame = oracle_frame(threads)
    for _ in range(args.warmup):
        frame()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        frame()
    dt = (time.perf_counter() - t0) / args.steps
    v = N_TRIS / dt / 1e6
    line = {"impl": "reference", "metric": "1080p Mtri/s", "value": v, "unit": "Mtri/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": bench_config(world),
            "cpu_baseline": {"value": v, "unit": "Mtri/s", "cores": threads, "kind": "port",
                             "sample": "full frames of the workload, C++ restatement of the Go CPU renderer "
                                       "(row-band threads, single-worker draw order)"},
            "e2e": {"value": v, "unit": "Mtri/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "frames_per_s": 1.0 / dt,
            "native_libraries": mapped_libraries()}
    print(json.dumps(line), flush=True)


def mapped_libraries():
    """The shared objects of this repository mapped into this process."""
    try:
        maps = open("/proc/self/maps").read().split("\n")
    except OSError:
        return None
    root = os.path.realpath(ROOT)
    found = set()
    for ln in maps:
        path = ln.split()[-1] if ln.split() else ""
        if path.startswith(root) and path.endswith(".so"):
            found.add(os.path.relpath(path, root))
    return sorted(found)


def cpu_baseline_sample(single_thread=True):
    """The oracle on one full frame with every host core, and (bounded: one
    frame each) with one thread, the parity order of render.Workers(1)."""
    threads = os.cpu_count() or 1
    frame = oracle_frame(threads, ("rgba",))
    t0 = time.perf_counter()
    frame()
    dt = time.perf_counter() - t0
    out = {"value": N_TRIS / dt / 1e6, "unit": "Mtri/s", "cores": threads, "kind": "port",
           "sample": "1 full frame of the workload (C++ restatement of the Go CPU renderer, row-band threads)"}
    if single_thread:
        one = oracle_frame(1, ("rgba",))
        t0 = time.perf_counter()
        one()
        d1 = time.perf_counter() - t0
        out["single_thread"] = {"value": N_TRIS / d1 / 1e6, "unit": "Mtri/s", "cores": 1, "s_per_frame": d1}
    return out


def max_over_ranks(ms, world, device):
    """The slowest rank's time (every rank renders its own replica of the
    workload; the job is done when the last one is)."""
    if world <= 1:
        return ms
    import torch
    import torch.distributed as dist
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(n_tris, world, ms):
    """Whole-job Mtri/s: every rank processes n_tris per step (weak scaling)."""
    return world * n_tris / (ms / 1e3) / 1e6


def measure_diff(dev, steps, adam_steps=0, cpu_baseline=True):
    """Differentiable shading on the 1M-triangle 1080p scene plus a
    vertex-coloured ground grid: device time of the forward frame
    (pr_diff_forward: full render + radiance) and of the backward pass
    (pr_diff_backward), L2 loss against a target rendered with Kd + 0.1,
    light position + (0.5, 0, 0) and vertex colours + N(0, 0.05). With
    adam_steps, also the Adam inverse-rendering loop over 16 views."""
    import numpy as np
    import torch
    from polyred_gb300 import diff, procedural, scene as sc
    s, cam = procedural.diff_scene(width=W, height=H)
    r = diff.DiffRenderer(s, [diff.View(cam, W, H)], device=dev, shadow_size=SHADOW)
    p = r.initial_params()
    g = torch.Generator(device="cpu").manual_seed(0x5EED0005)
    q = {k: v.clone() for k, v in p.items()}
    q["kd"] = (q["kd"] + 0.1).contiguous()
    q["light_pos"] = (q["light_pos"] + torch.tensor([0.5, 0.0, 0.0])).contiguous()
    q["vertex_color"] = (q["vertex_color"] + (torch.randn(q["vertex_color"].shape, generator=g) * 0.05).cuda())
    target = r.forward_raw(0, q)[0]
    stream = torch.cuda.ExternalStream(dev.stream())
    fwd, bwd, wall = [], [], []
    n = max(3, min(steps, 20))
    for it in range(n + 2):
        e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e[0].record(stream)
        rad, gbuf = r.forward_raw(0, p)
        e[1].record(stream)
        grad = torch.zeros_like(rad)
        grad[..., :3] = 2 * (rad[..., :3] - target[..., :3])
        torch.cuda.synchronize()
        e2 = torch.cuda.Event(enable_timing=True)
        e2.record(stream)
        r.backward_raw(0, p, gbuf, grad)
        e[2].record(stream)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        if it >= 2:
            fwd.append(e[0].elapsed_time(e[1]))
            bwd.append(e2.elapsed_time(e[2]))
            wall.append((t1 - t0) * 1e3)
    f, b = statistics.mean(fwd), statistics.mean(bwd)
    out = {"workload": "sphere_field_1M_1080p + 64x64 vertex-coloured ground grid", "n_tris": r.flat.n_tris,
           "fwd_ms": f, "bwd_ms": b, "fwd_bwd_over_fwd": (f + b) / f, "wall_ms_fwd_bwd": statistics.mean(wall),
           "steps": n, "gradients": "vertex colour, vertex normal, kd, ks, shininess, light pos, light intensity, ambient",
           "checked": "tests/test_gpu_diff_full.py: 64 parameters vs FP64 central differences (h=1e-4) within 1e-3 "
                      "relative at 1920x1080"}
    if cpu_baseline:
        # the FP64 reference adjoint (oracle/adjoint.cpp, one thread) on the same G-buffer: radiance and
        # loss, then every gradient
        import oracle
        fdesc = r.frame(0, p["light_pos"].numpy(), p["light_intensity"].numpy(), p["ambient"].numpy())
        npp = {k: v.detach().cpu().numpy().astype(np.float64) for k, v in p.items()}
        inp = oracle.DiffInputs(r.flat, gbuf.cpu().numpy(), npp, fdesc.desc, oracle.normal_matrices(r.flat))
        tgt = target.cpu().numpy()
        t0 = time.perf_counter()
        _, R64 = oracle.diff_forward64(inp, tgt)
        g64 = np.zeros_like(R64)
        g64[..., :3] = 2 * (R64[..., :3] - tgt[..., :3])
        oracle.diff_backward64(inp, g64)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": dt * 1e3, "unit": "ms per fwd+bwd", "cores": 1, "kind": "port",
                               "sample": "one forward + backward of the FP64 reference adjoint on the same "
                                         "1920x1080 G-buffer (shading only: the G-buffer is the GPU's)"}
    if adam_steps:
        cams = [sc.Perspective(position=(24 * np.cos(a), 4, 24 * np.sin(a)), target=(0, 0, 0), up=(0, 1, 0), fov=60,
                               aspect=W / H, near=0.1, far=100) for a in np.linspace(0, 2 * np.pi, 16, endpoint=False)]
        ra = diff.DiffRenderer(s, [diff.View(c, W, H) for c in cams], device=dev, shadow_size=SHADOW)
        targets = [ra.forward_raw(v, q)[0] for v in range(16)]
        x = {k: v.clone() for k, v in p.items()}
        for k in ("kd", "light_pos", "vertex_color"):
            x[k] = x[k].contiguous().requires_grad_(True)
        t0 = time.perf_counter()
        losses = diff.inverse_render(ra, targets, x, ("kd", "light_pos", "vertex_color"), steps=adam_steps, lr=0.01)
        el = time.perf_counter() - t0
        out["adam"] = {"views": 16, "steps": adam_steps, "loss_first": losses[0], "loss_last": losses[-1],
                       "s_total": el, "ms_per_view_step": el * 1e3 / (adam_steps * 16),
                       "trained": "kd, light position, vertex colours (lr 0.01)"}
    return out


def measure_soup(steps=10, n_tris=10_000_000, width=3840, height=2160, cpu_baseline=True):
    """The small-triangle stress workload: 10M soup triangles at 3840x2160
    (log-normal areas around 1 px, 30% back-facing, one point light, no
    shadows, gamma on), resident frames timed with CUDA events."""
    import torch
    from polyred_gb300 import _abi, native, procedural, render
    s, cam = procedural.soup_scene(n_tris, width, height)
    dev = render.Device(0)
    lib = native.load()
    flat = render.FlatScene(s)
    desc = flat.desc()
    native.check(lib.pr_scene_upload(dev.handle, C.byref(desc)))
    opts = dict(width=width, height=height, camera=cam, scene=s, perspective=True, shadow_map=False, gamma=True,
                background=(0, 0, 0, 0), shadow_size=None)
    fd = render.FrameDesc(opts, {})
    rgba = torch.empty((height, width, 4), dtype=torch.uint8, device="cuda")
    od = _abi.pr_outputs()
    od.size = C.sizeof(_abi.pr_outputs)
    od.flags = _abi.PR_OUT_DEVICE_PTRS
    od.rgba = rgba.data_ptr()
    for _ in range(3):
        native.check(lib.pr_render(dev.handle, C.byref(fd.desc), C.byref(od)))
    stream = torch.cuda.ExternalStream(dev.stream())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(steps):
        native.check(lib.pr_render_async(dev.handle, C.byref(fd.desc), C.byref(od)))
        native.check(lib.pr_sync(dev.handle))
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    st = _abi.pr_stats()
    st.size = C.sizeof(_abi.pr_stats)
    native.check(lib.pr_frame_stats(dev.handle, C.byref(st)))
    dev.close()
    res = {"workload": "triangle soup 10M at 3840x2160 (areas log-normal median 1 px, 30% back-facing)",
           "n_tris": n_tris, "value": n_tris / (ms / 1e3) / 1e6, "unit": "Mtri/s", "ms_per_frame": ms,
           "n_raster_tris": st.n_raster_tris, "ms_setup": st.ms_setup, "ms_raster": st.ms_raster,
           "ms_shade": st.ms_shade}
    if cpu_baseline:
        import numpy as np
        import oracle
        threads = os.cpu_count() or 1
        out = render.Outputs(width, height, ("rgba",))
        t0 = time.perf_counter()
        oracle.render(desc, fd.desc, out.desc, shadow_state=None, threads=threads)
        dt = time.perf_counter() - t0
        res["cpu_baseline"] = {"value": n_tris / dt / 1e6, "unit": "Mtri/s", "cores": threads, "kind": "port",
                               "sample": "1 full frame of the workload (C++ restatement of the Go CPU renderer, "
                                         "row-band threads)"}
    return res


def measure_obj(steps=20, n_tori=32, nu=128, nv=64, width=1920, height=1080):
    """OBJ ingestion (model.Load): a 41 MB Wavefront OBJ of 32 tori (524,288
    triangles from 262,144 quads, v/vt/vn, three .mtl materials, some
    triangle+quad objects) in a temporary directory. Host phases, best of 3
    wall-clock runs: native parse (file read included), mesh assembly, scene
    flatten + upload. Then resident frames of the loaded scene at
    width x height (one shadow-casting point light, 2048^2 map), CUDA
    events. CPU baseline: the oracle's pure-Python restatement of obj.go on
    the first 1 MB of the same text."""
    import tempfile
    import torch
    from oracle import objparse
    from polyred_gb300 import _abi, native, objload, procedural, render
    obj, mtl, n_tris = procedural.obj_tori(n_tori, nu, nv)
    tmp = tempfile.mkdtemp()
    path = os.path.join(tmp, "tori.obj")
    with open(path, "wb") as fh:
        fh.write(obj)
    with open(os.path.join(tmp, "tori.mtl"), "wb") as fh:
        fh.write(mtl)
    dev = render.Device(0)
    lib = native.load()
    t_parse = t_build = t_up = float("inf")
    for _ in range(3):
        t0 = time.perf_counter()
        f = objload.parse_file(path)
        t1 = time.perf_counter()
        g = objload.build_group(f, path)
        t2 = time.perf_counter()
        s, cam = procedural.obj_tori_scene(g, width, height)
        flat = render.FlatScene(s)
        desc = flat.desc()
        native.check(lib.pr_scene_upload(dev.handle, C.byref(desc)))
        torch.cuda.synchronize()
        t3 = time.perf_counter()
        t_parse, t_build, t_up = min(t_parse, t1 - t0), min(t_build, t2 - t1), min(t_up, t3 - t2)
    opts = dict(width=width, height=height, camera=cam, scene=s, perspective=True, shadow_map=True, gamma=True,
                background=(0, 0, 0, 0), shadow_size=(2048, 2048), directional_shadows=False)
    fd = render.FrameDesc(opts, shadow_cams(opts))
    rgba = torch.empty((height, width, 4), dtype=torch.uint8, device="cuda")
    od = _abi.pr_outputs()
    od.size = C.sizeof(_abi.pr_outputs)
    od.flags = _abi.PR_OUT_DEVICE_PTRS
    od.rgba = rgba.data_ptr()
    for _ in range(3):
        native.check(lib.pr_render(dev.handle, C.byref(fd.desc), C.byref(od)))
    stream = torch.cuda.ExternalStream(dev.stream())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(steps):
        native.check(lib.pr_render_async(dev.handle, C.byref(fd.desc), C.byref(od)))
        native.check(lib.pr_sync(dev.handle))
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    dev.close()
    sample = obj[:1 << 20]
    sample = sample[:sample.rindex(b"\n") + 1]
    spath = os.path.join(tmp, "sample.obj")
    with open(spath, "wb") as fh:
        fh.write(sample.replace(b"mtllib tori.mtl\n", b""))
    c0 = time.perf_counter()
    objparse.load_file(spath)
    c1 = time.perf_counter()
    mb = len(obj) / 1e6
    return {"workload": f"Wavefront OBJ, {n_tori} tori of {nu}x{nv} quads ({mb:.1f} MB, {n_tris} triangles), "
                        f"{width}x{height}",
            "file_mb": mb, "n_tris": n_tris, "parse_ms": t_parse * 1e3, "parse_mb_s": mb / t_parse,
            "assemble_ms": t_build * 1e3, "flatten_upload_ms": t_up * 1e3,
            "load_to_resident_ms": (t_parse + t_build + t_up) * 1e3,
            "frame_ms": ms, "frame_mtri_s": n_tris / (ms / 1e3) / 1e6,
            "cpu_baseline": {"value": len(sample) / 1e6 / (c1 - c0), "unit": "MB/s", "cores": 1, "kind": "port",
                             "sample": "obj.go restated in pure Python, first 1 MB of the same OBJ text"}}


def _resident_frames(s, cam, width, height, steps, msaa=1, shadow_size=SHADOW, shadow_map=True):
    """ms per resident frame of scene s (CUDA events on the context's stream)."""
    import torch
    from polyred_gb300 import _abi, native, render
    dev = render.Device(0)
    lib = native.load()
    flat = render.FlatScene(s)
    desc = flat.desc()
    native.check(lib.pr_scene_upload(dev.handle, C.byref(desc)))
    opts = dict(width=width, height=height, camera=cam, scene=s, perspective=True, shadow_map=shadow_map, gamma=True,
                background=(0, 0, 0, 0), shadow_size=shadow_size, directional_shadows=True, msaa=msaa)
    fd = render.FrameDesc(opts, shadow_cams(opts) if shadow_map else {})
    rgba = torch.empty((height, width, 4), dtype=torch.uint8, device="cuda")
    od = _abi.pr_outputs()
    od.size = C.sizeof(_abi.pr_outputs)
    od.flags = _abi.PR_OUT_DEVICE_PTRS
    od.rgba = rgba.data_ptr()
    for _ in range(3):
        native.check(lib.pr_render(dev.handle, C.byref(fd.desc), C.byref(od)))
    stream = torch.cuda.ExternalStream(dev.stream())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(steps):
        native.check(lib.pr_render_async(dev.handle, C.byref(fd.desc), C.byref(od)))
    e1.record(stream)
    native.check(lib.pr_sync(dev.handle))
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    dev.close()
    return ms


def measure_msaa(steps=20):
    """render.MSAA(2) on the workload: the 999,936-triangle sphere field into
    a 3840x2160 framebuffer (viewport test and clipping at 7680x4320, shadow
    maps 2048^2), resized to the 1920x1080 image."""
    s, cam = workload()
    ms = _resident_frames(s, cam, W, H, steps, msaa=2)
    return {"workload": "sphere field, 1920x1080 image, MSAA 2 (3840x2160 framebuffer)", "n_tris": N_TRIS,
            "ms_per_frame": ms, "value": N_TRIS / (ms / 1e3) / 1e6, "unit": "Mtri/s"}


def measure_small(steps=200, width=800, height=500, cpu_baseline=True):
    """The small CPU-runnable workload: the 64x32 UV sphere (3,968 triangles)
    on a 2-triangle ground, one point light, ambient 0.1, shadows off, gamma
    on, 800x500; resident frames, and the oracle on one frame (all host
    threads)."""
    from polyred_gb300 import procedural, render
    s, cam = procedural.small_scene(width, height)
    n = render.FlatScene(s).n_tris
    ms = _resident_frames(s, cam, width, height, steps, shadow_size=None, shadow_map=False)
    res = {"workload": "UV sphere 64x32 on a ground plane, 800x500, no shadows", "n_tris": n,
           "ms_per_frame": ms, "frames_per_s": 1e3 / ms, "value": n / (ms / 1e3) / 1e6, "unit": "Mtri/s"}
    if cpu_baseline:
        import oracle
        threads = os.cpu_count() or 1
        flat = render.FlatScene(s)
        opts = dict(width=width, height=height, camera=cam, scene=s, perspective=True, shadow_map=False, gamma=True,
                    background=(0, 0, 0, 0), shadow_size=None)
        fd = render.FrameDesc(opts, {})
        out = render.Outputs(width, height, ("rgba",))
        oracle.render(flat.desc(), fd.desc, out.desc, threads=threads)  # warm
        t0 = time.perf_counter()
        reps = 5
        for _ in range(reps):
            oracle.render(flat.desc(), fd.desc, out.desc, threads=threads)
        dt = (time.perf_counter() - t0) / reps
        res["cpu_baseline"] = {"value": 1.0 / dt, "unit": "frames/s", "cores": threads, "kind": "port",
                               "sample": "5 frames of the workload (C++ restatement of the Go CPU renderer, "
                                         "row-band threads)"}
    return res


def measure_textured(steps=50, width=1920, height=1080):
    """Image textures: procedural.textured_scene at 1920x1080 (a mipmapped
    256^2 texture, a 37x300 mipmapped texture, a 64x16 texture without
    mipmaps; 6,146 triangles; one shadow-casting light with a framebuffer-size
    map), resident frames."""
    from polyred_gb300 import procedural
    s, cam = procedural.textured_scene(width, height)
    ms = _resident_frames(s, cam, width, height, steps, shadow_size=None)
    return {"workload": "textured spheres and ground, 1920x1080", "ms_per_frame": ms, "frames_per_s": 1e3 / ms}


def measure_batch(reps=3, cpu_baseline=True):
    """The batched workload (32 sphere scenes of 1k-500k triangles, 8 ring
    views each at 1280x720, 16 casting point lights per scene with 1024^2
    maps, AO on): views/s of one tuned pr_batch_render against the same 256
    views rendered one pr_render_async at a time on one context per scene."""
    import torch
    from polyred_gb300 import _abi, batch as pb, native, render
    scenes, specs = pb.config4()
    b = pb.Batch(0)
    for s in scenes:
        b.add_scene(s)
    arr, outs, keep = b.views(specs, ("rgba",))
    tune = b.tune(arr)
    times = []
    for _ in range(reps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        b.render(arr)
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
    st_b = b.stats()
    bt = min(times)
    b.close()
    del outs, keep
    # plain: one context per scene, one frame per view (first-frame shadow maps)
    lib = native.load()
    devs = []
    for s in scenes:
        d = render.Device(0)
        fl = render.FlatScene(s)
        desc = fl.desc()
        native.check(lib.pr_scene_upload(d.handle, C.byref(desc)))
        devs.append(d)
    fds, ods, bufs = [], [], []
    for si, opts, cams in specs:
        fd = render.FrameDesc(opts, cams)
        t = torch.empty((opts["height"], opts["width"], 4), dtype=torch.uint8, device="cuda")
        od = _abi.pr_outputs()
        od.size = C.sizeof(_abi.pr_outputs)
        od.flags = _abi.PR_OUT_DEVICE_PTRS
        od.rgba = t.data_ptr()
        fds.append(fd)
        ods.append(od)
        bufs.append(t)

    def plain_pass():
        for (si, _, _), fd, od in zip(specs, fds, ods):
            native.check(lib.pr_shadow_reset(devs[si].handle))
            native.check(lib.pr_render_async(devs[si].handle, C.byref(fd.desc), C.byref(od)))
        for d in devs:
            native.check(lib.pr_sync(d.handle))

    for (si, _, _), fd, od in zip(specs, fds, ods):  # warm-up: synchronous frames size the buffers
        native.check(lib.pr_shadow_reset(devs[si].handle))
        native.check(lib.pr_render(devs[si].handle, C.byref(fd.desc), C.byref(od)))
    pt, ps = [], []
    for _ in range(reps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        plain_pass()
        torch.cuda.synchronize()
        pt.append(time.perf_counter() - t0)
    for _ in range(reps):  # one synchronous Render() per view
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for (si, _, _), fd, od in zip(specs, fds, ods):
            native.check(lib.pr_shadow_reset(devs[si].handle))
            native.check(lib.pr_render(devs[si].handle, C.byref(fd.desc), C.byref(od)))
        torch.cuda.synchronize()
        ps.append(time.perf_counter() - t0)
    # the synchronous plain views once more, each timed alone: wall time
    # against the frame's device span (CUDA events inside the library, from
    # the first kernel to the last), by scene size
    sizes = [render.FlatScene(s).n_tris for s in scenes]
    by_bucket = {}
    for (si, _, _), fd, od in zip(specs, fds, ods):
        t0 = time.perf_counter()
        native.check(lib.pr_shadow_reset(devs[si].handle))
        native.check(lib.pr_render(devs[si].handle, C.byref(fd.desc), C.byref(od)))
        wall = (time.perf_counter() - t0) * 1e3
        st = _abi.pr_stats()
        st.size = C.sizeof(_abi.pr_stats)
        native.check(lib.pr_frame_stats(devs[si].handle, C.byref(st)))
        n = sizes[si]
        key = "1k-10k" if n < 10_000 else ("10k-100k" if n < 100_000 else "100k-500k")
        b_ = by_bucket.setdefault(key, {"views": 0, "wall_ms": 0.0, "device_span_ms": 0.0,
                                        "kernel_launches_per_view": st.n_kernel_launches})
        b_["views"] += 1
        b_["wall_ms"] += wall
        b_["device_span_ms"] += st.ms_total
    for d in devs:
        d.close()
    n = len(specs)
    res = {"workload": "32 sphere scenes (1k-500k tris, log-uniform) x 8 views 1280x720, 16 casting point lights, "
                       "1024^2 maps, AO", "n_views": n, "n_tris_total": int(sum(sizes)),
           "n_passes": st_b["n_passes"], "batched_views_per_s": n / bt, "plain_views_per_s": n / min(ps),
           "batched_over_plain": min(ps) / bt, "plain": "one synchronous pr_render per view",
           "plain_async_views_per_s": n / min(pt), "batched_over_plain_async": min(pt) / bt,
           "plain_async": "pr_render_async per view, one context and stream per scene",
           "batched_ms": bt * 1e3, "batched_device_ms": st_b["ms_total"], "plain_ms": min(ps) * 1e3,
           "plain_by_bucket": by_bucket,
           "kernel_launches_per_batch": st_b["n_kernel_launches"],
           "graph_reused": st_b["graph_reused"], "device_gb": st_b["device_bytes"] / 1e9, "tuned": tune}
    if cpu_baseline:
        # the oracle on a bounded sample: view 0 of the smallest, a median and the largest scene
        import numpy as np
        import oracle
        threads = os.cpu_count() or 1
        order = np.argsort(sizes)
        pick = [int(order[0]), int(order[len(order) // 2]), int(order[-1])]
        t0 = time.perf_counter()
        for si in pick:
            k = [j for j, sp in enumerate(specs) if sp[0] == si][0]
            _, opts, cams = specs[k]
            flat = render.FlatScene(scenes[si])
            src, _ = opts["scene"].lights()
            sw, sh = opts["shadow_size"]
            out = render.Outputs(opts["width"], opts["height"], ("rgba",))
            oracle.render(flat.desc(), fds[k].desc, out.desc,
                          shadow_state=np.zeros((len(src), sh, sw), np.float32), threads=threads)
        dt = time.perf_counter() - t0
        res["cpu_baseline"] = {"value": len(pick) / dt, "unit": "views/s", "cores": threads, "kind": "port",
                               "sample": f"3 views (scenes of {sizes[pick[0]]}, {sizes[pick[1]]} and "
                                         f"{sizes[pick[2]]} triangles) rendered by the oracle, row-band threads"}
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-diff", action="store_true", help="skip the differentiable-shading measurement")
    ap.add_argument("--adam", type=int, default=200, help="Adam steps of the 16-view inverse-rendering loop (0: skip)")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-views measurement")
    ap.add_argument("--no-soup", action="store_true", help="skip the 10M-triangle 4K soup measurement")
    ap.add_argument("--no-obj", action="store_true", help="skip the OBJ ingestion measurement")
    ap.add_argument("--no-msaa", action="store_true", help="skip the MSAA and image-texture measurements")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        run_reference(args, rank)
        return

    import numpy as np
    import torch
    import torch.distributed as dist
    from polyred_gb300 import _abi, build, native, render

    build.build()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    lib = native.load()
    dev = render.Device(local)
    s, cam = workload()
    opts = frame_opts(s, cam)
    flat = render.FlatScene(s)
    # pinned host copies of the soup for the end-to-end leg
    pinned = {}
    for name in ("pos", "nor", "uv", "col", "mat_id"):
        a = getattr(flat, name)
        t = torch.empty(a.shape, dtype={np.float32: torch.float32, np.uint8: torch.uint8,
                                        np.int32: torch.int32}[a.dtype.type], pin_memory=True)
        t.numpy()[...] = a
        pinned[name] = t
        setattr(flat, name, t.numpy())
    desc = flat.desc()
    native.check(lib.pr_scene_upload(dev.handle, C.byref(desc)))
    fd = render.FrameDesc(opts, shadow_cams(opts))
    # device outputs for the resident leg
    rgba = torch.empty((H, W, 4), dtype=torch.uint8, device="cuda")
    tri = torch.empty((H, W), dtype=torch.int32, device="cuda")
    dep = torch.empty((H, W), dtype=torch.float32, device="cuda")
    od = _abi.pr_outputs()
    od.size = C.sizeof(_abi.pr_outputs)
    od.flags = _abi.PR_OUT_DEVICE_PTRS
    od.rgba, od.tri_id, od.depth = rgba.data_ptr(), tri.data_ptr(), dep.data_ptr()
    stream = torch.cuda.ExternalStream(dev.stream())

    def stats():
        st = _abi.pr_stats()
        st.size = C.sizeof(_abi.pr_stats)
        native.check(lib.pr_frame_stats(dev.handle, C.byref(st)))
        return st

    # warm-up (also sizes the internal buffers; the synchronous call retries on overflow)
    for _ in range(args.warmup):
        native.check(lib.pr_render(dev.handle, C.byref(fd.desc), C.byref(od)))

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    # ---- resident leg ----
    clocks = ClockSampler(local)
    clocks.start()
    barrier()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    phases = {"ms_shadow": [], "ms_setup": [], "ms_raster": [], "ms_shade": [], "ms_ao": [], "n_ao_pixels": []}
    # frames back to back on the library's stream, as a frame loop issues them
    ev0.record(stream)
    for _ in range(args.steps):
        native.check(lib.pr_render_async(dev.handle, C.byref(fd.desc), C.byref(od)))
    ev1.record(stream)
    barrier()
    clk = clocks.stop()
    ms = max_over_ranks(ev0.elapsed_time(ev1) / args.steps, world, "cuda")
    value = job_throughput(N_TRIS, world, ms)

    # per-phase device times (CUDA events inside the library, same stream) and
    # launch counts: three more frames, each synchronised so that its
    # statistics can be read (not timed)
    per_frame = 0
    for _ in range(3):
        native.check(lib.pr_render_async(dev.handle, C.byref(fd.desc), C.byref(od)))
        native.check(lib.pr_sync(dev.handle))
        st = stats()
        per_frame = st.n_kernel_launches
        for k in phases:
            phases[k].append(getattr(st, k))
    launches = per_frame * args.steps
    ph = {k: statistics.mean(v) for k, v in phases.items() if v}

    # ---- end-to-end leg (public C ABI, host buffers in page-locked memory) ----
    out = render.Outputs(W, H, ("rgba", "tri_id", "depth"), pinned=True)
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        # upload + frame + readback; the next step's upload overlaps this frame
        native.check(lib.pr_frame_submit(dev.handle, C.byref(desc), C.byref(fd.desc), C.byref(out.desc)))
    native.check(lib.pr_sync(dev.handle))
    e1.record(stream)
    barrier()
    ems = max_over_ranks(e0.elapsed_time(e1) / args.steps, world, "cuda")
    h2d = sum(getattr(flat, n).nbytes for n in ("pos", "nor", "uv", "col", "mat_id"))
    d2h = W * H * (4 + 4 + 4)

    # roofline of the dominant kernel, ao_kernel (AmbientOcclusionShade):
    # algorithmic bytes per launch = the depth buffer read once (4 B/px) +
    # per AO pixel its list entry (4 B) and its colour read and written (8 B)
    peak, peak_kind = measured_peaks()
    ao_ms = ph.get("ms_ao", 0.0)
    n_ao = ph.get("n_ao_pixels", 0.0)
    alg_bytes = W * H * 4 + n_ao * 12
    achieved = alg_bytes / (ao_ms / 1e3) / 1e9 if ao_ms > 0 else 0.0
    traffic = ncu_traffic()
    # the bound that limits it: instruction issue. Each SM issues at most one
    # warp instruction per clock on each of its 4 schedulers.
    n_sms = torch.cuda.get_device_properties(local).multi_processor_count
    sm_mhz = (clk or {}).get("sm_mhz") or 2070.0
    inst = ncu_instructions()
    issue = None
    if inst and ao_ms > 0:
        issue = {"kernel": "ao_kernel", "warp_instructions": inst, "duration_ms": ao_ms, "sm_mhz": sm_mhz,
                 "n_sms": n_sms, "frac": inst / (n_sms * 4 * sm_mhz * 1e6 * ao_ms / 1e3),
                 "source": "instructions per launch from the ncu summary "
                           "profiles/ao_kernel_sphere_field_1080p.txt, duration from this run's CUDA events"}

    if rank == 0:
        line = {"metric": "1080p Mtri/s", "value": value, "unit": "Mtri/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": bench_config(world),
                "frames_per_s": world * 1e3 / ms,
                "e2e": {"value": job_throughput(N_TRIS, world, ems), "unit": "Mtri/s", "h2d_bytes_per_step": h2d,
                        "d2h_bytes_per_step": d2h, "ms_per_step": ems},
                "phases_ms": ph,
                "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                             "frac": achieved / peak if peak else None, "traffic": traffic,
                             "kernel": "ao_kernel", "peak_source": peak_kind,
                             "algorithmic_bytes": alg_bytes,
                             "note": "issue-bound: 8 x 99 dependent depth taps per pixel (L1/L2 resident); "
                                     "see issue", "issue": issue},
                "gpu_launches": launches,
                "clocks": clk}
        if not args.no_diff:
            line["diff"] = measure_diff(dev, args.steps, args.adam, cpu_baseline=world == 1 and not args.no_cpu_baseline)
        if not args.no_soup:
            line["soup_4k"] = measure_soup(cpu_baseline=world == 1 and not args.no_cpu_baseline)
        if not args.no_batch:
            line["batched"] = measure_batch(cpu_baseline=world == 1 and not args.no_cpu_baseline)
        try:
            line["small_800x500"] = measure_small(cpu_baseline=world == 1 and not args.no_cpu_baseline)
        except Exception as e:  # the headline line must still print
            line["small_800x500"] = {"error": f"{type(e).__name__}: {e}"}
        if not args.no_msaa:
            try:
                line["msaa_2x"] = measure_msaa()
                line["textured_1080p"] = measure_textured()
            except Exception as e:  # the headline line must still print
                line["msaa_2x"] = {"error": f"{type(e).__name__}: {e}"}
        if not args.no_obj:
            try:
                line["obj_ingest"] = measure_obj()
            except Exception as e:  # the headline line must still print
                line["obj_ingest"] = {"error": f"{type(e).__name__}: {e}"}
        if world == 1 and not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline_sample()
        print(json.dumps(line), flush=True)
    dev.close()
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
