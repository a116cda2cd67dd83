"""Seeded procedural scenes for the render path's workloads.

  uv_sphere       latitude/longitude sphere, normals = positions
  ground_plane    two triangles, MaterialID -1 (vertex colour, like model/plane.go)
  small_scene     one UV sphere (64 lon x 32 lat = 3,968 triangles) on a 10x10
                  ground, 800x500, one point light + ambient 0.1
  sphere_field    256 spheres of 63 x 32 segments (999,936 triangles), centres
                  U[-10,10]^3, radii U[0.2,1.5], 4 materials, point +
                  directional light, AO and shadow maps
  triangle_soup   small random triangles with log-normal screen area
  textured_scene  spheres and a ground with image textures (mipmapped and
                  not, square and not)
  obj_tori        Wavefront OBJ / MTL text of a field of tori (quads with vt
                  and vn, three materials, some triangle+quad objects, some
                  negative indices) for the OBJ loading path

Random numbers: splitmix64 seeds a xoshiro128** generator; floats are the top
24 bits of a draw times 2^-24.
"""
import math

import numpy as np

from . import scene as sc

F32 = np.float32


class Xoshiro128:
    """xoshiro128** seeded from splitmix64 (public-domain generators by
    Blackman and Vigna)."""

    def __init__(self, seed):
        s = seed & 0xFFFFFFFFFFFFFFFF
        words = []
        for _ in range(2):
            s = (s + 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF
            z = s
            z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & 0xFFFFFFFFFFFFFFFF
            z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & 0xFFFFFFFFFFFFFFFF
            z ^= z >> 31
            words += [z & 0xFFFFFFFF, z >> 32]
        self.s = words

    @staticmethod
    def _rotl(x, k):
        return ((x << k) | (x >> (32 - k))) & 0xFFFFFFFF

    def next_u32(self):
        s = self.s
        result = (self._rotl((s[1] * 5) & 0xFFFFFFFF, 7) * 9) & 0xFFFFFFFF
        t = (s[1] << 9) & 0xFFFFFFFF
        s[2] ^= s[0]
        s[3] ^= s[1]
        s[1] ^= s[2]
        s[0] ^= s[3]
        s[2] ^= t
        s[3] = self._rotl(s[3], 11)
        return result

    def uniform(self, lo=0.0, hi=1.0):
        return lo + (hi - lo) * ((self.next_u32() >> 8) * (1.0 / 16777216.0))

    def integer(self, n):
        return self.next_u32() % n


def uv_sphere(lon=64, lat=32, radius=1.0, color=(255, 255, 255, 255)):
    """A UV sphere with 2*lon*(lat-1) triangles, wound counter-clockwise seen
    from outside; normals equal the unit positions (w = 0), positions w = 1."""
    th = np.pi * np.arange(lat + 1) / lat
    ph = 2 * np.pi * np.arange(lon + 1) / lon
    P = np.zeros((lat + 1, lon + 1, 3))
    P[..., 0] = np.sin(th)[:, None] * np.cos(ph)[None, :]
    P[..., 1] = np.cos(th)[:, None] * np.ones_like(ph)[None, :]
    P[..., 2] = -np.sin(th)[:, None] * np.sin(ph)[None, :]
    P[0, :] = (0, 1, 0)
    P[lat, :] = (0, -1, 0)
    UV = np.stack(np.meshgrid(np.arange(lon + 1) / lon, np.arange(lat + 1) / lat), -1)
    tris = []
    for j in range(lat):
        for i in range(lon):
            a, b, c, d = (j, i), (j, i + 1), (j + 1, i), (j + 1, i + 1)
            if j == 0:
                tris.append((a, c, d))
            elif j == lat - 1:
                tris.append((a, c, b))
            else:
                tris.append((a, c, d))
                tris.append((a, d, b))
    idx = np.array(tris)  # (n, 3, 2)
    pos = P[idx[..., 0], idx[..., 1]]
    # orient every triangle outward (counter-clockwise seen from outside)
    nrm = np.cross(pos[:, 1] - pos[:, 0], pos[:, 2] - pos[:, 0])
    flip = (nrm * pos.mean(axis=1)).sum(-1) < 0
    idx[flip] = idx[flip][:, [0, 2, 1]]
    pos = P[idx[..., 0], idx[..., 1]]
    uv = UV[idx[..., 0], idx[..., 1]]
    n = idx.shape[0]
    p4 = np.ones((n, 3, 4), F32)
    p4[..., :3] = pos * radius
    n4 = np.zeros((n, 3, 4), F32)
    n4[..., :3] = pos
    col = np.empty((n, 3, 4), np.uint8)
    col[:] = color
    return sc.Mesh(p4, n4, uv.astype(F32), col, np.zeros(n, np.int32))


def ground_plane(size=10.0, y=-1.0, color=(128, 128, 128, 255), material_id=-1):
    """Two triangles on y = const facing +y (like model/plane.go, which uses
    MaterialID -1 so the ground shows its vertex colour)."""
    h = size / 2
    q = np.array([[-h, y, h], [h, y, h], [h, y, -h], [-h, y, -h]], np.float64)
    tri = np.array([[0, 1, 2], [0, 2, 3]])
    pos = np.ones((2, 3, 4), F32)
    pos[..., :3] = q[tri]
    nor = np.zeros((2, 3, 4), F32)
    nor[..., 1] = 1
    uv = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], F32)[tri]
    col = np.empty((2, 3, 4), np.uint8)
    col[:] = color
    return sc.Mesh(pos, nor, uv, col, np.full(2, material_id, np.int32))


def small_scene(width=800, height=500):
    """The small CPU-runnable workload: a 64x32 UV sphere (3,968 triangles)
    on a 2-triangle ground, one point light, ambient 0.1, no shadows."""
    kd = sc.color_from_value(0.8, 0.3, 0.2, 1.0)
    ks = sc.color_from_value(0.5, 0.5, 0.5, 1.0)
    mat = sc.BlinnPhong(diffuse=kd, specular=ks, shininess=32)
    sphere = sc.Geometry(uv_sphere(64, 32, 1.0), mat)
    ground = sc.Geometry(ground_plane(10.0, -1.0))
    s = sc.Scene(sphere, ground, sc.Point(position=(4, 4, 2), intensity=1.0), sc.Ambient(intensity=0.1))
    cam = sc.Perspective(position=(0, 1.5, 4), target=(0, 0, 0), up=(0, 1, 0), fov=45, aspect=width / height,
                         near=0.1, far=100)
    return s, cam


def checkerboard_image(width, height, cells=8, seed=0x7E47):
    """A seeded RGBA8 test image: a colour checkerboard of cells x cells
    squares with a noise band and a transparent corner (rows top-down)."""
    y, x = np.mgrid[0:height, 0:width]
    cx, cy = (x * cells) // max(width, 1), (y * cells) // max(height, 1)
    img = np.zeros((height, width, 4), np.uint8)
    odd = (cx + cy) % 2 == 1
    img[..., 0] = np.where(odd, 230, 40)
    img[..., 1] = (x * 255 // max(width - 1, 1)).astype(np.uint8)
    img[..., 2] = (y * 255 // max(height - 1, 1)).astype(np.uint8)
    img[..., 3] = 255
    rng = np.random.default_rng(seed)
    band = slice(height // 3, height // 3 + max(height // 8, 1))
    img[band, :, :3] = rng.integers(0, 256, img[band, :, :3].shape, dtype=np.uint8)
    img[: height // 4, : width // 4, 3] = 0
    return img


def textured_scene(width=800, height=500):
    """Image textures: a 64x32 UV sphere with a mipmapped 256x256 checkerboard,
    a ground with a 64x16 texture sampled without mipmaps (queryL0), and a
    second sphere with a 37x300 mipmapped texture (non-square, not a power
    of two); one shadow-casting point light and ambient 0.15."""
    ks = sc.color_from_value(0.5, 0.5, 0.5, 1.0)
    m_sphere = sc.BlinnPhong(diffuse=sc.color_from_value(0.8, 0.8, 0.8, 1.0), specular=ks, shininess=32,
                             texture=sc.ImageTexture(checkerboard_image(256, 256), mipmap=True))
    m_ground = sc.BlinnPhong(diffuse=sc.color_from_value(0.6, 0.6, 0.6, 1.0), specular=ks, shininess=8,
                             texture=sc.ImageTexture(checkerboard_image(64, 16, cells=4, seed=3), mipmap=False))
    m_small = sc.BlinnPhong(diffuse=sc.color_from_value(0.9, 0.9, 0.9, 1.0), specular=ks, shininess=16,
                            texture=sc.ImageTexture(checkerboard_image(37, 300, cells=5, seed=5), mipmap=True))
    sphere = sc.Geometry(uv_sphere(64, 32, 1.0), m_sphere)
    small = sc.Geometry(uv_sphere(32, 16, 0.5), m_small).translate(1.6, -0.5, 0.6)
    ground = sc.Geometry(ground_plane(10.0, -1.0, material_id=0), m_ground)
    s = sc.Scene(sphere, small, ground, sc.Point(position=(4, 4, 2), intensity=1.0, cast_shadow=True),
                 sc.Ambient(intensity=0.15))
    cam = sc.Perspective(position=(0, 1.5, 4), target=(0, 0, 0), up=(0, 1, 0), fov=45, aspect=width / height,
                         near=0.1, far=100)
    return s, cam


def sphere_materials(ao=True):
    """The four Blinn-Phong materials of the sphere field."""
    return [
        sc.BlinnPhong(diffuse=sc.color_from_value(0.8, 0.3, 0.2), specular=sc.color_from_value(0.5, 0.5, 0.5),
                      shininess=32, ambient_occlusion=ao, receive_shadow=True),
        sc.BlinnPhong(diffuse=sc.color_from_value(0.2, 0.5, 0.8), specular=sc.color_from_value(0.5, 0.5, 0.5),
                      shininess=16, ambient_occlusion=ao, receive_shadow=True),
        sc.BlinnPhong(diffuse=sc.color_from_value(0.3, 0.8, 0.3), specular=sc.color_from_value(0.5, 0.5, 0.5),
                      shininess=64, ambient_occlusion=ao, receive_shadow=True, flat_shading=True),
        sc.BlinnPhong(diffuse=sc.color_from_value(0.9, 0.9, 0.9), specular=sc.color_from_value(0.5, 0.5, 0.5),
                      shininess=8, ambient_occlusion=ao, receive_shadow=True),
    ]


def sphere_field(n_spheres=256, lon=63, lat=32, seed=0x5EED0002, width=1920, height=1080, ao=True,
                 directional_shadow=True):
    """The 1M-triangle workload: 256 spheres of 3,906 triangles each."""
    rng = Xoshiro128(seed)
    materials = sphere_materials(ao)
    mesh = uv_sphere(lon, lat, 1.0)
    objs = []
    for _ in range(n_spheres):
        c = [rng.uniform(-10, 10) for _ in range(3)]
        r = rng.uniform(0.2, 1.5)
        m = materials[rng.integer(4)]
        g = sc.Geometry(mesh, m)
        g.scale(r, r, r).translate(*c)
        objs.append(g)
    s = sc.Scene(*objs)
    s.add(sc.Point(position=(14, 18, 12), intensity=1.0, cast_shadow=True),
          sc.Directional(direction=(-1, -1, -0.5), intensity=0.6, cast_shadow=directional_shadow),
          sc.Ambient(intensity=0.1))
    cam = sc.Perspective(position=(0, 4, 24), target=(0, 0, 0), up=(0, 1, 0), fov=60, aspect=width / height,
                         near=0.1, far=100)
    return s, cam


def ground_grid(n=64, size=24.0, y=-11.0, seed=0x5EED0005):
    """An n x n quad grid (2 n^2 triangles) on y = const facing +y, with
    random per-vertex colours and MaterialID -1 (shown with its vertex
    colours, as model/plane.go's ground)."""
    g = np.random.default_rng(seed)
    h = size / 2
    xs = np.linspace(-h, h, n + 1)
    X, Z = np.meshgrid(xs, xs, indexing="ij")
    P = np.stack([X, np.full_like(X, y), Z], -1)
    C = g.integers(40, 216, (n + 1, n + 1, 4))
    C[..., 3] = 255
    pos, col = [], []
    for i in range(n):
        for j in range(n):
            a, b, c, d = (i, j + 1), (i + 1, j + 1), (i + 1, j), (i, j)
            for tri in ((a, b, c), (a, c, d)):
                pos.append([P[v] for v in tri])
                col.append([C[v] for v in tri])
    pos = np.asarray(pos)
    nt = len(pos)
    p4 = np.ones((nt, 3, 4), F32)
    p4[..., :3] = pos
    nor = np.zeros((nt, 3, 4), F32)
    nor[..., 1] = 1
    uv = np.zeros((nt, 3, 2), F32)
    return sc.Mesh(p4, nor, uv, np.asarray(col, np.uint8), np.full(nt, -1, np.int32))


def diff_scene(width=1920, height=1080, n_spheres=256, lon=63, lat=32, grid=64):
    """The differentiation workload: the 1M-triangle sphere field (AO off,
    both lights casting shadows) over a vertex-coloured ground grid, so that
    per-vertex colours, normals, materials and lights all reach the image."""
    s, cam = sphere_field(n_spheres=n_spheres, lon=lon, lat=lat, width=width, height=height, ao=False)
    s.add(sc.Geometry(ground_grid(grid)))
    return s, cam


def triangle_soup(n_tris, width, height, seed=0x5EED0003, back_fraction=0.30, fov=60.0):
    """Small-triangle stress soup: centroids uniform on screen, view depth
    U[0.1, 100], area ~ LogNormal(ln 1 px^2, 1.0), random shape/orientation,
    winding flipped with probability back_fraction; unprojected to world
    space through a camera at the origin looking down -z."""
    g = np.random.default_rng(seed)
    cx = g.uniform(0, width, n_tris)
    cy = g.uniform(0, height, n_tris)
    depth = g.uniform(0.1, 100.0, n_tris)
    area = np.exp(g.normal(0.0, 1.0, n_tris))  # px^2, median 1
    ang = g.uniform(0, 2 * np.pi, n_tris)
    side = np.sqrt(4 * area / np.sqrt(3))  # equilateral of that area
    base = np.stack([np.cos(ang[:, None] + np.array([0, 2, 4]) * np.pi / 3),
                     np.sin(ang[:, None] + np.array([0, 2, 4]) * np.pi / 3)], -1)  # (n,3,2) unit circle
    jitter = g.uniform(0.6, 1.4, (n_tris, 3, 1))
    sx = cx[:, None] + base[..., 0] * side[:, None] / np.sqrt(3) * jitter[..., 0]
    sy = cy[:, None] + base[..., 1] * side[:, None] / np.sqrt(3) * jitter[..., 0]
    flip = g.uniform(0, 1, n_tris) < back_fraction
    sx[flip] = sx[flip][:, ::-1]
    sy[flip] = sy[flip][:, ::-1]
    t = math.tan(math.radians(fov) / 2)
    aspect = width / height
    ndc_x = sx / width * 2 - 1
    ndc_y = sy / height * 2 - 1
    z = -depth[:, None] * np.ones((1, 3))
    X = ndc_x * t * aspect * depth[:, None]
    Y = ndc_y * t * depth[:, None]
    pos = np.ones((n_tris, 3, 4), F32)
    pos[..., 0], pos[..., 1], pos[..., 2] = X, Y, z
    nrm = np.cross(pos[:, 1, :3] - pos[:, 0, :3], pos[:, 2, :3] - pos[:, 0, :3])
    nrm /= np.linalg.norm(nrm, axis=-1, keepdims=True) + 1e-30
    nor = np.zeros((n_tris, 3, 4), F32)
    nor[..., :3] = nrm[:, None, :]
    col = g.integers(0, 256, (n_tris, 3, 4), dtype=np.uint8)
    col[..., 3] = 255
    return sc.Mesh(pos, nor, None, col, np.zeros(n_tris, np.int32))


def soup_scene(n_tris, width, height, seed=0x5EED0003):
    """The small-triangle stress workload: a triangle soup (triangle_soup)
    with one Blinn-Phong material, one point light and ambient 0.1, seen by
    the camera the soup was unprojected through; no shadows."""
    mesh = triangle_soup(n_tris, width, height, seed=seed)
    mat = sc.BlinnPhong(diffuse=sc.color_from_value(0.8, 0.3, 0.2, 1.0), specular=sc.color_from_value(0.5, 0.5, 0.5, 1.0),
                        shininess=32)
    s = sc.Scene(sc.Geometry(mesh, mat), sc.Point(position=(0, 5, 5)), sc.Ambient(intensity=0.1))
    cam = sc.Perspective(position=(0, 0, 0), target=(0, 0, -1), up=(0, 1, 0), fov=60, aspect=width / height, near=0.1,
                         far=120)
    return s, cam


# ---------------------------------------------------------------- OBJ text

OBJ_TORI_MTL = (b"newmtl m0\nKa 1 1 1\nKd 0.8 0.3 0.2\nKs 0.5 0.5 0.5\nNs 32\nillum 2\n"
                b"newmtl m1\nKd 0.2 0.6 0.9\nKs 0.3 0.3 0.3\nNs 64\nd 1\nillum 2\n"
                b"newmtl m2\nKd 0.9 0.9 0.9\nKs 0.1 0.1 0.1\nNs 8\nillum 0\n")


def _rows(tag, arr, fmt):
    line = tag + " " + " ".join([fmt] * arr.shape[1])
    return "\n".join(line % tuple(r) for r in arr.tolist())


def obj_tori(n_tori=32, nu=128, nv=64, seed=0x0B17041, hybrid_every=3, relative_every=4):
    """OBJ and MTL text of n_tori tori, each 'o torus<k>' with 'usemtl
    m<k % 3>', nu x nv grid vertices (v, vt, vn) and nu x nv quad faces
    wound outward. Every hybrid_every-th torus writes its first 16 quads as
    two triangles each (triangles + quads: the reference's PolygonMesh,
    MaterialID -1); every relative_every-th uses negative (relative)
    indices. Centres U[-8,8] x U[-2,2] x U[-8,8], R U[0.8,1.6], r = R x
    U[0.2,0.4], tilted about x by U[0, pi). Returns (obj_bytes, mtl_bytes,
    n_tris)."""
    rng = Xoshiro128(seed)
    out = ["# tori field: %d tori of %d x %d quads" % (n_tori, nu, nv), "mtllib tori.mtl"]
    iu, jv = np.meshgrid(np.arange(nu), np.arange(nv), indexing="ij")
    u = (2.0 * np.pi * iu / nu).reshape(-1)
    v = (2.0 * np.pi * jv / nv).reshape(-1)
    a = (iu * nv + jv).reshape(-1)
    b = (((iu + 1) % nu) * nv + jv).reshape(-1)
    c = (((iu + 1) % nu) * nv + (jv + 1) % nv).reshape(-1)
    d = (iu * nv + (jv + 1) % nv).reshape(-1)
    quads = np.stack([a, d, c, b], axis=1)  # outward: (d - a) x (b - a) points away from the tube
    uv = np.stack([iu.reshape(-1) / nu, jv.reshape(-1) / nv], axis=1)
    count = 0
    n_tris = 0
    for k in range(n_tori):
        cx, cy, cz = rng.uniform(-8, 8), rng.uniform(-2, 2), rng.uniform(-8, 8)
        R = rng.uniform(0.8, 1.6)
        r = R * rng.uniform(0.2, 0.4)
        ang = rng.uniform(0.0, math.pi)
        ca, sa = math.cos(ang), math.sin(ang)
        x = (R + r * np.cos(v)) * np.cos(u)
        y = r * np.sin(v)
        z = (R + r * np.cos(v)) * np.sin(u)
        nx, ny, nz = np.cos(v) * np.cos(u), np.sin(v), np.cos(v) * np.sin(u)
        pos = np.stack([x + cx, y * ca - z * sa + cy, y * sa + z * ca + cz], axis=1)
        nor = np.stack([nx, ny * ca - nz * sa, ny * sa + nz * ca], axis=1)
        out += ["o torus%d" % k, "usemtl m%d" % (k % 3), _rows("v", pos, "%.6f"), _rows("vt", uv, "%.5f"),
                _rows("vn", nor, "%.5f"), "s 1"]
        first = count + 1
        count += nu * nv
        idx = quads + (first - count - 1 if k % relative_every == relative_every - 1 else first)
        faces = idx.tolist()
        lines = []
        start = 0
        if k % hybrid_every == hybrid_every - 1:
            for q in faces[:16]:
                lines.append("f %d/%d/%d %d/%d/%d %d/%d/%d" % (q[0], q[0], q[0], q[1], q[1], q[1], q[2], q[2], q[2]))
                lines.append("f %d/%d/%d %d/%d/%d %d/%d/%d" % (q[0], q[0], q[0], q[2], q[2], q[2], q[3], q[3], q[3]))
            start = 16
        lines += ["f %d/%d/%d %d/%d/%d %d/%d/%d %d/%d/%d" % (q[0], q[0], q[0], q[1], q[1], q[1], q[2], q[2], q[2],
                                                              q[3], q[3], q[3]) for q in faces[start:]]
        out.append("\n".join(lines))
        n_tris += 2 * nu * nv
    return ("\n".join(out) + "\n").encode(), OBJ_TORI_MTL, n_tris


def obj_tori_scene(group, width, height, shadows=True):
    """The tori group with a shadow-casting point light, a directional light
    and ambient 0.15, seen from (0, 9, 18) with a 45-degree perspective."""
    s = sc.Scene(group, sc.Point(position=(6, 10, 8), intensity=1.0, cast_shadow=shadows),
                 sc.Directional(direction=(-1, -2, -1), intensity=0.4), sc.Ambient(intensity=0.15))
    cam = sc.Perspective(position=(0, 9, 18), target=(0, 0, 0), up=(0, 1, 0), fov=45.0, aspect=width / height,
                         near=0.1, far=100.0)
    return s, cam
