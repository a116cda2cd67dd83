"""Host-side scene model mirroring polyred's camera, light, material,
geometry and scene packages, as far as the render path consumes them.

Everything here is plain data plus the reference's host float32 math; the
device never sees these objects, only the flattened descriptors that
polyred_gb300.render builds from them.
"""
import numpy as np

from . import pmath

F32 = np.float32


def color_from_value(r, g, b, a=1.0):
    """color.FromValue (color/color.go:33-44): round half away from zero."""
    vals = tuple(float(v) for v in (r, g, b, a))
    for v in vals:
        if v < 0 or v > 1:
            raise ValueError(f"out of range [0, 1], got {vals}")
    # Go infers T = float64 for untyped constant arguments; v*255 >= 0 here.
    return tuple(int(np.floor(v * 255 + 0.5)) for v in vals)


# ---------------------------------------------------------------- camera

class Perspective:
    """camera.Perspective (camera/perspective.go); fov in degrees."""

    def __init__(self, position=(0, 0, 1), target=(0, 0, 0), up=(0, 1, 0), fov=60.0, aspect=16.0 / 9,
                 near=0.01, far=1000.0):
        self.position = np.asarray(position, F32)
        self.target = np.asarray(target, F32)
        self.up = np.asarray(up, F32)
        self.fov, self.aspect, self.near, self.far = F32(fov), F32(aspect), F32(near), F32(far)

    def view_matrix(self):
        return pmath.view_matrix(self.position, self.target, self.up)

    def proj_matrix(self):
        return pmath.perspective_matrix(self.fov, self.aspect, self.near, self.far)


class Orthographic:
    """camera.Orthographic (camera/orthographic.go)."""

    def __init__(self, position=(0, 0, 1), target=(0, 0, 0), up=(0, 1, 0), left=-1, right=1, bottom=-1, top=1,
                 near=1, far=-1):
        self.position = np.asarray(position, F32)
        self.target = np.asarray(target, F32)
        self.up = np.asarray(up, F32)
        self.frustum = tuple(F32(v) for v in (left, right, bottom, top, near, far))

    def view_matrix(self):
        return pmath.view_matrix(self.position, self.target, self.up)

    def proj_matrix(self):
        return pmath.orthographic_matrix(*self.frustum)


# ---------------------------------------------------------------- lights

class Point:
    """light.Point (light/point.go)."""

    kind = "source"

    def __init__(self, position=(1, 1, 1), intensity=1.0, color=(255, 255, 255, 255), cast_shadow=False):
        self.position = np.asarray(position, F32)
        self.intensity = F32(intensity)
        self.color = tuple(int(c) for c in color)
        self.cast_shadow = bool(cast_shadow)

    def aabb(self):
        return self.position.copy(), self.position.copy()


class Directional:
    """light.Directional (light/directional.go); the direction is normalised
    at construction (light/directional.go:34-48)."""

    kind = "source"

    def __init__(self, direction=(0, -1, 0), intensity=1.0, color=(255, 255, 255, 255), cast_shadow=False,
                 position=(0, 0, 0)):
        self.direction = pmath.vec3_unit(direction)
        self.position = np.asarray(position, F32)
        self.intensity = F32(intensity)
        self.color = tuple(int(c) for c in color)
        self.cast_shadow = bool(cast_shadow)

    def aabb(self):
        z = np.zeros(3, F32)
        return z, z.copy()


class Ambient:
    """light.Ambient (light/ambient.go)."""

    kind = "environment"

    def __init__(self, intensity=0.1, color=(255, 255, 255, 255)):
        self.intensity = F32(intensity)
        self.color = tuple(int(c) for c in color)

    def aabb(self):
        z = np.zeros(3, F32)
        return z, z.copy()


# ---------------------------------------------------------------- material

class ImageTexture:
    """buffer.NewTexture(TextureImage(img), TextureIsoMipmap(mipmap))
    (buffer/texture.go:35-67, 216-226): an RGBA8 image, rows top-down as
    image.RGBA stores them; the library builds the mipmap levels."""

    def __init__(self, rgba, mipmap=True):
        a = np.ascontiguousarray(rgba, np.uint8)
        if a.ndim != 3 or a.shape[2] != 4 or a.shape[0] < 1 or a.shape[1] < 1:
            raise ValueError(f"texture image must be (height, width, 4) uint8, got {a.shape}")
        self.rgba = a
        self.mipmap = bool(mipmap)

    def size(self):
        """Texture.Size(): the image width."""
        return self.rgba.shape[1]


class BlinnPhong:
    """material.BlinnPhong (material/material.go:43-72). The texture is an
    RGBA8 tuple (buffer.NewUniformTexture) or an ImageTexture. Colours are
    RGBA8 tuples."""

    def __init__(self, diffuse=None, specular=None, shininess=1.0, texture=(255, 255, 255, 255), flat_shading=False,
                 ambient_occlusion=False, receive_shadow=False, mipmap=True):
        self.diffuse = tuple(diffuse) if diffuse is not None else color_from_value(0.5, 0.5, 0.5, 1.0)
        self.specular = tuple(specular) if specular is not None else color_from_value(0.5, 0.5, 0.5, 1.0)
        self.shininess = F32(shininess)
        self.texture = texture if isinstance(texture, ImageTexture) else tuple(int(c) for c in texture)
        self.flat_shading = bool(flat_shading)
        self.ambient_occlusion = bool(ambient_occlusion)
        self.receive_shadow = bool(receive_shadow)
        self.mipmap = texture.mipmap if isinstance(texture, ImageTexture) else bool(mipmap)


# ---------------------------------------------------------------- geometry

class Mesh:
    """A triangle soup (geometry/mesh/mesh_triangle.go): per triangle three
    vertices with pos (x,y,z,w), nor (x,y,z,w), uv, RGBA8 colour, and a
    geometry-local MaterialID (<0 = vertex colour)."""

    def __init__(self, pos, nor, uv=None, col=None, mat_id=None):
        self.pos = np.ascontiguousarray(pos, F32).reshape(-1, 3, 4)
        n = self.pos.shape[0]
        self.nor = np.ascontiguousarray(nor, F32).reshape(n, 3, 4)
        self.uv = np.zeros((n, 3, 2), F32) if uv is None else np.ascontiguousarray(uv, F32).reshape(n, 3, 2)
        self.col = (np.full((n, 3, 4), 255, np.uint8) if col is None
                    else np.ascontiguousarray(col, np.uint8).reshape(n, 3, 4))
        self.mat_id = (np.zeros(n, np.int32) if mat_id is None
                       else np.ascontiguousarray(mat_id, np.int32).reshape(n))

    @property
    def n_tris(self):
        return self.pos.shape[0]

    def aabb(self):
        """TriangleMesh.AABB over model-space positions."""
        p = self.pos[:, :, :3].reshape(-1, 3)
        return p.min(axis=0).astype(F32), p.max(axis=0).astype(F32)


class TransformContext:
    """math.TransformContext (math/context.go): Scale/Translate pre-multiply
    the internal matrix; rotation stays identity here."""

    def __init__(self):
        self._internal = pmath.identity()

    def scale(self, sx, sy, sz):
        self._internal = pmath.mat4_mul(pmath.scale_matrix(sx, sy, sz), self._internal)
        return self

    def translate(self, tx, ty, tz):
        self._internal = pmath.mat4_mul(pmath.translate_matrix(tx, ty, tz), self._internal)
        return self

    def model_matrix(self):
        # internal.MulM(rotation.ToRoMat()) with the identity rotation
        return pmath.mat4_mul(self._internal, pmath.identity())


class Geometry(TransformContext):
    """geometry.Geometry (geometry/geometry.go): a mesh plus the materials it
    owns, indexed by the mesh's local MaterialIDs."""

    def __init__(self, mesh, *materials):
        super().__init__()
        self.mesh = mesh
        self.materials = list(materials)

    def aabb(self):
        return self.mesh.aabb()


class Group(TransformContext):
    """scene.Group (scene/core.go:113-203)."""

    def __init__(self, *objects):
        super().__init__()
        self.objects = list(objects)

    def add(self, *objects):
        self.objects.extend(objects)
        return self

    def _iter(self, fn):
        # iterObjects (scene/core.go:187-203): leaf objects get this group's
        # model matrix; nested groups compose on the left.
        mm = self.model_matrix()
        for o in self.objects:
            if isinstance(o, Group):
                o._iter(lambda obj, m: fn(obj, pmath.mat4_mul(mm, m)))
            else:
                fn(o, mm)


class Scene:
    """scene.Scene (scene/core.go): objects in traversal order."""

    def __init__(self, *objects):
        self.root = Group()
        self.root.add(*objects)

    def add(self, *objects):
        self.root.add(*objects)
        return self.root

    def iter_objects(self):
        """IterObjects (scene/core.go:86-111): (object, modelMatrix) pairs;
        the render path then uses modelMatrix.MulM(o.ModelMatrix())."""
        out = []
        root_mm = self.root.model_matrix()
        for o in self.root.objects:
            if isinstance(o, Group):
                o._iter(lambda obj, m: out.append((obj, pmath.mat4_mul(root_mm, m))))
            else:
                out.append((o, root_mm))
        return out

    def lights(self):
        """Lights (scene/scene.go:35-47): sources and environments in order."""
        src, env = [], []
        for o, _ in self.iter_objects():
            if getattr(o, "kind", None) == "source":
                src.append(o)
            elif getattr(o, "kind", None) == "environment":
                env.append(o)
        return src, env

    def center(self):
        """Center (scene/scene.go:49-52): middle of the union of the objects'
        own AABBs (geometry in model space, lights at their positions)."""
        mn = mx = None
        for o, _ in self.iter_objects():
            a, b = o.aabb()
            mn = a if mn is None else np.minimum(mn, a)
            mx = b if mx is None else np.maximum(mx, b)
        if mn is None:
            return np.zeros(3, F32)
        return ((mn + mx).astype(F32) * F32(0.5)).astype(F32)
