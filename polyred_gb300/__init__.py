"""GB300-native (sm_103a) implementation of polyred's render path.

  render      NewRenderer/Render and options, with CUDA(dev) (render/raster.go)
  scene       cameras, lights, materials, geometry, scene graph (host data)
  procedural  seeded workloads (UV spheres, sphere field, triangle soup)
  objload     Wavefront OBJ / MTL loading (model.Load, model/obj) over the
              native pr_obj_* parser
  native      loader of the in-tree libpolyred_cuda.so (C ABI in include/)
  build       compiles libpolyred_cuda.so for sm_103a
"""
__all__ = ["render", "scene", "procedural", "objload", "native", "build", "pmath"]
