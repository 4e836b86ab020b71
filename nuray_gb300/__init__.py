"""GB300-native ptnee path tracer (nuRay's RendererPTLS) behind a C ABI.

The compute path is libnuray_gpu.so (include/nuray.h): host C++ for scene
flattening and the reference SAH BVH, hand-written sm_103a kernels for the
wavefront. This package only binds it (ctypes) and generates the seeded
procedural workloads.
"""
from ._lib import (MAT_BLINNPHONG, MAT_GGX, MAT_GGXR, MAT_GLASS, MAT_LAMBERT, MAT_LIGHT, Camera, Material,
                   NuRayError, Scene, camera_from_params, lib, make_material, parse_params)

__all__ = ["Scene", "Material", "Camera", "NuRayError", "lib", "make_material", "camera_from_params",
           "parse_params", "MAT_LAMBERT", "MAT_GGXR", "MAT_GGX", "MAT_GLASS", "MAT_BLINNPHONG", "MAT_LIGHT"]
