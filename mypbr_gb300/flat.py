"""ctypes views of the flat scene arrays (include/mypbr_gpu.h), for
inspection from Python: materials, textures, lights, primitives as numpy
record arrays."""
import ctypes

import numpy as np

_i32, _i64, _f64, _vp = ctypes.c_int32, ctypes.c_int64, ctypes.c_double, ctypes.c_void_p


class Environment(ctypes.Structure):
    _fields_ = [("width", _i32), ("height", _i32), ("pixels", _vp), ("intensity", _f64), ("rotation", _f64)]


class Sun(ctypes.Structure):
    _fields_ = [("enabled", _i32), ("disk_visible", _i32), ("direction", _f64 * 3), ("angular_diameter", _f64),
                ("irradiance", _f64 * 3)]


_ARRAYS = ["spheres", "quads", "positions", "normals", "uvs", "triangles", "meshes", "media", "xforms", "unbounded",
           "bvh_nodes", "bvh_prims", "materials", "textures", "texels_ldr", "texels_hdr", "lights", "light_members"]
_COUNTS = {"positions": "position_count", "normals": "normal_count", "uvs": "uv_count",
           "texels_ldr": "texels_ldr_bytes", "texels_hdr": "texels_hdr_count", "bvh_nodes": "bvh_node_count",
           "bvh_prims": "bvh_prim_count", "light_members": "light_member_count", "media": "medium_count",
           "meshes": "mesh_count", "unbounded": "unbounded_count"}


# Arrays after the sky fields, appended to the struct when voxels were added
_VOXEL_ARRAYS = ["voxel_models", "voxel_blocks", "voxel_palettes", "voxel_cells"]
_COUNTS.update({"voxel_models": "voxel_model_count", "voxel_blocks": "voxel_block_count",
                "voxel_palettes": "voxel_palette_count", "voxel_cells": "voxel_cell_bytes"})


def _count_name(a):
    return _COUNTS.get(a, a[:-1] + "_count")


class FlatScene(ctypes.Structure):
    _fields_ = ([("abi_version", ctypes.c_uint32), ("reserved0", ctypes.c_uint32)] +
                [f for a in _ARRAYS for f in ((a, _vp), (_count_name(a), _i64))] +
                [("environment", Environment), ("sun", Sun), ("use_sky", _i32), ("reserved1", _i32),
                 ("background", _f64 * 3)] +
                [f for a in _VOXEL_ARRAYS for f in ((a, _vp), (_count_name(a), _i64))])


DTYPES = {
    "spheres": np.dtype([("center", "<f8", 3), ("radius", "<f8"), ("material", "<i4"), ("xform", "<i4")]),
    "quads": np.dtype([("q", "<f8", 3), ("u", "<f8", 3), ("v", "<f8", 3), ("normal", "<f8", 3),
                       ("material", "<i4"), ("reserved", "<i4")]),
    "positions": np.dtype(("<f8", 3)),
    "normals": np.dtype(("<f8", 3)),
    "uvs": np.dtype(("<f8", 2)),
    "triangles": np.dtype([("v", "<i4", 3), ("n", "<i4", 3), ("t", "<i4", 3), ("material", "<i4"),
                           ("flags", "<i4"), ("mesh", "<i4")]),
    "meshes": np.dtype([("first_triangle", "<i8"), ("triangle_count", "<i8"), ("material", "<i4"),
                        ("alpha_mask", "<i4")]),
    "media": np.dtype([("shape", "<i4"), ("xform", "<i4"), ("material", "<i4"), ("reserved", "<i4"),
                       ("density", "<f8"), ("a", "<f8", 3), ("b", "<f8", 3)]),
    "xforms": np.dtype([("m", "<f8", (3, 3)), ("t", "<f8", 3), ("inv_m", "<f8", (3, 3)), ("inv_t", "<f8", 3)]),
    "unbounded": np.dtype([("kind", "<i4"), ("material", "<i4"), ("height", "<f8"), ("density", "<f8"),
                           ("scale_height", "<f8")]),
    "bvh_nodes": np.dtype([("bmin", "<f8", 3), ("bmax", "<f8", 3), ("offset", "<i4"), ("count", "<i4"),
                           ("axis", "<i4"), ("reserved", "<i4")]),
    "bvh_prims": np.dtype([("kind", "<i4"), ("index", "<i4")]),
    "materials": np.dtype([("type", "<i4"), ("flags", "<i4"), ("tex", "<i4", 8), ("normal_map", "<i4"),
                           ("emission_tex", "<i4"), ("p", "<f8", 16)]),
    "textures": np.dtype([("type", "<i4"), ("a", "<i4"), ("b", "<i4"), ("width", "<i4"), ("height", "<i4"),
                          ("flags", "<i4"), ("offset", "<i8"), ("p", "<f8", 6)]),
    "texels_ldr": np.dtype("u1"),
    "texels_hdr": np.dtype("<f4"),
    "lights": np.dtype([("kind", "<i4"), ("first_member", "<i4"), ("member_count", "<i4"), ("reserved", "<i4"),
                        ("probability", "<f8")]),
    "light_members": np.dtype([("prim_kind", "<i4"), ("prim_index", "<i4"), ("weight", "<f8")]),
    "voxel_models": np.dtype([("n", "<i4", 3), ("xform", "<i4"), ("cells", "<i8"), ("palette", "<i4"),
                              ("edge_material", "<i4"), ("edge_width", "<f8")]),
    "voxel_blocks": np.dtype([("model", "<i4"), ("lo", "<i4", 3), ("hi", "<i4", 3), ("reserved", "<i4")]),
    "voxel_palettes": np.dtype([("material", "<i4"), ("kind", "<i4")]),
    "voxel_cells": np.dtype("u1"),
}


def view(scene):
    """The flat scene of a mypbr_gb300.Scene as a dict of numpy arrays (copies)."""
    fs = FlatScene.from_address(scene.flat)
    out = {}
    for a in _ARRAYS + _VOXEL_ARRAYS:
        n = getattr(fs, _count_name(a))
        ptr = getattr(fs, a)
        dt = DTYPES[a]
        if n == 0 or not ptr:
            out[a] = np.zeros(0, dtype=dt)
            continue
        buf = (ctypes.c_char * (dt.itemsize * n)).from_address(ptr)
        out[a] = np.frombuffer(bytes(buf), dtype=dt, count=n)
    out["environment"] = fs.environment
    out["sun"] = fs.sun
    out["use_sky"] = fs.use_sky
    out["background"] = tuple(fs.background)
    return out
