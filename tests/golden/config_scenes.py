"""The benchmark workloads at test size, shared by the golden generator and the
GPU parity tests.

Each function writes one of mypbr_gb300.workloads' seeded scenes into a
directory at a reduced image size (same geometry, lights, materials and
depth as the full-size configuration) and returns (scene path, digest). The
digest is a SHA-1 over the generated files, stored in the golden .npz when the
reference renders the scene, and checked by the test before it compares
images, so a different numpy stream on another machine shows up as a clear
input mismatch, not as a parity failure.

  c2   the 1000-sphere field under the 1024 x 512 sky with the 5e4-peak sun
       lobe, 96 x 54 (1920 x 1080 / 20), depth 16
  c3   the triangle room at 60,000 triangles (32 principled materials, 16
       emissive quads), 64 x 36, depth 12
  c5   the 512^3 voxel hall lit through six slits (sun 0.54 deg, uniform sky),
       64 x 36, depth 16
"""
import hashlib
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from mypbr_gb300 import workloads  # noqa: E402


def _digest(directory):
    h = hashlib.sha1()
    for name in sorted(os.listdir(directory)):
        path = os.path.join(directory, name)
        if os.path.isfile(path):
            h.update(name.encode())
            with open(path, "rb") as f:
                for block in iter(lambda: f.read(1 << 20), b""):
                    h.update(block)
    return h.hexdigest()


def c2(directory, width=96, height=54):
    path = workloads.sphere_field_scene(directory, seed=2, spp=64, width=width, height=height, depth=16)
    return path, _digest(directory)


def c3(directory, width=64, height=36, triangles=60_000):
    path = workloads.triangle_room_scene(directory, triangles=triangles, seed=3, spp=64, width=width,
                                         height=height, depth=12)
    return path, _digest(directory)


def c5(directory, width=64, height=36):
    path = workloads.voxel_hall_scene(directory, size=512, seed=5, spp=64, width=width, height=height, depth=16)
    return path, _digest(directory)


CONFIGS = {"c2": c2, "c3": c3, "c5": c5}
