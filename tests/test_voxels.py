"""Voxel models: the .vox reader, the palette and the 3D DDA grid walk.

CPU: the host loader's layout; the oracle's grid walk against the reference's
own hits on the same scene (tests/golden/hits_voxels.npz, made by
tests/golden/gen_golden.py); and, as the reference's voxel test does
(tests/voxel_test.cpp), the grid finding exactly the surfaces that the same
model's faces do as quads in a BVH.
GPU: the device DDA against the oracle, grid against quads on the device, and
a full render against the reference's.
"""
import numpy as np
import pytest

import mypbr_gb300 as mp
import oracle as orc
from conftest import GOLDEN, scene_path
from mypbr_gb300 import flat

# material types of the flat scene (MYPBR_MAT_* in include/mypbr_gpu.h)
TYPES = {"LAMBERTIAN": 0, "METAL": 1, "DIELECTRIC": 2, "PRINCIPLED": 4, "DIFFUSE_LIGHT": 5}


def load_golden(name):
    return np.load(f"{GOLDEN}/{name}.npz")


def rays_of(g, tmax=np.inf):
    n = len(g["hit"])
    rays = np.zeros((n, 8))
    rays[:, 0:3] = g["o"]
    rays[:, 3:6] = g["d"]
    rays[:, 6] = 0.001
    rays[:, 7] = tmax
    return rays


def expected_ids(scene, materials):
    """What the reference harness reads back for a hit on each material: a
    lambertian's red albedo as round(1024 r) - 1, -2 for a light (it does not
    scatter); None where the readback says nothing about which material."""
    v = flat.view(scene)
    out = []
    for m in materials:
        mat = v["materials"][m]
        if mat["type"] == TYPES["LAMBERTIAN"]:
            out.append(int(round(v["textures"][mat["tex"][0]]["p"][0] * 1024)) - 1)
        elif mat["type"] == TYPES["DIFFUSE_LIGHT"]:
            out.append(-2)
        else:
            out.append(None)
    return out


def grid_rays(n, seed):
    """The reference voxel test's rays (tests/voxel_test.cpp:47-58) around the
    placed models: from outside aimed at a point inside, or from inside in any
    direction, a third of them with a finite tmax."""
    rng = np.random.default_rng(seed)
    sc = mp.load_scene(scene_path("voxels_grid.scene"))
    v = flat.view(sc)
    nodes = v["bvh_nodes"]
    lo, hi = nodes[0]["bmin"], nodes[0]["bmax"]
    target = lo + (hi - lo) * rng.random((n, 3))
    u = rng.normal(size=(n, 3))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    outside = np.arange(n) % 2 == 1
    origin = np.where(outside[:, None], target + 30 * u, target)
    u2 = rng.normal(size=(n, 3))
    u2 /= np.linalg.norm(u2, axis=1, keepdims=True)
    direction = np.where(outside[:, None], target - origin, u2 * rng.uniform(0.5, 2, size=(n, 1)))
    rays = np.zeros((n, 8))
    rays[:, 0:3] = origin
    rays[:, 3:6] = direction
    rays[:, 6] = 0.001
    rays[:, 7] = np.where(np.arange(n) % 3 == 0, rng.uniform(0.1, 40, size=n), np.inf)
    return rays


# ------------------------------------------------------------------- CPU

def test_vox_loader_layout():
    sc = mp.load_scene(scene_path("voxels.scene"))
    v = flat.view(sc)
    models, blocks, pal = v["voxel_models"], v["voxel_blocks"], v["voxel_palettes"]
    # model 0 (13 x 9 x 11) once, model 1 (5 x 4 x 3) twice, the default-palette model once
    dims = sorted(tuple(int(x) for x in m["n"]) for m in models)
    assert dims == [(5, 4, 3), (5, 4, 3), (6, 5, 4), (13, 9, 11)]
    # instances of one model share cells
    small = [m for m in models if tuple(m["n"]) == (5, 4, 3)]
    assert small[0]["cells"] == small[1]["cells"] and small[0]["xform"] != small[1]["xform"]
    # palettes: index 0 empty; glass (3, 4) transparent; others opaque
    assert len(pal) == 512
    kinds = pal["kind"][:256]
    assert kinds[0] == 0 and kinds[3] == 2 and kinds[4] == 2 and kinds[1] == 1 and kinds[5] == 1
    assert np.all(pal["kind"][256] == 0)
    # blocks are at most 8 cells a side and hold a voxel
    ext = blocks["hi"] - blocks["lo"]
    assert np.all(ext >= 1) and np.all(ext <= 8)
    cells = v["voxel_cells"]
    for b in blocks:
        m = models[b["model"]]
        nx, ny, nz = m["n"]
        grid = cells[m["cells"]:m["cells"] + nx * ny * nz].reshape(nz, ny, nx)
        sub = grid[b["lo"][2]:b["hi"][2], b["lo"][1]:b["hi"][1], b["lo"][0]:b["hi"][0]]
        assert (pal["kind"][m["palette"] + sub.astype(int)] != 0).any()
    # the edge material of the outlined file, none for the other
    edged = [m for m in models if m["edge_width"] > 0]
    assert len(edged) == 3 and all(m["edge_material"] >= 0 for m in edged)
    # emissive faces are quads outside the BVH, sampled by one light group
    assert (v["bvh_prims"]["kind"] == 4).sum() == len(blocks)
    assert (v["bvh_prims"]["kind"] == 1).sum() == 0
    assert len(v["lights"]) == 1 and v["lights"][0]["member_count"] == len(v["quads"])


def test_vox_errors_are_reported(tmp_path):
    bad = tmp_path / "bad.vox"
    i32 = lambda v: int(v).to_bytes(4, "little", signed=True)  # noqa: E731
    s = tmp_path / "s.scene"
    s.write_text(f"vox {bad}\n")
    # a SIZE chunk announcing 12 bytes of content with 4 left
    bad.write_bytes(b"VOX " + i32(150) + b"MAIN" + i32(0) + i32(16) + b"SIZE" + i32(12) + i32(0) + i32(1))
    with pytest.raises(mp.MypbrError, match="truncated or corrupt"):
        mp.load_scene(str(s))
    bad.write_bytes(b"VOX " + i32(150) + b"MAIN" + i32(0) + i32(0))
    with pytest.raises(mp.MypbrError, match="has no voxels"):
        mp.load_scene(str(s))
    bad.write_bytes(b"VOX " + i32(150) + b"MAIN" + i32(0) + i32(0) + b"SIZE" + i32(12) + i32(0) + i32(0) * 3)
    with pytest.raises(mp.MypbrError, match="invalid size"):
        mp.load_scene(str(s))
    s.write_text(f"vox {scene_path('voxels.vox')} lambertian 1 1 1\n")
    with pytest.raises(mp.MypbrError):
        mp.load_scene(str(s))
    s.write_text(f"vox {scene_path('voxels.vox')} edges 0.6\n")
    with pytest.raises(mp.MypbrError, match="expected 'vox"):
        mp.load_scene(str(s))


def test_voxel_hits_match_reference():
    sc = mp.load_scene(scene_path("voxels.scene"))
    g = load_golden("hits_voxels")
    hits, prim = orc.OracleScene(sc).trace(rays_of(g))
    hit = prim[:, 0] >= 0
    assert np.array_equal(hit, g["hit"] > 0), "hit/miss differs from the reference"
    assert hit.mean() > 0.2
    np.testing.assert_allclose(hits[hit, 0], g["t"][hit], rtol=1e-12)
    np.testing.assert_allclose(hits[hit, 1:4], g["normal"][hit], atol=1e-12)
    np.testing.assert_array_equal(hits[hit, 6], g["front"][hit])
    np.testing.assert_allclose(hits[hit, 4], g["u"][hit], atol=1e-9)
    np.testing.assert_allclose(hits[hit, 5], g["v"][hit], atol=1e-9)
    mats = hits[hit, 7].astype(int)
    ids = expected_ids(sc, mats)
    gold = g["material_id"][hit]
    known = np.array([i is not None for i in ids])
    np.testing.assert_array_equal(np.array([i for i in ids if i is not None]), gold[known])
    # outline hits are lambertian 0.9: id 921, and some rays find them
    assert (gold == 921).sum() > 50
    # the unread materials are the glass and metal palette entries, never a lambertian's id
    v = flat.view(sc)
    types = v["materials"]["type"][mats[~known]]
    assert set(types.tolist()) <= {TYPES["DIELECTRIC"], TYPES["PRINCIPLED"]}
    # glass scatters with attenuation 1 (read back as 1023)
    assert np.all(gold[~known][types == TYPES["DIELECTRIC"]] == 1023)


def test_voxel_grid_equals_its_faces():
    """voxel_test.cpp: the DDA finds the surfaces the faces do as quads."""
    grid = orc.OracleScene(mp.load_scene(scene_path("voxels_grid.scene")))
    quads = orc.OracleScene(mp.load_scene(scene_path("voxels_quads.scene")))
    rays = grid_rays(20000, 11)
    ha, pa = grid.trace(rays)
    hb, pb = quads.trace(rays)
    hit = pa[:, 0] >= 0
    np.testing.assert_array_equal(hit, pb[:, 0] >= 0)
    assert hit.mean() > 0.3
    np.testing.assert_allclose(ha[hit, 0], hb[hit, 0], rtol=1e-9, atol=1e-9)
    np.testing.assert_allclose(ha[hit, 1:4], hb[hit, 1:4], atol=1e-9)
    np.testing.assert_array_equal(ha[hit, 6], hb[hit, 6])
    np.testing.assert_array_equal(ha[hit, 7], hb[hit, 7])


# ------------------------------------------------------------------- GPU

_GPU = {}


def gpu_scene(name):
    if name not in _GPU:
        sc = mp.load_scene(scene_path(f"{name}.scene"))
        _GPU[name] = (sc, mp.GpuScene(sc))
    return _GPU[name]


def stable(O, rays, scale, trials=4, seed=0):
    """Rays whose oracle answer (primitive and material) keeps under origin
    moves of 1e-5 of the scene scale: away from cell edges, where an FP32
    walk must agree with the FP64 one."""
    rng = np.random.default_rng(seed)
    h0, p0 = O.trace(rays)
    ok = np.ones(len(rays), dtype=bool)
    for _ in range(trials):
        r = rays.copy()
        r[:, 0:3] += rng.normal(size=(len(r), 3)) * 1e-5 * scale
        h, p = O.trace(r)
        ok &= np.all(p == p0, axis=1) & (h[:, 7] == h0[:, 7]) & np.all(np.abs(h[:, 1:4] - h0[:, 1:4]) < 1e-6, axis=1)
    return ok


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["voxels", "voxels_grid"])
def test_gpu_voxel_trace_matches_oracle(name):
    sc, G = gpu_scene(name)
    O = orc.OracleScene(sc)
    rays = grid_rays(20000, 3) if name == "voxels_grid" else rays_of(load_golden("hits_voxels"), 3e38)
    rays[:, 7] = np.minimum(rays[:, 7], 3e38)
    rays32 = rays.astype(np.float32)
    rays = rays32.astype(np.float64)
    oh, op = O.trace(rays)
    hits, prim = G.trace(rays32)
    ok = stable(O, rays, 20.0)
    assert ok.mean() > 0.97, ok.mean()
    # A face on the plane between two blocks belongs to both (each block
    # reports the faces of its boundary, voxel.h:249-262), and the walk order
    # picks one: the face itself (kind, t, normal, side, material) is the
    # primitive identity compared here, the block index is not.
    np.testing.assert_array_equal(prim[ok, 0], op[ok, 0], err_msg="hit/miss or kind differs")
    both = ok & (prim[:, 0] >= 0)
    assert both.mean() > 0.2
    np.testing.assert_array_equal(hits[both, 7], oh[both, 7], err_msg="material differs")
    np.testing.assert_array_equal(hits[both, 6], oh[both, 6])
    dlen = np.linalg.norm(rays[both, 3:6], axis=1)
    dt = np.abs(hits[both, 0] - oh[both, 0]) * dlen
    bound = np.maximum(1e-5 * oh[both, 0] * dlen, 4 * 2.0 ** -23 * 40.0)
    assert np.all(dt <= bound), (dt / bound).max()
    assert np.abs(hits[both, 1:4] - oh[both, 1:4]).max() < 1e-5
    # u, v are fractions of a cell: FP32 resolves them to about 1e-5 here
    du = np.abs(hits[both, 4:6] - oh[both, 4:6])
    du = np.minimum(du, 1 - du)  # a point on a cell boundary is 0 or 1
    assert du.max() < 1e-3 and np.median(du) < 1e-5


@pytest.mark.gpu
def test_gpu_voxel_grid_equals_its_faces():
    _, Ga = gpu_scene("voxels_grid")
    _, Gb = gpu_scene("voxels_quads")
    sc = mp.load_scene(scene_path("voxels_grid.scene"))
    rays = grid_rays(20000, 5)
    rays[:, 7] = np.minimum(rays[:, 7], 3e38)
    rays32 = rays.astype(np.float32)
    ok = stable(orc.OracleScene(sc), rays32.astype(np.float64), 20.0)
    ha, pa = Ga.trace(rays32)
    hb, pb = Gb.trace(rays32)
    hit = ok & (pa[:, 0] >= 0)
    np.testing.assert_array_equal((pa[ok, 0] >= 0), (pb[ok, 0] >= 0))
    np.testing.assert_allclose(ha[hit, 0], hb[hit, 0], rtol=2e-5, atol=1e-5)
    np.testing.assert_array_equal(ha[hit, 7], hb[hit, 7])
    np.testing.assert_array_equal(ha[hit, 6], hb[hit, 6])
