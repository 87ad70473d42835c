"""ORACLE — test infrastructure only.

ctypes binding of the FP64 restatement (oracle/pt_oracle.cpp, built into
oracle/_build/libmypbr_oracle.so by oracle/Makefile). Imported only by the
tests, by __graft_entry__.smoke() as the checker, and by bench.py's CPU
baseline; the product package never imports it.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libmypbr_oracle.so")

_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            subprocess.run(["make", "-s", "-C", HERE], check=True)
        L = ctypes.CDLL(LIB_PATH)
        vp, i64 = ctypes.c_void_p, ctypes.c_int64
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int32)
        L.oracle_scene_create.restype = vp
        L.oracle_scene_create.argtypes = [vp]
        L.oracle_scene_destroy.argtypes = [vp]
        L.oracle_scene_destroy.restype = None
        L.oracle_ggx_table.argtypes = [dp]
        L.oracle_ggx_table.restype = None
        L.oracle_trace.argtypes = [vp, dp, i64, dp, ip, ctypes.c_int]
        L.oracle_trace.restype = None
        L.oracle_bsdf.argtypes = [vp, ctypes.c_int, dp, dp, dp, i64, dp]
        L.oracle_bsdf.restype = None
        L.oracle_light_pdf.argtypes = [vp, dp, dp, i64, dp]
        L.oracle_light_pdf.restype = None
        L.oracle_light_sample.argtypes = [vp, dp, i64, ctypes.c_uint64, dp]
        L.oracle_light_sample.restype = None
        L.oracle_environment.argtypes = [vp, dp, i64, dp, dp]
        L.oracle_environment.restype = None
        L.oracle_render.argtypes = [vp, vp, vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, vp, vp, vp, vp, vp, vp]
        L.oracle_render.restype = ctypes.c_int
        L.oracle_render_strided.argtypes = [vp, vp, vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                            vp, vp, vp, vp, vp, vp]
        L.oracle_render_strided.restype = ctypes.c_int
        L.oracle_denoise.argtypes = [dp, dp, dp, dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                     ctypes.c_double, ctypes.c_double, dp]
        L.oracle_denoise.restype = None
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def denoise(radiance, albedo, normal, variance, iterations=5, sigma_luminance=4.0, sigma_normal=0.1,
            sigma_albedo=0.1):
    """denoiser::run (denoiser.h:45-193) in FP64; inputs (H, W, 3) and (H, W)."""
    h, w = variance.shape
    arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (radiance, albedo, normal, variance)]
    out = np.zeros((h, w, 3))
    lib().oracle_denoise(*[_dp(a) for a in arrs], w, h, iterations, sigma_luminance, sigma_normal, sigma_albedo,
                         _dp(out))
    return out


def ggx_table():
    out = np.zeros(32 * 32 + 32)
    lib().oracle_ggx_table(_dp(out))
    return out[:1024].reshape(32, 32), out[1024:]


class OracleScene:
    """The oracle's view of a flat scene (kept alive with the Scene it reads)."""

    def __init__(self, scene):
        self.scene = scene  # keeps the flat arrays alive
        self._h = ctypes.c_void_p(lib().oracle_scene_create(scene.flat))

    def close(self):
        if self._h:
            lib().oracle_scene_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def trace(self, rays, brute_force=False):
        rays = np.ascontiguousarray(rays, dtype=np.float64)
        n = rays.shape[0]
        hits = np.zeros((n, 8))
        prim = np.zeros((n, 2), dtype=np.int32)
        lib().oracle_trace(self._h, _dp(rays), n, _dp(hits), prim.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                           int(brute_force))
        return hits, prim

    def bsdf(self, material, rec, r_in, wi):
        rec = np.ascontiguousarray(rec, dtype=np.float64)
        r_in = np.ascontiguousarray(r_in, dtype=np.float64)
        wi = np.ascontiguousarray(wi, dtype=np.float64)
        n = rec.shape[0]
        out = np.zeros((n, 6))
        lib().oracle_bsdf(self._h, int(material), _dp(rec), _dp(r_in), _dp(wi), n, _dp(out))
        return out

    def light_pdf(self, origin, direction):
        origin = np.ascontiguousarray(origin, dtype=np.float64)
        direction = np.ascontiguousarray(direction, dtype=np.float64)
        n = origin.shape[0]
        out = np.zeros(n)
        lib().oracle_light_pdf(self._h, _dp(origin), _dp(direction), n, _dp(out))
        return out

    def light_sample(self, origin, n, seed=1):
        origin = np.ascontiguousarray(origin, dtype=np.float64)
        out = np.zeros((n, 3))
        lib().oracle_light_sample(self._h, _dp(origin), n, seed, _dp(out))
        return out

    def environment(self, direction):
        direction = np.ascontiguousarray(direction, dtype=np.float64)
        n = direction.shape[0]
        rad = np.zeros((n, 3))
        pdf = np.zeros(n)
        lib().oracle_environment(self._h, _dp(direction), n, _dp(rad), _dp(pdf))
        return rad, pdf

    def render(self, camera, threads=0, rows=None, features=False, row_stride=1):
        """Renders with the oracle. Returns (radiance (H, W, 3), variance of the
        mean per channel (H, W, 3), extras dict). rows = (first, count) renders
        only those rows; with row_stride k, rows first, first + k, ... (count of
        them, 0: to the bottom) - the others are left at 0."""
        c, o = camera.structs()
        o.collect_features = int(features)
        w, h = c.image_width, c.image_height
        rad = np.zeros((h, w, 3))
        var = np.zeros((h, w, 3))
        alb = np.zeros((h, w, 3)) if features else None
        nrm = np.zeros((h, w, 3)) if features else None
        lv = np.zeros((h, w)) if features else None
        counts = np.zeros(3, dtype=np.uint64)
        first, count = (0, h) if rows is None else rows

        def p(a):
            return ctypes.c_void_p(a.ctypes.data) if a is not None else ctypes.c_void_p()

        lib().oracle_render_strided(self._h, ctypes.addressof(c), ctypes.addressof(o), int(threads), int(first),
                                    int(count) if rows is not None else 0, int(row_stride),
                                    p(rad), p(var), p(alb), p(nrm), p(lv), p(counts))
        return rad, var, {"albedo": alb, "normal": nrm, "lum_var": lv, "paths": int(counts[0]),
                          "extension_rays": int(counts[1]), "shadow_rays": int(counts[2])}
