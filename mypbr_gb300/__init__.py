"""mypbr_gb300 — the GB300 backend of mypbr's per-pixel path-tracing loop.

The Python side mirrors the reference's host interface for this path:

    scene.h:244   load_scene(path, scene&)        ->  load_scene(path) -> Scene
    camera.h:19   class camera (public settings)  ->  Camera (same attribute names)
    camera.h:79   frame camera::render(world, lights, save_every, on_pass)
                                                  ->  Camera.render(gpu_scene, save_every, on_pass) -> Frame
    denoiser.h:14 class frame                     ->  Frame (radiance, albedo, normal, variance)

Everything runs through the C ABI of include/mypbr_gpu.h, implemented by the
in-tree library mypbr_gb300/_lib/libmypbr_gb300.so (hand-written CUDA for
sm_103a plus the C++ host scene layer). There is no CPU fallback: if the
library is missing or no GPU is visible, rendering raises.
"""
import ctypes
import os

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "_lib", "libmypbr_gb300.so")

MYPBR_OK = 0
STATUS_NAMES = {
    0: "MYPBR_OK", 1: "MYPBR_ERR_CUDA", 2: "MYPBR_ERR_UNSUPPORTED", 3: "MYPBR_ERR_QUEUE_OVERFLOW",
    4: "MYPBR_ERR_DEVICE_TIMEOUT", 5: "MYPBR_ERR_INVALID_ARGUMENT", 6: "MYPBR_ERR_OUT_OF_MEMORY",
    7: "MYPBR_ERR_BAD_SCENE", 8: "MYPBR_ERR_IO", 9: "MYPBR_ERR_NO_DEVICE", 10: "MYPBR_ERR_DEVICE_CHECK",
}


class MypbrError(RuntimeError):
    """A non-zero mypbr_status, with the library's message."""

    def __init__(self, status, message):
        self.status = status
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")


class CameraStruct(ctypes.Structure):
    """mypbr_camera (include/mypbr_gpu.h)."""
    _fields_ = [("image_width", ctypes.c_int32), ("image_height", ctypes.c_int32),
                ("aspect_ratio", ctypes.c_double), ("vfov", ctypes.c_double),
                ("lookfrom", ctypes.c_double * 3), ("lookat", ctypes.c_double * 3), ("vup", ctypes.c_double * 3),
                ("defocus_angle", ctypes.c_double), ("focus_dist", ctypes.c_double),
                ("ortho_height", ctypes.c_double), ("blades", ctypes.c_int32), ("reserved", ctypes.c_int32),
                ("blade_rotation", ctypes.c_double)]


class RenderOptsStruct(ctypes.Structure):
    """mypbr_render_opts (include/mypbr_gpu.h)."""
    _fields_ = [("samples_per_pixel", ctypes.c_int32), ("max_depth", ctypes.c_int32),
                ("max_diffuse", ctypes.c_int32), ("max_specular", ctypes.c_int32),
                ("max_scatter", ctypes.c_int32), ("transparent_shadows", ctypes.c_int32),
                ("collect_features", ctypes.c_int32), ("guided", ctypes.c_int32), ("seed", ctypes.c_uint64),
                ("samples_per_wave", ctypes.c_int32), ("timing", ctypes.c_int32),
                ("first_row", ctypes.c_int32), ("row_count", ctypes.c_int32)]


class RenderStatsStruct(ctypes.Structure):
    """mypbr_render_stats (include/mypbr_gpu.h)."""
    _fields_ = [("paths", ctypes.c_uint64), ("extension_rays", ctypes.c_uint64),
                ("shadow_rays", ctypes.c_uint64), ("kernel_launches", ctypes.c_uint64),
                ("ms_generate", ctypes.c_double), ("ms_extend", ctypes.c_double), ("ms_shade", ctypes.c_double),
                ("ms_shadow", ctypes.c_double), ("ms_other", ctypes.c_double),
                ("launches_extend", ctypes.c_uint64), ("launches_shade", ctypes.c_uint64),
                ("launches_shadow", ctypes.c_uint64)]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


PASS_CALLBACK = ctypes.CFUNCTYPE(None, ctypes.c_int, ctypes.c_void_p)

TONEMAPPERS = {"none": 0, "reinhard": 1, "aces": 2}


class BatchJobStruct(ctypes.Structure):
    _fields_ = [("scene", ctypes.c_void_p), ("camera", ctypes.POINTER(CameraStruct)),
                ("opts", ctypes.POINTER(RenderOptsStruct)), ("radiance", ctypes.c_void_p),
                ("albedo", ctypes.c_void_p), ("normal", ctypes.c_void_p), ("variance", ctypes.c_void_p),
                ("status", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class BvhReportStruct(ctypes.Structure):
    _fields_ = [("primitives", ctypes.c_int64), ("nodes", ctypes.c_int64), ("depth", ctypes.c_int32),
                ("reserved", ctypes.c_int32), ("build_ms", ctypes.c_double), ("sah_cost", ctypes.c_double),
                ("sah_cost_before", ctypes.c_double)]


class SkySettingsStruct(ctypes.Structure):
    _fields_ = [("rayleigh", ctypes.c_double), ("mie", ctypes.c_double), ("mie_g", ctypes.c_double),
                ("ozone", ctypes.c_double), ("intensity", ctypes.c_double)]


class TuneResultStruct(ctypes.Structure):
    _fields_ = [("block", ctypes.c_int32), ("traversal", ctypes.c_int32), ("wave_paths", ctypes.c_int64),
                ("mpaths_per_s", ctypes.c_double), ("trial_mpaths", ctypes.c_double * 40)]


class DisplayOptsStruct(ctypes.Structure):
    _fields_ = [("exposure", ctypes.c_double), ("tonemap", ctypes.c_int32), ("reserved", ctypes.c_int32),
                ("bloom", ctypes.c_double), ("bloom_threshold", ctypes.c_double), ("bloom_radius", ctypes.c_double),
                ("vignette", ctypes.c_double)]

_lib = None


def lib():
    """The loaded C-ABI library (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise MypbrError(9, f"{LIB_PATH} is missing: build it with mypbr_gb300.build.build()")
    L = ctypes.CDLL(LIB_PATH)
    vp, i32, i64 = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64
    dp, fp, ip = ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_int32)
    L.mypbr_gpu_status_string.restype = ctypes.c_char_p
    L.mypbr_gpu_status_string.argtypes = [ctypes.c_int]
    L.mypbr_last_error.restype = ctypes.c_char_p
    L.mypbr_scene_load.argtypes = [ctypes.c_char_p, ctypes.POINTER(vp)]
    L.mypbr_scene_parse.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(vp)]
    L.mypbr_scene_flat.restype = vp
    L.mypbr_scene_flat.argtypes = [vp]
    L.mypbr_scene_camera.restype = ctypes.POINTER(CameraStruct)
    L.mypbr_scene_camera.argtypes = [vp]
    L.mypbr_scene_render_opts.restype = ctypes.POINTER(RenderOptsStruct)
    L.mypbr_scene_render_opts.argtypes = [vp]
    L.mypbr_scene_free.argtypes = [vp]
    L.mypbr_scene_free.restype = None
    L.mypbr_ggx_albedo_table.argtypes = [dp]
    L.mypbr_gpu_denoise.argtypes = [vp, vp, vp, vp, ctypes.c_int32, ctypes.c_int32, vp, vp, ctypes.c_int]
    L.mypbr_env_distribution.argtypes = [vp, ctypes.c_int32, ctypes.c_int32, vp, vp, ctypes.c_int]
    L.mypbr_gpu_test_wait_timeout.argtypes = []
    i32p = ctypes.POINTER(ctypes.c_int32)
    L.mypbr_image_read.argtypes = [ctypes.c_char_p, i32p, i32p, i32p, vp, ctypes.c_int64]
    L.mypbr_camera_init.argtypes = [ctypes.POINTER(CameraStruct)]
    L.mypbr_camera_init.restype = None
    L.mypbr_render_opts_init.argtypes = [ctypes.POINTER(RenderOptsStruct)]
    L.mypbr_render_opts_init.restype = None
    L.mypbr_gpu_scene_create.argtypes = [vp, ctypes.POINTER(vp)]
    L.mypbr_gpu_scene_destroy.argtypes = [vp]
    L.mypbr_gpu_scene_destroy.restype = None
    L.mypbr_gpu_render.argtypes = [vp, ctypes.POINTER(CameraStruct), ctypes.POINTER(RenderOptsStruct), vp, vp, vp,
                                   vp, ctypes.c_int, PASS_CALLBACK, vp]
    L.mypbr_gpu_render_device.argtypes = [vp, ctypes.POINTER(CameraStruct), ctypes.POINTER(RenderOptsStruct), vp,
                                          vp, vp, vp, vp, ctypes.POINTER(RenderStatsStruct)]
    L.mypbr_gpu_render_ex.argtypes = [vp, ctypes.POINTER(CameraStruct), ctypes.POINTER(RenderOptsStruct), vp, vp, vp,
                                      vp, vp, ctypes.c_int, PASS_CALLBACK, vp, ctypes.POINTER(RenderStatsStruct)]
    L.mypbr_gpu_trace.argtypes = [vp, fp, i64, fp, ip, ctypes.c_int]
    L.mypbr_gpu_bsdf_eval.argtypes = [vp, i32, fp, fp, fp, i64, fp]
    L.mypbr_gpu_render_batch.argtypes = [ctypes.POINTER(BatchJobStruct), i32]
    L.mypbr_gpu_set_launch.argtypes = [vp, i32, i64, i32]
    L.mypbr_gpu_scene_rebuild_bvh.argtypes = [vp, i32, ctypes.POINTER(BvhReportStruct)]
    L.mypbr_sky_settings_init.argtypes = [ctypes.POINTER(SkySettingsStruct)]
    L.mypbr_sky_settings_init.restype = None
    L.mypbr_sky_bake.argtypes = [ctypes.POINTER(SkySettingsStruct), dp, dp, i32, i32, dp, dp, ctypes.c_int]
    L.mypbr_gpu_autotune.argtypes = [vp, ctypes.POINTER(CameraStruct), ctypes.POINTER(RenderOptsStruct),
                                     ctypes.POINTER(TuneResultStruct)]
    L.mypbr_display_opts_init.argtypes = [ctypes.POINTER(DisplayOptsStruct)]
    L.mypbr_display_opts_init.restype = None
    L.mypbr_gpu_display.argtypes = [dp, i32, i32, ctypes.POINTER(DisplayOptsStruct), dp,
                                    ctypes.POINTER(ctypes.c_uint8), ctypes.c_int]
    L.mypbr_write_image.argtypes = [ctypes.c_char_p, dp, i32, i32, ctypes.POINTER(DisplayOptsStruct), ctypes.c_int]
    L.mypbr_guide_reset.argtypes = [vp]
    L.mypbr_guide_configure.argtypes = [vp, ctypes.c_float, i32, ctypes.c_float]
    L.mypbr_guide_schedule.argtypes = [vp, i32, i32, i32, i32, ctypes.c_float]
    L.mypbr_guide_test_encode.argtypes = [fp, i64, fp]
    L.mypbr_gpu_test_spawn.argtypes = [vp, fp, i64, ip]
    L.mypbr_guide_test_forward.argtypes = [ctypes.c_int, fp, fp, i64, fp]
    L.mypbr_guide_test_backward.argtypes = [ctypes.c_int, fp, fp, fp, i64, fp]
    L.mypbr_guide_test_loss.argtypes = [fp, fp, fp, i64, fp, fp]
    L.mypbr_guide_test_mixture.argtypes = [fp, fp, fp, i64, fp, fp, fp]
    _lib = L
    return L


def check(status):
    if status != MYPBR_OK:
        raise MypbrError(status, lib().mypbr_last_error().decode(errors="replace"))


class Frame:
    """What a render produces per pixel, rows from the top left (denoiser.h:14-20).
    radiance, albedo, normal: (H, W, 3) float64; variance: (H, W)."""

    def __init__(self, radiance, albedo=None, normal=None, variance=None):
        self.radiance = radiance
        self.albedo = albedo
        self.normal = normal
        self.variance = variance


class Scene:
    """A scene loaded on the host: the flat arrays of the C ABI plus the camera
    and render settings its file gives (scene.h:32-40)."""

    def __init__(self, handle):
        self._h = ctypes.c_void_p(handle)
        L = lib()
        self.camera = Camera(L.mypbr_scene_camera(self._h).contents, L.mypbr_scene_render_opts(self._h).contents)

    @property
    def flat(self):
        """Address of the mypbr_flat_scene (valid while this Scene lives)."""
        return lib().mypbr_scene_flat(self._h)

    def close(self):
        if self._h:
            lib().mypbr_scene_free(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def load_scene(path):
    """Parses a .scene file (the grammar of the reference's scene.h:44-243)."""
    out = ctypes.c_void_p()
    check(lib().mypbr_scene_load(os.fsencode(path), ctypes.byref(out)))
    return Scene(out.value)


def parse_scene(text, base_dir="."):
    """The same from text; relative file names resolve against base_dir."""
    out = ctypes.c_void_p()
    check(lib().mypbr_scene_parse(text.encode(), os.fsencode(base_dir), ctypes.byref(out)))
    return Scene(out.value)


class GpuScene:
    """The scene in HBM (mypbr_gpu_scene_create)."""

    def __init__(self, scene):
        out = ctypes.c_void_p()
        check(lib().mypbr_gpu_scene_create(scene.flat, ctypes.byref(out)))
        self._h = out

    @property
    def handle(self):
        return self._h

    def close(self):
        if self._h:
            lib().mypbr_gpu_scene_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def trace(self, rays):
        """Closest hits of rays (n, 8) float32 [o, d, tmin, tmax]: returns
        hits (n, 8) float32 [t, normal, u, v, front_face, -] and prim (n, 2) int32."""
        rays = np.ascontiguousarray(rays, dtype=np.float32)
        n = rays.shape[0]
        hits = np.zeros((n, 8), dtype=np.float32)
        prim = np.zeros((n, 2), dtype=np.int32)
        fp, ip = ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_int32)
        check(lib().mypbr_gpu_trace(self._h, rays.ctypes.data_as(fp), n, hits.ctypes.data_as(fp),
                                    prim.ctypes.data_as(ip), 0))
        return hits, prim

    def spawn_probe(self, rays):
        """Self-intersection probe (mypbr_gpu_test_spawn): for rays (n, 8)
        float32, (flags (n, 4) int32 [kind of the hit, reflected ray met its
        surface, continued ray met its surface, kind of the reflected ray's
        hit], detail (n, 4) float32 [t, origin offset, cosine to the normal,
        t_min] of the first spawned ray that met its surface, else the
        reflected one)."""
        rays = np.ascontiguousarray(rays, dtype=np.float32)
        out = np.zeros((rays.shape[0], 8), dtype=np.int32)
        fp, ip = ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_int32)
        check(lib().mypbr_gpu_test_spawn(self._h, rays.ctypes.data_as(fp), rays.shape[0], out.ctypes.data_as(ip)))
        return out[:, :4].copy(), out[:, 4:].copy().view(np.float32)

    def bsdf_eval(self, material, rec, r_in, wi):
        """eval rgb and scatter pdf of material at records rec (n, 16)."""
        rec = np.ascontiguousarray(rec, dtype=np.float32)
        r_in = np.ascontiguousarray(r_in, dtype=np.float32)
        wi = np.ascontiguousarray(wi, dtype=np.float32)
        n = rec.shape[0]
        out = np.zeros((n, 4), dtype=np.float32)
        fp = ctypes.POINTER(ctypes.c_float)
        check(lib().mypbr_gpu_bsdf_eval(self._h, int(material), rec.ctypes.data_as(fp), r_in.ctypes.data_as(fp),
                                        wi.ctypes.data_as(fp), n, out.ctypes.data_as(fp)))
        return out


class Camera:
    """The reference camera's settings (camera.h:20-56) as attributes."""

    _CAM = {"image_width", "aspect_ratio", "vfov", "lookfrom", "lookat", "vup", "defocus_angle", "focus_dist",
            "ortho_height", "blades", "blade_rotation"}
    _OPT = {"samples_per_pixel", "max_depth", "max_diffuse", "max_specular", "max_scatter", "transparent_shadows",
            "collect_features", "seed", "samples_per_wave", "guided", "timing", "first_row", "row_count"}

    def __init__(self, cam=None, opts=None):
        c = CameraStruct()
        o = RenderOptsStruct()
        if cam is None:
            lib().mypbr_camera_init(ctypes.byref(c))
        else:
            ctypes.memmove(ctypes.byref(c), ctypes.byref(cam), ctypes.sizeof(c))
        if opts is None:
            lib().mypbr_render_opts_init(ctypes.byref(o))
        else:
            ctypes.memmove(ctypes.byref(o), ctypes.byref(opts), ctypes.sizeof(o))
        object.__setattr__(self, "_c", c)
        object.__setattr__(self, "_o", o)

    def __getattr__(self, name):
        if name in Camera._CAM:
            v = getattr(self._c, name)
            return tuple(v) if name in ("lookfrom", "lookat", "vup") else v
        if name in Camera._OPT:
            return getattr(self._o, name)
        raise AttributeError(name)

    def __setattr__(self, name, value):
        if name in Camera._CAM:
            if name in ("lookfrom", "lookat", "vup"):
                arr = getattr(self._c, name)
                for k in range(3):
                    arr[k] = float(value[k])
            else:
                setattr(self._c, name, value)
        elif name in Camera._OPT:
            setattr(self._o, name, int(value))
        else:
            raise AttributeError(name)

    def height(self):
        h = int(self._c.image_width / self._c.aspect_ratio)
        return max(h, 1)

    def structs(self):
        """The (mypbr_camera, mypbr_render_opts) pair, with image_height set."""
        self._c.image_height = self.height()
        return self._c, self._o

    def render(self, gpu_scene, save_every=0, on_pass=None):
        """Renders on the GPU and returns the Frame (camera::render, camera.h:79-105).
        on_pass(done, frame) is called every save_every passes."""
        c, o = self.structs()
        w, h = c.image_width, c.image_height
        rad = np.zeros((h, w, 3), dtype=np.float64)
        feats = bool(o.collect_features)
        alb = np.zeros((h, w, 3), dtype=np.float64) if feats else None
        nrm = np.zeros((h, w, 3), dtype=np.float64) if feats else None
        var = np.zeros((h, w), dtype=np.float64) if feats else None

        def ptr(a):
            return ctypes.c_void_p(a.ctypes.data) if a is not None else ctypes.c_void_p()

        if on_pass is not None:
            def trampoline(done, _user):
                on_pass(done, Frame(rad.copy(), None if alb is None else alb.copy(),
                                    None if nrm is None else nrm.copy(), None if var is None else var.copy()))
            cb = PASS_CALLBACK(trampoline)
        else:
            cb = PASS_CALLBACK()
        check(lib().mypbr_gpu_render(gpu_scene.handle, ctypes.byref(c), ctypes.byref(o), ptr(rad), ptr(alb),
                                     ptr(nrm), ptr(var), int(save_every), cb, None))
        return Frame(rad, alb, nrm, var)


def render_ex(camera, gpu_scene):
    """Renders and returns (radiance (H, W, 3), per-channel variance of the
    mean (H, W, 3), stats dict) through mypbr_gpu_render_ex."""
    c, o = camera.structs()
    w, h = c.image_width, c.image_height
    rad = np.zeros((h, w, 3))
    chv = np.zeros((h, w, 3))
    st = RenderStatsStruct()
    check(lib().mypbr_gpu_render_ex(gpu_scene.handle, ctypes.byref(c), ctypes.byref(o),
                                    ctypes.c_void_p(rad.ctypes.data), None, None, None,
                                    ctypes.c_void_p(chv.ctypes.data), 0, PASS_CALLBACK(), None, ctypes.byref(st)))
    return rad, chv, st.as_dict()


def ggx_albedo_table():
    """The Kulla-Conty tables the device uses: (E[32, 32], E_avg[32])."""
    out = np.zeros(32 * 32 + 32, dtype=np.float64)
    check(lib().mypbr_ggx_albedo_table(out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
    return out[:1024].reshape(32, 32), out[1024:]


def read_image(path):
    """An 8-bit image file as image_texture decodes it: (RGBA bytes [H, W, 4], channels)."""
    w, h, c = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
    b = os.fsencode(path)
    check(lib().mypbr_image_read(b, ctypes.byref(w), ctypes.byref(h), ctypes.byref(c), None, 0))
    out = np.zeros((h.value, w.value, 4), dtype=np.uint8)
    check(lib().mypbr_image_read(b, ctypes.byref(w), ctypes.byref(h), ctypes.byref(c), out.ctypes.data, out.nbytes))
    return out, c.value


# ------------------------------------------------------------ path guiding

def guide_params(hidden):
    """Number of weights of a guiding network with `hidden` hidden layers."""
    return 64 * 128 + hidden * 64 * 64


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _fptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def guide_encode(scalars):
    """The network's encoded inputs (n, 128) of vertices given by their 7
    scalars (n, 7), as the forward kernels write them (BF16)."""
    s = _f32(scalars)
    out = np.zeros((s.shape[0], 128), dtype=np.float32)
    check(lib().mypbr_guide_test_encode(_fptr(s), s.shape[0], _fptr(out)))
    return out


def guide_forward(hidden, weights, inputs):
    """Network outputs (n, 64) for encoded inputs (n, 128), on the tensor cores."""
    w, x = _f32(weights), _f32(inputs)
    out = np.zeros((x.shape[0], 64), dtype=np.float32)
    check(lib().mypbr_guide_test_forward(int(hidden), _fptr(w), _fptr(x), x.shape[0], _fptr(out)))
    return out


def guide_backward(hidden, weights, inputs, dout):
    """Weight gradients of sum(dout * outputs), on the tensor cores."""
    w, x, g = _f32(weights), _f32(inputs), _f32(dout)
    grads = np.zeros(guide_params(hidden), dtype=np.float32)
    check(lib().mypbr_guide_test_backward(int(hidden), _fptr(w), _fptr(x), _fptr(g), x.shape[0], _fptr(grads)))
    return grads


def guide_loss(raw, dirs, c):
    """(gradient (n, 64), loss (n,)) of -c log q(dir) for mixtures given by raw outputs."""
    raw, dirs, c = _f32(raw), _f32(dirs), _f32(c)
    n = raw.shape[0]
    grad = np.zeros((n, 64), dtype=np.float32)
    loss = np.zeros(n, dtype=np.float32)
    check(lib().mypbr_guide_test_loss(_fptr(raw), _fptr(dirs), _fptr(c), n, _fptr(grad), _fptr(loss)))
    return grad, loss


def guide_mixture(raw, u, dirs):
    """(samples (n, 3), pdf at the samples (n,), pdf at dirs (n,)) of the packed mixtures."""
    raw, u, dirs = _f32(raw), _f32(u), _f32(dirs)
    n = raw.shape[0]
    samples = np.zeros((n, 3), dtype=np.float32)
    ps = np.zeros(n, dtype=np.float32)
    pd = np.zeros(n, dtype=np.float32)
    check(lib().mypbr_guide_test_mixture(_fptr(raw), _fptr(u), _fptr(dirs), n, _fptr(samples), _fptr(ps),
                                         _fptr(pd)))
    return samples, ps, pd


# ------------------------------------------------------------ display

def display_opts(exposure=0.0, tonemap="none", bloom=0.0, bloom_threshold=1.0, bloom_radius=0.04, vignette=0.0):
    """display_settings + post_settings (tonemap.h:12-18, postprocess.h:13-21)."""
    o = DisplayOptsStruct()
    lib().mypbr_display_opts_init(ctypes.byref(o))
    o.exposure = exposure
    o.tonemap = TONEMAPPERS[tonemap] if isinstance(tonemap, str) else int(tonemap)
    o.bloom, o.bloom_threshold, o.bloom_radius, o.vignette = bloom, bloom_threshold, bloom_radius, vignette
    return o


def display(radiance, opts=None):
    """(post-processed radiance (H, W, 3), display bytes (H, W, 3) uint8) on the GPU."""
    rad = np.ascontiguousarray(radiance, dtype=np.float64)
    h, w, _ = rad.shape
    lin = np.zeros_like(rad)
    rgb = np.zeros((h, w, 3), dtype=np.uint8)
    o = opts if opts is not None else display_opts()
    dp = ctypes.POINTER(ctypes.c_double)
    check(lib().mypbr_gpu_display(rad.ctypes.data_as(dp), w, h, ctypes.byref(o), lin.ctypes.data_as(dp),
                                  rgb.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), 0))
    return lin, rgb


def write_image(path, radiance, opts=None):
    """write_image (image_io.h:84-106): .png, .ppm, .hdr or .pfm by extension."""
    rad = np.ascontiguousarray(radiance, dtype=np.float64)
    h, w, _ = rad.shape
    o = opts if opts is not None else display_opts()
    check(lib().mypbr_write_image(str(path).encode(), rad.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), w, h,
                                  ctypes.byref(o), 0))


# ------------------------------------------------------------ batches and tuning

def render_batch(jobs):
    """jobs: [(gpu_scene, camera, radiance_device_pointer)] with the radiance
    buffers (H*W*3 float64) in device memory, or (gpu_scene, camera, radiance,
    albedo, normal, variance) pointers when the camera collects features.
    Renders them all (mypbr_gpu_render_batch); returns the per-job statuses."""
    n = len(jobs)
    arr = (BatchJobStruct * n)()
    keep = []
    for k, job in enumerate(jobs):
        gs, cam, ptr = job[:3]
        c, o = cam.structs()
        keep.append((c, o))
        arr[k].scene = gs.handle
        arr[k].camera = ctypes.pointer(c)
        arr[k].opts = ctypes.pointer(o)
        arr[k].radiance = int(ptr)
        if len(job) == 6:
            arr[k].albedo, arr[k].normal, arr[k].variance = (int(x) if x else None for x in job[3:6])
    status = lib().mypbr_gpu_render_batch(arr, n)
    codes = [arr[k].status for k in range(n)]
    check(status)
    return codes


def denoise(radiance, albedo, normal, variance, width, height, out, on_device=False):
    """denoiser::run with the default settings (mypbr_gpu_denoise). Arguments
    are numpy arrays (host) or device addresses (on_device); out receives the
    filtered radiance (H*W*3 float64)."""
    def addr(x):
        return int(x) if on_device else x.ctypes.data
    check(lib().mypbr_gpu_denoise(addr(radiance), addr(albedo), addr(normal), addr(variance), int(width),
                                  int(height), None, addr(out), int(bool(on_device))))


def env_distribution(rgb, on_gpu=False):
    """The environment's sampling tables for an (H, W, 3) float32 image:
    (texel pdf p*W*H [H, W], alias probabilities [H*W], alias indices [H*W])."""
    rgb = np.ascontiguousarray(rgb, dtype=np.float32)
    h, w = rgb.shape[:2]
    pdf = np.zeros((h, w), dtype=np.float32)
    alias = np.zeros((h * w, 2), dtype=np.float32)
    check(lib().mypbr_env_distribution(rgb.ctypes.data, w, h, pdf.ctypes.data, alias.ctypes.data, int(bool(on_gpu))))
    return pdf, alias[:, 0].copy(), alias[:, 1].copy().view(np.int32)


def autotune(camera, gpu_scene):
    """Runs the autotuner for this view; returns its choice and trial rates."""
    c, o = camera.structs()
    r = TuneResultStruct()
    check(lib().mypbr_gpu_autotune(gpu_scene.handle, ctypes.byref(c), ctypes.byref(o), ctypes.byref(r)))
    return {"block": r.block, "traversal": r.traversal, "wave_paths": r.wave_paths,
            "mpaths_per_s": r.mpaths_per_s, "trials": list(r.trial_mpaths)}


def set_launch(gpu_scene, block=0, wave_paths=0, traversal=0):
    """Launch settings of later renders of this handle (0 = default)."""
    check(lib().mypbr_gpu_set_launch(gpu_scene.handle, block, wave_paths, traversal))


def sky_bake(sun_direction, sun_irradiance, width=256, height=128, rayleigh=1.0, mie=1.0, mie_g=0.8, ozone=1.0,
             intensity=3.0, on_gpu=False):
    """atmosphere::bake + sun_transmittance: (image (H, W, 3), transmittance (3,))."""
    s = SkySettingsStruct(rayleigh, mie, mie_g, ozone, intensity)
    d = np.ascontiguousarray(sun_direction, dtype=np.float64)
    e = np.ascontiguousarray(sun_irradiance, dtype=np.float64)
    img = np.zeros((height, width, 3))
    t = np.zeros(3)
    dp = ctypes.POINTER(ctypes.c_double)
    check(lib().mypbr_sky_bake(ctypes.byref(s), d.ctypes.data_as(dp), e.ctypes.data_as(dp), width, height,
                               img.ctypes.data_as(dp), t.ctypes.data_as(dp), int(on_gpu)))
    return img, t


def guide_reset(gpu_scene):
    """The handle's guiding network back to its untrained weights (buffers kept)."""
    check(lib().mypbr_guide_reset(gpu_scene.handle))


def guide_configure(gpu_scene, alpha=0.5, depths=4, alpha_deep=-1.0):
    """Guided sampling of the handle: the mixture drawn with probability alpha
    (0 < alpha < 1, else the BSDF) at the first bounce and alpha_deep (below
    0: alpha) at the later ones of the first `depths` bounces of a path."""
    check(lib().mypbr_guide_configure(gpu_scene.handle if gpu_scene is not None else None, float(alpha),
                                      int(depths), float(alpha_deep)))


def guide_schedule(gpu_scene, steps_early=16, steps_late=4, max_steps=1500, use_after=128, weight_cap=256.0):
    """The training schedule of the scene handle's guiding network
    (mypbr_guide_schedule)."""
    check(lib().mypbr_guide_schedule(gpu_scene.handle, int(steps_early), int(steps_late), int(max_steps),
                                     int(use_after), float(weight_cap)))


def rebuild_bvh(gpu_scene):
    """Replaces the handle's BVH by a linear BVH built on the device; returns the report."""
    r = BvhReportStruct()
    check(lib().mypbr_gpu_scene_rebuild_bvh(gpu_scene.handle, 1, ctypes.byref(r)))
    return {k: getattr(r, k) for k, _ in BvhReportStruct._fields_ if k != "reserved"}
