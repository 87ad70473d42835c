// camera_gpu.h — the reference-side binding of the GB300 backend: a device
// version of camera::render (camera.h:79-105) for the reference's own tree.
//
// A maintainer drops this file next to include/camera.h of adriendjn/mypbr,
// adds this repository's include/ to the include path and links
// libmypbr_gb300.so. main.cpp then calls
//
//     frame f = render_device(scene_path, sc.cam, save_every, cb);
//
// in place of cam.render(world, sc.lights, save_every, cb) (main.cpp:93) when
// --gpu is given; the denoiser and image writers take the frame unchanged.
//
// The scene graph of the reference cannot cross a C ABI, so the backend
// reads the same scene file itself (the geometry, materials, lights,
// environment and sun it describes). Every setting the caller holds on the
// camera object is passed on: image size, view (lookfrom, lookat, vup,
// vfov), lens (defocus_angle, focus_dist, blades, blade_rotation,
// ortho_height), samples, bounce caps, transparent shadows, features, and
// the background (use_sky / background). threads has no meaning on the GPU.
#pragma once

#include <functional>
#include <stdexcept>
#include <string>
#include <vector>

#include "camera.h"
#include "mypbr_gpu.h"

namespace mypbr_binding {

// The camera's settings as the backend's camera and render options.
inline void settings_of(const camera& cam, mypbr_camera& c, mypbr_render_opts& o) {
    c.image_width = cam.image_width;
    int h = int(cam.image_width / cam.aspect_ratio);  // camera.h:143-144
    c.image_height = h < 1 ? 1 : h;
    c.aspect_ratio = cam.aspect_ratio;
    c.vfov = cam.vfov;
    for (int k = 0; k < 3; k++) {
        c.lookfrom[k] = cam.lookfrom[k];
        c.lookat[k] = cam.lookat[k];
        c.vup[k] = cam.vup[k];
    }
    c.defocus_angle = cam.defocus_angle;
    c.focus_dist = cam.focus_dist;
    c.ortho_height = cam.ortho_height;
    c.blades = cam.blades;
    c.blade_rotation = cam.blade_rotation;
    o.samples_per_pixel = cam.samples_per_pixel;
    o.max_depth = cam.max_depth;
    o.max_diffuse = cam.max_diffuse;
    o.max_specular = cam.max_specular;
    o.max_scatter = cam.max_scatter;
    o.transparent_shadows = cam.transparent_shadows;
    o.collect_features = cam.collect_features;
}

}  // namespace mypbr_binding

// Renders the scene file with the GB300 backend as `cam` is set up and
// returns the frame camera::render would (averages, rows from the top left,
// albedo / normal / variance with collect_features). on_pass gets the running
// average every save_every passes. Throws std::runtime_error with the
// backend's message on an error.
inline frame render_device(const std::string& scene_path, const camera& cam, int save_every,
                           const camera::pass_callback& on_pass) {
    mypbr_host_scene* hs = nullptr;
    if (mypbr_scene_load(scene_path.c_str(), &hs) != MYPBR_OK)
        throw std::runtime_error(mypbr_last_error());
    mypbr_flat_scene flat = *mypbr_scene_flat(hs);  // arrays stay owned by hs
    flat.use_sky = cam.use_sky;
    for (int k = 0; k < 3; k++)
        flat.background[k] = cam.background[k];
    mypbr_gpu_scene* gs = nullptr;
    if (mypbr_gpu_scene_create(&flat, &gs) != MYPBR_OK) {
        mypbr_scene_free(hs);
        throw std::runtime_error(mypbr_last_error());
    }
    mypbr_camera c = *mypbr_scene_camera(hs);
    mypbr_render_opts o = *mypbr_scene_render_opts(hs);
    mypbr_binding::settings_of(cam, c, o);

    size_t n = size_t(c.image_width) * size_t(c.image_height);
    std::vector<double> rad(3 * n), alb(3 * n), nrm(3 * n), var(n);
    auto to_frame = [&]() {
        frame f;
        f.radiance.resize(n);
        for (size_t k = 0; k < n; k++)
            f.radiance[k] = color(rad[3 * k], rad[3 * k + 1], rad[3 * k + 2]);
        if (o.collect_features) {
            f.albedo.resize(n);
            f.normal.resize(n);
            f.variance = var;
            for (size_t k = 0; k < n; k++) {
                f.albedo[k] = color(alb[3 * k], alb[3 * k + 1], alb[3 * k + 2]);
                f.normal[k] = color(nrm[3 * k], nrm[3 * k + 1], nrm[3 * k + 2]);
            }
        }
        return f;
    };
    struct Progress {
        const camera::pass_callback* cb;
        std::function<frame()>* make;
    };
    std::function<frame()> make = to_frame;
    Progress progress{&on_pass, &make};
    auto hook = [](int done, void* user) {
        auto* p = static_cast<Progress*>(user);
        if (*p->cb)
            (*p->cb)(done, (*p->make)());
    };
    int status = mypbr_gpu_render(gs, &c, &o, rad.data(), alb.data(), nrm.data(), var.data(), save_every,
                                  on_pass ? static_cast<mypbr_pass_callback>(hook) : nullptr, &progress);
    mypbr_gpu_scene_destroy(gs);
    mypbr_scene_free(hs);
    if (status != MYPBR_OK)
        throw std::runtime_error(mypbr_last_error());
    return to_frame();
}
