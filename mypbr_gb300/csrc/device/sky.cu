// The sky bake of `sky atmosphere` on the device: one thread per pixel of the
// equirectangular image, the same FP64 single-scattering march the host
// loader runs (sky_model.h). 256 x 128 pixels x 32 view steps x 16 sun steps
// are ~17M density evaluations: milliseconds here, about a second on one
// host core, which matters when the sun moves from frame to frame.
#include <vector>

#include "../host/sky_model.h"
#include "gpu_scene.h"

namespace mypbr_dev {
namespace {

__global__ void k_bake_sky(mypbr_sky::Settings st, double3 sun_dir, double3 sun_irr, int w, int h, double* out) {
    int n = w * h;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        double sd[3] = {sun_dir.x, sun_dir.y, sun_dir.z};
        mypbr_sky::C3 c = mypbr_sky::bake_pixel(st, k % w, k / w, w, h, sd, mypbr_sky::C3{sun_irr.x, sun_irr.y, sun_irr.z});
        out[3 * size_t(k)] = c.r;
        out[3 * size_t(k) + 1] = c.g;
        out[3 * size_t(k) + 2] = c.b;
    }
}

}  // namespace
}  // namespace mypbr_dev

using namespace mypbr_dev;

extern "C" {

void mypbr_sky_settings_init(mypbr_sky_settings* s) {
    if (!s)
        return;
    mypbr_sky::Settings d;
    s->rayleigh = d.rayleigh;
    s->mie = d.mie;
    s->mie_g = d.mie_g;
    s->ozone = d.ozone;
    s->intensity = d.intensity;
}

int mypbr_sky_bake(const mypbr_sky_settings* settings, const double sun_direction[3], const double sun_irradiance[3],
                   int32_t width, int32_t height, double* rgb, double* sun_transmittance, int on_gpu) {
    if (!sun_direction || !sun_irradiance || !rgb || width < 1 || height < 1) {
        set_error_message("mypbr_sky_bake: bad argument");
        return MYPBR_ERR_INVALID_ARGUMENT;
    }
    mypbr_sky::Settings st;
    if (settings) {
        st.rayleigh = settings->rayleigh;
        st.mie = settings->mie;
        st.mie_g = settings->mie_g;
        st.ozone = settings->ozone;
        st.intensity = settings->intensity;
    }
    size_t n = size_t(width) * height;
    if (on_gpu) {
        double* d = nullptr;
        MYPBR_CUDA(cudaMalloc(&d, 3 * n * sizeof(double)));
        k_bake_sky<<<int((n + 127) / 128), 128>>>(st, make_double3(sun_direction[0], sun_direction[1], sun_direction[2]),
                                                  make_double3(sun_irradiance[0], sun_irradiance[1], sun_irradiance[2]),
                                                  width, height, d);
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess)
            e = cudaMemcpy(rgb, d, 3 * n * sizeof(double), cudaMemcpyDeviceToHost);
        cudaFree(d);
        if (e != cudaSuccess)
            return cuda_fail(e, "mypbr_sky_bake");
    } else {
        mypbr_sky::C3 irr{sun_irradiance[0], sun_irradiance[1], sun_irradiance[2]};
        for (int j = 0; j < height; j++)
            for (int i = 0; i < width; i++) {
                mypbr_sky::C3 c = mypbr_sky::bake_pixel(st, i, j, width, height, sun_direction, irr);
                size_t k = (size_t(j) * width + i) * 3;
                rgb[k] = c.r;
                rgb[k + 1] = c.g;
                rgb[k + 2] = c.b;
            }
    }
    if (sun_transmittance) {
        mypbr_sky::C3 t = mypbr_sky::sun_transmittance(st, sun_direction);
        sun_transmittance[0] = t.r;
        sun_transmittance[1] = t.g;
        sun_transmittance[2] = t.b;
    }
    return MYPBR_OK;
}

}  // extern "C"
