// The storage behind a mypbr_host_scene: the vectors the flat scene points into.
#pragma once

#include <string>
#include <vector>

#include "../../../include/mypbr_gpu.h"
#include "host_math.h"

struct mypbr_host_scene {
    std::vector<mypbr_sphere> spheres;
    std::vector<mypbr_quad> quads;
    std::vector<double> positions, normals, uvs;
    std::vector<mypbr_triangle> triangles;
    std::vector<mypbr_mesh> meshes;
    std::vector<mypbr_medium> media;
    std::vector<mypbr_xform> xforms;
    std::vector<mypbr_unbounded> unbounded;
    std::vector<mypbr_bvh_node> bvh_nodes;
    std::vector<mypbr_prim_ref> bvh_prims;
    std::vector<mypbr_material> materials;
    std::vector<mypbr_texture> textures;
    std::vector<uint8_t> texels_ldr;
    std::vector<float> texels_hdr;
    std::vector<mypbr_light> lights;
    std::vector<mypbr_light_member> light_members;
    std::vector<mypbr_voxel_model> voxel_models;
    std::vector<mypbr_voxel_block> voxel_blocks;
    std::vector<mypbr_voxel_entry> voxel_palettes;
    std::vector<uint8_t> voxel_cells;
    std::vector<float> env_pixels;
    int env_width = 0, env_height = 0;
    double env_intensity = 1, env_rotation = 0;
    mypbr_sun sun{};
    bool use_sky = true;
    mypbr_host::V3 background;

    mypbr_camera camera{};
    mypbr_render_opts opts{};
    mypbr_flat_scene flat{};

    int64_t position_count() const { return int64_t(positions.size() / 3); }
    int64_t normal_count() const { return int64_t(normals.size() / 3); }
    int64_t uv_count() const { return int64_t(uvs.size() / 2); }

    // Points flat at the vectors (call after the last change) and sets the
    // camera's image height.
    void finalize();
};

namespace mypbr_host {
void set_error(const std::string& message);
void clear_error();
}  // namespace mypbr_host
