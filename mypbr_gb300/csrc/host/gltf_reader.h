// Reading glTF 2.0 models (.gltf with its buffers and images, or one .glb)
// into triangles in the file's world space plus a description of their
// materials, for the scene loader to map onto ours (gltf_loader.h:20-58 of
// the reference, which reads the same files with cgltf).
#pragma once

#include <cstdint>
#include <set>
#include <string>
#include <vector>

namespace mypbr_host {

// A texture as a material uses it (textureInfo, with KHR_texture_transform).
struct GltfTextureRef {
    int texture = -1;  // into GltfModel::textures; -1: none
    int texcoord = 0;  // the texture-coordinate set (the transform's texCoord wins)
    bool has_transform = false;
    double offset[2] = {0, 0}, rotation = 0, scale[2] = {1, 1};
    double strength = 1;  // normalTexture.scale
};

// A metallic-roughness material with the extensions the loader maps.
struct GltfMaterial {
    std::string name;
    double base_color[4] = {1, 1, 1, 1};
    double metallic = 1, roughness = 1;
    GltfTextureRef base_texture, metal_rough_texture, normal_texture, emissive_texture;
    double emissive[3] = {0, 0, 0};
    double emissive_strength = 1;  // KHR_materials_emissive_strength
    int alpha_mode = 0;            // 0 OPAQUE, 1 MASK, 2 BLEND
    double alpha_cutoff = 0.5;
    double ior = 1.5;                // KHR_materials_ior
    bool has_transmission = false;   // KHR_materials_transmission
    double transmission = 0;
    bool has_clearcoat = false;      // KHR_materials_clearcoat
    double clearcoat = 0, clearcoat_roughness = 0;
    GltfTextureRef clearcoat_texture, clearcoat_roughness_texture, clearcoat_normal_texture;
    std::vector<std::string> unsupported;  // extensions present that are left out (sheen, ...)
};

struct GltfImage {
    std::vector<uint8_t> bytes;  // the file inside a buffer view
    std::string path;            // else a file next to the model (URI decoded); empty for data URIs
    std::string label;           // the URI, the name or "embedded", for messages
};

struct GltfTexture {
    int image = -1;
    bool repeat = true;  // false only when both wrap modes clamp to the edge
};

struct GltfFace {
    int v[3], n[3], t[3];  // into positions / normals / uvs; -1 where absent
    int material;          // into materials; -1: the spec's default material
};

struct GltfModel {
    std::vector<GltfMaterial> materials;
    std::vector<GltfTexture> textures;
    std::vector<GltfImage> images;
    std::vector<double> positions;  // xyz, node transforms applied
    std::vector<double> normals;    // xyz, by the inverse transpose, not normalized
    std::vector<double> uvs;        // uv with v flipped to run up the image
    std::vector<GltfFace> faces;    // in the order the node walk meets them
    std::set<std::string> ignored;  // features present and left out
};

// Reads the model; false with a message in error ("cannot read glTF file ...",
// "cannot load the buffers of ...", or what is malformed).
bool read_gltf(const std::string& path, GltfModel& model, std::string& error);

}  // namespace mypbr_host
