// Host preparation of the device scene records from a HostScene.
#pragma once
#include <vector>

#include "device_types.h"
#include "scene_host.h"

namespace orion_gb300 {

struct PreparedScene {
  std::vector<PrimShade> prims;
  std::vector<DevMaterial> mats;
  std::vector<DevLight> lights;
  std::vector<float> light_func, light_cdf;  // Distribution1D over light power
  float light_func_int = 0.f;
  std::vector<int> env_idx;
  float world_center[3] = {0, 0, 0};
  float world_radius = 0.f;
  DevCamera cam{};
  // Image environment maps: every array in one float block; DevEnvMap
  // pointers are these offsets until the block is uploaded.
  std::vector<float> env_data;
  struct EnvMapLayout {
    int width, height;
    float marg_int;
    size_t texels, cond_func, cond_cdf, cond_int, marg_func, marg_cdf;
  };
  std::vector<EnvMapLayout> envmaps;
  // Image textures: texels in env_data too; per material its builder inputs
  // and texture slots; per primitive its three texture coordinates (only
  // when a material is textured).
  struct TextureLayout {
    int width, height;
    size_t texels;
  };
  std::vector<TextureLayout> textures;
  std::vector<DevMaterialSrc> mat_src;
  std::vector<float> prim_uv;  // T x 6, or empty
};

// Materials -> lobe lists (Material::getBSDF, src/material/*.cpp).
DevMaterial prepare_material(const orion_material& m);
// The builder inputs of a material: its constants and derived constants.
MaterialInputs material_inputs(const orion_material& m);
// True when an input of the material comes from an image texture.
bool material_textured(const orion_material& m);
// Everything else; returns false with `err` set on inconsistent input.
bool prepare_scene(const HostScene& s, PreparedScene* out, std::string* err);
DevCamera prepare_camera(const orion_camera& cam);

float roughness_to_alpha(float roughness);  // src/bsdf/microfacet.h:44-50
float spectrum_intensity(const float rgb[3]);  // src/core/spectrum.h:88-91

}  // namespace orion_gb300
