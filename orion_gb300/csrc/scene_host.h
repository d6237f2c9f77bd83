// Host-side scene: the .ori loader and the flat arrays it produces.
#pragma once
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/orion_gpu.h"

namespace orion_gb300 {

// 4x4 float matrix with the reference's row-major convention and
// left-to-right float arithmetic (src/core/transform.h:13-60,
// src/core/transform.cpp:34-100), so baked vertices, normals and the camera
// matrix come out bit-identical to the reference's.
struct Mat4 {
  float m[4][4];
  static Mat4 identity();
  static Mat4 make(float t00, float t01, float t02, float t03, float t10, float t11, float t12, float t13,
                   float t20, float t21, float t22, float t23, float t30, float t31, float t32, float t33);
  Mat4 operator*(const Mat4& b) const;
  Mat4 transposed() const;
  Mat4 inverse() const;  // Gauss-Jordan elimination with full pivoting
};

struct Xform {
  Mat4 m, minv;
  Xform() : m(Mat4::identity()), minv(Mat4::identity()) {}
  Xform(const Mat4& a, const Mat4& ainv) : m(a), minv(ainv) {}
  explicit Xform(const Mat4& a) : m(a), minv(a.inverse()) {}
  Xform inverse() const { return Xform(minv, m); }
  Xform operator*(const Xform& b) const { return Xform(m * b.m, b.minv * minv); }
  void point(const float in[3], float out[3]) const;
  void vector(const float in[3], float out[3]) const;
  void normal(const float in[3], float out[3]) const;

  static Xform translate(float x, float y, float z);
  static Xform scale(float x, float y, float z);
  static Xform rotate(float degrees, const float axis[3]);
  static Xform look_at(const float pos[3], const float look[3], const float up[3]);
};

struct HostImage {
  int32_t width = 0, height = 0;
  std::vector<float> rgb;         // width x height x 3, row 0 at the top
};

struct HostScene {
  std::vector<float> positions;   // T x 9
  std::vector<float> normals;     // T x 9
  std::vector<float> uvs;         // T x 6
  std::vector<int32_t> material_of_prim;
  std::vector<int32_t> light_of_prim;
  std::vector<orion_material> materials;
  std::vector<orion_light> lights;
  std::vector<HostImage> images;   // environment map and texture texels (orion_light.image, orion_material.tex = index + 1)
  std::vector<orion_image> image_desc;  // views of `images` for desc()
  orion_camera camera{};
  int32_t spp = 1;
  int32_t max_depth = 5;
  int32_t integrator = ORION_INTEGRATOR_PATH;
  orion_sppm_params sppm{0, 0, 0.f, 0};
  std::string source;             // file the scene was read from ("" if built from a desc)

  int64_t num_prims() const { return (int64_t)material_of_prim.size(); }
  void desc(orion_scene_desc* out) const;
  void index_images();  // refresh image_desc after `images` changes
};

// Returns ORION_OK or an error code; `err` receives a message.
int load_ori(const std::string& path, HostScene* out, std::string* err);
int scene_from_desc(const orion_scene_desc& d, HostScene* out, std::string* err);

// Shared float helpers with the reference's rounding.
float radians_f(float deg);
float degrees_f(float rad);

}  // namespace orion_gb300
