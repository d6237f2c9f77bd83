// Records shared by the host scene builder and the CUDA kernels.
//
// Everything a kernel reads about a scene is flattened into these plain
// structs at upload time: materials become fixed lobe lists (the BxDF list
// that Material::getBSDF builds per hit in the reference,
// src/material/*.cpp), lights become typed records with their derived
// constants, and the camera becomes its matrix and projection constants.
#pragma once
#include <stdint.h>

#ifdef __CUDACC__
#define ORION_HD __host__ __device__
#else
#define ORION_HD
#endif

namespace orion_gb300 {

// Deepest BVH (levels of the binary tree below the root) a scene upload accepts;
// the traversal stacks hold one entry per level.
constexpr int kMaxBvhDepth = 48;

// Shared memory a persistent trace block needs per warp beside its stacks:
// the scratch of the warp-cooperative triangle tests (TriScratch).
constexpr int kTriScratchBytes = 288;

// Sobol direction numbers (src/sampler/sobol.cpp): dimensions, numbers per
// dimension, and the index bytes those numbers cover.
constexpr int kSobolBits = 52;
constexpr int kSobolDims = 1024;
constexpr int kSobolBytes = (kSobolBits + 7) / 8;

// BxDFType bits (src/core/bsdf.h:16-24).
enum : int32_t {
  BXDF_REFLECTION = 1,
  BXDF_TRANSMISSION = 2,
  BXDF_DIFFUSE = 4,
  BXDF_GLOSSY = 8,
  BXDF_SPECULAR = 16,
  BXDF_ALL = 31,
};

enum LobeKind : int32_t {
  LOBE_LAMBERT_R = 0,      // src/bsdf/lambert.cpp:5-8
  LOBE_OREN_NAYAR = 1,     // src/bsdf/orennayar.cpp:5-37
  LOBE_MICROFACET_R = 2,   // src/bsdf/microfacet.cpp:42-74
  LOBE_MICROFACET_T = 3,   // src/bsdf/microfacet.cpp:76-120
  LOBE_SPECULAR_R = 4,     // src/bsdf/specular.cpp:20-25
  LOBE_SPECULAR_T = 5,     // src/bsdf/specular.cpp:4-18
  LOBE_FRESNEL_SPECULAR = 6,  // src/bsdf/specular.cpp:28-54
};

enum FresnelKind : int32_t {
  FRESNEL_NOOP = 0,        // src/core/bsdf.h:96-99
  FRESNEL_CONDUCTOR = 1,   // src/core/bsdf.cpp:124-147
  FRESNEL_DIELECTRIC = 2,  // src/core/bsdf.cpp:149-170
};

enum DistKind : int32_t { DIST_GGX = 0, DIST_BECKMANN = 1 };

struct DevLobe {       // 64 bytes
  int32_t kind;        // LobeKind
  int32_t type;        // BxDFType bits of this lobe
  int32_t fresnel;     // FresnelKind (reflection lobes)
  int32_t dist;        // DistKind (microfacet lobes)
  float c[3];          // R or T
  float alpha;         // microfacet alpha (roughnessToAlpha applied)
  float c2[3];         // FresnelSpecular: T
  float etaA;          // etaA / fresnel etaI
  float etaB;          // etaB / fresnel etaT (scalar dielectric)
  float on_a, on_b;    // Oren-Nayar A, B
  float fr_eta[3];     // conductor etaT
  float fr_k[3];       // conductor k
  int32_t photon;      // TransportMode::Photon: transmission without radiance scaling (SPPM photon pass)
};

constexpr int kMaxLobes = 5;

// Shading classes: materials whose lobe lists run the same code. Paths are
// sorted by the class of what they hit before shading, so a warp shades one
// kind of material.
enum ShadeClass : int32_t {
  SC_DIFFUSE = 0,     // Lambert
  SC_CONDUCTOR = 1,   // one microfacet reflection lobe (metal)
  SC_SPECULAR = 2,    // delta lobes only (mirror, smooth glass)
  SC_DIELECTRIC = 3,  // microfacet reflection + transmission (rough glass)
  SC_PLASTIC = 4,     // Lambert + microfacet reflection
  SC_GENERAL = 5,     // anything else (Oren-Nayar, uber, no lobes)
  SC_TEXTURED = 6,    // an input comes from an image texture: lobes built per hit
  SC_MISS = 7,        // the ray left the scene
  kShadeClasses = 8
};

struct DevMaterial {   // 16 + 5 * 64 = 336 bytes
  int32_t num_lobes;
  int32_t num_nonspecular;  // numBxDF(BxDF_ALL & ~BxDF_SPECULAR)
  int32_t shade_class;      // ShadeClass
  int32_t pad;
  DevLobe lobes[kMaxLobes];
};

// What Material::getBSDF reads (src/material/*.cpp), with every texture
// already evaluated: constants on the host, image texels at the hit in the
// textured shading kernel. Transcendental constants (alpha, Oren-Nayar A, B)
// are derived once on the host so both sides build identical lobes.
struct MaterialInputs {  // 128 bytes
  int32_t type;          // ORION_MAT_*
  int32_t dist;          // DistKind
  float Kd[3], Ks[3], Kr[3], Kt[3], opacity[3], eta_rgb[3], k[3];
  float sigma;           // matte: clamped at 0; 0 selects Lambert
  float roughness, eta;
  float alpha;           // roughnessToAlpha(roughness)
  float on_a, on_b;      // Oren-Nayar A, B for sigma
  float pad[3];
};
static_assert(sizeof(MaterialInputs) == 128, "MaterialInputs is 128 bytes");

constexpr int kTexSlots = 7;  // Kd, Ks, Kr, Kt, opacity, eta, k (ORION_TEX_*)

// A material with image-textured inputs: its constant inputs and, per
// input, the DevTexture it reads (-1: the constant).
struct DevMaterialSrc {  // 160 bytes
  MaterialInputs in;
  int32_t tex[8];
};
static_assert(sizeof(DevMaterialSrc) == 160, "DevMaterialSrc is 160 bytes");

// An image texture (ImageTexture, src/texture/imagetexture.cpp:4-12).
struct DevTexture {
  int32_t width, height;
  const float* texels;   // width x height x 3, row 0 at the top
};

enum DevLightKind : int32_t { DL_AREA = 0, DL_POINT = 1, DL_SPOT = 2, DL_DISTANT = 3, DL_ENV = 4 };

struct DevLight {      // 128 bytes
  int32_t kind;
  int32_t prim;        // area: emissive primitive
  float area;          // area: triangle area (src/core/triangle.cpp:77-83);
                       // env: intensity of the constant map (0 disables sampling)
  int32_t image;       // env: index of its DevEnvMap, -1 for a constant map
  float L[3];          // Le / I / L
  float pad1;
  float p[3];          // point/spot position; distant: direction
  float pad2;
  float m[9];          // spot: world->light 3x3; env: light->world 3x3
  float minv[9];       // spot: light->world 3x3; env: world->light 3x3
  float cos_total, cos_falloff;
  float pad3[2];
};

// An image environment map (src/light/envmap.cpp:9-44): texels already
// scaled by L, and the Distribution2D (src/sampler/sampling.h:127-151,
// sampling.cpp:63-76) over intensity x sin(theta) of each texel: one
// conditional Distribution1D per row and the marginal over the rows.
struct DevEnvMap {
  int32_t width, height;
  float marg_int;          // marginal funcInt
  int32_t pad;
  const float* texels;     // width x height x 3, row 0 at the top
  const float* cond_func;  // height rows of width
  const float* cond_cdf;   // height rows of width + 1
  const float* cond_int;   // height
  const float* marg_func;  // height
  const float* marg_cdf;   // height + 1
};

struct DevCamera {
  float c2w[16];       // camera-to-world 4x4 row-major
  float tan_half_fov;
  float aspect;
  float lens_radius;
  float focal_distance;
  int32_t width, height;
  int32_t pad[2];
};

// Per-primitive shading record, primID order: 96 bytes = 6 x float4.
struct PrimShade {
  float p[9];          // p0, p1, p2
  float n[9];          // n0, n1, n2
  int32_t material;
  int32_t light;       // area light index or -1
  int32_t pad[4];
};

// One BVH node: 32 bytes = 2 x float4. Children of an inner node are the
// adjacent pair (a, a + 1); a leaf holds triangles [a, a + b) of the
// leaf-ordered triangle array.
struct BvhNode {
  float lo[3];
  int32_t a;
  float hi[3];
  int32_t b;           // 0 = inner node, > 0 = leaf triangle count
};

// One node of the 8-wide BVH the kernels traverse: 80 bytes = 5 x float4.
// Child boxes are quantised to 8 bits per bound on a per-axis grid of
// power-of-two cells anchored at `p`: bound = p + q * 2^(e - 127).
// Internal children are stored contiguously from child_base in slot order;
// the triangles of all leaf children contiguously from tri_base.
// meta[s]: 0 = empty slot; internal child: 0x80; leaf child:
// (triangle count 1..3) << 5 | (first triangle - tri_base, 0..23).
// An empty slot's box is inverted (qlo = 255, qhi = 0), so it is never hit.
// Slots are assigned so that visiting them in order of (slot ^ octant),
// octant bit a set when the ray direction is negative along axis a, is
// roughly near to far.
struct WideNode {
  float p[3];
  uint8_t e[3];        // biased exponent of the cell size per axis
  uint8_t imask;       // bit s: slot s holds an internal child
  int32_t child_base;
  int32_t tri_base;
  uint8_t meta[8];
  uint8_t qlo[3][8];   // [axis][slot]
  uint8_t qhi[3][8];
};
static_assert(sizeof(WideNode) == 80, "WideNode is five float4");

}  // namespace orion_gb300
