// Declaration subset of framework/resource/material.h:16-80 and
// framework/render/material/predefine.h:15-22 (EMatType): the seven BSDF
// parameter sets and the tagged union resource::Material.
#pragma once
#include "util/texture.h"

namespace Pupil {
enum class EMatType : unsigned int {
    Unknown = 0, Diffuse, Dielectric, RoughDielectric, Conductor, RoughConductor, Plastic, RoughPlastic, Twosided, Count
};
}  // namespace Pupil

namespace Pupil::resource {
struct Diffuse { util::Texture reflectance; };
struct Dielectric {
    float int_ior;
    float ext_ior;
    util::Texture specular_reflectance;
    util::Texture specular_transmittance;
};
struct RoughDielectric {
    float int_ior;
    float ext_ior;
    util::Texture alpha;
    util::Texture specular_reflectance;
    util::Texture specular_transmittance;
};
struct Conductor {
    util::Texture eta;
    util::Texture k;
    util::Texture specular_reflectance;
};
struct RoughConductor {
    util::Texture alpha;
    util::Texture eta;
    util::Texture k;
    util::Texture specular_reflectance;
};
struct Plastic {
    float int_ior;
    float ext_ior;
    bool nonlinear;
    util::Texture diffuse_reflectance;
    util::Texture specular_reflectance;
};
struct RoughPlastic {
    float int_ior;
    float ext_ior;
    bool nonlinear;
    util::Texture alpha;
    util::Texture diffuse_reflectance;
    util::Texture specular_reflectance;
};
struct Material {
    EMatType type = EMatType::Unknown;
    bool twosided = false;
    union {
        Diffuse diffuse{};
        Dielectric dielectric;
        RoughDielectric rough_dielectric;
        Conductor conductor;
        RoughConductor rough_conductor;
        Plastic plastic;
        RoughPlastic rough_plastic;
    };
    Material() noexcept {}
};
}  // namespace Pupil::resource
