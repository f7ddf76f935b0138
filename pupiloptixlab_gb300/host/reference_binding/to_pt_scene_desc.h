// to_pt_scene_desc.h -- the one piece of code a PupilOptixLab maintainer adds
// besides the pass: conversion of the loaded resource::Scene
// (framework/resource/scene.h:39-57; ShapeInstance, Shape, Material, Emitter:
// framework/resource/shape.h:31-97, material.h:16-80, emitter.h:7-55) into the
// tracer's pt_scene_desc (include/pt_api.h).
//
// Compiled inside the PupilOptixLab tree against its framework headers, or
// here against the declaration subset in framework_subset/ (same names, same
// fields; tests/test_reference_binding_cpu.py builds both this file and
// wavefront_pass.cpp that way).
#pragma once

#include <string>
#include <unordered_map>
#include <vector>

#include "pt_api.h"
#include "resource/scene.h"

namespace Pupil::pt {

// What a pt_scene_desc points to.  The arrays of meshes, curves and bitmaps
// are NOT copied: they point into the resource::Scene's shapes and textures,
// which must stay alive until pt_scene_upload returns (it copies everything).
struct PtSceneDesc {
    pt_scene_desc desc{};
    std::vector<pt_mesh_desc> meshes;
    std::vector<pt_sphere_desc> spheres;
    std::vector<pt_curves_desc> curves;
    std::vector<pt_material_desc> materials;
    std::vector<pt_instance_desc> instances;
};

// Fills `out` from `scene`; `camera` is the optix::Camera of the world's camera
// helper (its device copy, world->camera->GetCudaMemory(), read back with
// cudaMemcpy), which already holds the sensor's fov, aspect and transform.
// Shapes shared by several instances (the built-in cube, rectangle and unit
// sphere, OBJ files loaded once) become one mesh / sphere each; an area
// emitter's radiance is its RGB value or its texture.  Returns false with a
// message in *error for a shape instance without a usable shape.  Point and
// directional emitters
// are skipped, as the reference's emitter tables skip them
// (framework/world/emitter.cpp:314-315).
bool ToPtSceneDesc(const resource::Scene &scene, const pt_camera_desc &camera, PtSceneDesc &out,
                   std::string *error = nullptr);

// One texture (util::Texture, framework/util/texture.h) as pt_texture_desc.
pt_texture_desc ToPtTexture(const util::Texture &t);

}  // namespace Pupil::pt
