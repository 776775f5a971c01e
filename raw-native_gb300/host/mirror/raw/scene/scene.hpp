#pragma once
// The scene the renderer draws (raw/scene/scene.hpp): meshes with one material albedo each,
// directional lights and the camera (aspect, near and far with the reference's defaults).
#include "raw/core/arena_allocator.hpp"
#include "raw/math/mat.hpp"
#include "raw/math/vec.hpp"
#include <vector>
namespace raw {
struct Material { Vec3 albedo{0.8f, 0.8f, 0.8f}; };
struct Mesh {
    std::vector<Vec3, ArenaAllocator<Vec3>> positions, normals;
    std::vector<int, ArenaAllocator<int>> indices;
    Material material;
};
struct Light { Vec3 dir{0, -1, 0}; float intensity{1.0f}; };
struct Camera {
    Vec3 eye{0, 0, 5}, center{0, 0, 0}, up{0, 1, 0};
    float fovy{1.0f}, aspect{1.0f}, nearZ{0.1f}, farZ{100.0f};
};
struct Scene {
    std::vector<Mesh, ArenaAllocator<Mesh>> meshes;
    std::vector<Light, ArenaAllocator<Light>> lights;
    Camera camera;
};
}  // namespace raw
