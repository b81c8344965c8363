// model.h — one imported model file (glTF or OBJ) before it joins a scene:
// meshes, materials, textures, lights and the node graph that instances the
// meshes; and the Assimp post-processing the reference asks for when it
// imports a model (src/scene/scene.cpp:537-550).
#ifndef PT_HOST_MODEL_H
#define PT_HOST_MODEL_H

#include <cstdint>
#include <vector>

#include "../../../include/pt_scene.h"

namespace pt::host {

struct Mat4 {
    float m[4][4]; // column-major, m[col][row] (the reference's glm::mat4)
    static Mat4 identity()
    {
        Mat4 r{};
        for (int i = 0; i < 4; i++)
            r.m[i][i] = 1.0f;
        return r;
    }
};

// glm-style column-major product, each entry summed left to right.
inline Mat4 mul(const Mat4& a, const Mat4& b)
{
    Mat4 r;
    for (int j = 0; j < 4; j++)
        for (int i = 0; i < 4; i++)
            r.m[j][i] = ((a.m[0][i] * b.m[j][0] + a.m[1][i] * b.m[j][1]) + a.m[2][i] * b.m[j][2]) + a.m[3][i] * b.m[j][3];
    return r;
}

// glm's mat4 * vec4 (type_mat4x4.inl): (m0*x + m1*y) + (m2*z + m3*w) per row.
inline void transform_point(const Mat4& m, const float v[3], float w, float out[3])
{
    for (int i = 0; i < 3; i++)
        out[i] = (m.m[0][i] * v[0] + m.m[1][i] * v[1]) + (m.m[2][i] * v[2] + m.m[3][i] * w);
}

// One texture as the reference's TextureData holds it: 8-bit texels with 1, 2
// or 4 channels (3-channel images widened to 4), srgb only meaningful for 4.
struct HostTexture {
    uint32_t width = 0, height = 0, channels = 0, srgb = 0;
    std::vector<uint8_t> texels;
};

// A node of the model's scene graph: its transform relative to its parent,
// the meshes it instances and its children.  `locked` nodes carry something
// the graph optimisation must keep in place (a light or a camera).
struct ModelNode {
    Mat4 local = Mat4::identity();
    std::vector<uint32_t> meshes;
    std::vector<int> children;
    bool locked = false;
};

struct Model {
    std::vector<float> vertices; // PT_VERTEX_FLOATS each
    std::vector<uint32_t> indices;
    std::vector<pt_mesh_range> meshes;
    std::vector<uint32_t> mesh_material;
    std::vector<std::vector<Mat4>> mesh_instances; // filled from the graph by assimp_postprocess
    std::vector<pt_material> materials;
    std::vector<float> point_lights, dir_lights;
    std::vector<HostTexture> textures;
    std::vector<ModelNode> nodes;
    std::vector<int> roots;
};

// The post-processing of the reference's import flags, in Assimp's order:
// RemoveRedundantMaterials, FindInstances, OptimizeGraph, OptimizeMeshes,
// FindDegenerates, JoinIdenticalVertices; then each mesh's instances are the
// graph's (pre-order, parents before children).  Texture indices of the
// materials that remain are renumbered in first-use order and unused
// textures dropped.  See assimp_post.cpp for what each pass does.
void assimp_postprocess(Model& md);

} // namespace pt::host

#endif
