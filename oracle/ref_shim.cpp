// ref_shim.cpp — C entry points into the reference's own CPU code, for pinning
// the oracle.  TEST INFRASTRUCTURE ONLY: compiled by oracle/Makefile together
// with the reference's sources where they lie (src/rng.cpp, lalgebra.cpp,
// colour.cpp, scene/camera.cpp, scene/lightsample.cpp, scene/material.cpp,
// io/tokenstream.cpp, io/parseutil.cpp, io/imagewrite.cpp for stb_image_write,
// scene/texturedata.cpp for stb_image) into oracle/_ref/libptref.so.  No
// reference source is copied into this repository.
#include <cstring>
#include <vector>

#include "aliastable.h"
#include "colour.h"
#include "io/parseutil.h"
#include "io/tokenstream.h"
#include "lalgebra.h"
#include "rng.h"
#include "scene/camera.h"
#include "scene/lightsample.h"
#include "scene/scene.h"

#include <stb/stb_image.h>
#include <stb/stb_image_write.h>

#include "../include/pt_scene.h"

// Scene grants its friend SceneBuilder access to its members; the reference's
// SceneBuilder (scenebuild.cpp) is not linked here, so this one fills a Scene
// from raw arrays the way read_scene_description would leave it.
class SceneBuilder {
  public:
    static void fill(Scene& s, const pt_raw_scene* raw)
    {
        s.meshes.resize(raw->mesh_count);
        s.object_variants.resize(raw->mesh_count);
        for (uint32_t m = 0; m < raw->mesh_count; m++) {
            const pt_mesh_range& r = raw->meshes[m];
            Mesh& mesh = s.meshes[m];
            mesh.get_vertices().resize(r.vertex_count);
            for (uint32_t v = 0; v < r.vertex_count; v++) {
                const float* f = raw->vertices + (size_t)(r.vertex_offset + v) * PT_VERTEX_FLOATS;
                Vertex& vx = mesh.get_vertices()[v];
                vx.position = Vec3(f[0], f[1], f[2]);
                vx.normal = Vec3(f[3], f[4], f[5]);
                vx.uv = Vec2(f[6], f[7]);
            }
            mesh.get_indexed_triangles().resize(r.tri_count);
            for (uint32_t t = 0; t < r.tri_count; t++)
                for (int k = 0; k < 3; k++)
                    mesh.get_indexed_triangles()[t].indices[k] = raw->indices[r.index_offset + 3 * t + k];
            ObjectVariant& var = s.object_variants[m];
            var.mesh_index = m;
            var.material_index = raw->mesh_material[m];
            for (uint32_t j = raw->mesh_instance_offset[m]; j < raw->mesh_instance_offset[m + 1]; j++) {
                Instance inst;
                std::memcpy(&inst.transform.matrix[0][0], raw->instance_matrices + 16 * (size_t)j, 64);
                var.instances.push_back(inst);
            }
        }
        s.materials.resize(raw->material_count);
        for (uint32_t i = 0; i < raw->material_count; i++)
            std::memcpy((void*)&s.materials[i], &raw->materials[i], sizeof(pt_material));
        for (uint32_t i = 0; i < raw->point_light_count; i++) {
            const float* L = raw->point_lights + 6 * i;
            s.point_lights.push_back(PointLight(Vec3(L[0], L[1], L[2]), Vec3(L[3], L[4], L[5])));
        }
        for (uint32_t i = 0; i < raw->directional_light_count; i++) {
            const float* L = raw->directional_lights + 6 * i;
            s.directional_lights.push_back(DirectionalLight(Vec3(L[0], L[1], L[2]), Vec3(L[3], L[4], L[5])));
        }
        for (uint32_t i = 0; i < raw->texture_count; i++) {
            const pt_texture& t = raw->textures[i];
            VkFormat f = t.channels == 4   ? (t.srgb ? VK_FORMAT_R8G8B8A8_SRGB : VK_FORMAT_R8G8B8A8_UNORM)
                         : t.channels == 2 ? (t.srgb ? VK_FORMAT_R8G8_SRGB : VK_FORMAT_R8G8_UNORM)
                                           : (t.srgb ? VK_FORMAT_R8_SRGB : VK_FORMAT_R8_UNORM);
            s.textures.emplace_back(raw->texels + t.offset, (size_t)t.width * t.height * t.channels, t.width, t.height, f);
        }
    }
};

extern "C" {

void ref_xshiro128_stream(const uint32_t seed4[4], uint32_t n, uint32_t* out_u32, float* out_f32)
{
    Xshiro128 r(seed4[0], seed4[1], seed4[2], seed4[3]);
    Xshiro128 rf(seed4[0], seed4[1], seed4[2], seed4[3]);
    for (uint32_t i = 0; i < n; i++) {
        out_u32[i] = r.next();
        out_f32[i] = rf.next_float();
    }
}

void ref_splitmix32_stream(uint32_t state, uint32_t n, uint32_t* out)
{
    Splitmix32 s(state);
    for (uint32_t i = 0; i < n; i++)
        out[i] = s.next();
}

// Returns the raw bin words of AliasTable<uint32_t> (p, q, alias, value).
void ref_alias_build(const float* weights, uint32_t n, uint32_t* out_words)
{
    std::vector<uint32_t> values(n);
    for (uint32_t i = 0; i < n; i++)
        values[i] = i;
    AliasTable<uint32_t> t(values.data(), weights, n);
    t.copy(out_words);
}

float ref_from_srgb(float x) { return from_srgb(x); }

// Camera chain of scenebuild.cpp:251-264 and pathtrace.cpp:381-396 with
// glm from the reference tree.
void ref_camera_params(const pt_camera_desc* c, uint32_t width, uint32_t height, float inv_view[16], float inv_proj[16])
{
    Vec3 look(c->lookdir[0], c->lookdir[1], c->lookdir[2]);
    Vec3 up(c->up[0], c->up[1], c->up[2]);
    Vec3 x = glm::normalize(look);
    Vec3 y = glm::normalize(glm::cross(up, x));
    Vec3 z = glm::cross(x, y);
    Camera cam(Vec3(c->position[0], c->position[1], c->position[2]), Quaternion(Mat3(y, z, x)), glm::radians(c->fov_degrees),
               1.0, c->near_plane, c->far_plane);
    cam.aspect_ratio = float(width) / height;
    Mat4 view = cam.view_matrix();
    Mat4 proj = cam.projection_matrix();
    Mat4 ip = glm::transpose(glm::inverse(proj));
    Mat4 iv = glm::transpose(glm::inverse(view));
    std::memcpy(inv_view, &iv[0][0], 64);
    std::memcpy(inv_proj, &ip[0][0], 64);
}

// InstanceData transform/normal of scenebuffer.cpp:215-216.
void ref_instance_matrices(const float* m_colmajor, float transform_rowmajor[16], float normal_rows[12])
{
    Mat4 M;
    std::memcpy(&M[0][0], m_colmajor, 64);
    Mat4 t = glm::transpose(M);
    Mat3x4 n = glm::transpose(glm::inverse(t));
    std::memcpy(transform_rowmajor, &t[0][0], 64);
    std::memcpy(normal_rows, &n[0][0], 48);
}

// The light-sampler stream of SceneBuffer::build (scenebuffer.cpp:225-232).
int ref_light_stream(const pt_raw_scene* raw, uint32_t* out, uint32_t cap, uint32_t* light_count)
{
    Scene scene;
    SceneBuilder::fill(scene, raw);
    std::vector<uint32_t> offsets(raw->mesh_count + 1);
    for (uint32_t i = 0; i <= raw->mesh_count; i++)
        offsets[i] = raw->mesh_instance_offset[i];
    size_t words = TableLightSampler::size_in_bytes(scene) / 4;
    if (words > cap)
        return -1;
    TableLightSampler ls(scene, offsets.data());
    size_t n = ls.copy(out) / 4;
    *light_count = (uint32_t)ls.light_count();
    return (int)n;
}

int ref_is_emitter(const pt_material* m)
{
    PbrMaterial pm;
    std::memcpy((void*)&pm, m, sizeof(pt_material));
    return pm.is_emitter() ? 1 : 0;
}

// One `t`/`r`/`s` line of a .scn objects section (parseutil.cpp); returns
// the column-major Mat4.
int ref_parse_transform(const char* line, float out_colmajor[16])
{
    try {
        TokenStream tokens(line, ' ');
        const std::string tok = tokens.next();
        Mat4 m;
        if (tok == "t")
            m = parse_translation(tokens);
        else if (tok == "r")
            m = parse_rotation(tokens);
        else if (tok == "s")
            m = parse_scaling(tokens);
        else
            return -1;
        std::memcpy(out_colmajor, &m[0][0], 64);
        return 0;
    } catch (...) {
        return -2;
    }
}

// A texture image decoded by the reference's stb_image as TextureData loads
// it (texturedata.cpp:64-76): the file's channel count with 3 widened to 4.
// Returns the byte count written (or -1).
int ref_image_decode(const uint8_t* data, int size, uint8_t* out, int cap, int* w, int* h, int* channels)
{
    int x, y, comp;
    if (!stbi_info_from_memory(data, size, &x, &y, &comp))
        return -1;
    const int want = comp == 3 ? 4 : comp;
    unsigned char* px = stbi_load_from_memory(data, size, &x, &y, &comp, want);
    if (!px)
        return -1;
    const int n = x * y * want;
    if (n > cap) {
        stbi_image_free(px);
        return -1;
    }
    std::memcpy(out, px, (size_t)n);
    stbi_image_free(px);
    *w = x;
    *h = y;
    *channels = want;
    return n;
}

namespace {
struct Sink {
    uint8_t* out;
    int cap, n;
};
void sink_write(void* ctx, void* data, int size)
{
    Sink* s = (Sink*)ctx;
    if (s->n + size <= s->cap)
        std::memcpy(s->out + s->n, data, (size_t)size);
    s->n += size;
}
} // namespace

// A JPEG written by the reference's vendored stb_image_write (baseline;
// chroma subsampled 2x2 at quality <= 90).  Returns the byte count (or -1).
int ref_jpeg_encode(const uint8_t* pixels, int w, int h, int comp, int quality, uint8_t* out, int cap)
{
    Sink s{out, cap, 0};
    if (!stbi_write_jpg_to_func(sink_write, &s, w, h, comp, pixels, quality))
        return -1;
    return s.n <= cap ? s.n : -1;
}

} // extern "C"
