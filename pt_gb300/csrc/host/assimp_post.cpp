// assimp_post.cpp — the post-processing the reference requests from Assimp
// 5.4.3 for every model file (src/scene/scene.cpp:537-550):
//
//   aiProcess_Triangulate | FlipUVs | GenNormals | JoinIdenticalVertices |
//   RemoveRedundantMaterials | FindDegenerates | FindInvalidData |
//   FindInstances | OptimizeMeshes | OptimizeGraph
//
// Triangulation, the UV flip and generated normals happen in the loaders.
// The passes below change which meshes, materials, vertices, triangles and
// instance transforms reach the packed scene; they run in the order Assimp's
// step registry runs them, each restating the published behaviour of
// Assimp's step (Assimp itself is not part of the reference tree and not
// installed here, so parity with it is unpinned):
//
//   RemoveRedundantMaterials  materials no mesh uses are dropped; a material
//                             equal to an earlier kept one (compared here as
//                             the packed material, Assimp compares a hash of
//                             its properties without the name) is merged
//                             into it; order kept
//   FindInstances             a mesh equal to an earlier one (same material,
//                             vertices and triangles) is replaced by it
//   OptimizeGraph             nodes that are not locked (by a light or camera)
//                             are removed and their children hoisted with
//                             the node's transform folded in (parent *
//                             child); under a locked node (and the root),
//                             childless hoisted nodes whose meshes are used
//                             once are joined into the first of them: their
//                             meshes are moved into its space (vertices by
//                             inverse(first) * node, normals by that
//                             matrix's inverse transpose, winding reversed
//                             for a negative determinant); a root left with
//                             one child is replaced by that child
//   OptimizeMeshes            meshes used more than once keep one mesh each,
//                             placed first in their original order; in every
//                             node (pre-order), each other mesh absorbs the
//                             later meshes of that node with its material
//                             (an absorbed mesh's slot takes the node's last
//                             mesh); the merged mesh holds the absorbed
//                             meshes' vertices and triangles first, its own
//                             last
//   FindDegenerates           (default settings: nothing is removed) a
//                             triangle with two equal vertex positions keeps
//                             fewer indices; the reference stores such faces
//                             as the triangle (0, 0, 0) (process_meshes,
//                             scene.cpp:416-431, default-initialised entries)
//   JoinIdenticalVertices     per mesh, vertices no face uses are dropped and
//                             vertices equal in position, normal and texture
//                             coordinate to an earlier one are replaced by
//                             it, first occurrence in vertex order kept
//
// FindInvalidData's checks are covered by the loaders' validation (non-finite
// positions are refused).
#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <functional>
#include <stdexcept>

#include "model.h"

namespace pt::host {
namespace {

inline uint32_t fbits(float f)
{
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
}
inline float bitsf(uint32_t u)
{
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}

struct MeshData {
    std::vector<float> v; // PT_VERTEX_FLOATS per vertex
    std::vector<std::array<uint32_t, 3>> f;
    std::vector<uint8_t> n; // indices a face keeps (3, or fewer after FindDegenerates)
    uint32_t material = 0;
};

std::vector<MeshData> split(const Model& md)
{
    std::vector<MeshData> out(md.meshes.size());
    for (size_t m = 0; m < md.meshes.size(); m++) {
        const pt_mesh_range& r = md.meshes[m];
        out[m].v.assign(md.vertices.begin() + (size_t)r.vertex_offset * PT_VERTEX_FLOATS,
                        md.vertices.begin() + (size_t)(r.vertex_offset + r.vertex_count) * PT_VERTEX_FLOATS);
        out[m].f.resize(r.tri_count);
        out[m].n.assign(r.tri_count, 3);
        for (uint32_t t = 0; t < r.tri_count; t++)
            for (int k = 0; k < 3; k++)
                out[m].f[t][k] = md.indices[r.index_offset + 3 * t + k];
        out[m].material = md.mesh_material[m];
    }
    return out;
}

void join(Model& md, const std::vector<MeshData>& ms)
{
    md.vertices.clear();
    md.indices.clear();
    md.meshes.clear();
    md.mesh_material.clear();
    for (const MeshData& m : ms) {
        pt_mesh_range r;
        r.vertex_offset = (uint32_t)(md.vertices.size() / PT_VERTEX_FLOATS);
        r.index_offset = (uint32_t)md.indices.size();
        r.vertex_count = (uint32_t)(m.v.size() / PT_VERTEX_FLOATS);
        r.tri_count = (uint32_t)m.f.size();
        md.vertices.insert(md.vertices.end(), m.v.begin(), m.v.end());
        for (size_t t = 0; t < m.f.size(); t++)
            for (int k = 0; k < 3; k++)
                md.indices.push_back(m.n[t] == 3 ? m.f[t][k] : 0u); // a degenerate face becomes (0, 0, 0)
        md.meshes.push_back(r);
        md.mesh_material.push_back(m.material);
    }
}

// ---------------------------------------------------------------- materials
void remove_redundant_materials(Model& md, std::vector<MeshData>& ms)
{
    const size_t n = md.materials.size();
    std::vector<char> used(n, 0);
    for (const MeshData& m : ms)
        used[m.material] = 1;
    std::vector<uint32_t> map(n, 0);
    std::vector<pt_material> kept;
    std::vector<size_t> kept_from;
    for (size_t i = 0; i < n; i++) {
        if (!used[i])
            continue;
        bool merged = false;
        for (size_t k = 0; k < kept.size(); k++)
            if (std::memcmp(&kept[k], &md.materials[i], sizeof(pt_material)) == 0) {
                map[i] = (uint32_t)k;
                merged = true;
                break;
            }
        if (!merged) {
            map[i] = (uint32_t)kept.size();
            kept.push_back(md.materials[i]);
            kept_from.push_back(i);
        }
    }
    for (MeshData& m : ms)
        m.material = map[m.material];
    md.materials = kept;
}

// The texture slots a material names, in the order the loaders (and the
// reference's material extraction, scene.cpp:358-383) look them up.
void for_each_map(pt_material& pm, const std::function<void(float&, bool srgb)>& fn)
{
    const uint32_t bits = fbits(pm.rough_metal_normal_map_bits[3]);
    if (bits & PT_BASE_COLOUR_MAP_BIT)
        fn(pm.base_colour[0], true);
    if (bits & PT_EMISSION_MAP_BIT)
        fn(pm.emission[0], true);
    if (bits & (PT_ROUGHNESS_MAP_BIT | PT_ROUGHNESS_METALNESS_MAP_BIT))
        fn(pm.rough_metal_normal_map_bits[0], false);
    if (bits & PT_METALNESS_MAP_BIT)
        fn(pm.rough_metal_normal_map_bits[1], false);
    if (bits & PT_NORMAL_MAP_BIT)
        fn(pm.rough_metal_normal_map_bits[2], false);
    if (bits & PT_SPECULAR_MAP_BIT)
        fn(pm.specular[0], false);
    if (bits & PT_SHEEN_MAP_BIT)
        fn(pm.sheen[0], false);
    if (bits & PT_CLEARCOAT_MAP_BIT)
        fn(pm.cc_ccrgh_aniso[0], false);
}

// Textures in first-use order over the remaining materials (the reference
// numbers them while extracting the post-processed materials, scene.cpp:50-72);
// the first use decides sRGB (4-channel base colour or emission maps).
void renumber_textures(Model& md)
{
    std::vector<int64_t> map(md.textures.size(), -1);
    std::vector<HostTexture> out;
    for (pt_material& pm : md.materials)
        for_each_map(pm, [&](float& slot, bool srgb) {
            const uint32_t old = fbits(slot);
            if (old >= md.textures.size())
                throw std::runtime_error("material names a missing texture");
            if (map[old] < 0) {
                map[old] = (int64_t)out.size();
                out.push_back(md.textures[old]);
                out.back().srgb = (srgb && out.back().channels == 4) ? 1u : 0u;
            }
            slot = bitsf((uint32_t)map[old]);
        });
    md.textures.swap(out);
}

// ---------------------------------------------------------------- instances
bool same_mesh(const MeshData& a, const MeshData& b)
{
    return a.material == b.material && a.v.size() == b.v.size() && a.f == b.f && a.n == b.n &&
           std::equal(a.v.begin(), a.v.end(), b.v.begin(), [](float x, float y) { return fbits(x) == fbits(y); });
}

void find_instances(Model& md, std::vector<MeshData>& ms)
{
    std::vector<uint32_t> map(ms.size());
    std::vector<MeshData> out;
    for (size_t i = 0; i < ms.size(); i++) {
        size_t j = 0;
        for (; j < out.size(); j++)
            if (same_mesh(out[j], ms[i]))
                break;
        if (j == out.size())
            out.push_back(ms[i]);
        map[i] = (uint32_t)j;
    }
    for (ModelNode& nd : md.nodes)
        for (uint32_t& m : nd.meshes)
            m = map[m];
    ms.swap(out);
}

// ---------------------------------------------------------------- graph
Mat4 inverse(const Mat4& a)
{
    // cofactor expansion in double, rounded once
    double m[16], inv[16];
    for (int c = 0; c < 4; c++)
        for (int r = 0; r < 4; r++)
            m[c * 4 + r] = a.m[c][r];
    inv[0] = m[5] * m[10] * m[15] - m[5] * m[11] * m[14] - m[9] * m[6] * m[15] + m[9] * m[7] * m[14] + m[13] * m[6] * m[11] - m[13] * m[7] * m[10];
    inv[4] = -m[4] * m[10] * m[15] + m[4] * m[11] * m[14] + m[8] * m[6] * m[15] - m[8] * m[7] * m[14] - m[12] * m[6] * m[11] + m[12] * m[7] * m[10];
    inv[8] = m[4] * m[9] * m[15] - m[4] * m[11] * m[13] - m[8] * m[5] * m[15] + m[8] * m[7] * m[13] + m[12] * m[5] * m[11] - m[12] * m[7] * m[9];
    inv[12] = -m[4] * m[9] * m[14] + m[4] * m[10] * m[13] + m[8] * m[5] * m[14] - m[8] * m[6] * m[13] - m[12] * m[5] * m[10] + m[12] * m[6] * m[9];
    inv[1] = -m[1] * m[10] * m[15] + m[1] * m[11] * m[14] + m[9] * m[2] * m[15] - m[9] * m[3] * m[14] - m[13] * m[2] * m[11] + m[13] * m[3] * m[10];
    inv[5] = m[0] * m[10] * m[15] - m[0] * m[11] * m[14] - m[8] * m[2] * m[15] + m[8] * m[3] * m[14] + m[12] * m[2] * m[11] - m[12] * m[3] * m[10];
    inv[9] = -m[0] * m[9] * m[15] + m[0] * m[11] * m[13] + m[8] * m[1] * m[15] - m[8] * m[3] * m[13] - m[12] * m[1] * m[11] + m[12] * m[3] * m[9];
    inv[13] = m[0] * m[9] * m[14] - m[0] * m[10] * m[13] - m[8] * m[1] * m[14] + m[8] * m[2] * m[13] + m[12] * m[1] * m[10] - m[12] * m[2] * m[9];
    inv[2] = m[1] * m[6] * m[15] - m[1] * m[7] * m[14] - m[5] * m[2] * m[15] + m[5] * m[3] * m[14] + m[13] * m[2] * m[7] - m[13] * m[3] * m[6];
    inv[6] = -m[0] * m[6] * m[15] + m[0] * m[7] * m[14] + m[4] * m[2] * m[15] - m[4] * m[3] * m[14] - m[12] * m[2] * m[7] + m[12] * m[3] * m[6];
    inv[10] = m[0] * m[5] * m[15] - m[0] * m[7] * m[13] - m[4] * m[1] * m[15] + m[4] * m[3] * m[13] + m[12] * m[1] * m[7] - m[12] * m[3] * m[5];
    inv[14] = -m[0] * m[5] * m[14] + m[0] * m[6] * m[13] + m[4] * m[1] * m[14] - m[4] * m[2] * m[13] - m[12] * m[1] * m[6] + m[12] * m[2] * m[5];
    inv[3] = -m[1] * m[6] * m[11] + m[1] * m[7] * m[10] + m[5] * m[2] * m[11] - m[5] * m[3] * m[10] - m[9] * m[2] * m[7] + m[9] * m[3] * m[6];
    inv[7] = m[0] * m[6] * m[11] - m[0] * m[7] * m[10] - m[4] * m[2] * m[11] + m[4] * m[3] * m[10] + m[8] * m[2] * m[7] - m[8] * m[3] * m[6];
    inv[11] = -m[0] * m[5] * m[11] + m[0] * m[7] * m[9] + m[4] * m[1] * m[11] - m[4] * m[3] * m[9] - m[8] * m[1] * m[7] + m[8] * m[3] * m[5];
    inv[15] = m[0] * m[5] * m[10] - m[0] * m[6] * m[9] - m[4] * m[1] * m[10] + m[4] * m[2] * m[9] + m[8] * m[1] * m[6] - m[8] * m[2] * m[5];
    const double det = m[0] * inv[0] + m[1] * inv[4] + m[2] * inv[8] + m[3] * inv[12];
    if (det == 0.0 || !std::isfinite(det))
        throw std::runtime_error("a node transform cannot be inverted");
    Mat4 r;
    for (int c = 0; c < 4; c++)
        for (int rr = 0; rr < 4; rr++)
            r.m[c][rr] = (float)(inv[c * 4 + rr] / det);
    return r;
}

double det3(const Mat4& a)
{
    const double m00 = a.m[0][0], m01 = a.m[1][0], m02 = a.m[2][0];
    const double m10 = a.m[0][1], m11 = a.m[1][1], m12 = a.m[2][1];
    const double m20 = a.m[0][2], m21 = a.m[1][2], m22 = a.m[2][2];
    return m00 * (m11 * m22 - m12 * m21) - m01 * (m10 * m22 - m12 * m20) + m02 * (m10 * m21 - m11 * m20);
}

// Moves a mesh into the space of `t` (OptimizeGraph's join).
void transform_mesh(MeshData& mesh, const Mat4& t)
{
    const double det = det3(t);
    // inverse transpose of the upper 3x3, in double, rounded once
    const double a = t.m[0][0], b = t.m[1][0], c = t.m[2][0], d = t.m[0][1], e = t.m[1][1], f = t.m[2][1], g = t.m[0][2],
                 h = t.m[1][2], i = t.m[2][2];
    float it[3][3] = {{(float)((e * i - f * h) / det), (float)((f * g - d * i) / det), (float)((d * h - e * g) / det)},
                      {(float)((c * h - b * i) / det), (float)((a * i - c * g) / det), (float)((b * g - a * h) / det)},
                      {(float)((b * f - c * e) / det), (float)((c * d - a * f) / det), (float)((a * e - b * d) / det)}};
    for (size_t k = 0; k + PT_VERTEX_FLOATS <= mesh.v.size(); k += PT_VERTEX_FLOATS) {
        float* v = &mesh.v[k];
        const float x = v[0], y = v[1], z = v[2];
        for (int r = 0; r < 3; r++)
            v[r] = ((t.m[0][r] * x + t.m[1][r] * y) + t.m[2][r] * z) + t.m[3][r];
        const float nx = v[3], ny = v[4], nz = v[5];
        for (int r = 0; r < 3; r++)
            v[3 + r] = (it[r][0] * nx + it[r][1] * ny) + it[r][2] * nz;
    }
    if (det < 0.0)
        for (auto& face : mesh.f)
            std::swap(face[0], face[2]);
}

// Mesh references of the nodes reachable from the roots.
std::vector<uint32_t> mesh_uses(const Model& md, size_t mesh_count)
{
    std::vector<uint32_t> uses(mesh_count, 0);
    std::function<void(int)> visit = [&](int ni) {
        for (uint32_t m : md.nodes[(size_t)ni].meshes)
            uses[m]++;
        for (int c : md.nodes[(size_t)ni].children)
            visit(c);
    };
    for (int r : md.roots)
        visit(r);
    return uses;
}

struct GraphOptimizer {
    Model& md;
    std::vector<MeshData>& ms;
    std::vector<uint32_t> uses;

    std::vector<int> collect(int nd)
    {
        std::vector<int> child_nodes;
        for (int c : md.nodes[(size_t)nd].children) {
            std::vector<int> sub = collect(c);
            child_nodes.insert(child_nodes.end(), sub.begin(), sub.end());
        }
        ModelNode& node = md.nodes[(size_t)nd];
        std::vector<int> out;
        if (!node.locked) {
            std::vector<int> kept;
            for (int c : child_nodes) {
                ModelNode& ch = md.nodes[(size_t)c];
                if (!ch.locked) {
                    ch.local = mul(node.local, ch.local);
                    out.push_back(c);
                } else {
                    kept.push_back(c);
                }
            }
            node.children = kept;
            if (!node.meshes.empty() || !kept.empty())
                out.push_back(nd);
            return out;
        }
        int master = -1;
        Mat4 inv = Mat4::identity();
        std::vector<int> remaining, joined;
        for (int c : child_nodes) {
            ModelNode& ch = md.nodes[(size_t)c];
            bool joinable = ch.children.empty() && !ch.locked;
            for (uint32_t m : ch.meshes)
                joinable = joinable && uses[m] <= 1;
            if (joinable) {
                if (master < 0) {
                    master = c;
                    inv = inverse(ch.local);
                } else {
                    ch.local = mul(inv, ch.local);
                    joined.push_back(c);
                    continue;
                }
            }
            remaining.push_back(c);
        }
        if (master >= 0)
            for (int c : joined) {
                for (uint32_t m : md.nodes[(size_t)c].meshes) {
                    transform_mesh(ms[m], md.nodes[(size_t)c].local);
                    md.nodes[(size_t)master].meshes.push_back(m);
                }
                md.nodes[(size_t)c].meshes.clear(); // the node leaves the graph
            }
        node.children = remaining;
        return {nd};
    }

    void run()
    {
        uses = mesh_uses(md, ms.size());
        ModelNode root;
        root.locked = true;
        root.children = md.roots;
        md.nodes.push_back(root);
        const int r = (int)md.nodes.size() - 1;
        collect(r);
        if (md.nodes[(size_t)r].children.size() == 1 && md.nodes[(size_t)r].meshes.empty())
            md.roots = {md.nodes[(size_t)r].children[0]};
        else
            md.roots = {r};
    }
};

// ---------------------------------------------------------------- meshes
void optimize_meshes(Model& md, std::vector<MeshData>& ms)
{
    const std::vector<uint32_t> uses = mesh_uses(md, ms.size());
    std::vector<MeshData> out;
    std::vector<int64_t> out_id(ms.size(), -1);
    for (size_t m = 0; m < ms.size(); m++)
        if (uses[m] > 1) {
            out_id[m] = (int64_t)out.size();
            out.push_back(ms[m]);
        }
    std::function<void(int)> process = [&](int ni) {
        ModelNode& nd = md.nodes[(size_t)ni];
        for (size_t i = 0; i < nd.meshes.size(); i++) {
            const uint32_t im = nd.meshes[i];
            if (uses[im] > 1) {
                nd.meshes[i] = (uint32_t)out_id[im];
                continue;
            }
            std::vector<uint32_t> merge;
            for (size_t a = i + 1; a < nd.meshes.size();) {
                const uint32_t am = nd.meshes[a];
                if (uses[am] == 1 && ms[am].material == ms[im].material) {
                    merge.push_back(am);
                    nd.meshes[a] = nd.meshes.back();
                    nd.meshes.pop_back();
                } else {
                    a++;
                }
            }
            MeshData mesh;
            if (merge.empty()) {
                mesh = ms[im];
            } else {
                merge.push_back(im);
                mesh.material = ms[im].material;
                for (uint32_t m : merge) {
                    const uint32_t base = (uint32_t)(mesh.v.size() / PT_VERTEX_FLOATS);
                    mesh.v.insert(mesh.v.end(), ms[m].v.begin(), ms[m].v.end());
                    for (size_t t = 0; t < ms[m].f.size(); t++) {
                        mesh.f.push_back({ms[m].f[t][0] + base, ms[m].f[t][1] + base, ms[m].f[t][2] + base});
                        mesh.n.push_back(ms[m].n[t]);
                    }
                }
            }
            out.push_back(std::move(mesh));
            nd.meshes[i] = (uint32_t)(out.size() - 1);
        }
        for (int c : nd.children)
            process(c);
    };
    for (int r : md.roots)
        process(r);
    ms.swap(out);
}

// ---------------------------------------------------------------- faces, vertices
void find_degenerates(std::vector<MeshData>& ms)
{
    for (MeshData& m : ms)
        for (size_t t = 0; t < m.f.size(); t++) {
            std::array<uint32_t, 3>& face = m.f[t];
            int n = 3;
            for (int i = 0; i < n; i++)
                for (int k = i + 1; k < n; k++) {
                    const float* a = &m.v[(size_t)face[i] * PT_VERTEX_FLOATS];
                    const float* b = &m.v[(size_t)face[k] * PT_VERTEX_FLOATS];
                    if (a[0] == b[0] && a[1] == b[1] && a[2] == b[2]) {
                        for (int s = k; s + 1 < n; s++)
                            face[s] = face[s + 1];
                        n--;
                        k--;
                    }
                }
            m.n[t] = (uint8_t)n;
        }
}

void join_identical_vertices(std::vector<MeshData>& ms)
{
    for (MeshData& m : ms) {
        const size_t nv = m.v.size() / PT_VERTEX_FLOATS;
        std::vector<char> used(nv, 0);
        for (size_t t = 0; t < m.f.size(); t++)
            for (int k = 0; k < m.n[t]; k++)
                used[m.f[t][k]] = 1;
        std::vector<uint32_t> map(nv, 0);
        std::vector<float> out;
        // hash on the 8 attribute words (+0 and -0 hash alike; equality is float ==)
        std::vector<std::vector<uint32_t>> buckets(std::max<size_t>(16, nv * 2));
        auto key = [](const float* v) {
            uint64_t h = 1469598103934665603ull;
            for (int k = 0; k < PT_VERTEX_FLOATS; k++) {
                const uint32_t u = v[k] == 0.0f ? 0u : fbits(v[k]);
                h = (h ^ u) * 1099511628211ull;
            }
            return h;
        };
        for (size_t i = 0; i < nv; i++) {
            if (!used[i])
                continue;
            const float* v = &m.v[i * PT_VERTEX_FLOATS];
            std::vector<uint32_t>& bucket = buckets[key(v) % buckets.size()];
            bool found = false;
            for (uint32_t u : bucket) {
                const float* w = &out[(size_t)u * PT_VERTEX_FLOATS];
                bool eq = true;
                for (int k = 0; k < PT_VERTEX_FLOATS && eq; k++)
                    eq = v[k] == w[k];
                if (eq) {
                    map[i] = u;
                    found = true;
                    break;
                }
            }
            if (!found) {
                const uint32_t u = (uint32_t)(out.size() / PT_VERTEX_FLOATS);
                out.insert(out.end(), v, v + PT_VERTEX_FLOATS);
                bucket.push_back(u);
                map[i] = u;
            }
        }
        for (size_t t = 0; t < m.f.size(); t++)
            for (int k = 0; k < m.n[t]; k++)
                m.f[t][k] = map[m.f[t][k]];
        m.v.swap(out);
    }
}

void instances_from_graph(Model& md)
{
    md.mesh_instances.assign(md.meshes.size(), {});
    std::function<void(int, const Mat4&)> visit = [&](int ni, const Mat4& parent) {
        const ModelNode& nd = md.nodes[(size_t)ni];
        const Mat4 M = mul(parent, nd.local);
        for (uint32_t m : nd.meshes)
            md.mesh_instances[m].push_back(M);
        for (int c : nd.children)
            visit(c, M);
    };
    for (int r : md.roots)
        visit(r, Mat4::identity());
}

} // namespace

void assimp_postprocess(Model& md)
{
    std::vector<MeshData> ms = split(md);
    const size_t materials_before = md.materials.size();
    remove_redundant_materials(md, ms);
    if (md.materials.size() != materials_before)
        renumber_textures(md);
    find_instances(md, ms);
    GraphOptimizer{md, ms, {}}.run();
    optimize_meshes(md, ms);
    find_degenerates(ms);
    join_identical_vertices(ms);
    join(md, ms);
    instances_from_graph(md);
}

} // namespace pt::host
