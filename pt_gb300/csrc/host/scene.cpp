// scene.cpp — host-side scene front end of libptgpu.so (include/pt_scene.h).
//
// Restates the reference's CPU scene path:
//   .scn parsing            src/scene/scenebuild.cpp:132-365, src/io/parseutil.cpp,
//                           src/io/tokenstream.cpp, src/io/ioutil.cpp
//   transforms              src/lalgebra.cpp:5-94
//   model import (glTF 2.0, src/scene/scene.cpp:74-488 (the reference imports
//   and Wavefront OBJ)      through Assimp 5.4.3, absent here; see the notes
//                           at load_gltf and load_obj for the Assimp behaviour
//                           reproduced)
//   packing                 src/scene/scenebuffer.cpp:65-168
//   light-sampler tables    src/scene/lightsample.cpp:5-221, src/aliastable.h:21-67
//   camera matrices         src/scene/camera.h:16, camera.cpp:21-26,
//                           scenebuild.cpp:251-264, pathtrace.cpp:381-396
//   image output            src/io/imagewrite.cpp:19-67
#include <algorithm>
#include <array>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <functional>
#include <limits>
#include <numeric>
#include <optional>
#include <sstream>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../../include/pt_scene.h"
#include "jpeg.h"
#include "model.h"
#include "json.h"
#include "png.h"

using pth::Json;
using pt::host::HostTexture;
using pt::host::Mat4;
using pt::host::Model;
using pt::host::ModelNode;
using pt::host::mul;
using pt::host::transform_point;

namespace {

thread_local std::string g_error;

// lalgebra.cpp:5-14
Mat4 translation(float x, float y, float z)
{
    Mat4 r = Mat4::identity();
    r.m[3][0] = x;
    r.m[3][1] = y;
    r.m[3][2] = z;
    return r;
}

// lalgebra.cpp:16-55: identity for angle < 1e-5 (negative angles too).
Mat4 rotation(float ux, float uy, float uz, float angle)
{
    if (angle < 1e-5)
        return Mat4::identity();
    float len = std::sqrt((ux * ux + uy * uy) + uz * uz);
    if (len < 1e-5)
        throw std::runtime_error("Rotation axis was (close to) zero");
    float inv = 1.0f / len;
    ux *= inv;
    uy *= inv;
    uz *= inv;
    float c = std::cos(angle);
    float s = std::sin(angle);
    Mat4 r{};
    r.m[0][0] = ux * ux + (1 - ux * ux) * c;
    r.m[0][1] = uy * ux * (1 - c) + uz * s;
    r.m[0][2] = uz * ux * (1 - c) - uy * s;
    r.m[1][0] = ux * uy * (1 - c) - uz * s;
    r.m[1][1] = uy * uy + (1 - uy * uy) * c;
    r.m[1][2] = uz * uy * (1 - c) + ux * s;
    r.m[2][0] = ux * uz * (1 - c) + uy * s;
    r.m[2][1] = uy * uz * (1 - c) - ux * s;
    r.m[2][2] = uz * uz + (1 - uz * uz) * c;
    r.m[3][3] = 1;
    return r;
}

Mat4 scaling(float x, float y, float z)
{
    Mat4 r{};
    r.m[0][0] = x;
    r.m[1][1] = y;
    r.m[2][2] = z;
    r.m[3][3] = 1;
    return r;
}

// colour.cpp:12-14: double arithmetic, float result.
float from_srgb(float x) { return (float)((x <= 0.04045) ? (x / 12.92) : std::pow((x + 0.055) / 1.055, 2.4)); }

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

// ---------------------------------------------------------------- tokens (tokenstream.cpp)
std::vector<std::string> split(const std::string& raw, char delim)
{
    std::vector<std::string> out;
    std::string cur;
    for (char c : raw) {
        if (c == delim) {
            if (!cur.empty())
                out.push_back(cur);
            cur.clear();
        } else {
            cur += c;
        }
    }
    if (!cur.empty())
        out.push_back(cur);
    return out;
}

struct Tokens {
    std::vector<std::string> t;
    size_t i = 0;
    Tokens(const std::string& raw, char d) : t(split(raw, d)) {}
    bool done() const { return i >= t.size(); }
    size_t remaining() const { return t.size() - i; }
    const std::string& next()
    {
        if (done())
            throw std::runtime_error("Token stream has no next token");
        return t[i++];
    }
    void rollback(size_t n)
    {
        if (i < n)
            throw std::runtime_error("Cannot roll further back than the start");
        i -= n;
    }
};

float to_float(const std::string& s) { return std::stof(s); }

void parse_vec3(Tokens& tk, float out[3])
{
    if (tk.remaining() < 3)
        throw std::runtime_error("Vectors need three components");
    for (int k = 0; k < 3; k++)
        out[k] = to_float(tk.next());
}

std::string read_file(const std::string& path)
{
    std::ifstream f(path, std::ios::binary);
    if (!f)
        throw std::runtime_error("Could not open file " + path);
    std::stringstream ss;
    ss << f.rdbuf();
    return ss.str();
}

std::string directory_of(const std::string& file)
{
    size_t i = file.find_last_of("\\/");
    return i == std::string::npos ? "" : file.substr(0, i + 1);
}

// ---------------------------------------------------------------- loaded model
// TextureData::has_alpha_less_than_one (texturedata.cpp:150-164).
bool has_alpha_below_one(const HostTexture& t)
{
    if (t.channels != 4)
        return false;
    for (size_t i = 0; i < (size_t)t.width * t.height; i++)
        if (t.texels[4 * i + 3] < 255)
            return true;
    return false;
}

// An encoded texture image as TextureData keeps it (texturedata.cpp:30-48:
// the file's channel count with 3 widened to 4; sRGB only for 4 channels).
// PNG and baseline JPEG; other formats are rejected.
HostTexture decode_texture(const std::vector<uint8_t>& bytes, const std::string& what, bool srgb)
{
    if (bytes.size() >= 3 && bytes[0] == 0xFF && bytes[1] == 0xD8 && bytes[2] == 0xFF) {
        pt::host::JpegImage jpg;
        std::string err;
        if (!pt::host::jpeg_decode(bytes.data(), bytes.size(), jpg, err))
            throw std::runtime_error("Failed to read texture " + what + ": " + err);
        HostTexture ht;
        ht.width = jpg.width;
        ht.height = jpg.height;
        ht.channels = jpg.channels;
        ht.srgb = (jpg.channels == 4 && srgb) ? 1u : 0u;
        ht.texels = std::move(jpg.texels);
        return ht;
    }
    pt::host::PngImage png;
    std::string err;
    if (!pt::host::png_decode(bytes.data(), bytes.size(), png, err))
        throw std::runtime_error("Failed to read texture " + what + ": " + err);
    HostTexture ht;
    ht.width = png.width;
    ht.height = png.height;
    ht.channels = png.channels;
    ht.srgb = (png.channels == 4 && srgb) ? 1u : 0u;
    ht.texels = std::move(png.texels);
    return ht;
}

// has_transparency (scene.cpp:344-355): a base-colour map with alpha below
// one, or a base-colour alpha (opacity) below one.
void mark_transparency(Model& md)
{
    for (pt_material& pm : md.materials) {
        uint32_t bits = fbits(pm.rough_metal_normal_map_bits[3]);
        bool transparent = (bits & PT_BASE_COLOUR_MAP_BIT) ? has_alpha_below_one(md.textures[fbits(pm.base_colour[0])])
                                                            : pm.base_colour[3] < 1.0f;
        if (transparent)
            pm.rough_metal_normal_map_bits[3] = bitsf(bits | PT_MATERIAL_IS_TRANSPARENT_BIT);
    }
}

std::vector<uint8_t> decode_base64(const std::string& s)
{
    auto val = [](char c) -> int {
        if (c >= 'A' && c <= 'Z')
            return c - 'A';
        if (c >= 'a' && c <= 'z')
            return c - 'a' + 26;
        if (c >= '0' && c <= '9')
            return c - '0' + 52;
        if (c == '+')
            return 62;
        if (c == '/')
            return 63;
        return -1;
    };
    std::vector<uint8_t> out;
    uint32_t acc = 0;
    int bits = 0;
    for (char c : s) {
        int v = val(c);
        if (v < 0)
            continue;
        acc = (acc << 6) | (uint32_t)v;
        bits += 6;
        if (bits >= 8) {
            bits -= 8;
            out.push_back((uint8_t)((acc >> bits) & 0xFF));
        }
    }
    return out;
}

struct Accessor {
    const uint8_t* data = nullptr;
    size_t count = 0, stride = 0;
    int comp = 0, ncomp = 0;
    bool normalized = false;
    double get(size_t i, int c) const
    {
        const uint8_t* p = data + i * stride;
        switch (comp) {
        case 5126: {
            float f;
            std::memcpy(&f, p + 4 * c, 4);
            return f;
        }
        case 5125: {
            uint32_t u;
            std::memcpy(&u, p + 4 * c, 4);
            return u;
        }
        case 5123: {
            uint16_t u;
            std::memcpy(&u, p + 2 * c, 2);
            return normalized ? u / 65535.0 : u;
        }
        case 5121: return normalized ? p[c] / 255.0 : p[c];
        case 5122: {
            int16_t v;
            std::memcpy(&v, p + 2 * c, 2);
            return normalized ? std::max(v / 32767.0, -1.0) : v;
        }
        case 5120: {
            int8_t v = (int8_t)p[c];
            return normalized ? std::max(v / 127.0, -1.0) : v;
        }
        }
        return 0.0;
    }
};

// The binary glTF container (.glb, glTF 2.0 section 4.4): a 12-byte header
// (magic "glTF", version 2, total length) and chunks of (length, type, data),
// the JSON chunk first and an optional BIN chunk that buffer 0 refers to when
// it has no uri.  Returns false when `file` is not a .glb.
bool split_glb(const std::string& file, std::string& json, std::vector<uint8_t>& bin, bool& has_bin)
{
    if (file.size() < 12 || std::memcmp(file.data(), "glTF", 4) != 0)
        return false;
    uint32_t version, length;
    std::memcpy(&version, file.data() + 4, 4);
    std::memcpy(&length, file.data() + 8, 4);
    if (version != 2)
        throw std::runtime_error("unsupported .glb version " + std::to_string(version));
    if (length > file.size() || length < 12)
        throw std::runtime_error(".glb shorter than its header says");
    has_bin = false;
    bool has_json = false;
    size_t off = 12;
    while (off + 8 <= length) {
        uint32_t clen, ctype;
        std::memcpy(&clen, file.data() + off, 4);
        std::memcpy(&ctype, file.data() + off + 4, 4);
        if ((uint64_t)off + 8 + clen > length)
            throw std::runtime_error(".glb chunk runs past the end of the file");
        if (ctype == 0x4E4F534Au && !has_json) {
            json.assign(file.data() + off + 8, clen);
            has_json = true;
        } else if (ctype == 0x004E4942u && !has_bin) {
            bin.assign(file.begin() + off + 8, file.begin() + off + 8 + clen);
            has_bin = true;
        }
        off += 8 + (size_t)clen;
    }
    if (!has_json)
        throw std::runtime_error(".glb without a JSON chunk");
    return true;
}

// glTF 2.0 import with the Assimp behaviour the reference relies on
// (scene.cpp:537-550 import flags, :74-296 material extraction):
//  - every mesh primitive becomes one mesh with one material (variant);
//  - node transforms are composed root to leaf (process_scene_node, :476-488);
//  - texture coordinates: Assimp's glTF importer flips v and aiProcess_FlipUVs
//    flips it back, so v is stored as 1 - (1 - v) in float;
//  - base colour and emission factors are sRGB-decoded (:94, :134);
//  - metallic/roughness come from the glTF factors (glTF defaults 1/1 when
//    absent, as Assimp reports them); specular defaults to 0.5 (:227),
//    sheen to 0, clearcoat 0 with roughness 0.5, anisotropy 0 (:263-295);
//  - KHR_materials_emissive_strength gives the emission strength (:140-143);
//  - KHR_materials_transmission gives opacity = 1 - transmission (:96-108).
// Textures: PNG and baseline JPEG images (files, data URIs or buffer views).
// Cameras inside glTF files are not imported: the reference hands the model
// import a dummy camera and keeps the .scn one (scenebuild.cpp:306-317).
// KHR_lights_punctual point and directional lights are (see below).
Model load_gltf(const std::string& path)
{
    std::string text = read_file(path);
    std::string glb_json;
    std::vector<uint8_t> glb_bin;
    bool has_glb_bin = false;
    if (split_glb(text, glb_json, glb_bin, has_glb_bin))
        text.swap(glb_json);
    Json doc = pth::JsonParser(text).parse();
    std::string dir = directory_of(path);
    std::vector<std::vector<uint8_t>> buffers;
    for (size_t b = 0; b < doc["buffers"].size(); b++) {
        const Json& jb = doc["buffers"][b];
        if (!jb.has("uri")) {
            if (b != 0 || !has_glb_bin)
                throw std::runtime_error("buffer " + std::to_string(b) + " has no uri and no .glb BIN chunk");
            buffers.push_back(glb_bin);
            if ((int64_t)buffers.back().size() < jb["byteLength"].integer(0))
                throw std::runtime_error("buffer 0 shorter than its byteLength");
            continue;
        }
        std::string uri = jb["uri"].str;
        if (uri.rfind("data:", 0) == 0) {
            size_t comma = uri.find(',');
            buffers.push_back(decode_base64(comma == std::string::npos ? "" : uri.substr(comma + 1)));
        } else {
            std::string bin = read_file(dir + uri);
            buffers.emplace_back(bin.begin(), bin.end());
        }
        if ((int64_t)buffers.back().size() < jb["byteLength"].integer(0))
            throw std::runtime_error("buffer " + std::to_string(b) + " shorter than its byteLength");
    }
    auto accessor = [&](int64_t idx) -> Accessor {
        const Json& a = doc["accessors"][(size_t)idx];
        if (a.kind != Json::OBJ)
            throw std::runtime_error("missing accessor " + std::to_string(idx));
        Accessor r;
        r.count = (size_t)a["count"].integer(0);
        r.comp = (int)a["componentType"].integer(0);
        r.normalized = a["normalized"].kind == Json::BOOL && a["normalized"].b;
        const std::string& type = a["type"].str;
        r.ncomp = type == "SCALAR" ? 1 : type == "VEC2" ? 2 : type == "VEC3" ? 3 : type == "VEC4" ? 4 : 0;
        int csize = (r.comp == 5126 || r.comp == 5125) ? 4 : (r.comp == 5123 || r.comp == 5122) ? 2 : 1;
        if (r.ncomp == 0)
            throw std::runtime_error("unsupported accessor type " + type);
        const Json& bv = doc["bufferViews"][(size_t)a["bufferView"].integer(-1)];
        if (bv.kind != Json::OBJ)
            throw std::runtime_error("accessor without a buffer view");
        size_t buf = (size_t)bv["buffer"].integer(0);
        if (buf >= buffers.size())
            throw std::runtime_error("buffer view names a missing buffer");
        size_t off = (size_t)bv["byteOffset"].integer(0) + (size_t)a["byteOffset"].integer(0);
        r.stride = (size_t)bv["byteStride"].integer(0);
        if (r.stride == 0)
            r.stride = (size_t)csize * r.ncomp;
        size_t need = r.count == 0 ? 0 : off + (r.count - 1) * r.stride + (size_t)csize * r.ncomp;
        if (need > buffers[buf].size())
            throw std::runtime_error("accessor outside its buffer");
        r.data = buffers[buf].data() + off;
        return r;
    };

    Model md;
    // Textures get an index per image in first-use order over the materials
    // (process_texture, scene.cpp:50-72), keyed by the image path (embedded
    // images by "*n"); the type of the first use decides sRGB (:42-48).
    struct TexSource {
        int64_t image;
        bool srgb;
    };
    std::unordered_map<std::string, uint32_t> tex_index;
    std::vector<TexSource> tex_src;
    auto texture = [&](const Json& info, bool srgb) -> int64_t {
        if (info.kind != Json::OBJ)
            return -1;
        const Json& t = doc["textures"][(size_t)info["index"].integer(-1)];
        if (t.kind != Json::OBJ)
            throw std::runtime_error("material names a missing texture");
        const int64_t img = t["source"].integer(-1);
        const Json& im = doc["images"][(size_t)img];
        if (im.kind != Json::OBJ)
            throw std::runtime_error("texture without an image");
        const bool external = im.has("uri") && im["uri"].str.rfind("data:", 0) != 0;
        const std::string key = external ? im["uri"].str : "*" + std::to_string(img);
        auto it = tex_index.find(key);
        if (it != tex_index.end())
            return it->second;
        const uint32_t idx = (uint32_t)tex_src.size();
        tex_index[key] = idx;
        tex_src.push_back({img, srgb});
        return idx;
    };
    // materials, in the reference's order of texture lookups (scene.cpp:358-383)
    for (size_t i = 0; i < doc["materials"].size(); i++) {
        const Json& m = doc["materials"][i];
        pt_material pm;
        std::memset(&pm, 0, sizeof(pm));
        uint32_t map_bits = 0;
        const Json& pbr = m["pbrMetallicRoughness"];
        const Json& ext = m["extensions"];
        // base colour (:74-112): a map stores its index and leaves alpha 0
        int64_t t = texture(pbr["baseColorTexture"], true);
        if (t >= 0) {
            map_bits |= PT_BASE_COLOUR_MAP_BIT;
            pm.base_colour[0] = bitsf((uint32_t)t);
        } else {
            const Json& bcf = pbr["baseColorFactor"];
            float base[3] = {(float)bcf[0].number(1.0), (float)bcf[1].number(1.0), (float)bcf[2].number(1.0)};
            float opacity = 1.0f;
            if (ext.has("KHR_materials_transmission"))
                opacity = 1.0f - (float)ext["KHR_materials_transmission"]["transmissionFactor"].number(0.0);
            for (int k = 0; k < 3; k++)
                pm.base_colour[k] = from_srgb(base[k]);
            pm.base_colour[3] = opacity;
        }
        // emission (:114-147)
        t = texture(m["emissiveTexture"], true);
        if (t >= 0) {
            map_bits |= PT_EMISSION_MAP_BIT;
            pm.emission[0] = bitsf((uint32_t)t);
        } else {
            const Json& ef = m["emissiveFactor"];
            for (int k = 0; k < 3; k++)
                pm.emission[k] = from_srgb((float)ef[(size_t)k].number(0.0));
        }
        pm.emission[3] = ext.has("KHR_materials_emissive_strength")
                             ? (float)ext["KHR_materials_emissive_strength"]["emissiveStrength"].number(1.0)
                             : 1.0f;
        // roughness / metalness / normal (:149-207): glTF has the combined map
        t = texture(pbr["metallicRoughnessTexture"], false);
        if (t >= 0) {
            map_bits |= PT_ROUGHNESS_METALNESS_MAP_BIT;
            pm.rough_metal_normal_map_bits[0] = bitsf((uint32_t)t);
        } else {
            pm.rough_metal_normal_map_bits[0] = (float)pbr["roughnessFactor"].number(1.0);
            pm.rough_metal_normal_map_bits[1] = (float)pbr["metallicFactor"].number(1.0);
        }
        t = texture(m["normalTexture"], false);
        if (t >= 0) {
            map_bits |= PT_NORMAL_MAP_BIT;
            pm.rough_metal_normal_map_bits[2] = bitsf((uint32_t)t);
        }
        // specular, sheen, clearcoat (:209-296) from the KHR extensions' textures
        t = texture(ext["KHR_materials_specular"]["specularColorTexture"], false);
        if (t >= 0) {
            map_bits |= PT_SPECULAR_MAP_BIT;
            pm.specular[0] = bitsf((uint32_t)t);
        } else {
            pm.specular[0] = pm.specular[1] = pm.specular[2] = 0.5f;
        }
        t = texture(ext["KHR_materials_sheen"]["sheenColorTexture"], false);
        if (t >= 0) {
            map_bits |= PT_SHEEN_MAP_BIT;
            pm.sheen[0] = bitsf((uint32_t)t);
        }
        t = texture(ext["KHR_materials_clearcoat"]["clearcoatTexture"], false);
        if (t >= 0) {
            map_bits |= PT_CLEARCOAT_MAP_BIT;
            pm.cc_ccrgh_aniso[0] = bitsf((uint32_t)t);
        } else {
            pm.cc_ccrgh_aniso[0] = 0.0f;
        }
        pm.cc_ccrgh_aniso[1] = 0.5f;
        pm.cc_ccrgh_aniso[2] = 0.0f;
        pm.rough_metal_normal_map_bits[3] = bitsf(map_bits);
        md.materials.push_back(pm);
    }
    // texture images (load_textures, scene.cpp:318-342; stb_image channel rules)
    for (const TexSource& src : tex_src) {
        const Json& im = doc["images"][(size_t)src.image];
        std::vector<uint8_t> bytes;
        std::string what;
        if (im.has("uri")) {
            const std::string& uri = im["uri"].str;
            what = uri;
            if (uri.rfind("data:", 0) == 0) {
                size_t comma = uri.find(',');
                bytes = decode_base64(comma == std::string::npos ? "" : uri.substr(comma + 1));
            } else {
                std::string f = read_file(dir + uri);
                bytes.assign(f.begin(), f.end());
            }
        } else {
            const Json& bv = doc["bufferViews"][(size_t)im["bufferView"].integer(-1)];
            if (bv.kind != Json::OBJ)
                throw std::runtime_error("image without data");
            size_t buf = (size_t)bv["buffer"].integer(0);
            size_t off = (size_t)bv["byteOffset"].integer(0), len = (size_t)bv["byteLength"].integer(0);
            if (buf >= buffers.size() || off + len > buffers[buf].size())
                throw std::runtime_error("image buffer view outside its buffer");
            bytes.assign(buffers[buf].begin() + off, buffers[buf].begin() + off + len);
            what = "embedded image " + std::to_string(src.image);
        }
        md.textures.push_back(decode_texture(bytes, what, src.srgb));
    }
    mark_transparency(md);
    // meshes: one entry per primitive
    std::vector<std::vector<uint32_t>> gltf_mesh_prims(doc["meshes"].size());
    for (size_t mi = 0; mi < doc["meshes"].size(); mi++) {
        const Json& prims = doc["meshes"][mi]["primitives"];
        for (size_t pi = 0; pi < prims.size(); pi++) {
            const Json& p = prims[pi];
            if (p["mode"].integer(4) != 4)
                continue; // points and lines are not triangles
            const Json& at = p["attributes"];
            if (!at.has("POSITION"))
                throw std::runtime_error("primitive without POSITION");
            Accessor pos = accessor(at["POSITION"].integer(0));
            std::optional<Accessor> nrm, uv;
            if (at.has("NORMAL"))
                nrm = accessor(at["NORMAL"].integer(0));
            if (at.has("TEXCOORD_0"))
                uv = accessor(at["TEXCOORD_0"].integer(0));
            if (!uv)
                std::fprintf(stderr, "Warning: mesh \"%s\" has no UVs.\n", doc["meshes"][mi]["name"].str.c_str());
            std::vector<uint32_t> idx;
            if (p.has("indices")) {
                Accessor ia = accessor(p["indices"].integer(0));
                for (size_t k = 0; k < ia.count; k++)
                    idx.push_back((uint32_t)ia.get(k, 0));
            } else {
                for (size_t k = 0; k < pos.count; k++)
                    idx.push_back((uint32_t)k);
            }
            idx.resize(idx.size() / 3 * 3);
            for (uint32_t ix : idx)
                if (ix >= pos.count)
                    throw std::runtime_error("index outside the vertex range");
            pt_mesh_range r;
            r.vertex_offset = (uint32_t)(md.vertices.size() / PT_VERTEX_FLOATS);
            r.index_offset = (uint32_t)md.indices.size();
            r.vertex_count = (uint32_t)pos.count;
            r.tri_count = (uint32_t)(idx.size() / 3);
            std::vector<float> flat_normals;
            if (!nrm) {
                // aiProcess_GenNormals: face normals (vertices shared by faces
                // take the normal of the last face that uses them).
                flat_normals.assign(3 * pos.count, 0.0f);
                for (size_t t = 0; t < idx.size(); t += 3) {
                    float a[3], b[3], c[3];
                    for (int k = 0; k < 3; k++) {
                        a[k] = (float)pos.get(idx[t], k);
                        b[k] = (float)pos.get(idx[t + 1], k);
                        c[k] = (float)pos.get(idx[t + 2], k);
                    }
                    float e1[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]}, e2[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
                    float n[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
                    float l = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
                    if (l > 0)
                        for (float& x : n)
                            x /= l;
                    for (int v = 0; v < 3; v++)
                        std::memcpy(&flat_normals[3 * idx[t + v]], n, sizeof(n));
                }
            }
            for (size_t k = 0; k < pos.count; k++) {
                float v[PT_VERTEX_FLOATS];
                for (int c = 0; c < 3; c++)
                    v[c] = (float)pos.get(k, c);
                for (int c = 0; c < 3; c++)
                    v[3 + c] = nrm ? (float)nrm->get(k, c) : flat_normals[3 * k + c];
                if (uv) {
                    v[6] = (float)uv->get(k, 0);
                    float flipped = 1.0f - (float)uv->get(k, 1);
                    v[7] = 1.0f - flipped;
                } else {
                    v[6] = v[7] = 0.0f;
                }
                md.vertices.insert(md.vertices.end(), v, v + PT_VERTEX_FLOATS);
            }
            md.indices.insert(md.indices.end(), idx.begin(), idx.end());
            gltf_mesh_prims[mi].push_back((uint32_t)md.meshes.size());
            md.meshes.push_back(r);
            int64_t mat = p["material"].integer(-1);
            if (mat < 0) {
                // Assimp adds a default material for primitives without one.
                pt_material dm;
                std::memset(&dm, 0, sizeof(dm));
                for (int k = 0; k < 3; k++)
                    dm.base_colour[k] = from_srgb(1.0f);
                dm.base_colour[3] = 1.0f;
                dm.emission[3] = 1.0f;
                dm.rough_metal_normal_map_bits[0] = 1.0f;
                dm.rough_metal_normal_map_bits[1] = 1.0f;
                dm.specular[0] = dm.specular[1] = dm.specular[2] = 0.5f;
                dm.cc_ccrgh_aniso[1] = 0.5f;
                mat = (int64_t)md.materials.size();
                md.materials.push_back(dm);
            }
            if ((size_t)mat >= md.materials.size())
                throw std::runtime_error("primitive names a missing material");
            md.mesh_material.push_back((uint32_t)mat);
        }
    }
    // nodes
    auto node_matrix = [&](const Json& n) -> Mat4 {
        if (n.has("matrix")) {
            Mat4 r;
            for (int k = 0; k < 16; k++)
                r.m[k / 4][k % 4] = (float)n["matrix"][(size_t)k].number(k % 5 == 0 ? 1.0 : 0.0);
            return r;
        }
        const Json& t = n["translation"];
        const Json& q = n["rotation"];
        const Json& s = n["scale"];
        float qx = (float)q[0].number(0), qy = (float)q[1].number(0), qz = (float)q[2].number(0), qw = (float)q[3].number(1);
        Mat4 R = Mat4::identity();
        R.m[0][0] = 1 - 2 * (qy * qy + qz * qz);
        R.m[0][1] = 2 * (qx * qy + qz * qw);
        R.m[0][2] = 2 * (qx * qz - qy * qw);
        R.m[1][0] = 2 * (qx * qy - qz * qw);
        R.m[1][1] = 1 - 2 * (qx * qx + qz * qz);
        R.m[1][2] = 2 * (qy * qz + qx * qw);
        R.m[2][0] = 2 * (qx * qz + qy * qw);
        R.m[2][1] = 2 * (qy * qz - qx * qw);
        R.m[2][2] = 1 - 2 * (qx * qx + qy * qy);
        Mat4 T = translation((float)t[0].number(0), (float)t[1].number(0), (float)t[2].number(0));
        Mat4 S = scaling((float)s[0].number(1), (float)s[1].number(1), (float)s[2].number(1));
        return mul(mul(T, R), S);
    };
    // KHR_lights_punctual: Assimp's glTF importer turns every light of the
    // extension's list, in list order, into an aiLight in the light's own node
    // space (position (0, 0, 0), direction (0, 0, -1)) with colour * intensity;
    // the reference keeps point and directional lights and skips spot lights
    // (process_lights, scene.cpp:440-466).  The node transform is not applied.
    const Json& lights = doc["extensions"]["KHR_lights_punctual"]["lights"];
    for (size_t li = 0; li < lights.size(); li++) {
        const Json& L = lights[li];
        const std::string& type = L["type"].str;
        const float intensity = (float)L["intensity"].number(1.0);
        float c[3];
        for (int k = 0; k < 3; k++)
            c[k] = (float)L["color"][(size_t)k].number(1.0) * intensity;
        if (type == "point")
            md.point_lights.insert(md.point_lights.end(), {0.0f, 0.0f, 0.0f, c[0], c[1], c[2]});
        else if (type == "directional")
            md.dir_lights.insert(md.dir_lights.end(), {0.0f, 0.0f, -1.0f, c[0], c[1], c[2]});
        else if (type != "spot")
            throw std::runtime_error("unknown KHR_lights_punctual light type " + type);
    }
    // The node graph reachable from the scene's roots (a forest: a node with
    // two parents or a cycle is refused).  Nodes that carry a light or a
    // camera are locked for the graph optimisation (Assimp locks the nodes
    // lights and cameras are named after).
    std::vector<int64_t> node_slot(doc["nodes"].size(), -1);
    std::function<int(int64_t)> add_node = [&](int64_t ni) -> int {
        const Json& n = doc["nodes"][(size_t)ni];
        if (ni < 0 || n.kind != Json::OBJ)
            throw std::runtime_error("missing node");
        if (node_slot[(size_t)ni] >= 0)
            throw std::runtime_error("node graph is not a tree (node " + std::to_string(ni) + " has two parents or a cycle)");
        const int slot = (int)md.nodes.size();
        node_slot[(size_t)ni] = slot;
        ModelNode mn;
        mn.local = node_matrix(n);
        if (n.has("mesh")) {
            size_t mi = (size_t)n["mesh"].integer(0);
            if (mi >= gltf_mesh_prims.size())
                throw std::runtime_error("node names a missing mesh");
            mn.meshes = gltf_mesh_prims[mi];
        }
        mn.locked = n.has("camera") || n["extensions"].has("KHR_lights_punctual");
        md.nodes.push_back(mn);
        std::vector<int> children;
        const Json& ch = n["children"];
        for (size_t k = 0; k < ch.size(); k++)
            children.push_back(add_node(ch[k].integer(-1)));
        md.nodes[(size_t)slot].children = children;
        return slot;
    };
    int64_t scene_idx = doc["scene"].integer(0);
    const Json& roots = doc["scenes"][(size_t)scene_idx]["nodes"];
    for (size_t k = 0; k < roots.size(); k++)
        md.roots.push_back(add_node(roots[k].integer(-1)));
    return md;
}

// Wavefront OBJ + MTL import with the behaviour of Assimp 5.4.3's OBJ importer
// as the reference's material extraction reads it (scene.cpp:74-296; Assimp is
// absent here, so this restates its documented format handling and parity is
// unpinned):
//  - one mesh per run of faces with the same object / group and material
//    (`o`, `g`, `usemtl`), all instanced once with the identity transform;
//  - polygons are fanned into triangles (aiProcess_Triangulate on convex
//    faces); negative indices count back from the last vertex read;
//  - aiProcess_FlipUVs: v is stored as 1 - v; faces without `vn` get the flat
//    face normal (aiProcess_GenNormals);
//  - material keys: Kd -> COLOR_DIFFUSE (the base colour, sRGB-decoded like
//    every factor, :94), `d` -> OPACITY (or 1 - `Tr`), Ke -> COLOR_EMISSIVE
//    (sRGB-decoded, strength 1), Pr / Pm -> roughness / metallic factors
//    (defaults 0.5 / 0, :190-202), `aniso` -> anisotropy; maps map_Kd
//    (diffuse), map_Ke (emissive), map_Pr (roughness), map_Pm (metalness; the
//    same image as map_Pr makes a combined map, :160-167), norm (normals),
//    map_Ks (specular colour); faces without a material use Assimp's default
//    material (diffuse 0.6, opacity 1).
struct ObjMaterial {
    float kd[3] = {0.6f, 0.6f, 0.6f}, ke[3] = {0.0f, 0.0f, 0.0f};
    float opacity = 1.0f, roughness = 0.5f, metallic = 0.0f, aniso = 0.0f;
    std::string map_kd, map_ke, map_pr, map_pm, norm, map_ks;
};

std::vector<std::string> line_tokens(const std::string& line)
{
    std::vector<std::string> out;
    std::istringstream is(line);
    std::string t;
    while (is >> t)
        out.push_back(t);
    return out;
}

// A map statement's file name: the last token (options such as -bm come first).
std::string map_file(const std::vector<std::string>& tk)
{
    if (tk.size() < 2)
        throw std::runtime_error("map statement without a file");
    return tk.back();
}

void load_mtl(const std::string& path, std::unordered_map<std::string, ObjMaterial>& out)
{
    std::istringstream in(read_file(path));
    std::string line;
    ObjMaterial* cur = nullptr;
    auto vec3 = [](const std::vector<std::string>& tk, float v[3]) {
        if (tk.size() < 2)
            throw std::runtime_error("colour without components");
        for (int k = 0; k < 3; k++)
            v[k] = std::stof(tk[std::min<size_t>(1 + k, tk.size() - 1)]);
    };
    while (std::getline(in, line)) {
        std::vector<std::string> tk = line_tokens(line);
        if (tk.empty() || tk[0][0] == '#')
            continue;
        const std::string& k = tk[0];
        if (k == "newmtl") {
            cur = &out[tk.size() > 1 ? tk[1] : ""];
            *cur = ObjMaterial();
            continue;
        }
        if (!cur)
            continue;
        if (k == "Kd")
            vec3(tk, cur->kd);
        else if (k == "Ke")
            vec3(tk, cur->ke);
        else if (k == "d" && tk.size() > 1)
            cur->opacity = std::stof(tk[1]);
        else if (k == "Tr" && tk.size() > 1)
            cur->opacity = 1.0f - std::stof(tk[1]);
        else if (k == "Pr" && tk.size() > 1)
            cur->roughness = std::stof(tk[1]);
        else if (k == "Pm" && tk.size() > 1)
            cur->metallic = std::stof(tk[1]);
        else if (k == "aniso" && tk.size() > 1)
            cur->aniso = std::stof(tk[1]);
        else if (k == "map_Kd")
            cur->map_kd = map_file(tk);
        else if (k == "map_Ke")
            cur->map_ke = map_file(tk);
        else if (k == "map_Pr")
            cur->map_pr = map_file(tk);
        else if (k == "map_Pm")
            cur->map_pm = map_file(tk);
        else if (k == "norm")
            cur->norm = map_file(tk);
        else if (k == "map_Ks")
            cur->map_ks = map_file(tk);
    }
}

Model load_obj(const std::string& path)
{
    const std::string dir = directory_of(path);
    std::istringstream in(read_file(path));
    std::vector<float> pos, uv, nrm;
    std::unordered_map<std::string, ObjMaterial> mtl;
    struct Face {
        uint32_t corners[3][3]; // position, uv, normal index (~0u: none)
    };
    struct Run {
        std::string material;
        std::vector<Face> faces;
    };
    std::vector<Run> runs(1);
    runs[0].material = "\x01default";
    std::string cur_mat = "\x01default";
    auto new_run = [&]() {
        if (!runs.back().faces.empty())
            runs.push_back(Run());
        runs.back().material = cur_mat;
    };
    auto index = [](const std::string& t, size_t count, const char* what) -> uint32_t {
        if (t.empty())
            return ~0u;
        long v = std::stol(t);
        long i = v > 0 ? v - 1 : (long)count + v;
        if (v == 0 || i < 0 || (size_t)i >= count)
            throw std::runtime_error(std::string("face refers to a missing ") + what);
        return (uint32_t)i;
    };
    std::string line;
    while (std::getline(in, line)) {
        std::vector<std::string> tk = line_tokens(line);
        if (tk.empty() || tk[0][0] == '#')
            continue;
        const std::string& k = tk[0];
        if (k == "v" && tk.size() >= 4) {
            for (int c = 0; c < 3; c++)
                pos.push_back(std::stof(tk[1 + c]));
        } else if (k == "vt" && tk.size() >= 2) {
            uv.push_back(std::stof(tk[1]));
            uv.push_back(tk.size() >= 3 ? std::stof(tk[2]) : 0.0f);
        } else if (k == "vn" && tk.size() >= 4) {
            for (int c = 0; c < 3; c++)
                nrm.push_back(std::stof(tk[1 + c]));
        } else if (k == "f" && tk.size() >= 4) {
            std::vector<std::array<uint32_t, 3>> poly;
            for (size_t t = 1; t < tk.size(); t++) {
                std::array<std::string, 3> part;
                size_t field = 0;
                for (char ch : tk[t]) {
                    if (ch == '/') {
                        if (++field > 2)
                            throw std::runtime_error("malformed face vertex " + tk[t]);
                        continue;
                    }
                    part[field] += ch;
                }
                poly.push_back({index(part[0], pos.size() / 3, "position"), index(part[1], uv.size() / 2, "texture coordinate"),
                                index(part[2], nrm.size() / 3, "normal")});
                if (poly.back()[0] == ~0u)
                    throw std::runtime_error("face vertex without a position");
            }
            for (size_t t = 1; t + 1 < poly.size(); t++) {
                Face f;
                const std::array<uint32_t, 3>* c3[3] = {&poly[0], &poly[t], &poly[t + 1]};
                for (int c = 0; c < 3; c++)
                    for (int a = 0; a < 3; a++)
                        f.corners[c][a] = (*c3[c])[a];
                runs.back().faces.push_back(f);
            }
        } else if (k == "usemtl") {
            cur_mat = tk.size() > 1 ? tk[1] : "";
            new_run();
        } else if (k == "o" || k == "g") {
            new_run();
        } else if (k == "mtllib") {
            for (size_t t = 1; t < tk.size(); t++)
                load_mtl(dir + tk[t], mtl);
        }
    }
    Model md;
    // materials in first-use order, textures in first-use order of the files
    std::unordered_map<std::string, uint32_t> mat_index, tex_index;
    std::vector<std::pair<std::string, bool>> tex_files;
    auto texture = [&](const std::string& file, bool srgb) -> uint32_t {
        auto it = tex_index.find(file);
        if (it != tex_index.end())
            return it->second;
        const uint32_t idx = (uint32_t)tex_files.size();
        tex_index[file] = idx;
        tex_files.push_back({file, srgb});
        return idx;
    };
    auto material = [&](const std::string& name) -> uint32_t {
        auto it = mat_index.find(name);
        if (it != mat_index.end())
            return it->second;
        ObjMaterial om;
        auto found = mtl.find(name);
        if (found != mtl.end())
            om = found->second;
        pt_material pm;
        std::memset(&pm, 0, sizeof(pm));
        uint32_t bits = 0;
        if (!om.map_kd.empty()) {
            bits |= PT_BASE_COLOUR_MAP_BIT;
            pm.base_colour[0] = bitsf(texture(om.map_kd, true));
        } else {
            for (int c = 0; c < 3; c++)
                pm.base_colour[c] = from_srgb(om.kd[c]);
            pm.base_colour[3] = om.opacity;
        }
        if (!om.map_ke.empty()) {
            bits |= PT_EMISSION_MAP_BIT;
            pm.emission[0] = bitsf(texture(om.map_ke, true));
        } else {
            for (int c = 0; c < 3; c++)
                pm.emission[c] = from_srgb(om.ke[c]);
        }
        pm.emission[3] = 1.0f;
        if (!om.map_pr.empty() && om.map_pr == om.map_pm) {
            bits |= PT_ROUGHNESS_METALNESS_MAP_BIT;
            pm.rough_metal_normal_map_bits[0] = bitsf(texture(om.map_pr, false));
        } else {
            if (!om.map_pr.empty()) {
                bits |= PT_ROUGHNESS_MAP_BIT;
                pm.rough_metal_normal_map_bits[0] = bitsf(texture(om.map_pr, false));
            } else {
                pm.rough_metal_normal_map_bits[0] = om.roughness;
            }
            if (!om.map_pm.empty()) {
                bits |= PT_METALNESS_MAP_BIT;
                pm.rough_metal_normal_map_bits[1] = bitsf(texture(om.map_pm, false));
            } else {
                pm.rough_metal_normal_map_bits[1] = om.metallic;
            }
        }
        if (!om.norm.empty()) {
            bits |= PT_NORMAL_MAP_BIT;
            pm.rough_metal_normal_map_bits[2] = bitsf(texture(om.norm, false));
        }
        if (!om.map_ks.empty()) {
            bits |= PT_SPECULAR_MAP_BIT;
            pm.specular[0] = bitsf(texture(om.map_ks, false));
        } else {
            pm.specular[0] = pm.specular[1] = pm.specular[2] = 0.5f;
        }
        pm.cc_ccrgh_aniso[1] = 0.5f;
        pm.cc_ccrgh_aniso[2] = om.aniso;
        pm.rough_metal_normal_map_bits[3] = bitsf(bits);
        md.materials.push_back(pm);
        mat_index[name] = (uint32_t)md.materials.size() - 1;
        return (uint32_t)md.materials.size() - 1;
    };
    for (const Run& r : runs) {
        if (r.faces.empty())
            continue;
        const uint32_t mi = material(r.material);
        pt_mesh_range range{(uint32_t)(md.vertices.size() / PT_VERTEX_FLOATS), (uint32_t)md.indices.size(),
                            (uint32_t)r.faces.size(), (uint32_t)(3 * r.faces.size())};
        for (const Face& f : r.faces) {
            float p[3][3];
            for (int c = 0; c < 3; c++)
                for (int a = 0; a < 3; a++)
                    p[c][a] = pos[3 * (size_t)f.corners[c][0] + a];
            // flat face normal for corners without one (aiProcess_GenNormals)
            float e1[3], e2[3], fn[3];
            for (int a = 0; a < 3; a++) {
                e1[a] = p[1][a] - p[0][a];
                e2[a] = p[2][a] - p[0][a];
            }
            fn[0] = e1[1] * e2[2] - e1[2] * e2[1];
            fn[1] = e1[2] * e2[0] - e1[0] * e2[2];
            fn[2] = e1[0] * e2[1] - e1[1] * e2[0];
            const float len = std::sqrt((fn[0] * fn[0] + fn[1] * fn[1]) + fn[2] * fn[2]);
            for (int a = 0; a < 3; a++)
                fn[a] = len > 0.0f ? fn[a] / len : 0.0f;
            for (int c = 0; c < 3; c++) {
                const uint32_t ti = f.corners[c][1], ni = f.corners[c][2];
                float v[PT_VERTEX_FLOATS] = {p[c][0], p[c][1], p[c][2], fn[0], fn[1], fn[2], 0.0f, 0.0f};
                if (ni != ~0u)
                    for (int a = 0; a < 3; a++)
                        v[3 + a] = nrm[3 * (size_t)ni + a];
                if (ti != ~0u) {
                    v[6] = uv[2 * (size_t)ti];
                    v[7] = 1.0f - uv[2 * (size_t)ti + 1];
                }
                md.indices.push_back((uint32_t)(md.vertices.size() / PT_VERTEX_FLOATS) - range.vertex_offset);
                md.vertices.insert(md.vertices.end(), v, v + PT_VERTEX_FLOATS);
            }
        }
        md.meshes.push_back(range);
        md.mesh_material.push_back(mi);
    }
    // Assimp's OBJ importer: a root node with one child per object/group run
    md.nodes.resize(1 + md.meshes.size());
    md.roots = {0};
    for (size_t m = 0; m < md.meshes.size(); m++) {
        md.nodes[0].children.push_back((int)m + 1);
        md.nodes[m + 1].meshes = {(uint32_t)m};
    }
    for (const auto& tf : tex_files) {
        std::string f = read_file(dir + tf.first);
        md.textures.push_back(decode_texture(std::vector<uint8_t>(f.begin(), f.end()), tf.first, tf.second));
    }
    mark_transparency(md);
    return md;
}

// Model import by file extension: .obj (Wavefront + MTL), otherwise glTF 2.0
// (.gltf or .glb), followed by the reference's Assimp post-processing.
Model load_model(const std::string& path)
{
    std::string ext;
    const size_t dot = path.find_last_of('.');
    if (dot != std::string::npos)
        for (char c : path.substr(dot + 1))
            ext += (char)std::tolower((unsigned char)c);
    Model md = ext == "obj" ? load_obj(path) : load_gltf(path);
    // the reference's import flags (scene.cpp:537-550), see assimp_post.cpp
    pt::host::assimp_postprocess(md);
    return md;
}

// ---------------------------------------------------------------- 4x4 inverse (FP64 cofactors)
void inverse4(const double a[16], double out[16])
{
    double inv[16];
    inv[0] = a[5] * a[10] * a[15] - a[5] * a[11] * a[14] - a[9] * a[6] * a[15] + a[9] * a[7] * a[14] + a[13] * a[6] * a[11] - a[13] * a[7] * a[10];
    inv[4] = -a[4] * a[10] * a[15] + a[4] * a[11] * a[14] + a[8] * a[6] * a[15] - a[8] * a[7] * a[14] - a[12] * a[6] * a[11] + a[12] * a[7] * a[10];
    inv[8] = a[4] * a[9] * a[15] - a[4] * a[11] * a[13] - a[8] * a[5] * a[15] + a[8] * a[7] * a[13] + a[12] * a[5] * a[11] - a[12] * a[7] * a[9];
    inv[12] = -a[4] * a[9] * a[14] + a[4] * a[10] * a[13] + a[8] * a[5] * a[14] - a[8] * a[6] * a[13] - a[12] * a[5] * a[10] + a[12] * a[6] * a[9];
    inv[1] = -a[1] * a[10] * a[15] + a[1] * a[11] * a[14] + a[9] * a[2] * a[15] - a[9] * a[3] * a[14] - a[13] * a[2] * a[11] + a[13] * a[3] * a[10];
    inv[5] = a[0] * a[10] * a[15] - a[0] * a[11] * a[14] - a[8] * a[2] * a[15] + a[8] * a[3] * a[14] + a[12] * a[2] * a[11] - a[12] * a[3] * a[10];
    inv[9] = -a[0] * a[9] * a[15] + a[0] * a[11] * a[13] + a[8] * a[1] * a[15] - a[8] * a[3] * a[13] - a[12] * a[1] * a[11] + a[12] * a[3] * a[9];
    inv[13] = a[0] * a[9] * a[14] - a[0] * a[10] * a[13] - a[8] * a[1] * a[14] + a[8] * a[2] * a[13] + a[12] * a[1] * a[10] - a[12] * a[2] * a[9];
    inv[2] = a[1] * a[6] * a[15] - a[1] * a[7] * a[14] - a[5] * a[2] * a[15] + a[5] * a[3] * a[14] + a[13] * a[2] * a[7] - a[13] * a[3] * a[6];
    inv[6] = -a[0] * a[6] * a[15] + a[0] * a[7] * a[14] + a[4] * a[2] * a[15] - a[4] * a[3] * a[14] - a[12] * a[2] * a[7] + a[12] * a[3] * a[6];
    inv[10] = a[0] * a[5] * a[15] - a[0] * a[7] * a[13] - a[4] * a[1] * a[15] + a[4] * a[3] * a[13] + a[12] * a[1] * a[7] - a[12] * a[3] * a[5];
    inv[14] = -a[0] * a[5] * a[14] + a[0] * a[6] * a[13] + a[4] * a[1] * a[14] - a[4] * a[2] * a[13] - a[12] * a[1] * a[6] + a[12] * a[2] * a[5];
    inv[3] = -a[1] * a[6] * a[11] + a[1] * a[7] * a[10] + a[5] * a[2] * a[11] - a[5] * a[3] * a[10] - a[9] * a[2] * a[7] + a[9] * a[3] * a[6];
    inv[7] = a[0] * a[6] * a[11] - a[0] * a[7] * a[10] - a[4] * a[2] * a[11] + a[4] * a[3] * a[10] + a[8] * a[2] * a[7] - a[8] * a[3] * a[6];
    inv[11] = -a[0] * a[5] * a[11] + a[0] * a[7] * a[9] + a[4] * a[1] * a[11] - a[4] * a[3] * a[9] - a[8] * a[1] * a[7] + a[8] * a[3] * a[5];
    inv[15] = a[0] * a[5] * a[10] - a[0] * a[6] * a[9] - a[4] * a[1] * a[10] + a[4] * a[2] * a[9] + a[8] * a[1] * a[6] - a[8] * a[2] * a[5];
    double det = a[0] * inv[0] + a[1] * inv[4] + a[2] * inv[8] + a[3] * inv[12];
    double id = 1.0 / det;
    for (int i = 0; i < 16; i++)
        out[i] = inv[i] * id;
}

// Vose alias table with the reference's float/double choices
// (aliastable.h:21-67); appends bins (p, q, alias, value words).
void append_alias(std::vector<uint32_t>& out, const std::vector<float>& w, const std::vector<std::vector<uint32_t>>& values)
{
    size_t n = w.size();
    double sum = std::accumulate(w.begin(), w.end(), 0.0);
    double inv_sum = 1.0 / sum;
    std::vector<float> p(n), q(n);
    std::vector<uint32_t> alias(n);
    for (size_t i = 0; i < n; i++) {
        p[i] = (float)((double)w[i] * inv_sum);
        alias[i] = (uint32_t)i;
    }
    std::vector<size_t> under, over;
    for (size_t i = 0; i < n; i++) {
        float u = p[i] * (float)n;
        q[i] = u;
        (u < 1.0f ? under : over).push_back(i);
    }
    while (!under.empty() && !over.empty()) {
        alias[under.back()] = (uint32_t)over.back();
        q[over.back()] += q[under.back()] - 1.0f;
        under.pop_back();
        if (q[over.back()] < 1.0f) {
            under.push_back(over.back());
            over.pop_back();
        }
    }
    for (size_t i : under)
        q[i] = 1.0f;
    for (size_t i : over)
        q[i] = 1.0f;
    for (size_t i = 0; i < n; i++) {
        out.push_back(fbits(p[i]));
        out.push_back(fbits(q[i]));
        out.push_back(alias[i]);
        out.insert(out.end(), values[i].begin(), values[i].end());
    }
}

bool is_emitter(const pt_material& m)
{
    uint32_t bits = fbits(m.rough_metal_normal_map_bits[3]);
    return ((bits & PT_EMISSION_MAP_BIT) || std::max(std::max(m.emission[0], m.emission[1]), m.emission[2]) > 0.0f) && m.emission[3] > 0.0f;
}

} // namespace

struct pt_host_scene {
    std::vector<float> vertices;
    std::vector<uint32_t> indices;
    std::vector<pt_mesh_range> meshes;
    std::vector<uint32_t> mesh_material;
    std::vector<uint32_t> mesh_instance_offset{0};
    std::vector<float> instance_matrices;
    std::vector<pt_material> materials;
    std::vector<float> point_lights, dir_lights;
    float env[3] = {0, 0, 0};
    pt_camera_desc camera{};
    std::vector<pt_texture> textures;
    std::vector<uint8_t> texels;
    std::vector<float> material_ior; // empty, or one per material (refractive extension)
    // packed
    bool packed = false;
    std::vector<pt_instance_data> inst;
    std::vector<uint32_t> inst_mesh;
    std::vector<float> w2o;
    std::vector<uint8_t> opaque;
    std::vector<uint32_t> light;
    uint32_t light_count = 0;

    void default_camera()
    {
        // scenebuild.cpp:138-144
        camera = pt_camera_desc{};
        camera.lookdir[2] = -1.0f;
        camera.up[1] = 1.0f;
        camera.fov_degrees = 45.0f;
        camera.near_plane = 0.1f;
        camera.far_plane = 1000.0f;
        camera.exposure = 1.0f;
    }

    void append_model(const Model& md, const std::vector<Mat4>& scene_instances)
    {
        uint32_t vbase = (uint32_t)(vertices.size() / PT_VERTEX_FLOATS);
        uint32_t ibase = (uint32_t)indices.size();
        uint32_t mbase = (uint32_t)materials.size();
        vertices.insert(vertices.end(), md.vertices.begin(), md.vertices.end());
        indices.insert(indices.end(), md.indices.begin(), md.indices.end());
        for (size_t m = 0; m < md.meshes.size(); m++) {
            pt_mesh_range r = md.meshes[m];
            r.vertex_offset += vbase;
            r.index_offset += ibase;
            meshes.push_back(r);
            mesh_material.push_back(md.mesh_material[m] + mbase);
            // scenebuild.cpp:345-352: scene instance x object instance
            for (const Mat4& si : scene_instances)
                for (const Mat4& oi : md.mesh_instances[m]) {
                    Mat4 M = mul(si, oi);
                    instance_matrices.insert(instance_matrices.end(), &M.m[0][0], &M.m[0][0] + 16);
                }
            mesh_instance_offset.push_back((uint32_t)(instance_matrices.size() / 16));
        }
        // textures of this object follow the scene's; its materials' map
        // indices move by the same offset (scenebuild.cpp:315-361, offset_maps_by
        // in material.cpp:16-42, which offsets the specular and sheen maps in the
        // .w slots while the shader reads them from .x)
        const uint32_t toff = (uint32_t)textures.size();
        for (pt_material pm : md.materials) {
            const uint32_t bits = fbits(pm.rough_metal_normal_map_bits[3]);
            auto shift = [&](float& f) { f = bitsf(fbits(f) + toff); };
            if (bits & PT_BASE_COLOUR_MAP_BIT)
                shift(pm.base_colour[0]);
            if (bits & PT_EMISSION_MAP_BIT)
                shift(pm.emission[0]);
            if ((bits & PT_ROUGHNESS_MAP_BIT) || (bits & PT_ROUGHNESS_METALNESS_MAP_BIT))
                shift(pm.rough_metal_normal_map_bits[0]);
            if (bits & PT_METALNESS_MAP_BIT)
                shift(pm.rough_metal_normal_map_bits[1]);
            if (bits & PT_SPECULAR_TINT_MAP_BIT)
                shift(pm.specular[0]);
            if (bits & PT_SPECULAR_MAP_BIT)
                shift(pm.specular[3]);
            if (bits & PT_SHEEN_TINT_MAP_BIT)
                shift(pm.sheen[0]);
            if (bits & PT_SHEEN_MAP_BIT)
                shift(pm.sheen[3]);
            if (bits & PT_CLEARCOAT_MAP_BIT)
                shift(pm.cc_ccrgh_aniso[0]);
            if (bits & PT_CLEARCOAT_ROUGHNESS_MAP_BIT)
                shift(pm.cc_ccrgh_aniso[1]);
            if (bits & PT_ANISOTROPY_MAP_BIT)
                shift(pm.cc_ccrgh_aniso[2]);
            if (bits & PT_NORMAL_MAP_BIT)
                shift(pm.rough_metal_normal_map_bits[2]);
            materials.push_back(pm);
        }
        for (const HostTexture& t : md.textures)
            add_texture(t.width, t.height, t.channels, t.srgb, t.texels.data());
    }

    void add_texture(uint32_t w, uint32_t h, uint32_t ch, uint32_t srgb, const uint8_t* data)
    {
        pt_texture d;
        d.offset = texels.size();
        d.width = w;
        d.height = h;
        d.channels = ch;
        d.srgb = srgb;
        textures.push_back(d);
        texels.insert(texels.end(), data, data + (size_t)w * h * ch);
    }
};

namespace {

// SceneBuilder::read_scene_description (scenebuild.cpp:279-365).
pt_host_scene* load_scn(const std::string& path)
{
    std::string text = read_file(path);
    text.erase(std::remove_if(text.begin(), text.end(), [](char c) { return c == '\r' || c == '\t'; }), text.end());
    Tokens lines(text, '\n');
    struct Subscene {
        std::string id, path;
        std::vector<Mat4> instances;
    };
    std::vector<Subscene> subs;
    std::unordered_map<std::string, size_t> sub_index;
    std::optional<std::string> current;
    Mat4 cur_tf = Mat4::identity();
    bool have_camera = false;
    auto host = std::make_unique<pt_host_scene>();
    host->default_camera();
    std::vector<float> plights, dlights;
    auto is_label = [](const std::string& t) { return !t.empty() && t.back() == ':'; };
    auto finish_instance = [&]() {
        if (current)
            subs[sub_index[*current]].instances.push_back(cur_tf);
    };
    auto parse_light = [&](Tokens& tk, std::vector<float>& out) {
        if (tk.remaining() != 7)
            throw std::runtime_error("Invalid light syntax.");
        float p[3], c[3];
        parse_vec3(tk, p);
        if (tk.next() != ",")
            throw std::runtime_error("Invalid light syntax.");
        parse_vec3(tk, c);
        out.insert(out.end(), {p[0], p[1], p[2], from_srgb(c[0]), from_srgb(c[1]), from_srgb(c[2])});
    };
    while (!lines.done()) {
        Tokens tk(lines.next(), ' ');
        if (tk.done())
            continue;
        std::string tok = tk.next();
        if (tok == "camera:") {
            if (have_camera)
                throw std::runtime_error("Camera already set.");
            have_camera = true;
            pt_camera_desc& cam = host->camera;
            while (!lines.done()) {
                Tokens ct(lines.next(), ' ');
                if (ct.done())
                    continue;
                std::string k = ct.next();
                if (k == "position")
                    parse_vec3(ct, cam.position);
                else if (k == "lookdir")
                    parse_vec3(ct, cam.lookdir);
                else if (k == "up")
                    parse_vec3(ct, cam.up);
                else if (k == "fov")
                    cam.fov_degrees = to_float(ct.next());
                else if (k == "near")
                    cam.near_plane = to_float(ct.next());
                else if (k == "far")
                    cam.far_plane = to_float(ct.next());
                else if (k == "focusdist")
                    cam.focus_dist = to_float(ct.next());
                else if (k == "lensradius")
                    cam.lens_radius = to_float(ct.next());
                else if (k == "exposure")
                    cam.exposure = to_float(ct.next());
                else if (k == "envcol") {
                    float e[3];
                    parse_vec3(ct, e);
                    for (int q = 0; q < 3; q++)
                        host->env[q] = from_srgb(e[q]);
                } else if (k == "envmap")
                    ct.next(); // environment maps are not part of the headless path
                else if (is_label(k)) {
                    lines.rollback(1);
                    break;
                } else
                    throw std::runtime_error("Unrecognised token in camera section " + k);
            }
        } else if (tok == "objects:") {
            while (!lines.done()) {
                Tokens ot(lines.next(), ' ');
                if (ot.done())
                    continue;
                std::string k = ot.next();
                if (k == "t" || k == "r" || k == "s") {
                    if (!current)
                        throw std::runtime_error(k == "t" ? "No instance to translate." : k == "r" ? "No instance to rotate." : "No instance to scale.");
                    Mat4 M;
                    if (k == "t") {
                        if (ot.remaining() != 3)
                            throw std::runtime_error("Translation did not have three coordinates");
                        float x = to_float(ot.next()), y = to_float(ot.next()), z = to_float(ot.next());
                        M = translation(x, y, z);
                    } else if (k == "r") {
                        if (ot.remaining() != 4)
                            throw std::runtime_error("Rotation did not have three coordinates and angle");
                        float x = to_float(ot.next()), y = to_float(ot.next()), z = to_float(ot.next());
                        float a = to_float(ot.next());
                        M = rotation(x, y, z, a);
                    } else {
                        if (ot.remaining() != 3)
                            throw std::runtime_error("Scaling did not have three coordinates");
                        float x = to_float(ot.next()), y = to_float(ot.next()), z = to_float(ot.next());
                        M = scaling(x, y, z);
                    }
                    cur_tf = mul(M, cur_tf);
                } else if (k == "basecol" || k == "roughness" || k == "metalness" || k == "specular") {
                    // accepted and ignored, as in the reference (scenebuild.cpp:222-237)
                    if (!current)
                        throw std::runtime_error("No instance to apply " + k + " parameter to.");
                } else if (k == "plight") {
                    parse_light(ot, plights);
                } else if (k == "dlight") {
                    parse_light(ot, dlights);
                } else if (is_label(k)) {
                    lines.rollback(1);
                    break;
                } else if (ot.done()) {
                    if (!sub_index.count(k))
                        throw std::runtime_error("Object " + k + " not recognised.");
                    finish_instance();
                    current = k;
                    cur_tf = Mat4::identity();
                } else {
                    sub_index[k] = subs.size();
                    subs.push_back(Subscene{k, ot.next(), {}});
                }
            }
            finish_instance();
            current.reset();
        } else {
            throw std::runtime_error("Unrecognised token " + tok);
        }
    }
    if (!have_camera)
        throw std::runtime_error("No camera section in scene description.");
    host->point_lights = plights;
    host->dir_lights = dlights;
    std::string dir = directory_of(path);
    for (const Subscene& s : subs) {
        if (s.instances.empty())
            continue;
        Model md = load_model(dir + s.path);
        // the model's own lights, once per scene instance, moved by the
        // instance transform (scenebuild.cpp:321-335)
        for (const Mat4& si : s.instances) {
            for (size_t k = 0; k + 6 <= md.point_lights.size(); k += 6) {
                float p[3];
                transform_point(si, &md.point_lights[k], 1.0f, p);
                host->point_lights.insert(host->point_lights.end(), {p[0], p[1], p[2], md.point_lights[k + 3],
                                                                     md.point_lights[k + 4], md.point_lights[k + 5]});
            }
            for (size_t k = 0; k + 6 <= md.dir_lights.size(); k += 6) {
                float d[3];
                transform_point(si, &md.dir_lights[k], 0.0f, d);
                host->dir_lights.insert(host->dir_lights.end(), {d[0], d[1], d[2], md.dir_lights[k + 3],
                                                                 md.dir_lights[k + 4], md.dir_lights[k + 5]});
            }
        }
        host->append_model(md, s.instances);
    }
    return host.release();
}

} // namespace

// ================================================================ C API
extern "C" {

const char* pt_scene_last_error(void) { return g_error.c_str(); }

pt_host_scene* pt_scene_load(const char* scn_path)
{
    if (!scn_path) {
        g_error = "null path";
        return nullptr;
    }
    try {
        return load_scn(scn_path);
    } catch (const std::exception& e) {
        g_error = e.what();
        return nullptr;
    }
}

pt_host_scene* pt_scene_from_raw(const pt_raw_scene* raw, const pt_camera_desc* camera)
{
    if (!raw) {
        g_error = "null raw scene";
        return nullptr;
    }
    try {
        auto s = std::make_unique<pt_host_scene>();
        if (camera)
            s->camera = *camera;
        else
            s->default_camera();
        s->vertices.assign(raw->vertices, raw->vertices + (size_t)raw->vertex_count * PT_VERTEX_FLOATS);
        s->indices.assign(raw->indices, raw->indices + raw->index_count);
        s->meshes.assign(raw->meshes, raw->meshes + raw->mesh_count);
        s->mesh_material.assign(raw->mesh_material, raw->mesh_material + raw->mesh_count);
        s->mesh_instance_offset.assign(raw->mesh_instance_offset, raw->mesh_instance_offset + raw->mesh_count + 1);
        s->instance_matrices.assign(raw->instance_matrices, raw->instance_matrices + 16 * (size_t)raw->instance_count);
        s->materials.assign(raw->materials, raw->materials + raw->material_count);
        if (raw->point_light_count)
            s->point_lights.assign(raw->point_lights, raw->point_lights + 6 * (size_t)raw->point_light_count);
        if (raw->directional_light_count)
            s->dir_lights.assign(raw->directional_lights, raw->directional_lights + 6 * (size_t)raw->directional_light_count);
        std::memcpy(s->env, raw->environment_colour, sizeof(s->env));
        for (uint32_t i = 0; i < raw->texture_count; i++) {
            const pt_texture& t = raw->textures[i];
            if (t.width == 0 || t.height == 0 || !(t.channels == 1 || t.channels == 2 || t.channels == 4) ||
                t.offset + (uint64_t)t.width * t.height * t.channels > raw->texel_bytes)
                throw std::runtime_error("texture " + std::to_string(i) + " is malformed");
            s->add_texture(t.width, t.height, t.channels, t.srgb ? 1u : 0u, raw->texels + t.offset);
        }
        if (raw->material_ior) {
            s->material_ior.assign(raw->material_ior, raw->material_ior + raw->material_count);
            for (uint32_t i = 0; i < raw->material_count; i++) {
                const float n = s->material_ior[i];
                if (!(n == 0.0f || (n >= 1.0f && std::isfinite(n))))
                    throw std::runtime_error("material " + std::to_string(i) + ": index of refraction must be 0 or >= 1");
            }
        }
        for (uint32_t m = 0; m < raw->mesh_count; m++) {
            if (s->mesh_material[m] >= raw->material_count)
                throw std::runtime_error("mesh " + std::to_string(m) + " names a missing material");
            if (s->mesh_instance_offset[m + 1] < s->mesh_instance_offset[m])
                throw std::runtime_error("instance offsets are not monotone");
        }
        if (s->mesh_instance_offset[raw->mesh_count] != raw->instance_count)
            throw std::runtime_error("instance offsets do not end at the instance count");
        return s.release();
    } catch (const std::exception& e) {
        g_error = e.what();
        return nullptr;
    }
}

void pt_scene_free(pt_host_scene* s) { delete s; }

int pt_scene_raw(const pt_host_scene* s, pt_raw_scene* out)
{
    if (!s || !out)
        return PT_ERR_INVALID;
    std::memset(out, 0, sizeof(*out));
    out->vertices = s->vertices.data();
    out->vertex_count = (uint32_t)(s->vertices.size() / PT_VERTEX_FLOATS);
    out->indices = s->indices.data();
    out->index_count = (uint32_t)s->indices.size();
    out->meshes = s->meshes.data();
    out->mesh_material = s->mesh_material.data();
    out->mesh_instance_offset = s->mesh_instance_offset.data();
    out->mesh_count = (uint32_t)s->meshes.size();
    out->instance_matrices = s->instance_matrices.data();
    out->instance_count = (uint32_t)(s->instance_matrices.size() / 16);
    out->materials = s->materials.data();
    out->material_count = (uint32_t)s->materials.size();
    out->point_lights = s->point_lights.data();
    out->point_light_count = (uint32_t)(s->point_lights.size() / 6);
    out->directional_lights = s->dir_lights.data();
    out->directional_light_count = (uint32_t)(s->dir_lights.size() / 6);
    std::memcpy(out->environment_colour, s->env, sizeof(s->env));
    out->texels = s->texels.data();
    out->texel_bytes = s->texels.size();
    out->textures = s->textures.data();
    out->texture_count = (uint32_t)s->textures.size();
    out->material_ior = s->material_ior.empty() ? nullptr : s->material_ior.data();
    return PT_OK;
}

int pt_scene_camera(const pt_host_scene* s, pt_camera_desc* out)
{
    if (!s || !out)
        return PT_ERR_INVALID;
    *out = s->camera;
    return PT_OK;
}

// The reference's generators (src/rng.cpp): xoshiro128++ and splitmix32.
struct Xshiro128 {
    uint32_t s[4];
    static uint32_t rotl(uint32_t x, int k) { return (x << k) | (x >> (32 - k)); }
    uint32_t next()
    {
        const uint32_t result = rotl(s[0] + s[3], 7) + s[0];
        const uint32_t t = s[1] << 9;
        s[2] ^= s[0];
        s[3] ^= s[1];
        s[1] ^= s[2];
        s[0] ^= s[3];
        s[2] ^= t;
        s[3] = rotl(s[3], 11);
        return result;
    }
    // static_cast<float>(next()) / UINT32_MAX: the divisor rounds to 2^32 in float
    float next_float() { return (float)next() / 4294967296.0f; }
};

struct Splitmix32 {
    uint32_t state;
    uint32_t next()
    {
        uint32_t z = (state += 0x9e3779b9u);
        z = (z ^ (z >> 16)) * 0x85ebca6bu;
        z = (z ^ (z >> 13)) * 0xc2b2ae35u;
        return z ^ (z >> 16);
    }
};

// Nearest texel of one coordinate: x = min((uint32_t)roundf(frac * size), size - 1)
// (lightsample.cpp:70-73).  The cast of a negative value is undefined in C++;
// GCC on x86 wraps it to a large number that the min() clamps, which is what
// happens here on every platform.
uint32_t nearest_texel(float f, uint32_t size)
{
    const float r = std::roundf(f);
    if (r < 0.0f || r >= 4294967296.0f)
        return size - 1;
    return std::min((uint32_t)r, size - 1);
}

// calculate_object_intensity (lightsample.cpp:41-87) for an emission map:
// 20 random points per triangle, nearest texel, raw 8-bit / 255 channels.
double textured_intensity(const pt_host_scene* s, size_t mesh, const pt_material& mat)
{
    Splitmix32 seeder{0xbd7a0d48u};
    // Xshiro128 rng(seeder.next() x 4): GCC evaluates those arguments right to left
    const uint32_t a = seeder.next(), b = seeder.next(), c = seeder.next(), d = seeder.next();
    Xshiro128 rng{{d, c, b, a}};
    const uint32_t ti = fbits(mat.emission[0]);
    if (ti >= s->textures.size())
        throw std::runtime_error("emission map names a missing texture");
    const pt_texture& tex = s->textures[ti];
    const uint8_t* texels = s->texels.data() + tex.offset;
    const pt_mesh_range& r = s->meshes[mesh];
    double total = 0.0;
    for (uint32_t t = 0; t < r.tri_count; t++) {
        const uint32_t* ix = &s->indices[r.index_offset + 3 * t];
        const float* va = &s->vertices[(size_t)(r.vertex_offset + ix[0]) * PT_VERTEX_FLOATS];
        const float* vb = &s->vertices[(size_t)(r.vertex_offset + ix[1]) * PT_VERTEX_FLOATS];
        const float* vc = &s->vertices[(size_t)(r.vertex_offset + ix[2]) * PT_VERTEX_FLOATS];
        double tri_sum = 0.0;
        for (int j = 0; j < 20; j++) {
            const float beta = 1.0f - std::sqrt(rng.next_float());
            const float gamma = (1.0f - beta) * rng.next_float();
            const float alpha = (1.0f - beta) - gamma;
            const float u = (alpha * va[6] + beta * vb[6]) + gamma * vc[6];
            const float v = (alpha * va[7] + beta * vb[7]) + gamma * vc[7];
            float integral;
            const uint32_t x = nearest_texel(std::modf(u, &integral) * (float)tex.width, tex.width);
            const uint32_t y = nearest_texel(std::modf(v, &integral) * (float)tex.height, tex.height);
            const uint8_t* p = texels + ((size_t)y * tex.width + x) * tex.channels;
            const float er = p[0] / 255.0f;
            const float eg = tex.channels >= 2 ? p[1] / 255.0f : 0.0f;
            const float eb = tex.channels == 4 ? p[2] / 255.0f : 0.0f;
            tri_sum += (er + eg) + eb;
        }
        total += tri_sum;
    }
    return total * (double)mat.emission[3] / (double)((size_t)r.tri_count * 20u);
}

// SceneBuffer::build (scenebuffer.cpp:65-168) + TableLightSampler
// (lightsample.cpp:89-178), including the reference's quirks: every emitter
// table offset starts from 0 (:126) and the offset shift counts unique
// emitter meshes (:150, :156-157).
int pt_scene_pack(pt_host_scene* s, pt_scene_view* v)
{
    if (!s || !v)
        return PT_ERR_INVALID;
    try {
        if (!s->packed) {
            s->inst.clear();
            s->inst_mesh.clear();
            s->w2o.clear();
            s->opaque.clear();
            s->light.clear();
            uint32_t emitter_index = 0;
            size_t nmesh = s->meshes.size();
            for (size_t m = 0; m < nmesh; m++) {
                const pt_material& mat = s->materials[s->mesh_material[m]];
                bool emits = is_emitter(mat);
                uint32_t bits = fbits(mat.rough_metal_normal_map_bits[3]);
                for (uint32_t j = s->mesh_instance_offset[m]; j < s->mesh_instance_offset[m + 1]; j++) {
                    const float* M = &s->instance_matrices[16 * (size_t)j];
                    pt_instance_data d;
                    d.vertex_index = s->meshes[m].vertex_offset;
                    d.index_index = s->meshes[m].index_offset;
                    d.emitter_index = emits ? emitter_index++ : PT_NO_EMITTER_INDEX;
                    d.material_index = s->mesh_material[m];
                    double Md[16], inv[16];
                    for (int r = 0; r < 4; r++)
                        for (int c = 0; c < 4; c++) {
                            d.transform[r][c] = M[c * 4 + r];
                            Md[r * 4 + c] = M[c * 4 + r];
                        }
                    inverse4(Md, inv);
                    for (int r = 0; r < 3; r++)
                        for (int c = 0; c < 4; c++)
                            d.normal[r][c] = (float)inv[c * 4 + r];
                    s->inst.push_back(d);
                    s->inst_mesh.push_back((uint32_t)m);
                    for (int k = 0; k < 12; k++)
                        s->w2o.push_back((float)inv[k]);
                    s->opaque.push_back((bits & PT_MATERIAL_IS_TRANSPARENT_BIT) ? 0 : 1);
                }
            }
            // light sampler
            size_t lights = s->point_lights.size() / 6 + s->dir_lights.size() / 6;
            for (size_t m = 0; m < nmesh; m++)
                if (is_emitter(s->materials[s->mesh_material[m]]))
                    lights += s->mesh_instance_offset[m + 1] - s->mesh_instance_offset[m];
            s->light_count = 0;
            if (lights > 0) {
                std::vector<float> weights;
                std::vector<std::vector<uint32_t>> values;
                std::vector<std::vector<float>> tw;
                std::vector<std::vector<std::vector<uint32_t>>> tv;
                std::unordered_map<uint32_t, size_t> table_of;
                for (size_t m = 0; m < nmesh; m++) {
                    const pt_material& mat = s->materials[s->mesh_material[m]];
                    if (!is_emitter(mat))
                        continue;
                    size_t ti;
                    auto it = table_of.find((uint32_t)m);
                    if (it == table_of.end()) {
                        ti = tw.size();
                        tw.emplace_back();
                        tv.emplace_back();
                        const pt_mesh_range& r = s->meshes[m];
                        for (uint32_t t = 0; t < r.tri_count; t++) {
                            const uint32_t* ix = &s->indices[r.index_offset + 3 * t];
                            const float* a = &s->vertices[(size_t)(r.vertex_offset + ix[0]) * PT_VERTEX_FLOATS];
                            const float* b = &s->vertices[(size_t)(r.vertex_offset + ix[1]) * PT_VERTEX_FLOATS];
                            const float* c = &s->vertices[(size_t)(r.vertex_offset + ix[2]) * PT_VERTEX_FLOATS];
                            float ab[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
                            float ac[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
                            float cr[3] = {ab[1] * ac[2] - ab[2] * ac[1], ab[2] * ac[0] - ab[0] * ac[2], ab[0] * ac[1] - ab[1] * ac[0]};
                            tw.back().push_back(std::sqrt((cr[0] * cr[0] + cr[1] * cr[1]) + cr[2] * cr[2]));
                            tv.back().push_back({ix[0], ix[1], ix[2]});
                        }
                        if (r.tri_count == 0)
                            throw std::runtime_error("emissive mesh without triangles");
                        table_of[(uint32_t)m] = ti;
                    } else {
                        ti = it->second;
                    }
                    float intensity = (fbits(mat.rough_metal_normal_map_bits[3]) & PT_EMISSION_MAP_BIT)
                                          ? (float)textured_intensity(s, m, mat)
                                          : (float)(double)(((mat.emission[0] + mat.emission[1]) + mat.emission[2]) * mat.emission[3]);
                    weights.push_back(intensity);
                    values.push_back({PT_LIGHT_TYPE_EMITTER, 0u, (uint32_t)tw[ti].size(), s->mesh_instance_offset[m],
                                      s->mesh_instance_offset[m + 1] - s->mesh_instance_offset[m], 0u, 0u});
                }
                uint32_t bin_count = (uint32_t)(s->point_lights.size() / 6 + s->dir_lights.size() / 6 + tw.size());
                for (auto& val : values)
                    val[1] += bin_count * PT_LIGHT_BIN_SIZE;
                auto add_inf = [&](const std::vector<float>& L, uint32_t type) {
                    for (size_t i = 0; i + 6 <= L.size(); i += 6) {
                        weights.push_back((L[i + 3] + L[i + 4]) + L[i + 5]);
                        values.push_back({type, fbits(L[i]), fbits(L[i + 1]), fbits(L[i + 2]), fbits(L[i + 3]), fbits(L[i + 4]), fbits(L[i + 5])});
                    }
                };
                add_inf(s->point_lights, PT_LIGHT_TYPE_POINT);
                add_inf(s->dir_lights, PT_LIGHT_TYPE_DIRECTIONAL);
                append_alias(s->light, weights, values);
                s->light_count = (uint32_t)weights.size();
                for (size_t t = 0; t < tw.size(); t++)
                    append_alias(s->light, tw[t], tv[t]);
            }
            s->packed = true;
        }
        std::memset(v, 0, sizeof(*v));
        v->vertices = s->vertices.data();
        v->vertex_count = (uint32_t)(s->vertices.size() / PT_VERTEX_FLOATS);
        v->indices = s->indices.data();
        v->index_count = (uint32_t)s->indices.size();
        v->meshes = s->meshes.data();
        v->mesh_count = (uint32_t)s->meshes.size();
        v->instances = s->inst.data();
        v->instance_mesh = s->inst_mesh.data();
        v->instance_world_to_object = s->w2o.data();
        v->instance_opaque = s->opaque.data();
        v->instance_count = (uint32_t)s->inst.size();
        v->materials = s->materials.data();
        v->material_count = (uint32_t)s->materials.size();
        v->light_words = s->light.data();
        v->light_word_count = (uint32_t)s->light.size();
        v->light_count = s->light_count;
        std::memcpy(v->environment_colour, s->env, sizeof(s->env));
        v->texels = s->texels.data();
        v->texel_bytes = s->texels.size();
        v->textures = s->textures.data();
        v->texture_count = (uint32_t)s->textures.size();
        v->material_ior = s->material_ior.empty() ? nullptr : s->material_ior.data();
        return PT_OK;
    } catch (const std::exception& e) {
        g_error = e.what();
        return PT_ERR_INVALID;
    }
}

// Camera chain of the reference evaluated in FP64 and rounded once:
// basis Mat3(y, z, x) with x = normalize(lookdir), y = normalize(cross(up, x)),
// z = cross(x, y) (scenebuild.cpp:251-257); the uploaded inverse view is
// translate(-position) * R (camera.h:16 inverted back, pathtrace.cpp:387-388),
// so rays start at -position and look along -lookdir; the projection is
// perspective with depth in [0, 1] and y flipped (camera.cpp:21-26), aspect
// = width / height (main.cpp:98).
int pt_camera_params(const pt_camera_desc* c, uint32_t width, uint32_t height, pt_render_params* P)
{
    if (!c || !P || width == 0 || height == 0)
        return PT_ERR_INVALID;
    double x[3] = {c->lookdir[0], c->lookdir[1], c->lookdir[2]};
    double xl = std::sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
    if (!(xl > 0))
        return PT_ERR_INVALID;
    for (double& v : x)
        v /= xl;
    double y[3] = {c->up[1] * x[2] - c->up[2] * x[1], c->up[2] * x[0] - c->up[0] * x[2], c->up[0] * x[1] - c->up[1] * x[0]};
    double yl = std::sqrt(y[0] * y[0] + y[1] * y[1] + y[2] * y[2]);
    if (!(yl > 0))
        return PT_ERR_INVALID;
    for (double& v : y)
        v /= yl;
    double z[3] = {x[1] * y[2] - x[2] * y[1], x[2] * y[0] - x[0] * y[2], x[0] * y[1] - x[1] * y[0]};
    double iv[16] = {y[0], z[0], x[0], -(double)c->position[0], y[1], z[1], x[1], -(double)c->position[1],
                     y[2], z[2], x[2], -(double)c->position[2], 0, 0, 0, 1};
    double aspect = (double)((float)width / (float)height);
    double fov = (double)(c->fov_degrees * 0.01745329251994329576923690768489f);
    double th = std::tan(fov / 2.0);
    double n = c->near_plane, f = c->far_plane;
    double pr[16] = {1.0 / (aspect * th), 0, 0, 0, 0, -1.0 / th, 0, 0, 0, 0, f / (n - f), -(f * n) / (f - n), 0, 0, -1, 0};
    double ip[16];
    inverse4(pr, ip);
    for (int i = 0; i < 16; i++) {
        P->inv_view[i] = (float)iv[i];
        P->inv_proj[i] = (float)ip[i];
    }
    P->near_plane = c->near_plane;
    P->far_plane = c->far_plane;
    P->focus_dist = c->focus_dist;
    P->lens_radius = c->lens_radius;
    P->exposure = c->exposure;
    P->width = width;
    P->height = height;
    return PT_OK;
}

float pt_from_srgb(float x) { return from_srgb(x); }

// Scene::scene_details (scene.cpp:490-518)
int pt_scene_details(const pt_host_scene* s, char* buf, size_t len)
{
    if (!s || !buf || len == 0)
        return PT_ERR_INVALID;
    size_t uv = s->vertices.size() / PT_VERTEX_FLOATS, ut = s->indices.size() / 3, inst = 0, tris = 0, emit = 0;
    for (size_t m = 0; m < s->meshes.size(); m++) {
        size_t n = s->mesh_instance_offset[m + 1] - s->mesh_instance_offset[m];
        inst += n;
        tris += n * s->meshes[m].tri_count;
        emit += is_emitter(s->materials[s->mesh_material[m]]) ? n : 0;
    }
    int w = std::snprintf(buf, len,
                          "Scene has:\n    %zu meshes\n    %zu materials\n    %zu point lights\n    %zu directional lights\n"
                          "    %zu instances with emission\n    %zu textures\n    %zu instances\n    %zu unique vertices\n"
                          "    %zu unique triangles\n    %zu total triangles\n",
                          s->meshes.size(), s->materials.size(), s->point_lights.size() / 6, s->dir_lights.size() / 6, emit,
                          s->textures.size(), inst,
                          uv, ut, tris);
    return w < 0 ? PT_ERR_INVALID : PT_OK;
}

} // extern "C"
