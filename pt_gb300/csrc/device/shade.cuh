// shade.cuh — per-segment shading of pt's path tracer on the device.
//
// Restates pathtrace.ch.hlsl:159-360 (closest hit, NEE, BSDF sampling),
// pathtrace.ms.hlsl:6-11 (miss), lightsample.hlsli:13-143 (light sampling),
// geometry.hlsli:38-69 and pathtrace.hlsli:118-139 (Russian roulette,
// radiance correction) in the operation order of the HLSL source.
//
// The reference traces the NEE shadow ray in the middle of the closest-hit
// shader.  Here shading stops at that point and returns the shadow ray as a
// request; BSDF sampling (which does not depend on visibility) runs before
// the ray is traced, and finish_nee() later adds the light term with the
// throughput the reference used.  The radiance sum is therefore formed in the
// reference's order whether the shadow ray is traced inline (megakernel) or
// in a later stage (wavefront).
#pragma once
#include "scene.cuh"

namespace pt {

constexpr uint32_t LIGHT_BIN_SIZE = 10;
constexpr uint32_t EMITTER_BIN_SIZE = 6;
constexpr uint32_t LIGHT_TYPE_POINT = 1;
constexpr uint32_t LIGHT_TYPE_DIRECTIONAL = 2;
constexpr uint32_t LIGHT_TYPE_EMITTER = 3;
constexpr uint32_t NO_EMITTER_INDEX = 0xFFFFFFFFu;

// Path state of one pixel sample: the reference's RayPayload
// (pathtrace.hlsli:36-45) plus the next ray.
struct PathState {
    f3 throughput;
    f3 radiance;
    float brdf_pdf; // < 0 on the first ray
    bool final_segment;
    Sampler smp;
    f3 next_o, next_d;
};

// Terms of light_contribution() that remain once the shadow ray is known.
struct NeeRequest {
    f3 origin, dir;
    float tmax;
    f3 emission, brdf;
    float w, cos_i, pdf; // w < 0 marks a delta light
    f3 tp_before;        // path throughput the light term is weighted by
    bool add;            // the reference adds light_contribution() (maybe 0)
    bool trace;          // a shadow ray decides the contribution
};

__device__ __forceinline__ void add_radiance(PathState& p, f3 r) { p.radiance = p.radiance + p.throughput * r; }

// Vertex position for an index taken from the light stream.  The reference
// reads through robust buffer access (out-of-range reads return zero), which
// this reproduces instead of reading outside the vertex array.
__device__ __forceinline__ f3 vpos(const DevScene& s, uint64_t i)
{
    if (i >= (uint64_t)s.vertex_count)
        return mk3(0.0f, 0.0f, 0.0f);
    float4 a = ldg4(s.vertices + 2 * (size_t)i);
    return mk3(a.x, a.y, a.z);
}

struct VertexF {
    f3 p, n;
    f2 uv;
};
__device__ __forceinline__ VertexF vfetch(const DevScene& s, uint32_t i)
{
    float4 a = ldg4(s.vertices + 2 * (size_t)i);
    float4 b = ldg4(s.vertices + 2 * (size_t)i + 1);
    VertexF v;
    v.p = mk3(a.x, a.y, a.z);
    v.n = mk3(a.w, b.x, b.y);
    v.uv = f2{b.z, b.w};
    return v;
}

__device__ __forceinline__ f3 mul3_rows(float4 r0, float4 r1, float4 r2, f3 v)
{
    return mk3((r0.x * v.x + r0.y * v.y) + r0.z * v.z, (r1.x * v.x + r1.y * v.y) + r1.z * v.z, (r2.x * v.x + r2.y * v.y) + r2.z * v.z);
}
__device__ __forceinline__ f3 mul_point_rows(float4 r0, float4 r1, float4 r2, f3 p)
{
    return mk3(((r0.x * p.x + r0.y * p.y) + r0.z * p.z) + r0.w * 1.0f, ((r1.x * p.x + r1.y * p.y) + r1.z * p.z) + r1.w * 1.0f,
               ((r2.x * p.x + r2.y * p.y) + r2.z * p.z) + r2.w * 1.0f);
}

__device__ __forceinline__ uint32_t sample_alias_table(const DevScene& s, uint32_t bin_count, uint32_t bin_size, uint32_t table_offset,
                                                       float& u, float& p)
{
    float ub = u * __uint2float_rn(bin_count);
    uint32_t i = min(bin_count - 1, __float2uint_rz(ub));
    uint32_t bin_offset = table_offset + i * bin_size;
    u = fminf(ub - __uint2float_rn(i), JUST_BELOW_ONE);
    float q = __uint_as_float(lw(s, bin_offset + 1));
    if (u < q) {
        u = fminf(u / q, JUST_BELOW_ONE);
    } else {
        i = lw(s, bin_offset + 2);
        bin_offset = table_offset + i * bin_size;
        u = fminf((u - q) / (1.0f - q), JUST_BELOW_ONE);
    }
    p = __uint_as_float(lw(s, bin_offset + 0));
    return bin_offset + 3;
}

__device__ __forceinline__ float light_pdf(const DevScene& s, uint32_t emitter_index, uint32_t primitive_index)
{
    if (emitter_index == NO_EMITTER_INDEX)
        return 0.0f;
    uint32_t bin_offset = emitter_index * LIGHT_BIN_SIZE;
    float p = __uint_as_float(lw(s, bin_offset + 0));
    uint32_t light_type = lw(s, bin_offset + 3);
    if (light_type == LIGHT_TYPE_EMITTER) {
        uint32_t table_offset = lw(s, bin_offset + 4);
        bin_offset = table_offset + primitive_index * EMITTER_BIN_SIZE;
        p = p * __uint_as_float(lw(s, bin_offset + 0));
    }
    return p;
}

// Material getters of material.hlsli:23-102: a set map bit replaces the
// constant with the texture sampled at uv.
__device__ __forceinline__ uint32_t map_bits(const DevMaterial* m)
{
    return __float_as_uint(__ldg(&m->rmn.w));
}

__device__ __forceinline__ f3 material_emission(const DevScene& s, const DevMaterial* m, f2 uv)
{
    float4 e = ldg4(&m->emission);
    if (map_bits(m) & MAP_EMISSION) {
        float4 t = sample_texture(s, __float_as_uint(e.x), uv);
        return mk3(t.x, t.y, t.z) * e.w;
    }
    return mk3(e.x, e.y, e.z) * e.w;
}

__device__ __forceinline__ float4 material_base_colour(const DevScene& s, const DevMaterial* m, f2 uv)
{
    float4 bc = ldg4(&m->base_colour);
    return (map_bits(m) & MAP_BASE_COLOUR) ? sample_texture(s, __float_as_uint(bc.x), uv) : bc;
}

__device__ __forceinline__ void material_rough_metal_normal(const DevScene& s, const DevMaterial* m, f2 uv, float& roughness,
                                                            float& metalness, f3& normal)
{
    const float4 rmn = ldg4(&m->rmn);
    const uint32_t bits = __float_as_uint(rmn.w);
    if (bits & MAP_ROUGHNESS_METALNESS) {
        const float4 t = sample_texture(s, __float_as_uint(rmn.x), uv);
        roughness = t.y;
        metalness = t.z;
    } else {
        roughness = (bits & MAP_ROUGHNESS) ? sample_texture(s, __float_as_uint(rmn.x), uv).x : rmn.x;
        metalness = (bits & MAP_METALNESS) ? sample_texture(s, __float_as_uint(rmn.y), uv).x : rmn.y;
    }
    if (bits & MAP_NORMAL) {
        const float4 t = sample_texture(s, __float_as_uint(rmn.z), uv);
        normal = normalize(mk3(t.x * 2.0f - 1.0f, t.y * 2.0f - 1.0f, t.z * 2.0f - 1.0f));
    } else {
        normal = mk3(0.0f, 0.0f, 1.0f);
    }
}

__device__ __forceinline__ f3 material_rgb(const DevScene& s, const float4* field, bool mapped, f2 uv)
{
    const float4 v = ldg4(field);
    if (mapped) {
        const float4 t = sample_texture(s, __float_as_uint(v.x), uv);
        return mk3(t.x, t.y, t.z);
    }
    return mk3(v.x, v.y, v.z);
}

// onb (util.hlsli:57-64): orthonormal basis around n (Duff et al. 2017).
__device__ __forceinline__ void onb(f3 n, f3& x, f3& y)
{
    const float sg = n.z < 0.0f ? -1.0f : 1.0f;
    const float a = -1.0f / (sg + n.z);
    const float b = (n.x * n.y) * a;
    x = mk3(1.0f + ((sg * n.x) * n.x) * a, sg * b, -sg * n.x);
    y = mk3(b, sg + (n.y * n.y) * a, -n.y);
}

__device__ __forceinline__ f3 sample_light(const DevScene& s, Sampler& smp, f3 pt, f3& light_dir, float& light_dist, float& pdf,
                                           bool& is_delta)
{
    float ux = sample_1d(smp);
    f2 u12 = sample_2d(smp);
    uint32_t bin_offset = sample_alias_table(s, s.light_count, LIGHT_BIN_SIZE, 0, ux, pdf);
    uint32_t light_type = lw(s, bin_offset + 0);
    if (light_type == LIGHT_TYPE_EMITTER) {
        uint32_t table_offset = lw(s, bin_offset + 1);
        uint32_t tri_count = lw(s, bin_offset + 2);
        uint32_t instance_offset = lw(s, bin_offset + 3);
        uint32_t instance_count = lw(s, bin_offset + 4);
        float p;
        bin_offset = sample_alias_table(s, tri_count, EMITTER_BIN_SIZE, table_offset, ux, p);
        pdf = pdf * p;
        uint32_t instance_id = instance_offset + min(instance_count - 1, __float2uint_rz(ux * __uint2float_rn(instance_count)));
        if (instance_id >= s.instance_count) {
            // outside the instance buffer: robust access yields no light
            light_dist = 0.0f;
            is_delta = true;
            return mk3(0.0f, 0.0f, 0.0f);
        }
        const DevInstanceData* id = s.inst_data + instance_id;
        float4 t0 = ldg4(&id->t0), t1 = ldg4(&id->t1), t2 = ldg4(&id->t2);
        uint32_t vbase = __ldg(&id->vertex_index);
        f3 pa = mul_point_rows(t0, t1, t2, vpos(s, (uint64_t)vbase + lw(s, bin_offset + 0)));
        f3 pb = mul_point_rows(t0, t1, t2, vpos(s, (uint64_t)vbase + lw(s, bin_offset + 1)));
        f3 pc = mul_point_rows(t0, t1, t2, vpos(s, (uint64_t)vbase + lw(s, bin_offset + 2)));
        f3 bary = random_barycentric(u12);
        f3 point = (bary.x * pa + bary.y * pb) + bary.z * pc;
        const unsigned long long ia = (unsigned long long)vbase + lw(s, bin_offset + 0);
        const unsigned long long ib = (unsigned long long)vbase + lw(s, bin_offset + 1);
        const unsigned long long ic = (unsigned long long)vbase + lw(s, bin_offset + 2);
        light_dir = point - pt;
        light_dist = 1.0f;
        f3 tn = cross(pb - pa, pc - pa);
        float area = sqrtf(dot(tn, tn)) * 0.5f;
        float cosine = fabsf(dot(normalize(light_dir), normalize(tn)));
        float dist2 = dot(light_dir, light_dir);
        pdf = pdf * (dist2 / (area * cosine));
        is_delta = false;
        if (!isfinite(pdf))
            return mk3(0.0f, 0.0f, 0.0f);
        // lightsample.hlsli:106-108: emission at the point's texture coordinate
        const DevMaterial* lm = s.materials + __ldg(&id->material_index);
        f2 luv = {0.0f, 0.0f};
        if (map_bits(lm) & MAP_EMISSION) {
            const f2 ua = vertex_uv(s, ia), ub = vertex_uv(s, ib), uc = vertex_uv(s, ic);
            luv = f2{(bary.x * ua.x + bary.y * ub.x) + bary.z * uc.x, (bary.x * ua.y + bary.y * ub.y) + bary.z * uc.y};
        }
        return material_emission(s, lm, luv);
    } else if (light_type == LIGHT_TYPE_POINT) {
        f3 lp = mk3(__uint_as_float(lw(s, bin_offset + 1)), __uint_as_float(lw(s, bin_offset + 2)), __uint_as_float(lw(s, bin_offset + 3)));
        light_dir = lp - pt;
        light_dist = 1.0f;
        is_delta = true;
        f3 col = mk3(__uint_as_float(lw(s, bin_offset + 4)), __uint_as_float(lw(s, bin_offset + 5)), __uint_as_float(lw(s, bin_offset + 6)));
        return (1.0f / dot(light_dir, light_dir)) * col;
    } else if (light_type == LIGHT_TYPE_DIRECTIONAL) {
        light_dir = mk3(__uint_as_float(lw(s, bin_offset + 1)), __uint_as_float(lw(s, bin_offset + 2)), __uint_as_float(lw(s, bin_offset + 3)));
        light_dist = __int_as_float(0x7f800000);
        is_delta = true;
        return mk3(__uint_as_float(lw(s, bin_offset + 4)), __uint_as_float(lw(s, bin_offset + 5)), __uint_as_float(lw(s, bin_offset + 6)));
    }
    light_dist = 0.0f;
    is_delta = true;
    return mk3(0.0f, 0.0f, 0.0f);
}

// Miss shader (pathtrace.ms.hlsl:6-11).
// First-hit features for the denoiser: base colour and the interpolated
// shading normal in world space, turned to face the ray.
__device__ __forceinline__ void hit_features(const DevScene& s, const Hit& h, f3 rd, f3& albedo, f3& normal)
{
    const DevInstanceData* id = s.inst_data + h.inst;
    const DevMaterial* mat = s.materials + __ldg(&id->material_index);
    const uint32_t vbase = __ldg(&id->vertex_index), ibase = __ldg(&id->index_index);
    const uint32_t i0 = __ldg(s.indices + ibase + h.prim * 3 + 0);
    const uint32_t i1 = __ldg(s.indices + ibase + h.prim * 3 + 1);
    const uint32_t i2 = __ldg(s.indices + ibase + h.prim * 3 + 2);
    VertexF va = vfetch(s, vbase + i0), vb = vfetch(s, vbase + i1), vc = vfetch(s, vbase + i2);
    const float ba = (1.0f - h.b1) - h.b2;
    f3 on = normalize((ba * va.n + h.b1 * vb.n) + h.b2 * vc.n);
    float4 n0 = ldg4(&id->n0), n1 = ldg4(&id->n1), n2 = ldg4(&id->n2);
    normal = normalize(mul3_rows(n0, n1, n2, on));
    if (dot(normal, rd) > 0.0f)
        normal = -normal;
    const f2 uv = {(ba * va.uv.x + h.b1 * vb.uv.x) + h.b2 * vc.uv.x, (ba * va.uv.y + h.b1 * vb.uv.y) + h.b2 * vc.uv.y};
    const float4 bc = material_base_colour(s, mat, uv);
    albedo = mk3(bc.x, bc.y, bc.z);
}

// Running mean of a feature vector, the image's accumulation rule.
__device__ __forceinline__ void feature_mean(float4& acc, float4 v, uint32_t si)
{
    if (si == 0) {
        acc = v;
    } else {
        float n = __uint2float_rn(si + 1u);
        acc.x = acc.x + (v.x - acc.x) / n;
        acc.y = acc.y + (v.y - acc.y) / n;
        acc.z = acc.z + (v.z - acc.z) / n;
        acc.w = acc.w + (v.w - acc.w) / n;
    }
}

__device__ __forceinline__ void shade_miss(const DevScene& s, PathState& pl)
{
    add_radiance(pl, s.env);
    pl.final_segment = true;
}

// Smooth dielectric: an extension of this library (the reference's BSDF has
// no refraction).  `o` is the direction to the viewer in the shading frame
// (o.z > 0), eta = index on the viewer's side / index on the far side.  The
// Fresnel reflectance of unpolarised light, F = (r_s^2 + r_p^2) / 2, picks
// reflection (probability F) or refraction, so the chosen lobe's weight is 1;
// refraction multiplies the throughput by the base colour (tint) and by eta^2
// (radiance is scaled by the squared index ratio across an interface; the
// factors cancel over a way in and out).  Total internal reflection gives
// F = 1.  One sampler dimension is used.  The next ray leaves from the side
// of the geometric normal `twn` (facing the viewer) it travels to.
__device__ __forceinline__ void shade_dielectric(PathState& pl, f3 tint, float eta, f3 o, f3 wx, f3 wy, f3 wn, f3 twn, f3 hit)
{
    const float cos_i = o.z;
    const float sin2_t = (eta * eta) * (1.0f - cos_i * cos_i);
    float F = 1.0f, cos_t = 0.0f;
    if (sin2_t < 1.0f) {
        cos_t = sqrtf(1.0f - sin2_t);
        const float rs = (eta * cos_i - cos_t) / (eta * cos_i + cos_t);
        const float rp = (cos_i - eta * cos_t) / (cos_i + eta * cos_t);
        F = 0.5f * (rs * rs + rp * rp);
    }
    f3 i;
    if (sample_1d(pl.smp) < F) {
        i = mk3(-o.x, -o.y, o.z);
        pl.next_o = hit + twn * ORIGIN_OFFSET;
    } else {
        i = mk3(-eta * o.x, -eta * o.y, -cos_t);
        pl.throughput = pl.throughput * (tint * (eta * eta));
        pl.next_o = hit - twn * ORIGIN_OFFSET;
    }
    pl.brdf_pdf = -1.0f; // a delta lobe: emission reached next counts in full
    f3 wi = mk3((wx.x * i.x + wy.x * i.y) + wn.x * i.z, (wx.y * i.x + wy.y * i.y) + wn.y * i.z, (wx.z * i.x + wy.z * i.y) + wn.z * i.z);
    pl.next_d = normalize(wi);
}

// Closest-hit shader (pathtrace.ch.hlsl:227-360) without the shadow ray.
// The NEE request is handed to `nee_out(pl, request)` as soon as it is
// formed, before the BSDF is sampled (nothing after it changes the radiance),
// so a caller that stores it at once does not carry it through the rest of
// the shader; it is not called when the shader ends before the light term.
template <class NeeOut>
__device__ __forceinline__ void shade_hit(const DevScene& s, PathState& pl, f3 ray_o, f3 ray_d, const Hit& h, NeeOut& nee_out)
{
    NeeRequest nee;
    nee.add = false;
    nee.trace = false;
    PT_CHECK_INDEX(h.inst < s.instance_count, s, {
        pl.final_segment = true;
        return;
    })
    const DevInstanceData* id = s.inst_data + h.inst;
    const DevInstance* di = s.dinst + h.inst;
    uint32_t vbase = __ldg(&id->vertex_index);
    uint32_t ibase = __ldg(&id->index_index);
    uint32_t emitter_index = __ldg(&id->emitter_index);
    const DevMaterial* mat = s.materials + __ldg(&id->material_index);
    PT_CHECK_INDEX((uint64_t)ibase + 3ull * h.prim + 3ull <= s.index_count, s, {
        pl.final_segment = true;
        return;
    })
    uint32_t i0 = __ldg(s.indices + ibase + h.prim * 3 + 0);
    uint32_t i1 = __ldg(s.indices + ibase + h.prim * 3 + 1);
    uint32_t i2 = __ldg(s.indices + ibase + h.prim * 3 + 2);
    PT_CHECK_INDEX((uint64_t)vbase + i0 < s.vertex_count && (uint64_t)vbase + i1 < s.vertex_count &&
                       (uint64_t)vbase + i2 < s.vertex_count,
                   s, {
                       pl.final_segment = true;
                       return;
                   })
    VertexF va = vfetch(s, vbase + i0), vb = vfetch(s, vbase + i1), vc = vfetch(s, vbase + i2);

    float ba = (1.0f - h.b1) - h.b2;
    f3 obj_normal = normalize((ba * va.n + h.b1 * vb.n) + h.b2 * vc.n);
    const f2 uv = {(ba * va.uv.x + h.b1 * vb.uv.x) + h.b2 * vc.uv.x, (ba * va.uv.y + h.b1 * vb.uv.y) + h.b2 * vc.uv.y};

    f3 emission = material_emission(s, mat, uv);
    if (maxc(emission) > 0.0f) {
        float4 w0 = ldg4(&di->w2o[0]), w1 = ldg4(&di->w2o[1]), w2 = ldg4(&di->w2o[2]);
        f3 obj_dir = mul3_rows(w0, w1, w2, ray_d);
        if (dot(obj_dir, obj_normal) < 0.0f) {
            if (pl.brdf_pdf < 0.0f) {
                add_radiance(pl, emission);
            } else {
                float4 t0 = ldg4(&id->t0), t1 = ldg4(&id->t1), t2 = ldg4(&id->t2);
                f3 wab = mul3_rows(t0, t1, t2, vb.p - va.p);
                f3 wac = mul3_rows(t0, t1, t2, vc.p - va.p);
                f3 en = cross(wab, wac);
                float area = sqrtf(dot(en, en)) * 0.5f;
                float dist2 = h.t * h.t;
                float cosine = fabsf(dot(ray_d, normalize(en)));
                float pdf_l = light_pdf(s, emitter_index, h.prim);
                pdf_l = pdf_l * (dist2 / (area * cosine));
                if (pdf_l > 0.0f && dist2 > 0.0f) {
                    float w = pl.brdf_pdf / (pl.brdf_pdf + pdf_l);
                    add_radiance(pl, w * emission);
                }
            }
        }
    }
    if (pl.final_segment)
        return;

    const float4 bc = material_base_colour(s, mat, uv);
    if (bc.w < sample_1d(pl.smp)) {
        pl.next_o = ray_o + ray_d * (h.t + ORIGIN_OFFSET);
        pl.next_d = ray_d;
        return;
    }
    const uint32_t bits = map_bits(mat);
    float anisotropy = __ldg(&mat->cc.z);
    BrdfInput bi;
    bi.base_colour = mk3(bc.x, bc.y, bc.z);
    float roughness;
    f3 mapped_normal;
    material_rough_metal_normal(s, mat, uv, roughness, bi.metalness, mapped_normal);
    bi.specular = material_rgb(s, &mat->specular, (bits & MAP_SPECULAR) != 0, uv);
    bi.sheen = material_rgb(s, &mat->sheen, (bits & MAP_SHEEN) != 0, uv);
    roughness = fmaxf(0.00001f, roughness * roughness);
    float aspect = sqrtf(1.0f - 0.9f * fabsf(anisotropy));
    bi.alpha = f2{roughness / aspect, roughness * aspect};
    if (anisotropy < 0.0f)
        bi.alpha = f2{bi.alpha.y, bi.alpha.x};

    // get_vertex_vectors (geometry.hlsli:49-69)
    f2 duv_ab = {vb.uv.x - va.uv.x, vb.uv.y - va.uv.y};
    f2 duv_ac = {vc.uv.x - va.uv.x, vc.uv.y - va.uv.y};
    f3 ab = vb.p - va.p, ac = vc.p - va.p;
    f3 true_obj_normal = cross(ab, ac);
    float denom = duv_ab.x * duv_ac.y - duv_ac.x * duv_ab.y;
    f3 tangent;
    if (fabsf(denom) < 1e-5f) {
        tangent = cross(obj_normal, fabsf(obj_normal.y) > 1e-5f ? mk3(1.0f, 0.0f, 0.0f) : mk3(0.0f, 1.0f, 0.0f));
    } else {
        tangent = (duv_ac.y * ab - duv_ab.y * ac) / denom;
        tangent = tangent - dot(tangent, obj_normal) * obj_normal;
    }
    f3 bitangent = cross(obj_normal, tangent);

    float4 n0 = ldg4(&id->n0), n1 = ldg4(&id->n1), n2 = ldg4(&id->n2);
    f3 wx = normalize(mul3_rows(n0, n1, n2, tangent));
    f3 wy = normalize(mul3_rows(n0, n1, n2, bitangent));
    f3 wn = normalize(mul3_rows(n0, n1, n2, obj_normal));
    const bool back_face = dot(wn, ray_d) > 0.0f; // the side the vertex normals point away from
    if (back_face) {
        wx = -wx;
        wy = -wy;
        wn = -wn;
    }
    f3 twn = normalize(mul3_rows(n0, n1, n2, true_obj_normal));
    if (dot(ray_d, twn) > 0.0f)
        twn = -twn;
    // mapped normal (pathtrace.ch.hlsl:321-326): rows of the world-to-shading
    // matrix become float3x3(mx, my, mn) x float3x3(wx, wy, wn)
    if (mapped_normal.z < 0.999f) {
        f3 mx, my;
        onb(mapped_normal, mx, my);
        const f3 rx = (mx.x * wx + mx.y * wy) + mx.z * wn;
        const f3 ry = (my.x * wx + my.y * wy) + my.z * wn;
        const f3 rn = (mapped_normal.x * wx + mapped_normal.y * wy) + mapped_normal.z * wn;
        wx = rx;
        wy = ry;
        wn = rn;
    }
    f3 nd = -ray_d;
    f3 o = normalize(mk3(dot(wx, nd), dot(wy, nd), dot(wn, nd)));
    if (o.z <= 0.0f) {
        pl.final_segment = true;
        return;
    }
    const f3 hit = ray_o + ray_d * h.t;
    if (s.material_ior) {
        const float ior = __ldg(s.material_ior + __ldg(&id->material_index));
        if (ior > 0.0f) {
            shade_dielectric(pl, bi.base_colour, back_face ? ior : 1.0f / ior, o, wx, wy, wn, twn, hit);
            return;
        }
    }
    f3 ip = hit + twn * ORIGIN_OFFSET;

    // light_contribution (pathtrace.ch.hlsl:159-225) up to the shadow ray.
    nee.add = true;
    nee.tp_before = pl.throughput;
    if (s.light_count != 0) {
        float pdf, light_dist;
        f3 light_dir;
        bool is_delta;
        f3 le = sample_light(s, pl.smp, ip, light_dir, light_dist, pdf, is_delta);
        if (maxc(le) > 0.0f) {
            f3 li = mk3(dot(wx, light_dir), dot(wy, light_dir), dot(wn, light_dir));
            if (li.z > 0.0f) {
                li = normalize(li);
                f3 m = normalize(li + o);
                float pdf_brdf;
                f3 brdf = evaluate_brdf(bi, li, o, m, pdf_brdf);
                nee.trace = true;
                nee.origin = ip;
                nee.dir = light_dir;
                nee.tmax = light_dist - 1e-5f;
                nee.emission = le;
                nee.brdf = brdf;
                nee.w = is_delta ? -1.0f : pdf / (pdf + pdf_brdf);
                nee.cos_i = cos_theta(li);
                nee.pdf = pdf;
            }
        }
    }
    nee_out(pl, nee);

    f3 m;
    float w, pdf;
    f3 i = sample_direction(o, bi.alpha, bi.metalness, pl.smp, m, w, pdf);
    if (i.z * o.z <= 0.0f) {
        pl.final_segment = true;
        return;
    }
    float pdf_brdf;
    f3 brdf = evaluate_brdf(bi, i, o, m, pdf_brdf);
    f3 tp = ((w * brdf) * cos_theta(i)) / pdf;
    pl.brdf_pdf = pdf_brdf;
    pl.throughput = pl.throughput * tp;
    f3 wi = mk3((wx.x * i.x + wy.x * i.y) + wn.x * i.z, (wx.y * i.x + wy.y * i.y) + wn.y * i.z, (wx.z * i.x + wy.z * i.y) + wn.z * i.z);
    pl.next_o = ip;
    pl.next_d = normalize(wi);
}

// shade_hit's NEE output for a caller that traces the shadow ray itself
// after the shader: the request is kept.
struct NeeKeep {
    NeeRequest& r;
    __device__ __forceinline__ void operator()(PathState&, const NeeRequest& n) { r = n; }
};

// Adds light_contribution() to the path radiance given the shadow ray's
// visibility (1 = unoccluded opaque path, 0 = occluded).
__device__ __forceinline__ void finish_nee(f3& radiance, const NeeRequest& nee, float vis)
{
    if (!nee.add)
        return;
    f3 L = mk3(0.0f, 0.0f, 0.0f);
    if (nee.trace && vis != 0.0f) {
        f3 e = nee.emission * vis;
        if (nee.w < 0.0f)
            L = ((e * nee.brdf) * nee.cos_i) / nee.pdf;
        else
            L = (((nee.w * e) * nee.brdf) * nee.cos_i) / nee.pdf;
    }
    radiance = radiance + nee.tp_before * L;
}

__device__ __forceinline__ bool russian_roulette(PathState& pl)
{
    f3 T = pl.throughput;
    float mt = fmaxf(fmaxf(T.x, T.y), T.z);
    float u = sample_1d(pl.smp);
    if (mt < 1.0f) {
        float q = fmaxf(0.0f, 1.0f - mt);
        if (u < q)
            return true;
        float sc = 1.0f / (1.0f - q);
        pl.throughput = pl.throughput * sc;
    }
    return false;
}

__device__ __forceinline__ f3 correct_radiance(f3 r)
{
    if (r.x < 0.0f || !isfinite(r.x))
        r.x = 0.0f;
    if (r.y < 0.0f || !isfinite(r.y))
        r.y = 0.0f;
    if (r.z < 0.0f || !isfinite(r.z))
        r.z = 0.0f;
    return r;
}

} // namespace pt
