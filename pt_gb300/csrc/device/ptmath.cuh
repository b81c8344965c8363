// ptmath.cuh — float vector math and the sampler of pt's shaders, on the device.
//
// Every expression is written in the operation order of the HLSL source
// (shaders/pathtrace/*.hlsl(i)) and this file is compiled with -fmad=false,
// so no multiply-add is fused: the device computes exactly what the CPU
// oracle computes, bit for bit.  Fused multiply-adds appear only where they
// are spelled out (fmaf in the conservative box test, where they cannot change
// a result).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace pt {

struct f2 { float x, y; };
struct f3 { float x, y, z; };

__host__ __device__ __forceinline__ f3 mk3(float x, float y, float z) { return f3{x, y, z}; }
__host__ __device__ __forceinline__ f3 operator+(f3 a, f3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__host__ __device__ __forceinline__ f3 operator-(f3 a, f3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__host__ __device__ __forceinline__ f3 operator-(f3 a) { return {-a.x, -a.y, -a.z}; }
__host__ __device__ __forceinline__ f3 operator*(f3 a, f3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
__host__ __device__ __forceinline__ f3 operator*(f3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__host__ __device__ __forceinline__ f3 operator*(float s, f3 a) { return {s * a.x, s * a.y, s * a.z}; }
__host__ __device__ __forceinline__ f3 operator/(f3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
__host__ __device__ __forceinline__ float dot(f3 a, f3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
__host__ __device__ __forceinline__ f3 cross(f3 a, f3 b)
{
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
// normalize(v) = v * (1 / sqrt(dot(v, v))), IEEE sqrt and division.
__device__ __forceinline__ f3 normalize(f3 v)
{
    float inv = 1.0f / sqrtf(dot(v, v));
    return v * inv;
}
__device__ __forceinline__ float maxc(f3 v) { return fmaxf(fmaxf(v.x, v.y), v.z); }
__device__ __forceinline__ float comp(f3 v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }
__device__ __forceinline__ float lerpf(float x, float y, float s) { return x + s * (y - x); }
__device__ __forceinline__ f3 lerp3(f3 x, f3 y, float s) { return {lerpf(x.x, y.x, s), lerpf(x.y, y.y, s), lerpf(x.z, y.z, s)}; }
__device__ __forceinline__ float sq(float x) { return x * x; }
__device__ __forceinline__ float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }

constexpr float PI_F = 3.141592654f;                   // util.hlsli:3
constexpr float JUST_BELOW_ONE = 0.99999994039535522f; // asfloat(0x3F7FFFFF)
constexpr float ORIGIN_OFFSET = 1e-5f;                 // pathtrace.hlsli:6

// ---------------------------------------------------------------- sin / cos
// Cody & Waite (1980) reduction by pi/2 with a three-part constant, then
// Taylor polynomials of sin and cos on [-pi/4, pi/4] by Horner's rule.  The
// CPU oracle implements the same method with the same constants, so both
// produce identical bits.  Valid for |x| <= 1e4; non-finite input gives NaN.
namespace sc {
constexpr float TWO_OVER_PI = 0.636619746685028076f;
constexpr float PIO2_HI = 1.5707855224609375f;
constexpr float PIO2_MID = 1.0804273188114166e-05f;
constexpr float PIO2_LO = 6.077094383272197e-11f;
constexpr float S3 = -0.16666667163372040f;
constexpr float S5 = 0.0083333337679505348f;
constexpr float S7 = -0.00019841270113829523f;
constexpr float S9 = 2.7557318844628753e-06f;
constexpr float C2 = -0.5f;
constexpr float C4 = 0.041666667908430099f;
constexpr float C6 = -0.0013888889225199819f;
constexpr float C8 = 2.4801587642286904e-05f;
constexpr float C10 = -2.7557319981497130e-07f;

__device__ __forceinline__ float reduce(float x, int* q)
{
    float k = rintf(x * TWO_OVER_PI);
    float r = ((x - k * PIO2_HI) - k * PIO2_MID) - k * PIO2_LO;
    *q = ((int)k) & 3;
    return r;
}
__device__ __forceinline__ float sin_poly(float r)
{
    float r2 = r * r;
    float p = S9;
    p = p * r2 + S7;
    p = p * r2 + S5;
    p = p * r2 + S3;
    return r + (r * r2) * p;
}
__device__ __forceinline__ float cos_poly(float r)
{
    float r2 = r * r;
    float p = C10;
    p = p * r2 + C8;
    p = p * r2 + C6;
    p = p * r2 + C4;
    p = p * r2 + C2;
    return 1.0f + r2 * p;
}
} // namespace sc

__device__ __forceinline__ float pt_sin(float x)
{
    if (!isfinite(x))
        return x - x;
    int q;
    float r = sc::reduce(x, &q);
    float s = (q & 1) ? sc::cos_poly(r) : sc::sin_poly(r);
    return (q & 2) ? -s : s;
}
__device__ __forceinline__ float pt_cos(float x)
{
    if (!isfinite(x))
        return x - x;
    int q;
    float r = sc::reduce(x, &q);
    float c = (q & 1) ? sc::sin_poly(r) : sc::cos_poly(r);
    return ((q + 1) & 2) ? -c : c;
}

// ---------------------------------------------------------------- sampler
// Owen-scrambled Sobol' sampler of shaders/pathtrace/sample.hlsli:94-166
// (Burley 2020 with the Laine-Karras permutation).  The 4x32 direction
// numbers come from the host (Joe & Kuo's primitive polynomials) as byte
// tables (g_sobol_bytes below, one copy per translation unit).

__device__ __forceinline__ uint32_t hash_combine(uint32_t seed, uint32_t x) { return seed ^ (x + (seed << 6) + (seed >> 2)); }
__device__ __forceinline__ uint32_t hash32(uint32_t x)
{
    x ^= x >> 16;
    x *= 0x85ebca6bu;
    x ^= x >> 13;
    x *= 0xc2b2ae35u;
    x ^= x >> 16;
    return x;
}
__device__ __forceinline__ uint32_t lk_permutation(uint32_t x, uint32_t seed)
{
    x += seed;
    x ^= x * 0x6c50b47cu;
    x ^= x * 0xb82f1e52u;
    x ^= x * 0xc7afe638u;
    x ^= x * 0x8d22f6e6u;
    return x;
}
__device__ __forceinline__ uint32_t scramble(uint32_t x, uint32_t seed) { return __brev(lk_permutation(__brev(x), seed)); }
// The Sobol' point of dimension `dim` (< 4) is the XOR of the direction
// numbers dir[dim][b] over the set bits b of the index.  XOR is
// associative, so it is taken a byte at a time from tables holding, for each
// byte position k and byte value v, the XOR over v's set bits j of
// dir[dim][8k + j]: four L1-resident loads instead of a 32-step loop over
// the (scrambled, so full-width) index.  Filled per translation unit from the
// same direction numbers (sobol_byte_tables).
static __device__ uint32_t g_sobol_bytes[4][4][256];

__host__ inline void sobol_byte_tables(const uint32_t* table128, uint32_t (*out)[4][256])
{
    for (int d = 0; d < 4; d++)
        for (int k = 0; k < 4; k++)
            for (int v = 0; v < 256; v++) {
                uint32_t x = 0;
                for (int j = 0; j < 8; j++)
                    if (v & (1 << j))
                        x ^= table128[d * 32 + 8 * k + j];
                out[d][k][v] = x;
            }
}

__device__ __forceinline__ uint32_t sobol(uint32_t index, uint32_t dim)
{
    const uint32_t* t = &g_sobol_bytes[dim][0][0];
    return (__ldg(t + (index & 255u)) ^ __ldg(t + 256u + ((index >> 8) & 255u))) ^
           (__ldg(t + 512u + ((index >> 16) & 255u)) ^ __ldg(t + 768u + (index >> 24)));
}

struct Sampler {
    uint32_t index, seed, dimension, shuffled;
};
constexpr uint32_t SOBOL_MAX_DIMENSION = 4;

__device__ __forceinline__ void sampler_start(Sampler& s, uint32_t px, uint32_t py, uint32_t sample_index, uint32_t seed)
{
    s.seed = hash_combine(seed, hash_combine(px, py));
    s.index = sample_index;
    s.dimension = SOBOL_MAX_DIMENSION;
    s.shuffled = 0;
}
__device__ __forceinline__ void sampler_pad(Sampler& s)
{
    s.dimension = 0;
    s.seed = hash32(s.seed);
    s.shuffled = scramble(s.index, s.seed);
}
__device__ __forceinline__ float u32_to_unit(uint32_t x)
{
    float r = 0x1p-32f * __uint2float_rn(x);
    return fminf(r, JUST_BELOW_ONE);
}
__device__ __forceinline__ float sample_1d(Sampler& s)
{
    if (s.dimension >= SOBOL_MAX_DIMENSION)
        sampler_pad(s);
    float r = u32_to_unit(scramble(sobol(s.shuffled, s.dimension), hash_combine(s.seed, s.dimension)));
    s.dimension += 1;
    return r;
}
__device__ __forceinline__ f2 sample_2d(Sampler& s)
{
    if (s.dimension + 1 >= SOBOL_MAX_DIMENSION)
        sampler_pad(s);
    f2 r;
    r.x = u32_to_unit(scramble(sobol(s.shuffled, s.dimension + 0), hash_combine(s.seed, s.dimension + 0)));
    r.y = u32_to_unit(scramble(sobol(s.shuffled, s.dimension + 1), hash_combine(s.seed, s.dimension + 1)));
    s.dimension += 2;
    return r;
}

// ---------------------------------------------------------------- warps (sample.hlsli:193-246)
__device__ __forceinline__ f3 cosine_weighted_rand_dir(f2 u)
{
    float su = sqrtf(u.x);
    float x = su * pt_cos((2.0f * PI_F) * u.y);
    float y = su * pt_sin((2.0f * PI_F) * u.y);
    float z = sqrtf(1.0f - u.x);
    return {x, y, z};
}
__device__ __forceinline__ f3 random_barycentric(f2 u)
{
    float beta = 1.0f - sqrtf(u.x);
    float gamma = (1.0f - beta) * u.y;
    float alpha = (1.0f - beta) - gamma;
    return {alpha, beta, gamma};
}
__device__ __forceinline__ f2 sample_concentric_disk(f2 u)
{
    float a = 2.0f * u.x - 1.0f;
    float b = 2.0f * u.y - 1.0f;
    float r, phi;
    if (a * a > b * b) {
        r = a;
        phi = (PI_F / 4.0f) * (b / a);
    } else {
        r = b;
        phi = (PI_F / 2.0f) - (PI_F / 4.0f) * (a / b);
    }
    return {r * pt_cos(phi), r * pt_sin(phi)};
}
__device__ __forceinline__ f3 sample_visible_micronormal(f3 v, f2 alpha, f2 u)
{
    v = normalize(mk3(alpha.x * v.x, alpha.y * v.y, v.z));
    f3 x = (v.z < 0.99999f) ? normalize(cross(mk3(0.0f, 0.0f, 1.0f), v)) : mk3(1.0f, 0.0f, 0.0f);
    f3 y = cross(v, x);
    float a = 1.0f / (1.0f + v.z);
    float r = sqrtf(u.x);
    float phi = (u.y < a) ? (u.y / a) * PI_F : PI_F + ((u.y - a) / (1.0f - a)) * PI_F;
    float p1 = r * pt_cos(phi);
    float p2 = (r * pt_sin(phi)) * ((u.y < a) ? 1.0f : v.z);
    float s = sqrtf(fmaxf(0.0f, (1.0f - p1 * p1) - p2 * p2));
    f3 m = (p1 * x + p2 * y) + s * v;
    return normalize(mk3(alpha.x * m.x, alpha.y * m.y, fmaxf(1e-6f, m.z)));
}

// ---------------------------------------------------------------- BSDF (pathtrace.ch.hlsl:22-157)
__device__ __forceinline__ float cos_theta(f3 v) { return v.z; }
__device__ __forceinline__ float cos2_theta(f3 v) { return sq(cos_theta(v)); }
__device__ __forceinline__ float sin2_theta(f3 v) { return fmaxf(0.0f, 1.0f - cos2_theta(v)); }
__device__ __forceinline__ float sin_theta(f3 v) { return sqrtf(sin2_theta(v)); }
__device__ __forceinline__ float tan2_theta(f3 v) { return sin2_theta(v) / cos2_theta(v); }

struct BrdfInput {
    f3 base_colour;
    f2 alpha;
    float metalness;
    f3 specular;
    f3 sheen;
};

__device__ __forceinline__ float fresnel_schlick(float cos_d)
{
    float b = 1.0f - cos_d;
    return (((b * b) * b) * b) * b;
}
__device__ __forceinline__ float lambda_fn(f3 m, f2 alpha)
{
    float tan2 = tan2_theta(m);
    if (isinf(tan2))
        return 0.0f;
    float s = sin_theta(m);
    float cos_phi = s == 0.0f ? 1.0f : clampf(m.x / s, -1.0f, 1.0f);
    float sin_phi = s == 0.0f ? 0.0f : clampf(m.y / s, -1.0f, 1.0f);
    float alpha2 = sq(cos_phi * alpha.x) + sq(sin_phi * alpha.y);
    return (sqrtf(1.0f + alpha2 * tan2) - 1.0f) / 2.0f;
}
__device__ __forceinline__ float g1_fn(f3 v, f2 alpha) { return 1.0f / (1.0f + lambda_fn(v, alpha)); }
__device__ __forceinline__ float masking(f3 o, f3 i, f2 alpha) { return 1.0f / ((1.0f + lambda_fn(o, alpha)) + lambda_fn(i, alpha)); }
__device__ __forceinline__ float distribution(f3 m, f2 alpha)
{
    float tan2 = tan2_theta(m);
    if (isinf(tan2))
        return 0.0f;
    float cos4 = sq(cos2_theta(m));
    float s = sin_theta(m);
    float cos_phi = s == 0.0f ? 1.0f : clampf(m.x / s, -1.0f, 1.0f);
    float sin_phi = s == 0.0f ? 0.0f : clampf(m.y / s, -1.0f, 1.0f);
    float e = tan2 * (sq(cos_phi / alpha.x) + sq(sin_phi / alpha.y));
    return 1.0f / ((((PI_F * alpha.x) * alpha.y) * cos4) * sq(1.0f + e));
}
__device__ __forceinline__ float diffuse_sample_probability(float metalness) { return lerpf(0.5f, 0.0f, metalness); }

__device__ __forceinline__ f3 evaluate_brdf(const BrdfInput& in, f3 i, f3 o, f3 m, float& pdf)
{
    f3 f0 = lerp3(in.specular * 0.08f, in.base_colour, in.metalness);
    float cos_d = dot(m, o);
    float f = fresnel_schlick(cos_d);
    float g = masking(o, i, in.alpha);
    float d = distribution(m, in.alpha);
    f3 lf = lerp3(f0, mk3(1.0f, 1.0f, 1.0f), f);
    float denom = (4.0f * cos_theta(i)) * cos_theta(o);
    f3 specular = ((d * lf) * g) / denom;
    f3 sheen = in.sheen * f;
    f3 diffuse = (((1.0f - in.metalness) * (in.base_colour + sheen)) / PI_F) * (1.0f - f);
    // The reference evaluates a clearcoat lobe but never adds it to the
    // result (pathtrace.ch.hlsl:93-100,114); it is omitted.
    float diffuse_prob = diffuse_sample_probability(in.metalness);
    float pdf_diffuse = cos_theta(i) / PI_F;
    float pdf_m = ((g1_fn(o, in.alpha) / fabsf(cos_theta(o))) * d) * fabsf(cos_d);
    float pdf_gtr = pdf_m / (4.0f * fabsf(cos_d));
    pdf = pdf_diffuse * diffuse_prob + pdf_gtr * (1.0f - diffuse_prob);
    return specular + diffuse;
}

__device__ __forceinline__ f3 sample_direction(f3 o, f2 alpha, float metalness, Sampler& smp, f3& m, float& w, float& pdf)
{
    f3 i;
    float diffuse_prob = diffuse_sample_probability(metalness);
    bool sample_diffuse = sample_1d(smp) < diffuse_prob;
    f2 ds = sample_2d(smp);
    if (sample_diffuse) {
        i = cosine_weighted_rand_dir(ds);
        m = normalize(o + i);
    } else {
        m = sample_visible_micronormal(o, alpha, ds);
        i = ((2.0f * dot(o, m)) * m) - o;
    }
    float pdf_diffuse = cos_theta(i) / PI_F;
    float cos_d = dot(m, o);
    float pdf_m = ((g1_fn(o, alpha) / fabsf(cos_theta(o))) * distribution(m, alpha)) * fabsf(cos_d);
    float pdf_gtr = pdf_m / (4.0f * fabsf(cos_d));
    pdf_diffuse = pdf_diffuse * diffuse_prob;
    pdf_gtr = pdf_gtr * (1.0f - diffuse_prob);
    pdf = sample_diffuse ? pdf_diffuse : pdf_gtr;
    w = pdf / (pdf_diffuse + pdf_gtr);
    return i;
}

} // namespace pt
