// pt_oracle.cpp — CPU oracle of pt's headless path-tracing path.
//
// TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and
// bench.py's CPU-baseline leg as the checker; never linked into the product.
// See pt_oracle.h for the list of reference functions restated here.
//
// Floating point: compiled with -ffp-contract=off so every expression is
// evaluated as written (no fused multiply-add), in the left-to-right order of
// the HLSL source.  The device code is compiled with -fmad=false and uses the
// same operation order, so the two agree bit for bit.
#include "pt_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <numeric>
#include <unordered_map>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---------------------------------------------------------------- vectors
struct V2 { float x, y; };
struct V3 { float x, y, z; };

inline V3 v3(float x, float y, float z) { return V3{x, y, z}; }
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator-(V3 a) { return {-a.x, -a.y, -a.z}; }
inline V3 operator*(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
inline V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline V3 operator*(float s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline V3 operator/(V3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
inline V3 operator/(V3 a, V3 b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
inline float dot(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline V3 cross(V3 a, V3 b)
{
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
// normalize(v) = v * (1 / sqrt(dot(v, v)))
inline V3 normalize(V3 v)
{
    float inv = 1.0f / std::sqrt(dot(v, v));
    return v * inv;
}
inline float maxc(V3 v) { return std::fmax(std::fmax(v.x, v.y), v.z); }
inline float comp(V3 v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }
// lerp(x, y, s) = x + s * (y - x)
inline float lerpf(float x, float y, float s) { return x + s * (y - x); }
inline V3 lerp3(V3 x, V3 y, float s) { return {lerpf(x.x, y.x, s), lerpf(x.y, y.y, s), lerpf(x.z, y.z, s)}; }
inline float sq(float x) { return x * x; }
inline bool is_finite(float x) { return std::isfinite(x); }
inline float clampf(float x, float lo, float hi) { return std::fmin(std::fmax(x, lo), hi); }

inline float asfloat(uint32_t u)
{
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}
inline uint32_t asuint(float f)
{
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
}

const float PI_F = 3.141592654f;                    // util.hlsli:3
const float JUST_BELOW_ONE = 0.99999994039535522f;  // asfloat(0x3F7FFFFF), util.hlsli:5
const float ORIGIN_OFFSET = 1e-5f;                  // pathtrace.hlsli:6
const float INF_F = std::numeric_limits<float>::infinity();

// Row-major 4x4: mul(M, v) = sum_j M[i][j] v[j], summed left to right.
inline V3 mul_point(const float m[4][4], V3 p)
{
    return {((m[0][0] * p.x + m[0][1] * p.y) + m[0][2] * p.z) + m[0][3] * 1.0f,
            ((m[1][0] * p.x + m[1][1] * p.y) + m[1][2] * p.z) + m[1][3] * 1.0f,
            ((m[2][0] * p.x + m[2][1] * p.y) + m[2][2] * p.z) + m[2][3] * 1.0f};
}
inline V3 mul_dir0(const float m[4][4], V3 d)
{
    return {((m[0][0] * d.x + m[0][1] * d.y) + m[0][2] * d.z) + m[0][3] * 0.0f,
            ((m[1][0] * d.x + m[1][1] * d.y) + m[1][2] * d.z) + m[1][3] * 0.0f,
            ((m[2][0] * d.x + m[2][1] * d.y) + m[2][2] * d.z) + m[2][3] * 0.0f};
}
// (float3x3)M * v
inline V3 mul3(const float m[4][4], V3 v)
{
    return {(m[0][0] * v.x + m[0][1] * v.y) + m[0][2] * v.z,
            (m[1][0] * v.x + m[1][1] * v.y) + m[1][2] * v.z,
            (m[2][0] * v.x + m[2][1] * v.y) + m[2][2] * v.z};
}
inline V3 mul3n(const float n[3][4], V3 v)
{
    return {(n[0][0] * v.x + n[0][1] * v.y) + n[0][2] * v.z,
            (n[1][0] * v.x + n[1][1] * v.y) + n[1][2] * v.z,
            (n[2][0] * v.x + n[2][1] * v.y) + n[2][2] * v.z};
}

// ---------------------------------------------------------------- sin/cos
// Cody & Waite (1980) argument reduction by pi/2 with a three-part constant,
// then Taylor polynomials of sin and cos on [-pi/4, pi/4] evaluated by Horner.
// Valid for |x| <= 1e4 (the path tracer uses |x| < 7).  The device code uses
// the same constants and operation order.
const float SC_TWO_OVER_PI = 0.636619746685028076f;
const float SC_PIO2_HI = 1.5707855224609375f;        // 17 significant bits
const float SC_PIO2_MID = 1.0804273188114166e-05f;   // 17 significant bits
const float SC_PIO2_LO = 6.077094383272197e-11f;
const float SC_S3 = -0.16666667163372040f;   // -1/3!
const float SC_S5 = 0.0083333337679505348f;  //  1/5!
const float SC_S7 = -0.00019841270113829523f;
const float SC_S9 = 2.7557318844628753e-06f;
const float SC_C2 = -0.5f;
const float SC_C4 = 0.041666667908430099f;
const float SC_C6 = -0.0013888889225199819f;
const float SC_C8 = 2.4801587642286904e-05f;
const float SC_C10 = -2.7557319981497130e-07f;

inline float sc_reduce(float x, int* quadrant)
{
    float k = std::nearbyint(x * SC_TWO_OVER_PI);
    float r = ((x - k * SC_PIO2_HI) - k * SC_PIO2_MID) - k * SC_PIO2_LO;
    *quadrant = ((int)k) & 3;
    return r;
}
inline float sc_sin_poly(float r)
{
    float r2 = r * r;
    float p = SC_S9;
    p = p * r2 + SC_S7;
    p = p * r2 + SC_S5;
    p = p * r2 + SC_S3;
    return r + (r * r2) * p;
}
inline float sc_cos_poly(float r)
{
    float r2 = r * r;
    float p = SC_C10;
    p = p * r2 + SC_C8;
    p = p * r2 + SC_C6;
    p = p * r2 + SC_C4;
    p = p * r2 + SC_C2;
    return 1.0f + r2 * p;
}
float pt_sin(float x)
{
    if (!std::isfinite(x))
        return x - x;
    int q;
    float r = sc_reduce(x, &q);
    float s = (q & 1) ? sc_cos_poly(r) : sc_sin_poly(r);
    return (q & 2) ? -s : s;
}
float pt_cos(float x)
{
    if (!std::isfinite(x))
        return x - x;
    int q;
    float r = sc_reduce(x, &q);
    float c = (q & 1) ? sc_sin_poly(r) : sc_cos_poly(r);
    return ((q + 1) & 2) ? -c : c;
}

// ---------------------------------------------------------------- sampler
// Sobol' direction numbers for 4 dimensions from the primitive polynomials
// and initial direction numbers of Joe & Kuo (2008): dim 0 is van der Corput;
// dims 1-3 use (s=1,a=0,m=1), (s=2,a=1,m=1,3), (s=3,a=1,m=1,3,1).  These are
// the values tabulated in shaders/pathtrace/sample.hlsli:31-67.
struct SobolTable {
    uint32_t v[4][32];
    SobolTable()
    {
        for (int b = 0; b < 32; b++)
            v[0][b] = 1u << (31 - b);
        const int s_[3] = {1, 2, 3};
        const uint32_t a_[3] = {0, 1, 1};
        const uint32_t m_[3][3] = {{1, 0, 0}, {1, 3, 0}, {1, 3, 1}};
        for (int d = 1; d < 4; d++) {
            int s = s_[d - 1];
            uint32_t a = a_[d - 1];
            for (int k = 0; k < s; k++)
                v[d][k] = m_[d - 1][k] << (31 - k);
            for (int k = s; k < 32; k++) {
                uint32_t x = v[d][k - s] ^ (v[d][k - s] >> s);
                for (int j = 1; j < s; j++)
                    if ((a >> (s - 1 - j)) & 1u)
                        x ^= v[d][k - j];
                v[d][k] = x;
            }
        }
    }
};
const SobolTable& sobol_table()
{
    static SobolTable t;
    return t;
}

inline uint32_t hash_combine(uint32_t seed, uint32_t x) { return seed ^ (x + (seed << 6) + (seed >> 2)); }
inline uint32_t hash32(uint32_t x)
{
    x ^= x >> 16;
    x *= 0x85ebca6bu;
    x ^= x >> 13;
    x *= 0xc2b2ae35u;
    x ^= x >> 16;
    return x;
}
inline uint32_t reverse_bits(uint32_t x)
{
    x = ((x >> 1) & 0x55555555u) | ((x & 0x55555555u) << 1);
    x = ((x >> 2) & 0x33333333u) | ((x & 0x33333333u) << 2);
    x = ((x >> 4) & 0x0F0F0F0Fu) | ((x & 0x0F0F0F0Fu) << 4);
    x = ((x >> 8) & 0x00FF00FFu) | ((x & 0x00FF00FFu) << 8);
    return (x >> 16) | (x << 16);
}
inline uint32_t lk_permutation(uint32_t x, uint32_t seed)
{
    x += seed;
    x ^= x * 0x6c50b47cu;
    x ^= x * 0xb82f1e52u;
    x ^= x * 0xc7afe638u;
    x ^= x * 0x8d22f6e6u;
    return x;
}
inline uint32_t scramble(uint32_t x, uint32_t seed) { return reverse_bits(lk_permutation(reverse_bits(x), seed)); }
inline uint32_t sobol(uint32_t index, uint32_t dim)
{
    const SobolTable& t = sobol_table();
    uint32_t x = 0;
    for (int b = 0; b < 32; b++)
        if ((index >> b) & 1u)
            x ^= t.v[dim][b];
    return x;
}
inline uint32_t scrambled_sobol(uint32_t shuffled, uint32_t dim, uint32_t seed)
{
    return scramble(sobol(shuffled, dim), hash_combine(seed, dim));
}

struct Sampler {
    uint32_t index, seed, dimension, shuffled;
};
const uint32_t SOBOL_MAX_DIMENSION = 4;

inline void sampler_start(Sampler& s, uint32_t px, uint32_t py, uint32_t sample_index, uint32_t seed)
{
    s.seed = hash_combine(seed, hash_combine(px, py));
    s.index = sample_index;
    s.dimension = SOBOL_MAX_DIMENSION;
    s.shuffled = 0;
}
inline void sampler_pad(Sampler& s)
{
    s.dimension = 0;
    s.seed = hash32(s.seed);
    s.shuffled = scramble(s.index, s.seed);
}
inline float u32_to_unit(uint32_t x)
{
    float r = 0x1p-32f * (float)x;
    return std::fmin(r, JUST_BELOW_ONE);
}
inline float sample_1d(Sampler& s)
{
    if (s.dimension >= SOBOL_MAX_DIMENSION)
        sampler_pad(s);
    float r = u32_to_unit(scrambled_sobol(s.shuffled, s.dimension, s.seed));
    s.dimension += 1;
    return r;
}
inline V2 sample_2d(Sampler& s)
{
    if (s.dimension + 1 >= SOBOL_MAX_DIMENSION)
        sampler_pad(s);
    V2 r;
    r.x = u32_to_unit(scrambled_sobol(s.shuffled, s.dimension + 0, s.seed));
    r.y = u32_to_unit(scrambled_sobol(s.shuffled, s.dimension + 1, s.seed));
    s.dimension += 2;
    return r;
}

// ---------------------------------------------------------------- warps (sample.hlsli)
inline V3 cosine_weighted_rand_dir(V2 u)
{
    float su = std::sqrt(u.x);
    float x = su * pt_cos((2.0f * PI_F) * u.y);
    float y = su * pt_sin((2.0f * PI_F) * u.y);
    float z = std::sqrt(1.0f - u.x);
    return {x, y, z};
}
inline V3 random_barycentric(V2 u)
{
    float beta = 1.0f - std::sqrt(u.x);
    float gamma = (1.0f - beta) * u.y;
    float alpha = (1.0f - beta) - gamma;
    return {alpha, beta, gamma};
}
inline V2 sample_concentric_disk(V2 u)
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
inline V3 sample_visible_micronormal(V3 v, V2 alpha, V2 u)
{
    v = normalize(v3(alpha.x * v.x, alpha.y * v.y, v.z));
    V3 x = (v.z < 0.99999f) ? normalize(cross(v3(0.0f, 0.0f, 1.0f), v)) : v3(1.0f, 0.0f, 0.0f);
    V3 y = cross(v, x);
    float a = 1.0f / (1.0f + v.z);
    float r = std::sqrt(u.x);
    float phi = (u.y < a) ? (u.y / a) * PI_F : PI_F + ((u.y - a) / (1.0f - a)) * PI_F;
    float p1 = r * pt_cos(phi);
    float p2 = (r * pt_sin(phi)) * ((u.y < a) ? 1.0f : v.z);
    float s = std::sqrt(std::fmax(0.0f, (1.0f - p1 * p1) - p2 * p2));
    V3 m = (p1 * x + p2 * y) + s * v;
    return normalize(v3(alpha.x * m.x, alpha.y * m.y, std::fmax(1e-6f, m.z)));
}

// ---------------------------------------------------------------- BSDF (pathtrace.ch.hlsl:22-157)
inline float cos_theta(V3 v) { return v.z; }
inline float cos2_theta(V3 v) { return sq(cos_theta(v)); }
inline float sin2_theta(V3 v) { return std::fmax(0.0f, 1.0f - cos2_theta(v)); }
inline float sin_theta(V3 v) { return std::sqrt(sin2_theta(v)); }
inline float tan2_theta(V3 v) { return sin2_theta(v) / cos2_theta(v); }

struct BrdfInput {
    V3 base_colour;
    V2 alpha;
    float metalness;
    V3 specular;
    V3 sheen;
};

inline float fresnel_schlick(float cos_d)
{
    float b = 1.0f - cos_d;
    return (((b * b) * b) * b) * b;
}
inline float lambda_fn(V3 m, V2 alpha)
{
    float tan2 = tan2_theta(m);
    if (std::isinf(tan2))
        return 0.0f;
    float s = sin_theta(m);
    float cos_phi = s == 0.0f ? 1.0f : clampf(m.x / s, -1.0f, 1.0f);
    float sin_phi = s == 0.0f ? 0.0f : clampf(m.y / s, -1.0f, 1.0f);
    float alpha2 = sq(cos_phi * alpha.x) + sq(sin_phi * alpha.y);
    return (std::sqrt(1.0f + alpha2 * tan2) - 1.0f) / 2.0f;
}
inline float g1_fn(V3 v, V2 alpha) { return 1.0f / (1.0f + lambda_fn(v, alpha)); }
inline float masking(V3 o, V3 i, V2 alpha) { return 1.0f / ((1.0f + lambda_fn(o, alpha)) + lambda_fn(i, alpha)); }
inline float distribution(V3 m, V2 alpha)
{
    float tan2 = tan2_theta(m);
    if (std::isinf(tan2))
        return 0.0f;
    float cos4 = sq(cos2_theta(m));
    float s = sin_theta(m);
    float cos_phi = s == 0.0f ? 1.0f : clampf(m.x / s, -1.0f, 1.0f);
    float sin_phi = s == 0.0f ? 0.0f : clampf(m.y / s, -1.0f, 1.0f);
    float e = tan2 * (sq(cos_phi / alpha.x) + sq(sin_phi / alpha.y));
    return 1.0f / ((((PI_F * alpha.x) * alpha.y) * cos4) * sq(1.0f + e));
}
inline float diffuse_sample_probability(float metalness) { return lerpf(0.5f, 0.0f, metalness); }

inline V3 evaluate_brdf(const BrdfInput& in, V3 i, V3 o, V3 m, float& pdf)
{
    V3 f0 = lerp3(in.specular * 0.08f, in.base_colour, in.metalness);
    float cos_d = dot(m, o);
    float f = fresnel_schlick(cos_d);
    float g = masking(o, i, in.alpha);
    float d = distribution(m, in.alpha);
    V3 lf = lerp3(f0, v3(1.0f, 1.0f, 1.0f), f);
    float denom = (4.0f * cos_theta(i)) * cos_theta(o);
    V3 specular = ((d * lf) * g) / denom;
    V3 sheen = in.sheen * f;
    V3 diffuse = (((1.0f - in.metalness) * (in.base_colour + sheen)) / PI_F) * (1.0f - f);
    // The clearcoat lobe of the reference is evaluated but never added to the
    // result (pathtrace.ch.hlsl:93-100,114), so it is left out here.
    float diffuse_prob = diffuse_sample_probability(in.metalness);
    float pdf_diffuse = cos_theta(i) / PI_F;
    float pdf_m = ((g1_fn(o, in.alpha) / std::fabs(cos_theta(o))) * d) * std::fabs(cos_d);
    float pdf_gtr = pdf_m / (4.0f * std::fabs(cos_d));
    pdf = pdf_diffuse * diffuse_prob + pdf_gtr * (1.0f - diffuse_prob);
    return specular + diffuse;
}

inline V3 sample_direction(V3 o, V2 alpha, float metalness, Sampler& smp, V3& m, float& w, float& pdf)
{
    V3 i;
    float diffuse_prob = diffuse_sample_probability(metalness);
    bool sample_diffuse = sample_1d(smp) < diffuse_prob;
    V2 ds = sample_2d(smp);
    if (sample_diffuse) {
        i = cosine_weighted_rand_dir(ds);
        m = normalize(o + i);
    } else {
        m = sample_visible_micronormal(o, alpha, ds);
        i = ((2.0f * dot(o, m)) * m) - o;
    }
    float pdf_diffuse = cos_theta(i) / PI_F;
    float cos_d = dot(m, o);
    float pdf_m = ((g1_fn(o, alpha) / std::fabs(cos_theta(o))) * distribution(m, alpha)) * std::fabs(cos_d);
    float pdf_gtr = pdf_m / (4.0f * std::fabs(cos_d));
    pdf_diffuse = pdf_diffuse * diffuse_prob;
    pdf_gtr = pdf_gtr * (1.0f - diffuse_prob);
    pdf = sample_diffuse ? pdf_diffuse : pdf_gtr;
    w = pdf / (pdf_diffuse + pdf_gtr);
    return i;
}

// ---------------------------------------------------------------- BVH2 (binned SAH)
struct Box {
    float lo[3], hi[3];
    void reset()
    {
        for (int k = 0; k < 3; k++) {
            lo[k] = INF_F;
            hi[k] = -INF_F;
        }
    }
    void grow(const float p[3])
    {
        for (int k = 0; k < 3; k++) {
            lo[k] = std::min(lo[k], p[k]);
            hi[k] = std::max(hi[k], p[k]);
        }
    }
    void grow(const Box& b)
    {
        for (int k = 0; k < 3; k++) {
            lo[k] = std::min(lo[k], b.lo[k]);
            hi[k] = std::max(hi[k], b.hi[k]);
        }
    }
    double area() const
    {
        double e[3];
        for (int k = 0; k < 3; k++)
            e[k] = std::max(0.0, (double)hi[k] - (double)lo[k]);
        return 2.0 * (e[0] * e[1] + e[1] * e[2] + e[2] * e[0]);
    }
};

// Pad a box outward so that it strictly contains its primitives with a margin
// of 1e-5 of the largest coordinate magnitude: together with the rounding
// slack of the slab test this keeps box culling conservative.
inline void pad_box(Box& b)
{
    float mag = 0.0f;
    for (int k = 0; k < 3; k++)
        mag = std::max(mag, std::max(std::fabs(b.lo[k]), std::fabs(b.hi[k])));
    float eps = mag * 1e-5f + 1e-30f;
    for (int k = 0; k < 3; k++) {
        b.lo[k] -= eps;
        b.hi[k] += eps;
    }
}

struct Node {
    Box box;
    uint32_t left, right; // interior children
    uint32_t first, count; // leaf range into prim order (count > 0 = leaf)
};

struct Bvh {
    std::vector<Node> nodes;
    std::vector<uint32_t> prims;
};

void build_bvh(Bvh& bvh, const std::vector<Box>& boxes, uint32_t max_leaf)
{
    const uint32_t n = (uint32_t)boxes.size();
    bvh.nodes.clear();
    bvh.prims.resize(n);
    std::iota(bvh.prims.begin(), bvh.prims.end(), 0u);
    if (n == 0)
        return;
    std::vector<float> cent(3 * (size_t)n);
    for (uint32_t i = 0; i < n; i++)
        for (int k = 0; k < 3; k++)
            cent[3 * (size_t)i + k] = 0.5f * (boxes[i].lo[k] + boxes[i].hi[k]);

    struct Task { uint32_t node, first, count; };
    std::vector<Task> stack;
    bvh.nodes.push_back(Node{});
    stack.push_back({0, 0, n});
    const int BINS = 16;
    while (!stack.empty()) {
        Task t = stack.back();
        stack.pop_back();
        Box bb, cb;
        bb.reset();
        cb.reset();
        for (uint32_t i = t.first; i < t.first + t.count; i++) {
            uint32_t p = bvh.prims[i];
            bb.grow(boxes[p]);
            cb.grow(&cent[3 * (size_t)p]);
        }
        Node& nd = bvh.nodes[t.node];
        nd.box = bb;
        nd.count = 0;
        if (t.count <= max_leaf) {
            nd.first = t.first;
            nd.count = t.count;
            continue;
        }
        // binned SAH over the three axes
        double best_cost = std::numeric_limits<double>::infinity();
        int best_axis = -1, best_split = -1;
        for (int axis = 0; axis < 3; axis++) {
            float lo = cb.lo[axis], hi = cb.hi[axis];
            if (!(hi > lo))
                continue;
            Box bin_box[BINS];
            uint32_t bin_cnt[BINS] = {0};
            for (int b = 0; b < BINS; b++)
                bin_box[b].reset();
            float scale = BINS / (hi - lo);
            for (uint32_t i = t.first; i < t.first + t.count; i++) {
                uint32_t p = bvh.prims[i];
                int b = std::min(BINS - 1, (int)((cent[3 * (size_t)p + axis] - lo) * scale));
                bin_cnt[b]++;
                bin_box[b].grow(boxes[p]);
            }
            double right_area[BINS];
            uint32_t right_cnt[BINS];
            Box acc;
            acc.reset();
            uint32_t c = 0;
            for (int b = BINS - 1; b > 0; b--) {
                acc.grow(bin_box[b]);
                c += bin_cnt[b];
                right_area[b] = acc.area();
                right_cnt[b] = c;
            }
            acc.reset();
            c = 0;
            for (int b = 0; b < BINS - 1; b++) {
                acc.grow(bin_box[b]);
                c += bin_cnt[b];
                if (c == 0 || right_cnt[b + 1] == 0)
                    continue;
                double cost = acc.area() * c + right_area[b + 1] * right_cnt[b + 1];
                if (cost < best_cost) {
                    best_cost = cost;
                    best_axis = axis;
                    best_split = b;
                }
            }
        }
        uint32_t mid;
        if (best_axis < 0) {
            // all centroids coincide: split the range in half
            mid = t.first + t.count / 2;
        } else {
            double leaf_cost = bb.area() * t.count;
            double split_cost = 0.5 + best_cost; // traversal step ~ half a triangle test
            if (t.count <= 8 && leaf_cost <= split_cost * 1.0) {
                nd.first = t.first;
                nd.count = t.count;
                continue;
            }
            float lo = cb.lo[best_axis], hi = cb.hi[best_axis];
            float scale = BINS / (hi - lo);
            auto it = std::stable_partition(bvh.prims.begin() + t.first, bvh.prims.begin() + t.first + t.count,
                                            [&](uint32_t p) {
                                                int b = std::min(BINS - 1, (int)((cent[3 * (size_t)p + best_axis] - lo) * scale));
                                                return b <= best_split;
                                            });
            mid = (uint32_t)(it - bvh.prims.begin());
            if (mid == t.first || mid == t.first + t.count)
                mid = t.first + t.count / 2;
        }
        uint32_t l = (uint32_t)bvh.nodes.size();
        bvh.nodes.push_back(Node{});
        bvh.nodes.push_back(Node{});
        bvh.nodes[t.node].left = l;
        bvh.nodes[t.node].right = l + 1;
        stack.push_back({l, t.first, mid - t.first});
        stack.push_back({l + 1, mid, t.first + t.count - mid});
    }
    for (Node& nd : bvh.nodes)
        pad_box(nd.box);
}

// Robust slab test (Ize 2013, as in PBRT-v3): the far distance is scaled by
// 1 + 2*gamma(3) so float rounding never culls a box the ray meets.
const float SLAB_SCALE = 1.0f + 2.0f * (3.0f * 0x1p-24f) / (1.0f - 3.0f * 0x1p-24f);

inline bool slab(const Box& b, V3 o, V3 inv_d, float tmin, float tmax)
{
    float t0 = tmin, t1 = tmax;
    const float oo[3] = {o.x, o.y, o.z};
    const float id[3] = {inv_d.x, inv_d.y, inv_d.z};
    for (int k = 0; k < 3; k++) {
        float tn = (b.lo[k] - oo[k]) * id[k];
        float tf = (b.hi[k] - oo[k]) * id[k];
        if (tn > tf)
            std::swap(tn, tf);
        tf *= SLAB_SCALE;
        // NaN (0 * inf: origin on a slab plane of a zero direction) is
        // ignored by fmin/fmax; the padded box makes this case a true miss.
        t0 = std::fmax(t0, tn);
        t1 = std::fmin(t1, tf);
        if (t0 > t1)
            return false;
    }
    return true;
}

// ---------------------------------------------------------------- watertight test
struct ObjRay {
    V3 o, d;
    int kx, ky, kz;
    float sx, sy, sz;
    V3 inv_d;
};

inline void setup_obj_ray(ObjRay& r)
{
    float ax = std::fabs(r.d.x), ay = std::fabs(r.d.y), az = std::fabs(r.d.z);
    int kz = (ax > ay) ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
    int kx = kz + 1;
    if (kx == 3)
        kx = 0;
    int ky = kx + 1;
    if (ky == 3)
        ky = 0;
    if (comp(r.d, kz) < 0.0f)
        std::swap(kx, ky);
    r.kx = kx;
    r.ky = ky;
    r.kz = kz;
    float dz = comp(r.d, kz);
    r.sx = comp(r.d, kx) / dz;
    r.sy = comp(r.d, ky) / dz;
    r.sz = 1.0f / dz;
    r.inv_d = v3(1.0f / r.d.x, 1.0f / r.d.y, 1.0f / r.d.z);
}

// Woop, Benthin & Wald 2013, "Watertight Ray/Triangle Intersection", without
// back-face culling; falls back to FP64 edge functions when one is zero.
inline bool watertight(const ObjRay& r, V3 p0, V3 p1, V3 p2, float& t, float& b1, float& b2)
{
    V3 A = p0 - r.o, B = p1 - r.o, C = p2 - r.o;
    float Akx = comp(A, r.kx), Aky = comp(A, r.ky), Akz = comp(A, r.kz);
    float Bkx = comp(B, r.kx), Bky = comp(B, r.ky), Bkz = comp(B, r.kz);
    float Ckx = comp(C, r.kx), Cky = comp(C, r.ky), Ckz = comp(C, r.kz);
    float Ax = Akx - r.sx * Akz, Ay = Aky - r.sy * Akz;
    float Bx = Bkx - r.sx * Bkz, By = Bky - r.sy * Bkz;
    float Cx = Ckx - r.sx * Ckz, Cy = Cky - r.sy * Ckz;
    float U = Cx * By - Cy * Bx;
    float V = Ax * Cy - Ay * Cx;
    float W = Bx * Ay - By * Ax;
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        U = (float)((double)Cx * (double)By - (double)Cy * (double)Bx);
        V = (float)((double)Ax * (double)Cy - (double)Ay * (double)Cx);
        W = (float)((double)Bx * (double)Ay - (double)By * (double)Ax);
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f))
        return false;
    float det = (U + V) + W;
    if (det == 0.0f)
        return false;
    float Az = r.sz * Akz, Bz = r.sz * Bkz, Cz = r.sz * Ckz;
    float T = (U * Az + V * Bz) + W * Cz;
    float inv = 1.0f / det;
    t = T * inv;
    b1 = V * inv;
    b2 = W * inv;
    return true;
}

// ---------------------------------------------------------------- scene
struct Instance {
    pt_instance_data data;
    float w2o[3][4];
    uint32_t mesh;
    bool opaque;
    Box world_box;
};

struct Vertex {
    V3 position, normal;
    V2 uv;
};

struct Stats {
    uint64_t segments = 0, shadow_rays = 0, paths = 0, node_visits = 0, tri_tests = 0, inst_visits = 0, rays = 0;
    void add(const Stats& o)
    {
        segments += o.segments;
        shadow_rays += o.shadow_rays;
        paths += o.paths;
        node_visits += o.node_visits;
        tri_tests += o.tri_tests;
        inst_visits += o.inst_visits;
        rays += o.rays;
    }
};

} // namespace

struct or_scene {
    std::vector<float> vertices;
    std::vector<uint32_t> indices;
    std::vector<pt_mesh_range> meshes;
    std::vector<Instance> instances;
    std::vector<pt_material> materials;
    std::vector<uint32_t> light;
    uint32_t light_count = 0;
    V3 env{0, 0, 0};
    bool brute = false;
    std::vector<uint8_t> texels;
    std::vector<pt_texture> textures;
    std::vector<float> material_ior; // empty, or per material: > 0 = smooth dielectric
    float srgb[256]; // sRGB decode of 8-bit values, FP64 curve rounded once
    std::vector<Bvh> blas;
    Bvh tlas;

    Vertex vertex(uint32_t i) const
    {
        const float* v = &vertices[(size_t)i * PT_VERTEX_FLOATS];
        return Vertex{{v[0], v[1], v[2]}, {v[3], v[4], v[5]}, {v[6], v[7]}};
    }
    V3 position(uint32_t i) const
    {
        const float* v = &vertices[(size_t)i * PT_VERTEX_FLOATS];
        return {v[0], v[1], v[2]};
    }
    uint32_t lw(uint64_t i) const { return i < light.size() ? light[i] : 0u; } // robust buffer access
    // Position for an index read from the light stream, with robust buffer
    // access (zeros outside the vertex array).
    V3 position_robust(uint64_t i) const
    {
        if (i >= vertices.size() / PT_VERTEX_FLOATS)
            return {0.0f, 0.0f, 0.0f};
        return position((uint32_t)i);
    }
    V2 uv_robust(uint64_t i) const
    {
        if (i >= vertices.size() / PT_VERTEX_FLOATS)
            return {0.0f, 0.0f};
        const float* v = &vertices[(size_t)i * PT_VERTEX_FLOATS];
        return {v[6], v[7]};
    }
};

namespace {

// Texture sampling (material.hlsli SampleLevel(uv, 0) with the sampler of
// src/graphics/sampler.cpp:8-22: linear, REPEAT, level 0) in the library's
// stated arithmetic: uv wrapped to [0, 1), texel centres at (i + 0.5) / size,
// neighbours wrapped, weights (1-a)(1-b), a(1-b), (1-a)b, ab summed in that
// order.  Texels decode as UNORM (/255) or, for sRGB textures, through the
// FP64 sRGB curve rounded once; 1- and 2-channel textures read (r, 0, 0, 1)
// and (r, g, 0, 1).  Out-of-range texture indices read zero.
struct F4 {
    float x, y, z, w;
};

F4 texel(const or_scene& s, const pt_texture& t, uint32_t x, uint32_t y)
{
    const uint8_t* p = s.texels.data() + t.offset + ((size_t)y * t.width + x) * t.channels;
    if (t.channels == 4) {
        if (t.srgb)
            return {s.srgb[p[0]], s.srgb[p[1]], s.srgb[p[2]], (float)p[3] / 255.0f};
        return {(float)p[0] / 255.0f, (float)p[1] / 255.0f, (float)p[2] / 255.0f, (float)p[3] / 255.0f};
    }
    if (t.channels == 2)
        return {(float)p[0] / 255.0f, (float)p[1] / 255.0f, 0.0f, 1.0f};
    return {(float)p[0] / 255.0f, 0.0f, 0.0f, 1.0f};
}

F4 sample_texture(const or_scene& s, uint32_t index, V2 uv)
{
    if (index >= s.textures.size())
        return {0.0f, 0.0f, 0.0f, 0.0f};
    const pt_texture& t = s.textures[index];
    float u = uv.x - std::floor(uv.x), v = uv.y - std::floor(uv.y);
    if (!(u >= 0.0f && u < 1.0f))
        u = 0.0f;
    if (!(v >= 0.0f && v < 1.0f))
        v = 0.0f;
    const float x = u * (float)t.width - 0.5f, y = v * (float)t.height - 0.5f;
    const float fx = std::floor(x), fy = std::floor(y);
    const float a = x - fx, b = y - fy;
    int x0 = (int)fx, y0 = (int)fy;
    if (x0 < 0)
        x0 += (int)t.width;
    if (y0 < 0)
        y0 += (int)t.height;
    if (x0 >= (int)t.width)
        x0 = (int)t.width - 1;
    if (y0 >= (int)t.height)
        y0 = (int)t.height - 1;
    const uint32_t x1 = (uint32_t)x0 + 1 == t.width ? 0u : (uint32_t)x0 + 1;
    const uint32_t y1 = (uint32_t)y0 + 1 == t.height ? 0u : (uint32_t)y0 + 1;
    const F4 t00 = texel(s, t, x0, y0), t10 = texel(s, t, x1, y0), t01 = texel(s, t, x0, y1), t11 = texel(s, t, x1, y1);
    const float w00 = (1.0f - a) * (1.0f - b), w10 = a * (1.0f - b), w01 = (1.0f - a) * b, w11 = a * b;
    return {((w00 * t00.x + w10 * t10.x) + w01 * t01.x) + w11 * t11.x, ((w00 * t00.y + w10 * t10.y) + w01 * t01.y) + w11 * t11.y,
            ((w00 * t00.z + w10 * t10.z) + w01 * t01.z) + w11 * t11.z, ((w00 * t00.w + w10 * t10.w) + w01 * t01.w) + w11 * t11.w};
}

inline uint32_t map_bits_of(const pt_material& m)
{
    uint32_t b;
    std::memcpy(&b, &m.rough_metal_normal_map_bits[3], 4);
    return b;
}

inline uint32_t index_of(float f)
{
    uint32_t b;
    std::memcpy(&b, &f, 4);
    return b;
}

} // namespace

namespace {

struct Hit {
    float t, b1, b2;
    uint32_t inst, prim;
    bool valid;
};

inline bool better(float t, uint32_t inst, uint32_t prim, const Hit& h)
{
    if (t < h.t)
        return true;
    if (t > h.t)
        return false;
    return inst < h.inst || (inst == h.inst && prim < h.prim);
}

inline ObjRay to_object(const Instance& in, V3 o, V3 d)
{
    const float(*w)[4] = in.w2o;
    ObjRay r;
    r.o = v3(((w[0][0] * o.x + w[0][1] * o.y) + w[0][2] * o.z) + w[0][3],
             ((w[1][0] * o.x + w[1][1] * o.y) + w[1][2] * o.z) + w[1][3],
             ((w[2][0] * o.x + w[2][1] * o.y) + w[2][2] * o.z) + w[2][3]);
    r.d = v3((w[0][0] * d.x + w[0][1] * d.y) + w[0][2] * d.z,
             (w[1][0] * d.x + w[1][1] * d.y) + w[1][2] * d.z,
             (w[2][0] * d.x + w[2][1] * d.y) + w[2][2] * d.z);
    setup_obj_ray(r);
    return r;
}

inline void tri_positions(const or_scene& s, const Instance& in, uint32_t prim, V3& p0, V3& p1, V3& p2)
{
    const pt_mesh_range& m = s.meshes[in.mesh];
    const uint32_t* ix = &s.indices[(size_t)m.index_offset + 3 * (size_t)prim];
    p0 = s.position(m.vertex_offset + ix[0]);
    p1 = s.position(m.vertex_offset + ix[1]);
    p2 = s.position(m.vertex_offset + ix[2]);
}

// Closest hit over instance `ii` (object space), shrinking h.
void blas_closest(const or_scene& s, uint32_t ii, V3 o, V3 d, float tmin, Hit& h, Stats& st)
{
    const Instance& in = s.instances[ii];
    ObjRay r = to_object(in, o, d);
    st.inst_visits++;
    const pt_mesh_range& m = s.meshes[in.mesh];
    auto test = [&](uint32_t prim) {
        V3 p0, p1, p2;
        tri_positions(s, in, prim, p0, p1, p2);
        float t, b1, b2;
        st.tri_tests++;
        if (watertight(r, p0, p1, p2, t, b1, b2) && t >= tmin && t <= h.t && better(t, ii, prim, h)) {
            h.t = t;
            h.b1 = b1;
            h.b2 = b2;
            h.inst = ii;
            h.prim = prim;
            h.valid = true;
        }
    };
    if (s.brute) {
        for (uint32_t p = 0; p < m.tri_count; p++)
            test(p);
        return;
    }
    const Bvh& b = s.blas[in.mesh];
    if (b.nodes.empty())
        return;
    uint32_t stack[128];
    int sp = 0;
    stack[sp++] = 0;
    while (sp > 0) {
        const Node& nd = b.nodes[stack[--sp]];
        if (!slab(nd.box, r.o, r.inv_d, tmin, h.t))
            continue;
        if (nd.count > 0) {
            for (uint32_t k = nd.first; k < nd.first + nd.count; k++)
                test(b.prims[k]);
        } else {
            st.node_visits++;
            stack[sp++] = nd.right;
            stack[sp++] = nd.left;
        }
    }
}

Hit closest_hit(const or_scene& s, V3 o, V3 d, float tmin, float tmax, Stats& st)
{
    Hit h;
    h.t = tmax;
    h.inst = 0xFFFFFFFFu;
    h.prim = 0xFFFFFFFFu;
    h.valid = false;
    st.rays++;
    if (s.brute) {
        for (uint32_t i = 0; i < (uint32_t)s.instances.size(); i++)
            blas_closest(s, i, o, d, tmin, h, st);
        return h;
    }
    if (s.tlas.nodes.empty())
        return h;
    V3 inv_d = v3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
    uint32_t stack[128];
    int sp = 0;
    stack[sp++] = 0;
    while (sp > 0) {
        const Node& nd = s.tlas.nodes[stack[--sp]];
        if (!slab(nd.box, o, inv_d, tmin, h.t))
            continue;
        if (nd.count > 0) {
            for (uint32_t k = nd.first; k < nd.first + nd.count; k++)
                blas_closest(s, s.tlas.prims[k], o, d, tmin, h, st);
        } else {
            st.node_visits++;
            stack[sp++] = nd.right;
            stack[sp++] = nd.left;
        }
    }
    return h;
}

// shadowray.ah.hlsl:29-34: the base colour's alpha at the hit (a map is
// sampled at the hit's texture coordinate).
inline float material_alpha(const or_scene& s, uint32_t inst, uint32_t prim, float b1, float b2)
{
    const pt_instance_data& id = s.instances[inst].data;
    const pt_material& m = s.materials[id.material_index];
    if (!(map_bits_of(m) & PT_BASE_COLOUR_MAP_BIT))
        return m.base_colour[3];
    const uint32_t* ix = &s.indices[(size_t)id.index_index + (size_t)prim * 3];
    const V2 ua = s.uv_robust((uint64_t)id.vertex_index + ix[0]);
    const V2 ub = s.uv_robust((uint64_t)id.vertex_index + ix[1]);
    const V2 uc = s.uv_robust((uint64_t)id.vertex_index + ix[2]);
    const float ba = (1.0f - b1) - b2;
    const V2 uv = {(ba * ua.x + b1 * ub.x) + b2 * uc.x, (ba * ua.y + b1 * ub.y) + b2 * uc.y};
    return sample_texture(s, index_of(m.base_colour[0]), uv).w;
}

// Shadow ray (shadowray.ah.hlsl / shadowray.ms.hlsl): any opaque hit in
// [tmin, tmax] occludes; transparent instances attenuate by (1 - alpha).
// Returns the visibility throughput (0 when occluded).
float shadow_visibility(const or_scene& s, V3 o, V3 d, float tmin, float tmax, Stats& st)
{
    float throughput = 1.0f;
    bool occluded = false;
    st.rays++;
    auto visit_instance = [&](uint32_t ii) -> bool {
        const Instance& in = s.instances[ii];
        ObjRay r = to_object(in, o, d);
        st.inst_visits++;
        const pt_mesh_range& m = s.meshes[in.mesh];
        auto test = [&](uint32_t prim) -> bool {
            V3 p0, p1, p2;
            tri_positions(s, in, prim, p0, p1, p2);
            float t, b1, b2;
            st.tri_tests++;
            if (watertight(r, p0, p1, p2, t, b1, b2) && t >= tmin && t <= tmax) {
                if (in.opaque) {
                    occluded = true;
                    return true;
                }
                throughput *= (1.0f - material_alpha(s, ii, prim, b1, b2));
                if (throughput < 1e-5f) {
                    occluded = true;
                    return true;
                }
            }
            return false;
        };
        if (s.brute) {
            for (uint32_t p = 0; p < m.tri_count; p++)
                if (test(p))
                    return true;
            return false;
        }
        const Bvh& b = s.blas[in.mesh];
        if (b.nodes.empty())
            return false;
        uint32_t stack[128];
        int sp = 0;
        stack[sp++] = 0;
        while (sp > 0) {
            const Node& nd = b.nodes[stack[--sp]];
            if (!slab(nd.box, r.o, r.inv_d, tmin, tmax))
                continue;
            if (nd.count > 0) {
                for (uint32_t k = nd.first; k < nd.first + nd.count; k++)
                    if (test(b.prims[k]))
                        return true;
            } else {
                st.node_visits++;
                stack[sp++] = nd.right;
                stack[sp++] = nd.left;
            }
        }
        return false;
    };
    if (s.brute) {
        for (uint32_t i = 0; i < (uint32_t)s.instances.size(); i++)
            if (visit_instance(i))
                break;
    } else if (!s.tlas.nodes.empty()) {
        V3 inv_d = v3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
        uint32_t stack[128];
        int sp = 0;
        stack[sp++] = 0;
        while (sp > 0 && !occluded) {
            const Node& nd = s.tlas.nodes[stack[--sp]];
            if (!slab(nd.box, o, inv_d, tmin, tmax))
                continue;
            if (nd.count > 0) {
                for (uint32_t k = nd.first; k < nd.first + nd.count && !occluded; k++)
                    visit_instance(s.tlas.prims[k]);
            } else {
                st.node_visits++;
                stack[sp++] = nd.right;
                stack[sp++] = nd.left;
            }
        }
    }
    if (occluded || throughput < 1e-5f)
        return 0.0f;
    return throughput;
}

// ---------------------------------------------------------------- light sampling (lightsample.hlsli)
inline uint32_t sample_alias_table(const or_scene& s, uint32_t bin_count, uint32_t bin_size, uint32_t table_offset,
                                   float& u, float& p)
{
    float ub = u * (float)bin_count;
    uint32_t i = std::min(bin_count - 1, (uint32_t)ub);
    uint32_t bin_offset = table_offset + i * bin_size;
    u = std::fmin(ub - (float)i, JUST_BELOW_ONE);
    float q = asfloat(s.lw(bin_offset + 1));
    if (u < q) {
        u = std::fmin(u / q, JUST_BELOW_ONE);
    } else {
        i = s.lw(bin_offset + 2);
        bin_offset = table_offset + i * bin_size;
        u = std::fmin((u - q) / (1.0f - q), JUST_BELOW_ONE);
    }
    p = asfloat(s.lw(bin_offset + 0));
    return bin_offset + 3;
}

inline float light_pdf(const or_scene& s, uint32_t emitter_index, uint32_t primitive_index)
{
    if (emitter_index == PT_NO_EMITTER_INDEX)
        return 0.0f;
    uint32_t bin_offset = emitter_index * PT_LIGHT_BIN_SIZE;
    float p = asfloat(s.lw(bin_offset + 0));
    uint32_t light_type = s.lw(bin_offset + 3);
    if (light_type == PT_LIGHT_TYPE_EMITTER) {
        uint32_t table_offset = s.lw(bin_offset + 4);
        bin_offset = table_offset + primitive_index * PT_EMITTER_BIN_SIZE;
        p = p * asfloat(s.lw(bin_offset + 0));
    }
    return p;
}

// get_emission / get_base_colour / get_roughness_metalness_normal /
// get_specular / get_sheen (material.hlsli:23-88)
inline V3 material_emission(const or_scene& s, const pt_material& m, V2 uv)
{
    if (map_bits_of(m) & PT_EMISSION_MAP_BIT) {
        F4 t = sample_texture(s, index_of(m.emission[0]), uv);
        return v3(t.x, t.y, t.z) * m.emission[3];
    }
    return v3(m.emission[0], m.emission[1], m.emission[2]) * m.emission[3];
}

inline F4 material_base_colour(const or_scene& s, const pt_material& m, V2 uv)
{
    if (map_bits_of(m) & PT_BASE_COLOUR_MAP_BIT)
        return sample_texture(s, index_of(m.base_colour[0]), uv);
    return {m.base_colour[0], m.base_colour[1], m.base_colour[2], m.base_colour[3]};
}

void material_rough_metal_normal(const or_scene& s, const pt_material& m, V2 uv, float& roughness, float& metalness, V3& normal)
{
    const float* rmn = m.rough_metal_normal_map_bits;
    const uint32_t bits = map_bits_of(m);
    if (bits & PT_ROUGHNESS_METALNESS_MAP_BIT) {
        F4 t = sample_texture(s, index_of(rmn[0]), uv);
        roughness = t.y;
        metalness = t.z;
    } else {
        roughness = (bits & PT_ROUGHNESS_MAP_BIT) ? sample_texture(s, index_of(rmn[0]), uv).x : rmn[0];
        metalness = (bits & PT_METALNESS_MAP_BIT) ? sample_texture(s, index_of(rmn[1]), uv).x : rmn[1];
    }
    if (bits & PT_NORMAL_MAP_BIT) {
        F4 t = sample_texture(s, index_of(rmn[2]), uv);
        normal = normalize(v3(t.x * 2.0f - 1.0f, t.y * 2.0f - 1.0f, t.z * 2.0f - 1.0f));
    } else {
        normal = v3(0.0f, 0.0f, 1.0f);
    }
}

inline V3 material_rgb(const or_scene& s, const float* field, bool mapped, V2 uv)
{
    if (mapped) {
        F4 t = sample_texture(s, index_of(field[0]), uv);
        return v3(t.x, t.y, t.z);
    }
    return v3(field[0], field[1], field[2]);
}

// onb (util.hlsli:57-64)
inline void onb(V3 n, V3& x, V3& y)
{
    const float sg = n.z < 0.0f ? -1.0f : 1.0f;
    const float a = -1.0f / (sg + n.z);
    const float b = (n.x * n.y) * a;
    x = v3(1.0f + ((sg * n.x) * n.x) * a, sg * b, -sg * n.x);
    y = v3(b, sg + (n.y * n.y) * a, -n.y);
}

V3 sample_light(const or_scene& s, Sampler& smp, V3 pt, V3& light_dir, float& light_dist, float& pdf, bool& is_delta)
{
    float u0 = sample_1d(smp);
    V2 u12 = sample_2d(smp);
    float ux = u0;
    uint32_t bin_offset = sample_alias_table(s, s.light_count, PT_LIGHT_BIN_SIZE, 0, ux, pdf);
    uint32_t light_type = s.lw(bin_offset + 0);
    if (light_type == PT_LIGHT_TYPE_EMITTER) {
        uint32_t table_offset = s.lw(bin_offset + 1);
        uint32_t tri_count = s.lw(bin_offset + 2);
        uint32_t instance_offset = s.lw(bin_offset + 3);
        uint32_t instance_count = s.lw(bin_offset + 4);
        float p;
        bin_offset = sample_alias_table(s, tri_count, PT_EMITTER_BIN_SIZE, table_offset, ux, p);
        pdf = pdf * p;
        uint32_t instance_id = instance_offset + std::min(instance_count - 1, (uint32_t)(ux * (float)instance_count));
        if (instance_id >= s.instances.size()) {
            light_dist = 0.0f;
            is_delta = true;
            return v3(0, 0, 0);
        }
        const pt_instance_data& id = s.instances[instance_id].data;
        V3 pa = mul_point(id.transform, s.position_robust((uint64_t)id.vertex_index + s.lw(bin_offset + 0)));
        V3 pb = mul_point(id.transform, s.position_robust((uint64_t)id.vertex_index + s.lw(bin_offset + 1)));
        V3 pc = mul_point(id.transform, s.position_robust((uint64_t)id.vertex_index + s.lw(bin_offset + 2)));
        V3 bary = random_barycentric(u12);
        V3 point = (bary.x * pa + bary.y * pb) + bary.z * pc;
        const uint64_t ia = (uint64_t)id.vertex_index + s.lw(bin_offset + 0);
        const uint64_t ib = (uint64_t)id.vertex_index + s.lw(bin_offset + 1);
        const uint64_t ic = (uint64_t)id.vertex_index + s.lw(bin_offset + 2);
        light_dir = point - pt;
        light_dist = 1.0f;
        V3 tn = cross(pb - pa, pc - pa);
        float area = std::sqrt(dot(tn, tn)) * 0.5f;
        float cosine = std::fabs(dot(normalize(light_dir), normalize(tn)));
        float dist2 = dot(light_dir, light_dir);
        pdf = pdf * (dist2 / (area * cosine));
        is_delta = false;
        if (!is_finite(pdf))
            return v3(0, 0, 0);
        // lightsample.hlsli:106-108: emission at the point's texture coordinate
        const pt_material& lm = s.materials[id.material_index];
        V2 luv = {0.0f, 0.0f};
        if (map_bits_of(lm) & PT_EMISSION_MAP_BIT) {
            const V2 ua = s.uv_robust(ia), ub = s.uv_robust(ib), uc = s.uv_robust(ic);
            luv = {(bary.x * ua.x + bary.y * ub.x) + bary.z * uc.x, (bary.x * ua.y + bary.y * ub.y) + bary.z * uc.y};
        }
        return material_emission(s, lm, luv);
    } else if (light_type == PT_LIGHT_TYPE_POINT) {
        V3 lp = v3(asfloat(s.lw(bin_offset + 1)), asfloat(s.lw(bin_offset + 2)), asfloat(s.lw(bin_offset + 3)));
        light_dir = lp - pt;
        light_dist = 1.0f;
        is_delta = true;
        V3 col = v3(asfloat(s.lw(bin_offset + 4)), asfloat(s.lw(bin_offset + 5)), asfloat(s.lw(bin_offset + 6)));
        return (1.0f / dot(light_dir, light_dir)) * col;
    } else if (light_type == PT_LIGHT_TYPE_DIRECTIONAL) {
        light_dir = v3(asfloat(s.lw(bin_offset + 1)), asfloat(s.lw(bin_offset + 2)), asfloat(s.lw(bin_offset + 3)));
        light_dist = INF_F;
        is_delta = true;
        return v3(asfloat(s.lw(bin_offset + 4)), asfloat(s.lw(bin_offset + 5)), asfloat(s.lw(bin_offset + 6)));
    }
    light_dist = 0.0f;
    is_delta = true;
    return v3(0, 0, 0);
}

// ---------------------------------------------------------------- path state (RayPayload)
struct Payload {
    V3 throughput;
    bool final_segment;
    V3 radiance;
    float brdf_pdf; // < 0 on the first ray
    Sampler smp;
    V3 next_origin, next_dir;
};

inline void add_radiance(Payload& p, V3 r) { p.radiance = p.radiance + p.throughput * r; }

V3 light_contribution(const or_scene& s, const BrdfInput& bi, V3 o, V3 pt, const V3 fw[3], Payload& pl, Stats& st)
{
    if (s.light_count == 0)
        return v3(0, 0, 0);
    float pdf, light_dist;
    V3 light_dir;
    bool is_delta;
    V3 emission = sample_light(s, pl.smp, pt, light_dir, light_dist, pdf, is_delta);
    if (maxc(emission) <= 0.0f)
        return v3(0, 0, 0);
    V3 i = v3(dot(fw[0], light_dir), dot(fw[1], light_dir), dot(fw[2], light_dir));
    if (i.z <= 0.0f)
        return v3(0, 0, 0);
    st.shadow_rays++;
    float vis = shadow_visibility(s, pt, light_dir, 0.0f, light_dist - 1e-5f, st);
    if (vis == 0.0f)
        return v3(0, 0, 0);
    emission = emission * vis;
    i = normalize(i);
    V3 m = normalize(i + o);
    float pdf_brdf;
    V3 brdf = evaluate_brdf(bi, i, o, m, pdf_brdf);
    if (is_delta)
        return ((emission * brdf) * cos_theta(i)) / pdf;
    float w = pdf / (pdf + pdf_brdf);
    return (((w * emission) * brdf) * cos_theta(i)) / pdf;
}

// Smooth dielectric, this library's extension (the reference has no
// refraction), restated from the Fresnel equations for unpolarised light:
// with eta = n(viewer side) / n(far side), cos_t = sqrt(1 - eta^2 sin^2_i),
// r_s = (eta cos_i - cos_t) / (eta cos_i + cos_t),
// r_p = (cos_i - eta cos_t) / (cos_i + eta cos_t), F = (r_s^2 + r_p^2) / 2
// (1 under total internal reflection).  Reflection with probability F,
// else refraction t = -eta o_xy - cos_t z with throughput x tint x eta^2.
void shade_dielectric(Payload& pl, V3 tint, float eta, V3 o, const V3 fw[3], V3 twn, V3 hit)
{
    const float cos_i = o.z;
    const float sin2_t = (eta * eta) * (1.0f - cos_i * cos_i);
    float F = 1.0f, cos_t = 0.0f;
    if (sin2_t < 1.0f) {
        cos_t = std::sqrt(1.0f - sin2_t);
        const float rs = (eta * cos_i - cos_t) / (eta * cos_i + cos_t);
        const float rp = (cos_i - eta * cos_t) / (cos_i + eta * cos_t);
        F = 0.5f * (rs * rs + rp * rp);
    }
    V3 i;
    if (sample_1d(pl.smp) < F) {
        i = v3(-o.x, -o.y, o.z);
        pl.next_origin = hit + twn * ORIGIN_OFFSET;
    } else {
        i = v3(-eta * o.x, -eta * o.y, -cos_t);
        pl.throughput = pl.throughput * (tint * (eta * eta));
        pl.next_origin = hit - twn * ORIGIN_OFFSET;
    }
    pl.brdf_pdf = -1.0f; // delta lobe: the next emitter hit counts in full
    const V3 &wx = fw[0], &wy = fw[1], &wn = fw[2];
    V3 wi = v3((wx.x * i.x + wy.x * i.y) + wn.x * i.z, (wx.y * i.x + wy.y * i.y) + wn.y * i.z,
               (wx.z * i.x + wy.z * i.y) + wn.z * i.z);
    pl.next_dir = normalize(wi);
}

// pathtrace.ch.hlsl:227-360 for a hit; pathtrace.ms.hlsl for a miss.
void shade(const or_scene& s, Payload& pl, V3 ray_o, V3 ray_d, const Hit& h, Stats& st)
{
    if (!h.valid) {
        add_radiance(pl, s.env);
        pl.final_segment = true;
        return;
    }
    const Instance& inst = s.instances[h.inst];
    const pt_instance_data& id = inst.data;
    const pt_material& mat = s.materials[id.material_index];
    const uint32_t* ix = &s.indices[(size_t)id.index_index + (size_t)h.prim * 3];
    Vertex va = s.vertex(id.vertex_index + ix[0]);
    Vertex vb = s.vertex(id.vertex_index + ix[1]);
    Vertex vc = s.vertex(id.vertex_index + ix[2]);

    // get_vertex_attributes (geometry.hlsli:38-47)
    float ba = (1.0f - h.b1) - h.b2;
    V3 obj_normal = normalize((ba * va.normal + h.b1 * vb.normal) + h.b2 * vc.normal);
    const V2 uv = {(ba * va.uv.x + h.b1 * vb.uv.x) + h.b2 * vc.uv.x, (ba * va.uv.y + h.b1 * vb.uv.y) + h.b2 * vc.uv.y};

    V3 emission = material_emission(s, mat, uv);
    V3 obj_dir = v3((inst.w2o[0][0] * ray_d.x + inst.w2o[0][1] * ray_d.y) + inst.w2o[0][2] * ray_d.z,
                    (inst.w2o[1][0] * ray_d.x + inst.w2o[1][1] * ray_d.y) + inst.w2o[1][2] * ray_d.z,
                    (inst.w2o[2][0] * ray_d.x + inst.w2o[2][1] * ray_d.y) + inst.w2o[2][2] * ray_d.z);
    if (maxc(emission) > 0.0f && dot(obj_dir, obj_normal) < 0.0f) {
        if (pl.brdf_pdf < 0.0f) {
            add_radiance(pl, emission);
        } else {
            V3 wab = mul3(id.transform, vb.position - va.position);
            V3 wac = mul3(id.transform, vc.position - va.position);
            V3 en = cross(wab, wac);
            float area = std::sqrt(dot(en, en)) * 0.5f;
            float dist2 = h.t * h.t;
            float cosine = std::fabs(dot(ray_d, normalize(en)));
            float pdf_l = light_pdf(s, id.emitter_index, h.prim);
            pdf_l = pdf_l * (dist2 / (area * cosine));
            if (pdf_l > 0.0f && dist2 > 0.0f) {
                float w = pl.brdf_pdf / (pl.brdf_pdf + pdf_l);
                add_radiance(pl, w * emission);
            }
        }
    }
    if (pl.final_segment)
        return;

    const F4 bc = material_base_colour(s, mat, uv);
    V3 base = v3(bc.x, bc.y, bc.z);
    float base_a = bc.w;
    if (base_a < sample_1d(pl.smp)) {
        V3 ip = ray_o + ray_d * (h.t + ORIGIN_OFFSET);
        pl.next_origin = ip;
        pl.next_dir = ray_d;
        return;
    }
    BrdfInput bi;
    bi.base_colour = base;
    float roughness;
    V3 mapped_normal;
    material_rough_metal_normal(s, mat, uv, roughness, bi.metalness, mapped_normal);
    const uint32_t bits = map_bits_of(mat);
    bi.specular = material_rgb(s, mat.specular, (bits & PT_SPECULAR_MAP_BIT) != 0, uv);
    float anisotropy = mat.cc_ccrgh_aniso[2];
    bi.sheen = material_rgb(s, mat.sheen, (bits & PT_SHEEN_MAP_BIT) != 0, uv);
    roughness = std::fmax(0.00001f, roughness * roughness);
    float aspect = std::sqrt(1.0f - 0.9f * std::fabs(anisotropy));
    bi.alpha = {roughness / aspect, roughness * aspect};
    if (anisotropy < 0.0f)
        bi.alpha = {bi.alpha.y, bi.alpha.x};

    // get_vertex_vectors (geometry.hlsli:49-69)
    V2 duv_ab = {vb.uv.x - va.uv.x, vb.uv.y - va.uv.y};
    V2 duv_ac = {vc.uv.x - va.uv.x, vc.uv.y - va.uv.y};
    V3 ab = vb.position - va.position, ac = vc.position - va.position;
    V3 true_obj_normal = cross(ab, ac);
    float denom = duv_ab.x * duv_ac.y - duv_ac.x * duv_ab.y;
    V3 tangent;
    if (std::fabs(denom) < 1e-5f) {
        tangent = cross(obj_normal, std::fabs(obj_normal.y) > 1e-5f ? v3(1, 0, 0) : v3(0, 1, 0));
    } else {
        tangent = (duv_ac.y * ab - duv_ab.y * ac) / denom;
        tangent = tangent - dot(tangent, obj_normal) * obj_normal;
    }
    V3 bitangent = cross(obj_normal, tangent);

    V3 wx = normalize(mul3n(id.normal, tangent));
    V3 wy = normalize(mul3n(id.normal, bitangent));
    V3 wn = normalize(mul3n(id.normal, obj_normal));
    const bool back_face = dot(wn, ray_d) > 0.0f;
    if (back_face) {
        wx = -wx;
        wy = -wy;
        wn = -wn;
    }
    V3 twn = normalize(mul3n(id.normal, true_obj_normal));
    if (dot(ray_d, twn) > 0.0f)
        twn = -twn;
    // mapped normal (pathtrace.ch.hlsl:321-326): from_world becomes
    // float3x3(mapped_x, mapped_y, mapped_normal) x float3x3(wx, wy, wn)
    if (mapped_normal.z < 0.999f) {
        V3 mx, my;
        onb(mapped_normal, mx, my);
        const V3 rx = (mx.x * wx + mx.y * wy) + mx.z * wn;
        const V3 ry = (my.x * wx + my.y * wy) + my.z * wn;
        const V3 rn = (mapped_normal.x * wx + mapped_normal.y * wy) + mapped_normal.z * wn;
        wx = rx;
        wy = ry;
        wn = rn;
    }
    V3 fw[3] = {wx, wy, wn};
    V3 nd = -ray_d;
    V3 o = normalize(v3(dot(fw[0], nd), dot(fw[1], nd), dot(fw[2], nd)));
    if (o.z <= 0.0f) {
        pl.final_segment = true;
        return;
    }
    const V3 hit = ray_o + ray_d * h.t;
    if (!s.material_ior.empty() && s.material_ior[id.material_index] > 0.0f) {
        const float ior = s.material_ior[id.material_index];
        shade_dielectric(pl, bi.base_colour, back_face ? ior : 1.0f / ior, o, fw, twn, hit);
        return;
    }
    V3 ip = hit + twn * ORIGIN_OFFSET;
    add_radiance(pl, light_contribution(s, bi, o, ip, fw, pl, st));

    V3 m;
    float w, pdf;
    V3 i = sample_direction(o, bi.alpha, bi.metalness, pl.smp, m, w, pdf);
    if (i.z * o.z <= 0.0f) {
        pl.final_segment = true;
        return;
    }
    float pdf_brdf;
    V3 brdf = evaluate_brdf(bi, i, o, m, pdf_brdf);
    V3 tp = ((w * brdf) * cos_theta(i)) / pdf;
    pl.brdf_pdf = pdf_brdf;
    pl.throughput = pl.throughput * tp;
    // to_world = transpose(from_world)
    V3 wi = v3((wx.x * i.x + wy.x * i.y) + wn.x * i.z, (wx.y * i.x + wy.y * i.y) + wn.y * i.z,
               (wx.z * i.x + wy.z * i.y) + wn.z * i.z);
    pl.next_origin = ip;
    pl.next_dir = normalize(wi);
}

inline bool russian_roulette(Payload& pl)
{
    V3 T = pl.throughput;
    float mt = std::fmax(std::fmax(T.x, T.y), T.z);
    float u = sample_1d(pl.smp);
    if (mt < 1.0f) {
        float q = std::fmax(0.0f, 1.0f - mt);
        if (u < q)
            return true;
        float s = 1.0f / (1.0f - q);
        pl.throughput = pl.throughput * s;
    }
    return false;
}

inline V3 correct_radiance(V3 r)
{
    if (r.x < 0.0f || !is_finite(r.x))
        r.x = 0.0f;
    if (r.y < 0.0f || !is_finite(r.y))
        r.y = 0.0f;
    if (r.z < 0.0f || !is_finite(r.z))
        r.z = 0.0f;
    return r;
}

inline void camera_ray(const pt_render_params& P, uint32_t px, uint32_t py, V2 u_pixel, V2 u_lens, V3& origin, V3& dir)
{
    float fx = (float)px + u_pixel.x, fy = (float)py + u_pixel.y;
    float nx = (fx / (float)P.width) * 2.0f - 1.0f;
    float ny = (fy / (float)P.height) * 2.0f - 1.0f;
    const float* ip = P.inv_proj;
    V3 target = v3(((ip[0] * nx + ip[1] * ny) + ip[2] * 1.0f) + ip[3] * 1.0f,
                   ((ip[4] * nx + ip[5] * ny) + ip[6] * 1.0f) + ip[7] * 1.0f,
                   ((ip[8] * nx + ip[9] * ny) + ip[10] * 1.0f) + ip[11] * 1.0f);
    V3 ro = v3(0, 0, 0), rd = target;
    if (P.lens_radius > 0.0f) {
        V2 d = sample_concentric_disk(u_lens);
        V2 lp = {P.lens_radius * d.x, P.lens_radius * d.y};
        float t = P.focus_dist / -rd.z;
        V3 fp = ro + t * rd;
        ro = v3(lp.x, lp.y, 0.0f);
        rd = fp - ro;
    }
    const float* iv = P.inv_view;
    origin = v3(((iv[0] * ro.x + iv[1] * ro.y) + iv[2] * ro.z) + iv[3] * 1.0f,
                ((iv[4] * ro.x + iv[5] * ro.y) + iv[6] * ro.z) + iv[7] * 1.0f,
                ((iv[8] * ro.x + iv[9] * ro.y) + iv[10] * ro.z) + iv[11] * 1.0f);
    dir = normalize(v3(((iv[0] * rd.x + iv[1] * rd.y) + iv[2] * rd.z) + iv[3] * 0.0f,
                       ((iv[4] * rd.x + iv[5] * rd.y) + iv[6] * rd.z) + iv[7] * 0.0f,
                       ((iv[8] * rd.x + iv[9] * rd.y) + iv[10] * rd.z) + iv[11] * 0.0f));
}

// One sample of one pixel (pathtrace.rg.hlsl:16-56).  Returns the radiance
// before exposure/correction; optionally records the hit sequence.
V3 trace_sample(const or_scene& s, const pt_render_params& P, uint32_t px, uint32_t py, uint32_t sample_index, Stats& st,
                uint64_t* sig, uint32_t sig_cap, uint32_t* sig_n)
{
    Payload pl;
    pl.radiance = v3(0, 0, 0);
    sampler_start(pl.smp, px, py, sample_index, 0);
    V2 u_pixel = sample_2d(pl.smp);
    V2 u_lens = sample_2d(pl.smp);
    V3 ro, rd;
    camera_ray(P, px, py, u_pixel, u_lens, ro, rd);
    sampler_start(pl.smp, px, py, sample_index, 1);
    pl.throughput = v3(1, 1, 1);
    pl.brdf_pdf = -1.0f;
    pl.final_segment = (P.max_bounces == 0);
    auto record = [&](const Hit& h) {
        if (sig && *sig_n < sig_cap)
            sig[(*sig_n)++] = h.valid ? (((uint64_t)h.inst << 32) | h.prim) : ~0ull;
    };
    st.paths++;
    st.segments++;
    Hit h = closest_hit(s, ro, rd, P.near_plane, P.far_plane, st);
    record(h);
    shade(s, pl, ro, rd, h, st);
    if (!pl.final_segment) {
        for (uint32_t segment = 1; segment <= P.max_bounces; segment++) {
            sampler_start(pl.smp, px, py, sample_index, segment + 1);
            ro = pl.next_origin;
            rd = pl.next_dir;
            pl.final_segment = segment >= P.max_bounces;
            st.segments++;
            h = closest_hit(s, ro, rd, 0.0f, INF_F, st);
            record(h);
            shade(s, pl, ro, rd, h, st);
            if (pl.final_segment)
                break;
            if (segment >= P.rr_start && russian_roulette(pl))
                break;
        }
    }
    return pl.radiance;
}

// ---------------------------------------------------------------- packing helpers
// 4x4 inverse by cofactor expansion in FP64 (the adjugate over the
// determinant), rounded to float.  `m` is row-major.
void inverse4(const double m[4][4], double out[4][4])
{
    double a[16];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++)
            a[i * 4 + j] = m[i][j];
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
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++)
            out[i][j] = inv[i * 4 + j] * id;
}

} // namespace

// ================================================================ C API
extern "C" {

uint32_t or_hash(uint32_t x) { return hash32(x); }
uint32_t or_hash_combine(uint32_t seed, uint32_t x) { return hash_combine(seed, x); }
uint32_t or_sobol(uint32_t index, uint32_t dimension) { return sobol(index, dimension & 3u); }
uint32_t or_scramble(uint32_t x, uint32_t seed) { return scramble(x, seed); }
float or_sin(float x) { return pt_sin(x); }
float or_cos(float x) { return pt_cos(x); }

uint32_t or_sampler_sequence(uint32_t px, uint32_t py, uint32_t sample_index, uint32_t seed, const uint8_t* kinds,
                             uint32_t n, float* out)
{
    Sampler s;
    sampler_start(s, px, py, sample_index, seed);
    uint32_t k = 0;
    for (uint32_t i = 0; i < n; i++) {
        if (kinds[i] == 2) {
            V2 v = sample_2d(s);
            out[k++] = v.x;
            out[k++] = v.y;
        } else {
            out[k++] = sample_1d(s);
        }
    }
    return k;
}

// src/rng.cpp:24-60 (xoshiro128++ named Xshiro128, and Splitmix32)
static inline uint32_t rotl32(uint32_t x, int k) { return (x << k) | (x >> (32 - k)); }
void or_xshiro128_stream(const uint32_t seed4[4], uint32_t n, uint32_t* out_u32, float* out_f32)
{
    uint32_t s[4] = {seed4[0], seed4[1], seed4[2], seed4[3]};
    for (uint32_t i = 0; i < n; i++) {
        uint32_t result = rotl32(s[0] + s[3], 7) + s[0];
        uint32_t t = s[1] << 9;
        s[2] ^= s[0];
        s[3] ^= s[1];
        s[1] ^= s[2];
        s[0] ^= s[3];
        s[2] ^= t;
        s[3] = rotl32(s[3], 11);
        if (out_u32)
            out_u32[i] = result;
        if (out_f32)
            out_f32[i] = (float)result / (float)UINT32_MAX;
    }
}
void or_splitmix32_stream(uint32_t state, uint32_t n, uint32_t* out)
{
    for (uint32_t i = 0; i < n; i++) {
        state += 0x9e3779b9u;
        uint32_t z = state;
        z = (z ^ (z >> 16)) * 0x85ebca6bu;
        z = (z ^ (z >> 13)) * 0xc2b2ae35u;
        out[i] = z ^ (z >> 16);
    }
}

// src/aliastable.h:21-67 (Vose's alias method with the reference's
// float/double choices and stack discipline).
void or_alias_build(const float* weights, uint32_t n, float* p, float* q, uint32_t* alias)
{
    double sum = 0.0;
    for (uint32_t i = 0; i < n; i++)
        sum += (double)weights[i];
    double inv_sum = 1.0 / sum;
    for (uint32_t i = 0; i < n; i++) {
        p[i] = (float)((double)weights[i] * inv_sum);
        alias[i] = i;
    }
    std::vector<uint32_t> under, over;
    for (uint32_t i = 0; i < n; i++) {
        float u = p[i] * (float)n;
        q[i] = u;
        if (u < 1.0f)
            under.push_back(i);
        else
            over.push_back(i);
    }
    while (!under.empty() && !over.empty()) {
        alias[under.back()] = over.back();
        q[over.back()] += q[under.back()] - 1.0f;
        under.pop_back();
        if (q[over.back()] < 1.0f) {
            under.push_back(over.back());
            over.pop_back();
        }
    }
    for (uint32_t i : under)
        q[i] = 1.0f;
    for (uint32_t i : over)
        q[i] = 1.0f;
}

// src/colour.cpp:12-14: evaluated in double, returned as float.
float or_from_srgb(float x)
{
    return (float)((x <= 0.04045) ? (x / 12.92) : std::pow((x + 0.055) / 1.055, 2.4));
}

// Camera chain: basis Mat3(y, z, x) (scenebuild.cpp:184-190), view =
// inverse(T(-position) * R) (camera.h:16), projection = perspective with
// depth in [0, 1] and y flipped (camera.cpp:21-26), uploaded as
// transpose(inverse(.)) (pathtrace.cpp:381-396).  The oracle evaluates the
// chain in FP64 and rounds once; the reference rounds at every float step.
void or_camera_params(const pt_camera_desc* c, uint32_t width, uint32_t height, pt_render_params* P)
{
    double x[3] = {c->lookdir[0], c->lookdir[1], c->lookdir[2]};
    double xl = std::sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
    for (double& v : x)
        v /= xl;
    double up[3] = {c->up[0], c->up[1], c->up[2]};
    double y[3] = {up[1] * x[2] - up[2] * x[1], up[2] * x[0] - up[0] * x[2], up[0] * x[1] - up[1] * x[0]};
    double yl = std::sqrt(y[0] * y[0] + y[1] * y[1] + y[2] * y[2]);
    for (double& v : y)
        v /= yl;
    double z[3] = {x[1] * y[2] - x[2] * y[1], x[2] * y[0] - x[0] * y[2], x[0] * y[1] - x[1] * y[0]};
    // rotation matrix with columns (y, z, x); the quaternion round trip of
    // the reference is a rotation, so R is used directly.
    double inv_view[4][4] = {{y[0], z[0], x[0], -c->position[0]},
                             {y[1], z[1], x[1], -c->position[1]},
                             {y[2], z[2], x[2], -c->position[2]},
                             {0, 0, 0, 1}};
    double aspect = (double)(float)((float)width / (float)height);
    double fov = (double)(float)(c->fov_degrees * 0.01745329251994329576923690768489f);
    double th = std::tan(fov / 2.0);
    double n = c->near_plane, f = c->far_plane;
    double proj[4][4] = {{1.0 / (aspect * th), 0, 0, 0},
                         {0, -1.0 / th, 0, 0},
                         {0, 0, f / (n - f), -(f * n) / (f - n)},
                         {0, 0, -1, 0}};
    double inv_proj[4][4];
    inverse4(proj, inv_proj);
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) {
            P->inv_view[i * 4 + j] = (float)inv_view[i][j];
            P->inv_proj[i * 4 + j] = (float)inv_proj[i][j];
        }
    P->near_plane = c->near_plane;
    P->far_plane = c->far_plane;
    P->focus_dist = c->focus_dist;
    P->lens_radius = c->lens_radius;
    P->exposure = c->exposure;
    P->width = width;
    P->height = height;
}

} // extern "C"

// ---------------------------------------------------------------- packing
struct or_packed {
    std::vector<float> vertices;
    std::vector<uint32_t> indices;
    std::vector<pt_mesh_range> meshes;
    std::vector<pt_instance_data> instances;
    std::vector<uint32_t> instance_mesh;
    std::vector<float> w2o;
    std::vector<uint8_t> opaque;
    std::vector<pt_material> materials;
    std::vector<uint32_t> light;
    uint32_t light_count = 0;
    float env[3] = {0, 0, 0};
    std::vector<uint8_t> texels;
    std::vector<pt_texture> textures;
    std::vector<float> material_ior;
};

namespace {
bool is_emitter(const pt_material& m)
{
    uint32_t bits = asuint(m.rough_metal_normal_map_bits[3]);
    return ((bits & PT_EMISSION_MAP_BIT) || std::max(std::max(m.emission[0], m.emission[1]), m.emission[2]) > 0.0f) &&
           m.emission[3] > 0.0f;
}

// Xshiro128 (xoshiro128++) and Splitmix32 of src/rng.cpp.
struct OrXoshiro {
    uint32_t s[4];
    static uint32_t rotl(uint32_t x, int k) { return (x << k) | (x >> (32 - k)); }
    uint32_t next()
    {
        uint32_t r = rotl(s[0] + s[3], 7) + s[0];
        uint32_t t = s[1] << 9;
        s[2] ^= s[0];
        s[3] ^= s[1];
        s[1] ^= s[2];
        s[0] ^= s[3];
        s[2] ^= t;
        s[3] = rotl(s[3], 11);
        return r;
    }
    // float(next()) / float(UINT32_MAX); the float divisor is 2^32
    float next_float() { return (float)next() / 4294967296.0f; }
};

uint32_t splitmix32(uint32_t& state)
{
    uint32_t z = (state += 0x9e3779b9u);
    z = (z ^ (z >> 16)) * 0x85ebca6bu;
    z = (z ^ (z >> 13)) * 0xc2b2ae35u;
    return z ^ (z >> 16);
}

// static_cast<uint32_t>(roundf(f)) clamped by min(., size - 1)
// (lightsample.cpp:70-73): a negative or huge value lands on size - 1.
uint32_t texel_coordinate(float f, uint32_t size)
{
    float r = std::roundf(f);
    if (!(r >= 0.0f) || r >= 4294967296.0f)
        return size - 1;
    uint32_t x = (uint32_t)r;
    return x < size - 1 ? x : size - 1;
}

// calculate_object_intensity (lightsample.cpp:41-87) for an emission-mapped
// material: 20 barycentric samples per triangle from Xshiro128 seeded by four
// Splitmix32(0xbd7a0d48) draws, nearest texel, channels as UNORM / 255 (no
// sRGB decode), summed per triangle in double.  The four seed draws reach the
// constructor in reverse order: GCC evaluates call arguments right to left.
double emission_map_intensity(const pt_raw_scene* raw, const pt_mesh_range& m, const pt_material& mat)
{
    uint32_t st = 0xbd7a0d48u;
    uint32_t d0 = splitmix32(st), d1 = splitmix32(st), d2 = splitmix32(st), d3 = splitmix32(st);
    OrXoshiro rng{{d3, d2, d1, d0}};
    const pt_texture& t = raw->textures[asuint(mat.emission[0])];
    double total = 0.0;
    for (uint32_t i = 0; i < m.tri_count; i++) {
        const uint32_t* ix = raw->indices + m.index_offset + 3 * i;
        const float* a = raw->vertices + (size_t)(m.vertex_offset + ix[0]) * PT_VERTEX_FLOATS;
        const float* b = raw->vertices + (size_t)(m.vertex_offset + ix[1]) * PT_VERTEX_FLOATS;
        const float* c = raw->vertices + (size_t)(m.vertex_offset + ix[2]) * PT_VERTEX_FLOATS;
        double sum = 0.0;
        for (int j = 0; j < 20; j++) {
            float beta = 1.0f - std::sqrt(rng.next_float());
            float gamma = (1.0f - beta) * rng.next_float();
            float alpha = (1.0f - beta) - gamma;
            float u = (alpha * a[6] + beta * b[6]) + gamma * c[6];
            float v = (alpha * a[7] + beta * b[7]) + gamma * c[7];
            float ip;
            uint32_t x = texel_coordinate(std::modf(u, &ip) * (float)t.width, t.width);
            uint32_t y = texel_coordinate(std::modf(v, &ip) * (float)t.height, t.height);
            const uint8_t* px = raw->texels + t.offset + ((size_t)y * t.width + x) * t.channels;
            float r = px[0] / 255.0f;
            float g = t.channels >= 2 ? px[1] / 255.0f : 0.0f;
            float bl = t.channels == 4 ? px[2] / 255.0f : 0.0f;
            sum += (r + g) + bl;
        }
        total += sum;
    }
    return total * mat.emission[3] / (double)((size_t)m.tri_count * 20);
}

// AliasTable<T> bins as u32 words: p, q, alias, value words.
void append_alias_table(std::vector<uint32_t>& out, const std::vector<float>& weights,
                        const std::vector<std::vector<uint32_t>>& values)
{
    uint32_t n = (uint32_t)weights.size();
    std::vector<float> p(n), q(n);
    std::vector<uint32_t> a(n);
    or_alias_build(weights.data(), n, p.data(), q.data(), a.data());
    for (uint32_t i = 0; i < n; i++) {
        out.push_back(asuint(p[i]));
        out.push_back(asuint(q[i]));
        out.push_back(a[i]);
        for (uint32_t w : values[i])
            out.push_back(w);
    }
}
} // namespace

extern "C" {

or_packed* or_pack(const pt_raw_scene* raw)
{
    or_packed* P = new or_packed();
    P->vertices.assign(raw->vertices, raw->vertices + (size_t)raw->vertex_count * PT_VERTEX_FLOATS);
    P->indices.assign(raw->indices, raw->indices + raw->index_count);
    P->meshes.assign(raw->meshes, raw->meshes + raw->mesh_count);
    P->materials.assign(raw->materials, raw->materials + raw->material_count);
    for (int k = 0; k < 3; k++)
        P->env[k] = raw->environment_colour[k];
    if (raw->texture_count) {
        P->texels.assign(raw->texels, raw->texels + raw->texel_bytes);
        P->textures.assign(raw->textures, raw->textures + raw->texture_count);
    }
    if (raw->material_ior)
        P->material_ior.assign(raw->material_ior, raw->material_ior + raw->material_count);

    // scenebuffer.cpp:201-220
    uint32_t emitter_index = 0;
    for (uint32_t v = 0; v < raw->mesh_count; v++) {
        const pt_material& mat = raw->materials[raw->mesh_material[v]];
        bool emits = is_emitter(mat);
        for (uint32_t j = raw->mesh_instance_offset[v]; j < raw->mesh_instance_offset[v + 1]; j++) {
            const float* M = raw->instance_matrices + 16 * (size_t)j; // column-major
            pt_instance_data d;
            d.vertex_index = raw->meshes[v].vertex_offset;
            d.index_index = raw->meshes[v].index_offset;
            d.emitter_index = emits ? emitter_index++ : PT_NO_EMITTER_INDEX;
            d.material_index = raw->mesh_material[v];
            double Md[4][4];
            for (int r = 0; r < 4; r++)
                for (int c = 0; c < 4; c++) {
                    d.transform[r][c] = M[c * 4 + r];
                    Md[r][c] = M[c * 4 + r];
                }
            double inv[4][4];
            inverse4(Md, inv);
            for (int r = 0; r < 3; r++)
                for (int c = 0; c < 4; c++)
                    d.normal[r][c] = (float)inv[c][r]; // rows of inverse-transpose
            P->instances.push_back(d);
            P->instance_mesh.push_back(v);
            for (int r = 0; r < 3; r++)
                for (int c = 0; c < 4; c++)
                    P->w2o.push_back((float)inv[r][c]);
            uint32_t bits = asuint(mat.rough_metal_normal_map_bits[3]);
            P->opaque.push_back((bits & PT_MATERIAL_IS_TRANSPARENT_BIT) ? 0 : 1);
        }
    }

    // lightsample.cpp:89-178 (TableLightSampler), quirks included.
    uint32_t n_lights = raw->point_light_count + raw->directional_light_count;
    for (uint32_t v = 0; v < raw->mesh_count; v++)
        if (is_emitter(raw->materials[raw->mesh_material[v]]))
            n_lights += raw->mesh_instance_offset[v + 1] - raw->mesh_instance_offset[v];
    if (n_lights > 0) {
        std::vector<float> weights;
        std::vector<std::vector<uint32_t>> values;
        std::vector<std::vector<float>> tri_weights;
        std::vector<std::vector<std::vector<uint32_t>>> tri_values;
        std::unordered_map<uint32_t, uint32_t> mesh_table; // mesh -> table index
        for (uint32_t v = 0; v < raw->mesh_count; v++) {
            const pt_material& mat = raw->materials[raw->mesh_material[v]];
            if (!is_emitter(mat))
                continue;
            uint32_t table_index;
            auto it = mesh_table.find(v);
            if (it == mesh_table.end()) {
                table_index = (uint32_t)tri_weights.size();
                tri_weights.emplace_back();
                tri_values.emplace_back();
                const pt_mesh_range& m = raw->meshes[v];
                for (uint32_t t = 0; t < m.tri_count; t++) {
                    const uint32_t* ix = raw->indices + m.index_offset + 3 * t;
                    const float* va = raw->vertices + (size_t)(m.vertex_offset + ix[0]) * PT_VERTEX_FLOATS;
                    const float* vb = raw->vertices + (size_t)(m.vertex_offset + ix[1]) * PT_VERTEX_FLOATS;
                    const float* vc = raw->vertices + (size_t)(m.vertex_offset + ix[2]) * PT_VERTEX_FLOATS;
                    V3 ab = v3(vb[0] - va[0], vb[1] - va[1], vb[2] - va[2]);
                    V3 ac = v3(vc[0] - va[0], vc[1] - va[1], vc[2] - va[2]);
                    V3 cr = cross(ab, ac);
                    float double_area = std::sqrt(dot(cr, cr));
                    tri_weights.back().push_back(double_area);
                    tri_values.back().push_back({ix[0], ix[1], ix[2]});
                }
                mesh_table[v] = table_index;
            } else {
                table_index = it->second;
            }
            // calculate_object_intensity (lightsample.cpp:41-87)
            float intensity = (asuint(mat.rough_metal_normal_map_bits[3]) & PT_EMISSION_MAP_BIT)
                                  ? (float)emission_map_intensity(raw, raw->meshes[v], mat)
                                  : (float)(double)(((mat.emission[0] + mat.emission[1]) + mat.emission[2]) * mat.emission[3]);
            weights.push_back(intensity);
            // table_offset stays 0: the reference accumulates the size of the
            // still-empty light table (lightsample.cpp:126).
            values.push_back({PT_LIGHT_TYPE_EMITTER, 0u, (uint32_t)tri_weights[table_index].size(), raw->mesh_instance_offset[v],
                              raw->mesh_instance_offset[v + 1] - raw->mesh_instance_offset[v], 0u, 0u});
        }
        uint32_t bin_count = raw->point_light_count + raw->directional_light_count + (uint32_t)tri_weights.size();
        for (auto& val : values)
            val[1] += bin_count * PT_LIGHT_BIN_SIZE;
        for (uint32_t i = 0; i < raw->point_light_count; i++) {
            const float* L = raw->point_lights + 6 * (size_t)i;
            weights.push_back((L[3] + L[4]) + L[5]);
            values.push_back({PT_LIGHT_TYPE_POINT, asuint(L[0]), asuint(L[1]), asuint(L[2]), asuint(L[3]), asuint(L[4]), asuint(L[5])});
        }
        for (uint32_t i = 0; i < raw->directional_light_count; i++) {
            const float* L = raw->directional_lights + 6 * (size_t)i;
            weights.push_back((L[3] + L[4]) + L[5]);
            values.push_back({PT_LIGHT_TYPE_DIRECTIONAL, asuint(L[0]), asuint(L[1]), asuint(L[2]), asuint(L[3]), asuint(L[4]), asuint(L[5])});
        }
        append_alias_table(P->light, weights, values);
        P->light_count = (uint32_t)weights.size();
        for (size_t t = 0; t < tri_weights.size(); t++)
            append_alias_table(P->light, tri_weights[t], tri_values[t]);
    }
    return P;
}

void or_packed_view(const or_packed* P, pt_scene_view* v)
{
    std::memset(v, 0, sizeof(*v));
    v->vertices = P->vertices.data();
    v->vertex_count = (uint32_t)(P->vertices.size() / PT_VERTEX_FLOATS);
    v->indices = P->indices.data();
    v->index_count = (uint32_t)P->indices.size();
    v->meshes = P->meshes.data();
    v->mesh_count = (uint32_t)P->meshes.size();
    v->instances = P->instances.data();
    v->instance_mesh = P->instance_mesh.data();
    v->instance_world_to_object = P->w2o.data();
    v->instance_opaque = P->opaque.data();
    v->instance_count = (uint32_t)P->instances.size();
    v->materials = P->materials.data();
    v->material_count = (uint32_t)P->materials.size();
    v->light_words = P->light.data();
    v->light_word_count = (uint32_t)P->light.size();
    v->light_count = P->light_count;
    for (int k = 0; k < 3; k++)
        v->environment_colour[k] = P->env[k];
    v->texels = P->texels.data();
    v->texel_bytes = P->texels.size();
    v->textures = P->textures.data();
    v->texture_count = (uint32_t)P->textures.size();
    v->material_ior = P->material_ior.empty() ? nullptr : P->material_ior.data();
}

void or_packed_free(or_packed* p) { delete p; }

or_scene* or_scene_create(const pt_scene_view* v, int brute_force)
{
    or_scene* s = new or_scene();
    s->vertices.assign(v->vertices, v->vertices + (size_t)v->vertex_count * PT_VERTEX_FLOATS);
    s->indices.assign(v->indices, v->indices + v->index_count);
    s->meshes.assign(v->meshes, v->meshes + v->mesh_count);
    s->materials.assign(v->materials, v->materials + v->material_count);
    if (v->light_words)
        s->light.assign(v->light_words, v->light_words + v->light_word_count);
    s->light_count = v->light_count;
    s->env = v3(v->environment_colour[0], v->environment_colour[1], v->environment_colour[2]);
    s->brute = brute_force != 0;
    if (v->texture_count) {
        s->texels.assign(v->texels, v->texels + v->texel_bytes);
        s->textures.assign(v->textures, v->textures + v->texture_count);
    }
    if (v->material_ior)
        s->material_ior.assign(v->material_ior, v->material_ior + v->material_count);
    for (int i = 0; i < 256; i++) {
        const double c = i / 255.0;
        s->srgb[i] = (float)(c <= 0.04045 ? c / 12.92 : std::pow((c + 0.055) / 1.055, 2.4));
    }

    // BLAS per mesh
    s->blas.resize(v->mesh_count);
    std::vector<Box> mesh_box(v->mesh_count);
    for (uint32_t m = 0; m < v->mesh_count; m++) {
        const pt_mesh_range& r = v->meshes[m];
        std::vector<Box> boxes(r.tri_count);
        Box all;
        all.reset();
        for (uint32_t t = 0; t < r.tri_count; t++) {
            Box& b = boxes[t];
            b.reset();
            for (int k = 0; k < 3; k++) {
                uint32_t vi = r.vertex_offset + v->indices[r.index_offset + 3 * t + k];
                b.grow(&v->vertices[(size_t)vi * PT_VERTEX_FLOATS]);
            }
            all.grow(b);
        }
        if (!brute_force)
            build_bvh(s->blas[m], boxes, 4);
        pad_box(all);
        mesh_box[m] = all;
    }
    // instances
    s->instances.resize(v->instance_count);
    std::vector<Box> inst_boxes(v->instance_count);
    for (uint32_t i = 0; i < v->instance_count; i++) {
        Instance& in = s->instances[i];
        in.data = v->instances[i];
        in.mesh = v->instance_mesh[i];
        in.opaque = v->instance_opaque ? v->instance_opaque[i] != 0 : true;
        if (v->instance_world_to_object) {
            std::memcpy(in.w2o, v->instance_world_to_object + 12 * (size_t)i, 48);
        } else {
            double Md[4][4], inv[4][4];
            for (int r = 0; r < 4; r++)
                for (int c = 0; c < 4; c++)
                    Md[r][c] = in.data.transform[r][c];
            inverse4(Md, inv);
            for (int r = 0; r < 3; r++)
                for (int c = 0; c < 4; c++)
                    in.w2o[r][c] = (float)inv[r][c];
        }
        // world box: transform the 8 corners of the padded mesh box in FP64;
        // a mesh without triangles is a point at the instance origin
        const Box& mb = mesh_box[in.mesh];
        Box wb;
        wb.reset();
        if (v->meshes[in.mesh].tri_count == 0) {
            const float o[3] = {in.data.transform[0][3], in.data.transform[1][3], in.data.transform[2][3]};
            wb.grow(o);
            inst_boxes[i] = wb;
            in.world_box = wb;
            continue;
        }
        for (int corner = 0; corner < 8; corner++) {
            double p[3] = {(corner & 1) ? mb.hi[0] : mb.lo[0], (corner & 2) ? mb.hi[1] : mb.lo[1], (corner & 4) ? mb.hi[2] : mb.lo[2]};
            float w[3];
            for (int r = 0; r < 3; r++)
                w[r] = (float)(in.data.transform[r][0] * p[0] + in.data.transform[r][1] * p[1] + in.data.transform[r][2] * p[2] +
                               in.data.transform[r][3]);
            wb.grow(w);
        }
        pad_box(wb);
        in.world_box = wb;
        inst_boxes[i] = wb;
    }
    if (!brute_force)
        build_bvh(s->tlas, inst_boxes, 1);
    return s;
}

void or_scene_destroy(or_scene* s) { delete s; }

void or_texture_sample(const or_scene* s, uint32_t index, float u, float v, float out[4])
{
    F4 t = sample_texture(*s, index, V2{u, v});
    out[0] = t.x;
    out[1] = t.y;
    out[2] = t.z;
    out[3] = t.w;
}

int or_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

int or_render(or_scene* s, const pt_render_params* P, uint32_t row_begin, uint32_t row_end, float* rgba, double* sum64,
              or_stats* stats_out, int threads)
{
    if (!s || !P || !rgba || P->width == 0 || P->height == 0 || P->samples == 0)
        return -1;
    row_end = std::min(row_end, P->height);
    const uint32_t W = P->width;
    const int64_t n_pix = (int64_t)(row_end - row_begin) * W;
    Stats total;
#ifdef _OPENMP
    int nt = threads > 0 ? threads : omp_get_max_threads();
#pragma omp parallel num_threads(nt)
#endif
    {
        Stats st;
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 64)
#endif
        for (int64_t k = 0; k < n_pix; k++) {
            uint32_t py = row_begin + (uint32_t)(k / W), px = (uint32_t)(k % W);
            float* dst = rgba + ((size_t)py * W + px) * 4;
            double* d64 = sum64 ? sum64 + ((size_t)py * W + px) * 4 : nullptr;
            for (uint32_t si = P->sample_index; si < P->sample_index + P->samples; si++) {
                V3 r = trace_sample(*s, *P, px, py, si, st, nullptr, 0, nullptr);
                r = correct_radiance(r * P->exposure);
                // running mean of pathtrace.rg.hlsl:62-67 with one sample per update
                if (si == 0) {
                    dst[0] = r.x / 1.0f;
                    dst[1] = r.y / 1.0f;
                    dst[2] = r.z / 1.0f;
                    dst[3] = 1.0f;
                } else {
                    float n = (float)(si + 1u);
                    dst[0] = dst[0] + (r.x - 1.0f * dst[0]) / n;
                    dst[1] = dst[1] + (r.y - 1.0f * dst[1]) / n;
                    dst[2] = dst[2] + (r.z - 1.0f * dst[2]) / n;
                }
                if (d64) {
                    d64[0] += (double)r.x;
                    d64[1] += (double)r.y;
                    d64[2] += (double)r.z;
                    d64[3] += 1.0;
                }
            }
        }
#ifdef _OPENMP
#pragma omp critical
#endif
        total.add(st);
    }
    if (stats_out) {
        stats_out->segments = total.segments;
        stats_out->shadow_rays = total.shadow_rays;
        stats_out->paths = total.paths;
        stats_out->node_visits = total.node_visits;
        stats_out->tri_tests = total.tri_tests;
        stats_out->inst_visits = total.inst_visits;
        stats_out->ray_count = total.rays;
    }
    return 0;
}

uint32_t or_path_signature(or_scene* s, const pt_render_params* P, uint32_t px, uint32_t py, uint32_t sample_index,
                           uint64_t* out, uint32_t cap)
{
    Stats st;
    uint32_t n = 0;
    trace_sample(*s, *P, px, py, sample_index, st, out, cap, &n);
    return n;
}

int or_intersect(or_scene* s, const float o[3], const float d[3], float tmin, float tmax, float* t, float* b1, float* b2,
                 uint32_t* instance, uint32_t* primitive)
{
    Stats st;
    Hit h = closest_hit(*s, v3(o[0], o[1], o[2]), v3(d[0], d[1], d[2]), tmin, tmax, st);
    if (!h.valid)
        return 0;
    *t = h.t;
    *b1 = h.b1;
    *b2 = h.b2;
    *instance = h.inst;
    *primitive = h.prim;
    return 1;
}

double or_meansq(const float* ref, const float* img, uint32_t w, uint32_t h)
{
    double sse = 0.0;
    for (size_t i = 0; i < (size_t)w * h * 4; i++) {
        if ((i % 4) == 3)
            continue;
        // meansq.cpp:39: `double error = image[i] - reference[i];` — the
        // difference is taken in float, then widened.
        double e = (double)(img[i] - ref[i]);
        sse += e * e;
    }
    return sse / ((double)w * h * 3 - 1);
}

double or_meansq64(const double* ref, const float* img, uint32_t w, uint32_t h)
{
    double sse = 0.0;
    for (size_t i = 0; i < (size_t)w * h * 4; i++) {
        if ((i % 4) == 3)
            continue;
        double e = (double)img[i] - ref[i];
        sse += e * e;
    }
    return sse / ((double)w * h * 3 - 1);
}

} // extern "C"

// ---------------------------------------------------------------- tone map (tonemap.cs.hlsl:17-77)
// ACES fit of the reference (src_is_srgb = false, dst_is_srgb = true, as
// ptdispatch.cpp:29 configures it): sRGB encode with the reference's
// threshold 0.00031308, sRGB->RRT matrix, RRT/ODT rational fit, ODT->sRGB
// matrix, saturate.  Alpha is passed through.
namespace {
inline float to_srgb_f(float x) { return x <= 0.00031308f ? 12.92f * x : 1.055f * std::pow(x, 1.0f / 2.4f) - 0.055f; }
} // namespace

extern "C" void or_tonemap(float* rgba, uint64_t pixels)
{
    static const float A[3][3] = {{0.59719f, 0.35458f, 0.04823f}, {0.07600f, 0.90834f, 0.01566f}, {0.02840f, 0.13383f, 0.83777f}};
    static const float B[3][3] = {{1.60475f, -0.53108f, -0.07367f}, {-0.10208f, 1.10813f, -0.00605f}, {-0.00327f, -0.07276f, 1.07602f}};
    for (uint64_t p = 0; p < pixels; p++) {
        float* c = rgba + 4 * p;
        float s[3] = {to_srgb_f(c[0]), to_srgb_f(c[1]), to_srgb_f(c[2])};
        float r[3], o[3];
        for (int i = 0; i < 3; i++)
            r[i] = (A[i][0] * s[0] + A[i][1] * s[1]) + A[i][2] * s[2];
        for (int i = 0; i < 3; i++) {
            float v = r[i];
            float a = v * (v + 0.0245786f) - 0.000090537f;
            float b = v * (0.983729f * v + 0.4329510f) + 0.238081f;
            r[i] = a / b;
        }
        for (int i = 0; i < 3; i++)
            o[i] = (B[i][0] * r[0] + B[i][1] * r[1]) + B[i][2] * r[2];
        for (int i = 0; i < 3; i++)
            c[i] = std::fmin(std::fmax(o[i], 0.0f), 1.0f); // saturate (NaN -> 0)
        for (int i = 0; i < 3; i++)
            if (std::isnan(o[i]))
                c[i] = 0.0f;
    }
}
