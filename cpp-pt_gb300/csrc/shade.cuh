// Device-side BxDFs, light sampling and random numbers for the PT+NEE+MIS
// integrator.  Each function names the reference code it follows; the
// arithmetic is single precision (the reference's double-literal steps are
// evaluated in float here, which changes results only in the last bits).
// Vector arithmetic and the BxDF formulas round every product and sum
// separately (__fmul_rn / __fadd_rn), in the reference's order: the
// reference's float code has no fused multiply-adds, and a contracted
// 1 - z*z near the normal (sin theta of GGX, the cosine-weighted
// hemisphere) would round differently from its own where the subtraction
// cancels.
#pragma once
#include "dev_types.h"

namespace cpppt_gb300 {

#define PT_MAT_DIFFUSE_ 0
#define PT_MAT_GGX_ 1
#define PT_MAT_DIELECTRIC_ 2
#define PT_MAT_EMISSIVE_ 3
#define PT_FLAG_THROUGHPUT_RR_ 16u  // PT_FLAG_THROUGHPUT_RR of the C ABI

constexpr float kPi = 3.14159265358979323846f;
constexpr float kInvPi = 0.318309886183790671538f;
constexpr float kEps = 1e-4f;  // EPS, src/math/math.h:11

struct f3 {
    float x, y, z;
};
// unfused single-precision steps
__device__ __forceinline__ float fm(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fa(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fs(float a, float b) { return __fsub_rn(a, b); }

__device__ __forceinline__ f3 mk(float x, float y, float z) { return {x, y, z}; }
__device__ __forceinline__ f3 operator+(f3 a, f3 b) { return {fa(a.x, b.x), fa(a.y, b.y), fa(a.z, b.z)}; }
__device__ __forceinline__ f3 operator-(f3 a, f3 b) { return {fs(a.x, b.x), fs(a.y, b.y), fs(a.z, b.z)}; }
__device__ __forceinline__ f3 operator*(f3 a, f3 b) { return {fm(a.x, b.x), fm(a.y, b.y), fm(a.z, b.z)}; }
__device__ __forceinline__ f3 operator*(f3 a, float s) { return {fm(a.x, s), fm(a.y, s), fm(a.z, s)}; }
__device__ __forceinline__ f3 operator-(f3 a) { return {-a.x, -a.y, -a.z}; }
__device__ __forceinline__ float dot(f3 a, f3 b) { return fa(fa(fm(a.x, b.x), fm(a.y, b.y)), fm(a.z, b.z)); }
__device__ __forceinline__ f3 cross(f3 a, f3 b) {
    return {fs(fm(a.y, b.z), fm(a.z, b.y)), fs(fm(a.z, b.x), fm(a.x, b.z)), fs(fm(a.x, b.y), fm(a.y, b.x))};
}
__device__ __forceinline__ float length(f3 a) { return sqrtf(dot(a, a)); }
__device__ __forceinline__ f3 normalized(f3 a) { return a * (1.0f / length(a)); }
__device__ __forceinline__ f3 f3of(float4 v) { return {v.x, v.y, v.z}; }

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw: "Parallel Random Numbers: As
// Easy as 1, 2, 3", SC 2011).  Counter-based: a path's numbers depend only on
// (seed, sample, pixel, bounce), so batching and scheduling cannot change them.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint4 philox4x32(uint4 c, uint2 k) {
#pragma unroll
    for (int r = 0; r < 10; r++) {
        const uint32_t lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
        const uint32_t lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
        c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
        k.x += 0x9E3779B9u;
        k.y += 0xBB67AE85u;
    }
    return c;
}
__device__ __forceinline__ float u01(uint32_t x) { return (float)(x >> 8) * (1.0f / 16777216.0f); }

// ---------------------------------------------------------------------------
// Film: signed 32.32 fixed point, one 64-bit integer per pixel and channel.
// Integer addition is associative, so a render's image does not depend on
// the order in which contributions arrive.  A contribution below
// ctr->film_safe cannot carry the sum out of range (fire-and-forget add);
// a larger one adds with the returned old value and counts a sum that left
// the range (and one that cannot be represented at all is dropped and
// counted); the host then fails the render.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void film_add1(unsigned long long* cell, float v, float safe, WaveCounters* ctr) {
    if (v == 0.f) return;
    const float a = fabsf(v);
    const float s = 4294967296.0f;
    if (a < safe) {
        atomicAdd(cell, (unsigned long long)__float2ll_rn(v * s));
        return;
    }
    if (a >= 2147483648.0f) {  // the contribution alone exceeds the range
        atomicAdd(&ctr->stat_film_overflow, 1ull);
        return;
    }
    const long long q = __float2ll_rn(v * s);
    const long long old = (long long)atomicAdd(cell, (unsigned long long)q);
    const long long sum = (long long)((unsigned long long)old + (unsigned long long)q);
    if ((q > 0 && sum < old) || (q < 0 && sum > old)) atomicAdd(&ctr->stat_film_overflow, 1ull);
}

// One pixel's contribution (r, g, b); inf / NaN ones are dropped and counted.
__device__ __forceinline__ void film_add_rgb(unsigned long long* film, size_t pix, float r, float g, float b,
                                             WaveCounters* ctr) {
    if (!isfinite(r) || !isfinite(g) || !isfinite(b)) {
        atomicAdd(&ctr->stat_nonfinite, 1ull);
        return;
    }
    const float safe = ctr->film_safe;
    film_add1(film + 3 * pix, r, safe, ctr);
    film_add1(film + 3 * pix + 1, g, safe, ctr);
    film_add1(film + 3 * pix + 2, b, safe, ctr);
}

struct Rng4 {
    float v[4];
};
// stream: 0,1 = per-bounce streams; 0xffff = camera
__device__ __forceinline__ Rng4 rng4(uint32_t seed, uint32_t sample, uint32_t pixel, uint32_t bounce, uint32_t stream) {
    uint4 r = philox4x32(make_uint4(pixel, bounce, stream, sample), make_uint2(seed, 0x5eed1234u ^ sample));
    return {{u01(r.x), u01(r.y), u01(r.z), u01(r.w)}};
}

// ---------------------------------------------------------------------------
// Surface interaction (Triangle::intersect, triangle.h:83-114; then
// Intersection::get_bxdf, intersection.h:25-33).
// ---------------------------------------------------------------------------
struct Surf {
    f3 p, n, ng, t, b;  // hitpoint, shading normal, geometric normal, tangent, bitangent
    int32_t mat;
};

// ---------------------------------------------------------------------------
// Image textures (ImageTexture::sample, src/texture/image_texture.h:24-41,
// on Image::get_pixel with the default REPEAT border, src/image/rgb_image.h:
// 210-250).  The reference leaves ImageTexture::filtering uninitialised; the
// bilinear branch is used here.  Where the reference's wrap of a negative
// multiple of the size yields the size itself (i % n + n), the pixel index
// runs on into the next row as there, and is clamped to the image.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int tex_wrap(int i, int n) {
    if (i >= n) return i % n;
    if (i < 0) return i % n + n;
    return i;
}

__device__ __forceinline__ f3 tex_pixel(const DevScene& S, int4 info, int i, int j) {
    const int w = info.y, h = info.z;
    int idx = tex_wrap(i, w) + tex_wrap(j, h) * w;
    idx = min(max(idx, 0), w * h - 1);
    const float* p = S.tex_px + info.x + (size_t)idx * info.w;
    if (info.w == 1) {
        const float v = __ldg(p);
        return mk(v, v, v);
    }
    return mk(__ldg(p), __ldg(p + 1), __ldg(p + 2));
}

__device__ __forceinline__ f3 tex_sample(const DevScene& S, uint32_t t, float u, float v) {
    const int4 info = __ldg(S.tex_info + t);
    float x = u * (float)info.y;
    float y = (float)((1.0 - (double)v) * (double)info.z);
    x = (float)((double)x - 0.5);
    y = (float)((double)y - 0.5);
    const int i = (int)floorf(x), j = (int)floorf(y);
    x = x - (float)i;
    y = y - (float)j;
    const f3 p00 = tex_pixel(S, info, i, j), p10 = tex_pixel(S, info, i + 1, j);
    const f3 p01 = tex_pixel(S, info, i, j + 1), p11 = tex_pixel(S, info, i + 1, j + 1);
    return (p00 * (1.0f - x) + p10 * x) * (1.0f - y) + (p01 * (1.0f - x) + p11 * x) * y;
}

// StandardMaterial::get_bxdf / EmissiveMaterial::get_bxdf at uv
// (standard_material.h:46-61, emissive_material.h:28-30): the textured
// albedo or emission colour, the BxDF picked by the metal value and the
// GGX parameters from the roughness value.
__device__ __forceinline__ void apply_textures(const DevScene& S, DevMaterial& m, float u, float v) {
    const uint32_t ta = m.tex & 0xffu, tr = (m.tex >> 8) & 0xffu, tm = (m.tex >> 16) & 0xffu;
    if (m.kind == PT_MAT_EMISSIVE_) {
        if (ta != kNoTex) {
            const f3 c = tex_sample(S, ta, u, v);
            m.r = c.x * m.alpha;
            m.g = c.y * m.alpha;
            m.b = c.z * m.alpha;
        }
        return;
    }
    if (ta != kNoTex) {
        const f3 c = tex_sample(S, ta, u, v);
        m.r = c.x; m.g = c.y; m.b = c.z;
    }
    if (tm != kNoTex) m.kind = (double)tex_sample(S, tm, u, v).x < 0.1 ? PT_MAT_DIFFUSE_ : PT_MAT_GGX_;
    if (tr != kNoTex) {
        const float r = tex_sample(S, tr, u, v).x;
        m.alpha = fmaxf(r * r, 0.01f);  // glossy_bxdf.h:23, 77-79
        m.delta = (double)r < 0.01 ? 1 : 0;
    }
}

__device__ __forceinline__ Surf make_surf(const DevScene& S, int32_t prim, f3 o, f3 d, float t, float beta, float gamma,
                                          bool first_hit, int32_t* kind_out, DevMaterial* mat_out) {
    const int4 vi = __ldg(S.tri_vidx + prim);
    const float alpha = 1.0f - (gamma + beta);
    const f3 a = f3of(__ldg(S.v_pos + vi.x)), b = f3of(__ldg(S.v_pos + vi.y)), c = f3of(__ldg(S.v_pos + vi.z));
    const f3 n = normalized(f3of(__ldg(S.v_nrm + vi.x)) * alpha + f3of(__ldg(S.v_nrm + vi.y)) * beta +
                            f3of(__ldg(S.v_nrm + vi.z)) * gamma);
    const f3 bt = normalized(f3of(__ldg(S.v_btan + vi.x)) * alpha + f3of(__ldg(S.v_btan + vi.y)) * beta +
                             f3of(__ldg(S.v_btan + vi.z)) * gamma);
    Surf s;
    s.p = o + d * t;
    s.n = n;
    s.ng = normalized(cross(b - a, c - a));
    s.b = bt;
    s.t = normalized(cross(bt, n));
    s.mat = vi.w;
    DevMaterial m = S.mats[vi.w];
    f3 nmap = mk(0.f, 0.f, 1.f);  // tangent-space normal of a normal-map texture
    bool mapped = false;          // the constant map rgb(0.5,0.5,1) is the identity
    if (m.tex != kNoTextures) {
        // triangle.h:91-94: uv1 * alpha + uv2 * beta + uv3 * gamma
        const float2 t0 = __ldg(S.v_uv + vi.x), t1 = __ldg(S.v_uv + vi.y), t2 = __ldg(S.v_uv + vi.z);
        const float u = fa(fa(fm(t0.x, alpha), fm(t1.x, beta)), fm(t2.x, gamma));
        const float v = fa(fa(fm(t0.y, alpha), fm(t1.y, beta)), fm(t2.y, gamma));
        const uint32_t tn = m.tex >> 24;
        if (first_hit && tn != kNoTex && (m.kind == PT_MAT_DIFFUSE_ || m.kind == PT_MAT_GGX_)) {
            const f3 c = tex_sample(S, tn, u, v);  // standard_material.h:64-71
            nmap = mk(c.x * 2.0f - 1.0f, c.y * 2.0f - 1.0f, c.z);
            mapped = true;
        }
        apply_textures(S, m, u, v);
    }
    *mat_out = m;
    *kind_out = m.kind;
    // The reference's Intersection is reused for all bounces of a path and
    // its computed_normal flag is never reset, so normal mapping
    // (standard_material.h:64-71: Mat3(tangent, bitangent, normal) times the
    // map's value) and the re-orthogonalisation only run at the first hit.
    if (first_hit) {
        if (m.kind == PT_MAT_DIFFUSE_ || m.kind == PT_MAT_GGX_)
            s.n = normalized(mapped ? s.t * nmap.x + s.b * nmap.y + s.n * nmap.z : s.n);
        s.b = normalized(cross(s.n, s.t));
        s.t = normalized(cross(s.b, s.n));
    }
    return s;
}

// BxDF::same_hemisphere (bxdf.h:42-45)
__device__ __forceinline__ bool same_hemisphere(const Surf& s, f3 wo, f3 wi) {
    const float sign = dot(wo, s.ng);
    return sign * dot(wi, s.n) > 0.f && sign * dot(wi, s.ng) > 0.f;
}

// ---------------------------------------------------------------------------
// GGX (MicrofacetDistribution, microfacet_distribution.h:9-168), isotropic.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float sin_t(f3 w) { return sqrtf(fmaxf(0.0f, fs(1.0f, fm(w.z, w.z)))); }
__device__ __forceinline__ float cos_p(f3 w) { const float s = sin_t(w); return s == 0.f ? 1.f : w.x / s; }
__device__ __forceinline__ float sin_p(f3 w) { const float s = sin_t(w); return s == 0.f ? 1.f : w.y / s; }

__device__ __forceinline__ float ggx_d(float a, f3 wh) {
    float tan2 = sin_t(wh) / wh.z;
    tan2 = fm(tan2, tan2);
    if (isinf(tan2)) return 0.f;
    const float cos4 = fm(fm(wh.z, wh.z), fm(wh.z, wh.z));
    const float cp = cos_p(wh), sp = sin_p(wh);
    const float a2 = fm(a, a);
    const float e = fm(fa(fm(cp, cp) / a2, fm(sp, sp) / a2), tan2);
    const float e1 = fa(1.f, e);
    return 1.0f / fm(fm(fm(fm(fm(kPi, a), a), cos4), e1), e1);
}
// |cos(theta)/sin(theta)| as written at microfacet_distribution.h:138
// The reference evaluates (-1 + sqrt(1 + x)) / 2 in double; the same value
// in float without the cancellation is x / (2 (1 + sqrt(1 + x))).
__device__ __forceinline__ float ggx_lambda(float a, f3 w) {
    const float abs_tan = fabsf(w.z / sin_t(w));
    if (isinf(abs_tan)) return 0.f;
    const float cp = cos_p(w), sp = sin_p(w);
    const float al = sqrtf(fa(fm(fm(fm(cp, cp), a), a), fm(fm(fm(sp, sp), a), a)));
    const float at = fm(al, abs_tan);
    const float a2t2 = fm(at, at);
    return a2t2 / fm(2.0f, fa(1.0f, sqrtf(fa(1.0f, a2t2))));
}
__device__ __forceinline__ float ggx_g(float a, f3 wo, f3 wi) {
    return 1.0f / fa(fa(1.0f, ggx_lambda(a, wo)), ggx_lambda(a, wi));
}
__device__ __forceinline__ float ggx_g1(float a, f3 w) { return 1.0f / fa(1.0f, ggx_lambda(a, w)); }
__device__ __forceinline__ float ggx_pdf_h(float a, f3 wo, f3 wh) {
    return fm(fm(ggx_d(a, wh), ggx_g1(a, wo)), fabsf(dot(wo, wh))) / fabsf(wo.z);
}

// sample11 (microfacet_distribution.h:13-58), PBRT-3 visible-normal sampling
__device__ __forceinline__ void ggx_sample11(float cos_theta, float U1, float U2, float& sx, float& sy) {
    if (cos_theta > .9999f) {
        const float r = sqrtf(U1 / fs(1.f, U1));
        const float phi = fm(6.28318530718f, U2);
        float sn, cs;
        sincosf(phi, &sn, &cs);
        sx = fm(r, cs);
        sy = fm(r, sn);
        return;
    }
    const float sin_theta = sqrtf(fmaxf(0.f, fs(1.f, fm(cos_theta, cos_theta))));
    const float tan_theta = sin_theta / cos_theta;
    const float a = 1.f / tan_theta;
    const float G1 = 2.f / fa(1.f, sqrtf(fa(1.f, 1.f / fm(a, a))));
    const float A = fs(fm(2.f, U1) / G1, 1.f);
    float tmp = 1.f / fs(fm(A, A), 1.f);
    if (tmp > 1e10f) tmp = 1e10f;
    const float B = tan_theta;
    const float D = sqrtf(fmaxf(fs(fm(fm(fm(B, B), tmp), tmp), fm(fs(fm(A, A), fm(B, B)), tmp)), 0.f));
    const float s1 = fs(fm(B, tmp), D), s2 = fa(fm(B, tmp), D);
    sx = (A < 0.f || s2 > 1.f / tan_theta) ? s1 : s2;
    float S;
    if (U2 > 0.5f) { S = 1.f; U2 = fm(2.f, fs(U2, .5f)); }
    else { S = -1.f; U2 = fm(2.f, fs(.5f, U2)); }
    const float z = fm(U2, fa(fm(U2, fs(fm(U2, 0.27385f), 0.73369f)), 0.46341f)) /
                    fa(fm(U2, fs(fm(U2, fa(fm(U2, 0.093073f), 0.309420f)), 1.000000f)), 0.597999f);
    sy = fm(fm(S, z), sqrtf(fa(1.f, fm(sx, sx))));
    if (isinf(sy) || isnan(sy)) sy = 0.f;
}

__device__ __forceinline__ f3 ggx_sample_wh(float a, f3 wi, float U1, float U2) {
    const f3 ws = normalized(mk(fm(a, wi.x), fm(a, wi.y), wi.z));
    float sx, sy;
    ggx_sample11(ws.z, U1, U2, sx, sy);
    const float cp = cos_p(ws), sp = sin_p(ws);
    const float tmp = fs(fm(cp, sx), fm(sp, sy));
    sy = fa(fm(sp, sx), fm(cp, sy));
    sx = tmp;
    return normalized(mk(-fm(a, sx), -fm(a, sy), 1.f));
}

// frame helpers: Mat3(tangent, bitangent, normal) and its transpose
__device__ __forceinline__ f3 to_local(const Surf& s, f3 v) { return mk(dot(s.t, v), dot(s.b, v), dot(s.n, v)); }
__device__ __forceinline__ f3 to_world(const Surf& s, f3 v) { return s.t * v.x + s.b * v.y + s.n * v.z; }
__device__ __forceinline__ f3 reflect(f3 wo, f3 wh) { return normalized(-wo + wh * (dot(wh, wo) * 2.0f)); }

// ---------------------------------------------------------------------------
// BxDF dispatch: eval includes the cosine (diffuse_bxdf.h:25-27).
// ---------------------------------------------------------------------------
__device__ __forceinline__ f3 bsdf_eval(const DevMaterial& m, const Surf& s, f3 wo, f3 wi) {
    if (m.kind == PT_MAT_DIFFUSE_) {  // albedo * |n.wi| divided by pi (a product with 1/pi, as vdivs)
        const float c = fabsf(dot(s.n, wi));
        return mk(fm(m.r, c), fm(m.g, c), fm(m.b, c)) * kInvPi;
    }
    if (m.kind == PT_MAT_GGX_) {  // glossy_bxdf.h:23-33: white, no Fresnel, signed cos
        const f3 wol = normalized(to_local(s, wo)), wil = normalized(to_local(s, wi));
        const f3 wh = normalized(wol + wil);
        const float v = fm(ggx_g(m.alpha, wol, wil), ggx_d(m.alpha, wh)) / fm(4.0f, dot(wo, s.n));
        return mk(v, v, v);
    }
    if (m.kind == PT_MAT_DIELECTRIC_) return mk(1.f, 1.f, 1.f);
    return mk(0.f, 0.f, 0.f);
}

__device__ __forceinline__ float bsdf_pdf(const DevMaterial& m, const Surf& s, f3 wo, f3 wi) {
    if (m.kind == PT_MAT_DIFFUSE_) return fabsf(dot(s.n, wi)) * kInvPi;
    if (m.kind == PT_MAT_GGX_) {  // glossy_bxdf.h:55-72
        const f3 wol = normalized(to_local(s, wo));
        const f3 wh = normalized(to_local(s, wo + wi));
        return ggx_pdf_h(m.alpha, wol, wh) / fm(4.0f, fabsf(dot(wol, wh)));
    }
    return 1.0f;
}

struct BSample {
    f3 wi;
    float pdf;
    bool delta;
};

// math.h:663-688
__device__ __forceinline__ void orthogonal(f3 v1, f3& x, f3& y, f3& z) {
    const float ax = fabsf(v1.x), ay = fabsf(v1.y), az = fabsf(v1.z);
    f3 aux;
    if (ax < ay) aux = ax < az ? mk(1, 0, 0) : mk(0, 0, 1);
    else aux = ay < az ? mk(0, 1, 0) : mk(0, 0, 1);
    const f3 aux2 = cross(v1, aux);
    x = normalized(v1);
    y = normalized(cross(aux2, v1));
    z = normalized(aux2);
}

__device__ __forceinline__ BSample bsdf_sample(const DevMaterial& m, const Surf& s, f3 wo, float u1, float u2) {
    BSample r;
    if (m.kind == PT_MAT_DIFFUSE_) {  // diffuse_bxdf.h:28-41 + sample_hemisphere_cos (math.h:647-653)
        const float theta = fm(fm(u1, 2.0f), kPi);
        const float sin_phi = sqrtf(u2);
        const float cos_phi = sqrtf(fmaxf(0.f, fs(1.0f, fm(sin_phi, sin_phi))));
        float sn, cs;
        sincosf(theta, &sn, &cs);
        const f3 sm = mk(fm(cs, sin_phi), fm(sn, sin_phi), cos_phi);
        f3 n = s.n;
        if (dot(n, wo) < 0.f) n = -n;  // correct_normal, bxdf.h:52-57
        f3 x, y, z;
        orthogonal(n, x, y, z);
        r.wi = y * sm.x + z * sm.y + x * sm.z;  // Mat3(y, z, x) * sample
        r.pdf = fm(sm.z, kInvPi);
        r.delta = false;
        return r;
    }
    if (m.kind == PT_MAT_GGX_) {  // glossy_bxdf.h:34-46
        if (m.delta) {
            r.wi = reflect(wo, s.n);
            r.pdf = 1.0f;
            r.delta = true;
            return r;
        }
        const f3 wol = normalized(to_local(s, wo));
        const f3 whl = normalized(ggx_sample_wh(m.alpha, wol, u1, u2));
        const f3 wh = normalized(to_world(s, whl));
        r.wi = reflect(wo, wh);
        r.pdf = bsdf_pdf(m, s, wo, r.wi);
        r.delta = false;
        return r;
    }
    // RefractionBxDF::sample (refraction_bxdf.h:26-52)
    f3 n = s.n;
    float n2 = 1.0f / m.ior;
    if (dot(n, wo) < 0.f) { n2 = 1.0f / n2; n = -n; }
    const float ci = dot(wo, n);
    const float ct2 = fs(1.0f, fm(fm(n2, n2), fs(1.0f, fm(ci, ci))));
    f3 w;
    if (ct2 < 0.f) w = normalized(-wo + s.n * fm(dot(s.n, wo), 2.0f));
    else w = normalized((-wo) * n2 + n * fs(fm(n2, ci), sqrtf(ct2)));
    r.wi = w;
    r.pdf = 1.0f;
    r.delta = true;
    return r;
}

// Russian roulette survival (pathtracerMIS.h:24-27), computed on eval
__device__ __forceinline__ float russian_roulette(f3 ev) {
    return fabsf(ev.x * 0.2f + ev.y * 0.5f + ev.z * 0.3f) * 0.5f + 0.4f;
}

// LightGroup::connect_eye_path + ShapeLight::connect_eye_path + Triangle::sample
// (light_group.h:25-30, shape_light.h:24-44, triangle.h:209-269)
struct LSample {
    f3 pos, n, le;  // le = Le * |n_l . normalize(from - pos)|
    float pdf;      // (1/n_lights) * (1/area)
};
__device__ __forceinline__ LSample sample_light(const DevScene& S, f3 from, float u0, float u1, float u2) {
    LSample ls;
    const int nl = S.n_lights;
    int k = (int)(u0 * (float)nl) % nl;
    const int32_t prim = __ldg(S.light_prim + k);
    const int4 vi = __ldg(S.tri_vidx + prim);
    float al = u1, be = u2;
    if (al + be > 1.0f) { al = 1.0f - al; be = 1.0f - be; }
    const float ga = fs(fs(1.0f, al), be);
    const f3 a = f3of(__ldg(S.v_pos + vi.x)), b = f3of(__ldg(S.v_pos + vi.y)), c = f3of(__ldg(S.v_pos + vi.z));
    ls.pos = a * al + b * be + c * ga;
    ls.n = normalized(f3of(__ldg(S.v_nrm + vi.x)) * al + f3of(__ldg(S.v_nrm + vi.y)) * be +
                      f3of(__ldg(S.v_nrm + vi.z)) * ga);
    DevMaterial m = S.mats[vi.w];
    if (m.tex != kNoTextures) {
        // triangle.h:244-249 interpolates the sampled point's uv as
        // uv1 * alpha + uv2 * beta + uv2 * gamma (the second vertex twice)
        const float2 t0 = __ldg(S.v_uv + vi.x), t1 = __ldg(S.v_uv + vi.y);
        apply_textures(S, m, fa(fa(fm(t0.x, al), fm(t1.x, be)), fm(t1.x, ga)),
                       fa(fa(fm(t0.y, al), fm(t1.y, be)), fm(t1.y, ga)));
    }
    const float cosl = fabsf(dot(ls.n, normalized(from - ls.pos)));
    ls.le = mk(fm(m.r, cosl), fm(m.g, cosl), fm(m.b, cosl));
    ls.pdf = fm(1.0f / __ldg(S.light_area + k), 1.0f / (float)nl);
    return ls;
}

}  // namespace cpppt_gb300
