// BSDFs of the reference's materials, evaluated in the local frame (x = dpdu, y = N, z = dpdv).
//
// Every material of the reference builds exactly one BxDF per hit (Materials/*.cpp), so the
// BSDF container (BSDFs/BSDF.cpp:25-130) reduces to: world->local by the transposed TNB frame
// and fixVector, the reflect/transmit selection of Pdf and DistributionFunction (with the
// operator-precedence behaviour of BSDF.cpp:39-40), and one sampled BxDF.
#pragma once
#include "dev_common.cuh"

namespace c2g {

struct Frame {
    float3 T, N, B;  // dpdu, shading normal (facing the incoming ray), dpdv
};

__device__ __forceinline__ float3 to_local(const Frame& f, float3 w) {
    return clamp1(f3(dot(f.T, w), dot(f.N, w), dot(f.B, w)));
}
__device__ __forceinline__ float3 to_world(const Frame& f, float3 w) {
    return clamp1(f.T * w.x + f.N * w.y + f.B * w.z);
}

struct BxDF {
    int mtype;
    int flags;          // BxDFType of the material's BxDF
    float3 R;           // color / kd
    float3 S;           // ks (plastic)
    float ax, ay;
    float etaA, etaB;
};

__device__ __forceinline__ int material_flags(int mtype) {
    switch (mtype) {
        case MAT_DIFFUSE: return BXDF_DIFFUSE | BXDF_REFLECTION;
        case MAT_MIRROR: return BXDF_SPECULAR | BXDF_REFLECTION;
        case MAT_GLASS_ROUGH: return BXDF_TRANSMISSION | BXDF_REFLECTION | BXDF_GLOSSY;
        case MAT_GLASS_SMOOTH: return BXDF_TRANSMISSION | BXDF_REFLECTION | BXDF_SPECULAR;
        case MAT_MICRO_GGX:
        case MAT_MICRO_BECKMANN: return BXDF_REFLECTION | BXDF_GLOSSY;
        case MAT_PLASTIC_GGX:
        case MAT_PLASTIC_BECKMANN: return BXDF_REFLECTION | BXDF_GLOSSY;
        case MAT_ORENNAYAR: return BXDF_DIFFUSE | BXDF_REFLECTION;
        case MAT_BLINNPHONG: return BXDF_GLOSSY | BXDF_REFLECTION;
    }
    return 0;
}

__device__ __forceinline__ BxDF make_bxdf(const Material& m, bool front_face) {
    BxDF b;
    b.mtype = m.type;
    b.flags = material_flags(m.type);
    b.R = f3(m.color[0], m.color[1], m.color[2]);
    b.S = f3(m.ks[0], m.ks[1], m.ks[2]);
    b.ax = m.ax;
    b.ay = m.ay;
    // Glass / Micro swap the IORs on back faces (Glass.cpp:19-20, MicrofacetMaterial.cpp:20-21);
    // Mirror uses 1, 1 (MirrorMaterial.cpp:11-13).
    b.etaA = 1.f;
    const bool dielectric = m.type != MAT_MIRROR && m.type != MAT_DIFFUSE && m.type != MAT_ORENNAYAR && m.type != MAT_BLINNPHONG;
    b.etaB = dielectric ? m.ior : 1.f;
    if (!front_face && dielectric) { float t = b.etaA; b.etaA = b.etaB; b.etaB = t; }
    if (m.type == MAT_BLINNPHONG) b.ax = m.ior;  // the exponent K
    return b;
}

__device__ __forceinline__ float sq(float x) { return x * x; }

// ---- Fresnel (BSDFs/Models/Fresnel.cpp) -------------------------------------------------
__device__ __forceinline__ float fresnel_dielectric(float etaA, float etaB, float cosI) {
    float sinI = sqrtf(fmaxf(0.f, 1.f - cosI * cosI));
    float sinT = etaA / etaB * sinI;
    if (sinT >= 1.f) return 1.f;
    float cosT = sqrtf(fmaxf(0.f, 1.f - sinT * sinT));
    float rparl = ((etaB * cosI) - (etaA * cosT)) / ((etaB * cosI) + (etaA * cosT));
    float rperp = ((etaA * cosI) - (etaB * cosT)) / ((etaA * cosI) + (etaB * cosT));
    return (rparl * rparl + rperp * rperp) / 2;
}
__device__ __forceinline__ float fresnel_schlick(float r0, float etaA, float etaB, float cosI) {
    float sinI = sqrtf(fmaxf(0.f, 1.f - cosI * cosI));
    float sinT = etaA / etaB * sinI;
    if (sinT >= 1.f) return 1.f;
    return r0 + (1.f - r0) * powf(1.f - cosI, 5.f);
}
// Micro uses Schlick with R0 = 0.99 (MicrofacetMaterial.cpp:23); glass uses the dielectric.
__device__ __forceinline__ float bxdf_fresnel(const BxDF& b, float cosI) {
    if (b.mtype == MAT_MICRO_GGX || b.mtype == MAT_MICRO_BECKMANN) return fresnel_schlick(0.99f, b.etaA, b.etaB, cosI);
    return fresnel_dielectric(b.etaA, b.etaB, cosI);
}

// ---- microfacet distributions (BSDFs/Models/MicrofacetDistribution.cpp) -------------------
__device__ __forceinline__ bool is_beckmann(int mtype) { return mtype == MAT_MICRO_BECKMANN || mtype == MAT_PLASTIC_BECKMANN; }

__device__ __forceinline__ float2 cos_sin_phi(float3 w, float sinT) {
    if (sinT == 0.f) return make_float2(1.f, 0.f);
    return make_float2(fminf(fmaxf(w.x / sinT, -1.f), 1.f), fminf(fmaxf(-w.z / sinT, -1.f), 1.f));
}

__device__ __forceinline__ float ndf_D(const BxDF& b, float3 wh) {
    if (!is_beckmann(b.mtype)) {
        float cos2 = wh.y * wh.y;
        float sin2 = fmaxf(0.f, 1.f - cos2);
        float2 p = cos_sin_phi(wh, sqrtf(sin2));
        float A = sq(p.x) / sq(b.ax) + sq(p.y) / sq(b.ay);
        return 1.f / (kPiF * b.ax * b.ay * sq(A - cos2 * (A - 1)));
    }
    float cos2 = wh.y * wh.y;
    float sin2 = 1.f - cos2;
    float tan2 = sin2 / cos2;
    if (isinf(tan2)) return 0.f;
    float cos4 = cos2 * cos2;
    float2 v = cos_sin_phi(wh, sqrtf(sin2));
    float bot = kPiF * b.ax * b.ay * cos4;
    float top = expf(-tan2 * (sq(v.x) / sq(b.ax) + sq(v.y) / sq(b.ay)));
    return top / bot;
}

__device__ __forceinline__ float ndf_lambda(const BxDF& b, float3 w) {
    if (!is_beckmann(b.mtype)) {
        float cos2 = w.y * w.y;
        float sin2 = 1.f - cos2;
        float tan2 = sin2 / cos2;
        if (isinf(tan2)) return 0.f;
        float2 p = cos_sin_phi(w, sqrtf(sin2));
        float a2 = sq(p.x) * sq(b.ax) + sq(p.y) * sq(b.ay);
        return (-1 + sqrtf(1 + a2 * tan2)) / 2;
    }
    float cosT = w.y;
    float sinT = sqrtf(1.f - cosT * cosT);
    float tanT = fabsf(sinT / cosT);
    if (isinf(tanT)) return 0.f;
    float2 v = cos_sin_phi(w, sinT);
    float alpha = sqrtf(sq(v.x) * sq(b.ax) + sq(v.y) * sq(b.ay));
    float a = 1.f / (tanT * alpha);
    if (a >= 1.6f) return 0.f;
    return (1 - 1.259f * a + 0.396f * a * a) / (3.535f * a + 2.181f * a * a);
}

__device__ __forceinline__ float ndf_G(const BxDF& b, float3 wo, float3 wi) {
    return 1.f / (1.f + ndf_lambda(b, wo) + ndf_lambda(b, wi));
}

__device__ __forceinline__ float ndf_pdf(const BxDF& b, float3 wh) { return ndf_D(b, wh) * fabsf(wh.y); }

// GetUnitVectorUsingCos (Utils.h:79-83)
__device__ __forceinline__ float3 unit_from_cos(float cosT, float phi) {
    float r = sqrtf(1 - cosT * cosT);
    float s, c;
    sincosf(phi, &s, &c);
    return f3(r * c, cosT, -r * s);
}

__device__ __forceinline__ float3 ndf_sample(const BxDF& b, float2 u) {
    float cosT, phi;
    if (!is_beckmann(b.mtype)) {
        if (b.ax == b.ay) {
            cosT = sqrtf((1 - u.x) / (u.x * (b.ax * b.ax - 1) + 1));
            phi = kTwoPiF * u.y;
        } else {
            phi = atanf(b.ay / b.ax * tanf(kTwoPiF * u.y + kHalfPiF));
            if (u.y > 0.5f) phi += kPiF;
            float s, c;
            sincosf(phi, &s, &c);
            float A = sq(c) / sq(b.ax) + sq(s) / sq(b.ay);
            float cos2 = A * (u.x - 1) / (u.x * (A - 1) - A);
            cosT = sqrtf(cos2);
        }
        return unit_from_cos(cosT, phi);
    }
    float logS = logf(1.f - u.x);
    if (isinf(logS)) logS = 0;
    float tan2;
    if (b.ax == b.ay) {
        tan2 = -sq(b.ax) * logS;
        phi = u.y * kTwoPiF;
    } else {
        phi = atanf(b.ay / b.ax * tanf(kTwoPiF * u.y + kHalfPiF));
        if (u.y > 0.5f) phi += kPiF;
        float s, c;
        sincosf(phi, &s, &c);
        tan2 = -logS / (c * c / sq(b.ax) + s * s / sq(b.ay));
    }
    cosT = 1.f / sqrtf(1.f + tan2);
    return unit_from_cos(cosT, phi);
}

__device__ __forceinline__ float3 reflect(float3 I, float3 N) { return I - N * dot(N, I) * 2.f; }

// refract(wo, wh, eta, wt) (Utils.h:102-112)
__device__ __forceinline__ bool refract(float3 wo, float3 wh, float eta, float3& wt) {
    float cosO = fminf(fmaxf(dot(wo, wh), -1.f), 1.f);
    float sin2O = fmaxf(0.f, 1.f - cosO * cosO);
    float sin2I = eta * eta * sin2O;
    if (sin2I > 1.f) return false;
    float cosI = sqrtf(1.f - sin2I);
    wt = eta * (-wo) + (eta * cosO - cosI) * wh;
    return true;
}

// ---- microfacet BxDFs (BSDFs/Microfacet.cpp) --------------------------------------------
__device__ __forceinline__ float mf_refl_pdf(const BxDF& b, float3 wo, float3 wi) {
    float3 H = normalize(wo + wi);
    return ndf_pdf(b, H) / (4 * dot(wo, H));
}
__device__ __forceinline__ float3 mf_refl_f(const BxDF& b, float3 wo, float3 wi) {
    if (wo.y * wi.y < 0) return f3(0.f, 0.f, 0.f);
    float3 H = normalize(wo + wi);
    float F = bxdf_fresnel(b, fmaxf(0.f, dot(wo, H)));
    float G = ndf_G(b, wo, wi);
    float D = ndf_D(b, H);
    return b.R * D * G * F / (4 * fmaxf(0.f, wi.y) * fmaxf(0.f, wo.y));
}
__device__ __forceinline__ float mf_trans_pdf(const BxDF& b, float3 wo, float3 wi) {
    if (wo.y * wi.y > 0) return 0.f;
    float eta = b.etaB / b.etaA;
    float3 H = normalize(wo + wi * eta);
    float absDot = fabsf(dot(H, wi));
    float dwh = eta * eta * absDot / sq(dot(wo, H) + eta * dot(wi, H));
    return ndf_pdf(b, H) * dwh;
}
__device__ __forceinline__ float3 mf_trans_f(const BxDF& b, float3 wo, float3 wi) {
    if (wi.y * wo.y > 0) return f3(0.f, 0.f, 0.f);
    if (wo.y == 0.f) return f3(0.f, 0.f, 0.f);
    float eta = b.etaB / b.etaA;
    float3 H = normalize(wo + wi * eta);
    if (H.y < 0) H = -H;
    float bot = sq(dot(wo, H) + eta * dot(wi, H));
    float F = 1.f - bxdf_fresnel(b, fmaxf(0.f, dot(wo, H)));
    float G = ndf_G(b, wo, wi);
    float D = ndf_D(b, H);
    return b.R * D * G * F * fabsf(dot(H, wo)) * fabsf(dot(H, wi)) / (bot * fmaxf(0.f, -wi.y) * fmaxf(0.f, wo.y));
}

// ---- FresnelBlend (BSDFs/FresnelBlend.cpp) ----------------------------------------------
__device__ __forceinline__ float fb_pdf(const BxDF& b, float3 wo, float3 wi) {
    float3 H = normalize(wo + wi);
    return 0.5f * (fmaxf(0.f, wi.y) / kPiF + ndf_pdf(b, H) / (4 * dot(wo, H)));
}
__device__ __forceinline__ float3 fb_f(const BxDF& b, float3 wo, float3 wi) {
    float cosI = fmaxf(0.f, wi.y), cosO = fmaxf(0.f, wo.y);
    float k = (28.f / (23.f * kPiF));
    float3 diffuse = k * b.R * (f3(1.f, 1.f, 1.f) - b.S) * (1.f - powf(1.f - 0.5f * cosO, 5.f)) * (1.f - powf(1.f - 0.5f * cosI, 5.f));
    float3 H = normalize(wo + wi);
    float cwh = dot(wi, H);
    float s = ndf_D(b, H) / (4 * cwh * fmaxf(cosI, cosO));
    float p5 = powf(1.f - cwh, 5.f);
    float3 schlick = b.S + (f3(1.f, 1.f, 1.f) - b.S) * p5;
    return diffuse + s * schlick;
}

// ---- Oren-Nayar (BSDFs/Reflections.cpp:7-66); A, B in ax, ay -----------------------------
__device__ __forceinline__ float3 on_f(const BxDF& b, float3 wo, float3 wi) {
    const float sinO = sqrtf(fmaxf(0.f, 1.f - wo.y * wo.y)), sinI = sqrtf(fmaxf(0.f, 1.f - wi.y * wi.y));
    float sinA, tanB;
    if (wo.y < wi.y) { sinA = sinI; tanB = sinO / wo.y; }
    else { sinA = sinO; tanB = sinI / wi.y; }
    float dcos = 0.f;
    if (sinI > 1e-5f && sinO > 1e-5f) {
        const float2 dI = cos_sin_phi(wi, sinI), dO = cos_sin_phi(wo, sinO);
        dcos = fmaxf(0.f, dI.x * dO.x + dI.y * dO.y);
    }
    return b.R / kPiF * (b.ax + b.ay * (dcos * sinA * tanB));
}

// ---- Blinn-Phong (BSDFs/BlinnPhongReflection.cpp:14-58); exponent K in ax -------------------
// The reference raises float to int powers with std::pow, i.e. in double: so does this.
__device__ __forceinline__ float bp_pdf(const BxDF& b, float3 wo, float3 wi) {
    const float3 wh = normalize(wo + wi);
    const float k = b.ax;
    return (float)((double)((k + 2.f) / kTwoPiF) * pow((double)fmaxf(0.f, wh.y), (double)(k + 1.f)));
}
__device__ __forceinline__ float3 bp_f(const BxDF& b, float3 wo, float3 wi) {
    const float3 wh = normalize(wo + wi);
    const float k = b.ax;
    const float s = (float)pow((double)fmaxf(0.f, wh.y), (double)k) * (k + 2.f) / kTwoPiF;
    return b.R * s / (4.f * fmaxf(0.f, wi.y) * fmaxf(0.f, wo.y));
}
// A rejected half vector is redrawn.  The reference redraws from a static std::mt19937 shared by
// all render threads (BlinnPhongReflection.cpp:33-56), which no other run can reproduce; here the
// next pair is a hash of the rejected pair and the attempt number, and the loop stops after
// kPhongAttempts draws (the sample then fails) instead of looping without bound.
constexpr int kPhongAttempts = 64;
__device__ __forceinline__ float2 phong_redraw(float2 u, int attempt) {
    const uint32_t h = hash32(__float_as_uint(u.x) ^ hash32(__float_as_uint(u.y) + 0x9E3779B9u * (uint32_t)(attempt + 1)));
    const uint32_t g = hash32(h ^ 0x85EBCA6Bu);
    return make_float2((float)(h >> 8) * 0x1p-24f, (float)(g >> 8) * 0x1p-24f);
}

// ---- per-BxDF dispatch (local frame) ------------------------------------------------------
__device__ __forceinline__ float3 bxdf_f(const BxDF& b, float3 wo, float3 wi) {
    switch (b.mtype) {
        case MAT_DIFFUSE: return b.R / kPiF;
        case MAT_MICRO_GGX:
        case MAT_MICRO_BECKMANN: return mf_refl_f(b, wo, wi);
        case MAT_GLASS_ROUGH: return (wo.y * wi.y < 0) ? mf_trans_f(b, wo, wi) : mf_refl_f(b, wo, wi);
        case MAT_PLASTIC_GGX:
        case MAT_PLASTIC_BECKMANN: return fb_f(b, wo, wi);
        case MAT_ORENNAYAR: return on_f(b, wo, wi);
        case MAT_BLINNPHONG: return bp_f(b, wo, wi);
    }
    return f3(0.f, 0.f, 0.f);  // specular BxDFs
}
__device__ __forceinline__ float bxdf_pdf(const BxDF& b, float3 wo, float3 wi) {
    switch (b.mtype) {
        case MAT_DIFFUSE: return fmaxf(0.f, wi.y) / kPiF;
        case MAT_MICRO_GGX:
        case MAT_MICRO_BECKMANN: return mf_refl_pdf(b, wo, wi);
        case MAT_GLASS_ROUGH: return (wo.y * wi.y < 0) ? mf_trans_pdf(b, wo, wi) : mf_refl_pdf(b, wo, wi);
        case MAT_PLASTIC_GGX:
        case MAT_PLASTIC_BECKMANN: return fb_pdf(b, wo, wi);
        case MAT_ORENNAYAR: return fmaxf(0.f, wi.y) / kPiF;
        case MAT_BLINNPHONG: return bp_pdf(b, wo, wi);
    }
    return 0.f;
}

// f and pdf of the BxDF at one (wo, wi) pair, sharing the half vector and D() between them.
// Same values as bxdf_f / bxdf_pdf.
__device__ __forceinline__ float3 mf_refl_f_pdf(const BxDF& b, float3 wo, float3 wi, float& pdf) {
    float3 H = normalize(wo + wi);
    float D = ndf_D(b, H);
    pdf = D * fabsf(H.y) / (4 * dot(wo, H));
    if (wo.y * wi.y < 0) return f3(0.f, 0.f, 0.f);
    float F = bxdf_fresnel(b, fmaxf(0.f, dot(wo, H)));
    float G = ndf_G(b, wo, wi);
    return b.R * D * G * F / (4 * fmaxf(0.f, wi.y) * fmaxf(0.f, wo.y));
}
__device__ __forceinline__ float3 mf_trans_f_pdf(const BxDF& b, float3 wo, float3 wi, float& pdf) {
    const float3 zero = f3(0.f, 0.f, 0.f);
    if (wo.y * wi.y > 0) { pdf = 0.f; return zero; }
    float eta = b.etaB / b.etaA;
    float3 H = normalize(wo + wi * eta);
    float D = ndf_D(b, H);  // D is even in H
    float s = dot(wo, H) + eta * dot(wi, H);
    pdf = D * fabsf(H.y) * (eta * eta * fabsf(dot(H, wi)) / sq(s));
    if (wo.y == 0.f) return zero;
    if (H.y < 0) H = -H;
    float bot = sq(dot(wo, H) + eta * dot(wi, H));
    float F = 1.f - bxdf_fresnel(b, fmaxf(0.f, dot(wo, H)));
    float G = ndf_G(b, wo, wi);
    return b.R * D * G * F * fabsf(dot(H, wo)) * fabsf(dot(H, wi)) / (bot * fmaxf(0.f, -wi.y) * fmaxf(0.f, wo.y));
}
__device__ __forceinline__ float3 fb_f_pdf(const BxDF& b, float3 wo, float3 wi, float& pdf) {
    float3 H = normalize(wo + wi);
    float D = ndf_D(b, H);
    pdf = 0.5f * (fmaxf(0.f, wi.y) / kPiF + D * fabsf(H.y) / (4 * dot(wo, H)));
    float cosI = fmaxf(0.f, wi.y), cosO = fmaxf(0.f, wo.y);
    float k = (28.f / (23.f * kPiF));
    float3 diffuse = k * b.R * (f3(1.f, 1.f, 1.f) - b.S) * (1.f - powf(1.f - 0.5f * cosO, 5.f)) * (1.f - powf(1.f - 0.5f * cosI, 5.f));
    float cwh = dot(wi, H);
    float sp = D / (4 * cwh * fmaxf(cosI, cosO));
    float3 schlick = b.S + (f3(1.f, 1.f, 1.f) - b.S) * powf(1.f - cwh, 5.f);
    return diffuse + sp * schlick;
}
__device__ __forceinline__ float3 bxdf_f_pdf(const BxDF& b, float3 wo, float3 wi, float& pdf) {
    switch (b.mtype) {
        case MAT_DIFFUSE: pdf = fmaxf(0.f, wi.y) / kPiF; return b.R / kPiF;
        case MAT_MICRO_GGX:
        case MAT_MICRO_BECKMANN: return mf_refl_f_pdf(b, wo, wi, pdf);
        case MAT_GLASS_ROUGH: return (wo.y * wi.y < 0) ? mf_trans_f_pdf(b, wo, wi, pdf) : mf_refl_f_pdf(b, wo, wi, pdf);
        case MAT_PLASTIC_GGX:
        case MAT_PLASTIC_BECKMANN: return fb_f_pdf(b, wo, wi, pdf);
        case MAT_ORENNAYAR: pdf = fmaxf(0.f, wi.y) / kPiF; return on_f(b, wo, wi);
        case MAT_BLINNPHONG: pdf = bp_pdf(b, wo, wi); return bp_f(b, wo, wi);
    }
    pdf = 0.f;
    return f3(0.f, 0.f, 0.f);
}

// NextCosineUnitHemiSphere (Utils.h:114-123)
__device__ __forceinline__ float3 cosine_hemisphere(float2 u, float& pdf) {
    float r = sqrtf(u.x);
    float phi = u.y * kTwoPiF;
    float s, c;
    sincosf(phi, &s, &c);
    float x = r * c, z = r * s;
    float y = sqrtf(1.0f - r * r);
    pdf = y / kPiF;
    return f3(x, y, z);
}

// BxDF::SampleDirection.  Returns f; writes wi (local), pdf and the sampled type.  A zero return
// leaves pdf as it was, like the reference.
__device__ __forceinline__ float3 bxdf_sample(const BxDF& b, float2 u, float3 wo, float3& wi, float& pdf, int& stype) {
    const float3 zero = f3(0.f, 0.f, 0.f);
    switch (b.mtype) {
        case MAT_DIFFUSE: {
            wi = cosine_hemisphere(u, pdf);
            return b.R / kPiF;
        }
        case MAT_MIRROR: {
            wi = f3(-wo.x, wo.y, -wo.z);
            pdf = 1.0f;
            return b.R;  // FresnelNoOp
        }
        case MAT_GLASS_SMOOTH: {  // SpecularFresnel (SpecularFresnel.cpp:28-46)
            float fr = fresnel_dielectric(b.etaA, b.etaB, wo.y);
            if (u.x < fr) {
                stype = BXDF_REFLECTION | BXDF_SPECULAR;
                wi = f3(-wo.x, wo.y, -wo.z);
                pdf = fr;
                return fr * b.R;
            }
            stype = BXDF_TRANSMISSION | BXDF_SPECULAR;
            refract(wo, f3(0.f, 1.f, 0.f), b.etaA / b.etaB, wi);
            pdf = 1.f - fr;
            return (1.f - fr) * b.R;
        }
        case MAT_MICRO_GGX:
        case MAT_MICRO_BECKMANN: {
            float3 wh = ndf_sample(b, u);
            if (dot(wo, wh) <= 0) return zero;
            wi = reflect(-wo, wh);
            pdf = mf_refl_pdf(b, wo, wi);
            wi = clamp1(wi);
            return mf_refl_f(b, wo, wi);
        }
        case MAT_GLASS_ROUGH: {  // MicrofacetBlend (Microfacet.cpp:164-199)
            float3 wh = ndf_sample(b, u);
            if (dot(wo, wh) <= 0) return zero;
            float fr = fresnel_dielectric(b.etaA, b.etaB, dot(wo, wh));
            if (u.x < fr) {
                stype = BXDF_REFLECTION | BXDF_GLOSSY;
                wi = reflect(-wo, wh);
                pdf = bxdf_pdf(b, wo, wi) * fr;
                wi = clamp1(wi);
                return mf_refl_f(b, wo, wi);
            }
            float3 t;
            if (refract(wo, wh, b.etaA / b.etaB, t)) {
                stype = BXDF_TRANSMISSION | BXDF_GLOSSY;
                wi = t;
                pdf = bxdf_pdf(b, wo, wi) * (1 - fr);
                wi = clamp1(wi);
                return mf_trans_f(b, wo, wi);
            }
            stype = BXDF_REFLECTION | BXDF_GLOSSY;
            wi = reflect(-wo, wh);
            pdf = bxdf_pdf(b, wo, wi) * (1 - fr);
            wi = clamp1(wi);
            return mf_refl_f(b, wo, wi);
        }
        case MAT_PLASTIC_GGX:
        case MAT_PLASTIC_BECKMANN: {  // FresnelBlend::SampleDirection
            float2 s = u;
            if (s.x < 0.5f) {
                s.x = s.x * 2.f;
                wi = cosine_hemisphere(s, pdf);
            } else {
                s.x = (s.x - 0.5f) * 2.f;
                float3 wh = ndf_sample(b, s);
                float3 L = reflect(-wo, wh);
                if (L.y * wo.y <= 0) return zero;
                wi = clamp1(L);
            }
            pdf = fb_pdf(b, wo, wi);
            return fb_f(b, wo, wi);
        }
        case MAT_ORENNAYAR: {
            wi = cosine_hemisphere(u, pdf);
            return on_f(b, wo, wi);
        }
        case MAT_BLINNPHONG: {
            float2 s = u;
            for (int attempt = 0; attempt < kPhongAttempts; attempt++) {
                const float cosT = (float)pow((double)s.x, 1.0 / (double)(b.ax + 2.f));
                const float phi = kTwoPiF * s.y;
                const float3 N = unit_from_cos(cosT, phi);
                if (dot(N, wo) < 0.f) { s = phong_redraw(s, attempt); continue; }
                const float3 w = reflect(-wo, N);
                if (w.y < 0.f) { s = phong_redraw(s, attempt); continue; }
                wi = w;
                pdf = bp_pdf(b, wo, wi);
                return bp_f(b, wo, wi);
            }
            return zero;
        }
    }
    return zero;
}

// ---- BSDF container (BSDF.cpp) --------------------------------------------------------------
__device__ __forceinline__ bool matches(int bxdf_flags, int flags) { return (bxdf_flags & flags) == bxdf_flags; }

__device__ __forceinline__ float3 bsdf_f(const BxDF& b, const Frame& fr, float3 wo_w, float3 wi_w) {
    float3 wo = to_local(fr, wo_w), wi = to_local(fr, wi_w);
    bool refl = wi.y * wo.y > 0;
    if ((refl && (b.flags & BXDF_REFLECTION)) || (!refl && (b.flags & BXDF_TRANSMISSION))) return bxdf_f(b, wo, wi);
    return f3(0.f, 0.f, 0.f);
}

__device__ __forceinline__ float bsdf_pdf(const BxDF& b, const Frame& fr, float3 wo_w, float3 wi_w, int flags) {
    float3 wo = to_local(fr, wo_w), wi = to_local(fr, wi_w);
    bool refl = wi.y * wo.y > 0;
    // `Matches(flags) && (reflect && R) || (!reflect && T)` parses as (A && B) || C (BSDF.cpp:39-40)
    if ((matches(b.flags, flags) && refl && (b.flags & BXDF_REFLECTION)) || (!refl && (b.flags & BXDF_TRANSMISSION)))
        return bxdf_pdf(b, wo, wi);
    return 0.f;
}

// BSDF::DistributionFunction and BSDF::Pdf(flags) of one direction pair in one pass.
__device__ __forceinline__ float3 bsdf_f_pdf(const BxDF& b, const Frame& fr, float3 wo_w, float3 wi_w, int flags, float& pdf) {
    float3 wo = to_local(fr, wo_w), wi = to_local(fr, wi_w);
    bool refl = wi.y * wo.y > 0;
    bool fcond = (refl && (b.flags & BXDF_REFLECTION)) || (!refl && (b.flags & BXDF_TRANSMISSION));
    bool pcond = (matches(b.flags, flags) && refl && (b.flags & BXDF_REFLECTION)) || (!refl && (b.flags & BXDF_TRANSMISSION));
    pdf = 0.f;
    float3 f = f3(0.f, 0.f, 0.f);
    if (fcond || pcond) {
        float p;
        float3 v = bxdf_f_pdf(b, wo, wi, p);
        if (fcond) f = v;
        if (pcond) pdf = p;
    }
    return f;
}

// Returns f; wi_w, pdf, stype written when the BxDF matches `flags`.  ok = false when the BSDF
// returned zero (no matching BxDF, or the sampled value/pdf is zero).
__device__ __forceinline__ float3 bsdf_sample(const BxDF& b, const Frame& fr, float u1, float2 u2, float3 wo_w,
                                              float3& wi_w, float& pdf, int flags, int& stype, bool& ok) {
    ok = false;
    const float3 zero = f3(0.f, 0.f, 0.f);
    if (!matches(b.flags, flags)) return zero;
    (void)u1;  // one BxDF: (int)(min(0.9999999404f, u1) * 1) == 0
    stype = b.flags;
    float3 wo = to_local(fr, wo_w);
    float3 wi = zero;
    float3 L = bxdf_sample(b, u2, wo, wi, pdf, stype);
    if (is_zero(L) || pdf == 0.f) return zero;
    wi_w = to_world(fr, wi);
    ok = true;
    return L;
}

}  // namespace c2g
