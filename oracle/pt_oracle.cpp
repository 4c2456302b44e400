// pt_oracle.cpp -- CPU restatement of the reference's path integrator.
//
// ORACLE: test infrastructure only.  Only tests/, __graft_entry__.smoke()
// and bench.py's CPU-baseline leg load this library, as the checker of the
// CUDA path; nothing in the product links it.
//
// What it restates (reference file:line at each piece):
//   * samplers: HaltonSampler None / PermuteDigits / Owen (pt_oracle_math.hpp)
//   * scene: BVHNode (bvh.hpp:27-102), MeshBVHNode (meshBVH.cpp:6-143),
//     TriangleMesh (triangleMesh.cpp:28-54), AARectangle (primitive.cpp),
//     Sphere (primitive.hpp:124-170), FlipFace (objectTransform.hpp:5-38)
//   * materials: pt_oracle_bsdf.hpp / below
//   * lights: QuadLight, SphereLight, EnvironmentLight + HDRITexture
//     (light.hpp, envLight.hpp, texture.hpp, texture.cpp:95-149),
//     discover_emissive_objects_as_lights (lightDiscovery.hpp:5-81)
//   * integrator: getRayColor of maxdepth_nee.hpp:9-256 (recursive, REF_NEE)
//     and the build's NEE+MIS / medium / roulette extensions (iterative)
//   * the pixel loop of SceneInfo::render (renderManager.hpp:97-155)
// Every draw the reference takes from gl::rand_num uses the build's
// counter-based generator with the same (path, bounce, slot) keys as the CUDA
// path, so the two can be compared path by path; Halton dimensions are the
// reference's.
//
// Parity is pinned by tests/golden/ (fixtures written by running the
// reference itself, tests/golden/make_golden.py).
#include <algorithm>
#include <array>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <numeric>
#include <thread>
#include <vector>

#include "../include/pathtracer_gb300.h"
#include "pt_oracle_bsdf.hpp"

namespace orc {

// ================================================================ materials
Material make_material(int type, int flags, const float *p) {
  Material m;
  m.type = type;
  m.flags = flags;
  std::memcpy(m.p, p, sizeof m.p);
  if (type == PT_MAT_CONDUCTOR) m.tr = TR{p[6], p[7]};
  if (type == PT_MAT_MF_DIELECTRIC) m.tr = TR{p[1], p[2]};
  if (type == PT_MAT_DISNEY) {  // disneyPrincipledBSDF.hpp:34-66
    const float st = p[3], metallic = p[4], sheen = p[10], cc = p[12];
    m.w[0] = (1 - metallic) * (1 - st);
    m.w[1] = (1 - st * (1 - metallic));
    m.w[2] = (1 - metallic) * st;
    m.w[3] = (float)(0.25 * cc);
    m.w[4] = (1 - metallic) * sheen;
    m.tr = TR::from_rough(p[7], p[9]);
    m.cc = CC{(1.f - p[13]) * 0.1f + p[13] * 0.001f};
  }
  if (type == PT_MAT_HAIR) {  // hairMarsch.hpp:9-34
    const float bm = p[5], bn = p[6], alpha = p[7];
    m.v[0] = sqr(0.726f * bm + 0.812f * sqr(bm) + 3.7f * std::pow(bm, 20.f));
    m.v[1] = (float)(.25 * m.v[0]);
    m.v[2] = 4 * m.v[0];
    m.v[3] = m.v[2];
    m.s = 0.626657069f * (0.265f * bn + 1.194f * sqr(bn) + 5.372f * std::pow(bn, 22.f));
    m.s2k[0] = std::sin(alpha);
    m.c2k[0] = safe_sqrt(1 - sqr(m.s2k[0]));
    for (int i = 1; i < 3; ++i) {
      m.s2k[i] = 2 * m.c2k[i - 1] * m.s2k[i - 1];
      m.c2k[i] = sqr(m.c2k[i - 1]) - sqr(m.s2k[i - 1]);
    }
    if (flags & PT_MAT_FLAG_MELANIN)  // pbrt-v3 SigmaAFromConcentration (extension)
      m.sigma_a = V(0.419f, 0.697f, 1.37f) * p[8] + V(0.187f, 0.4f, 1.05f) * p[9];
    else
      m.sigma_a = V(p[0], p[1], p[2]);
  }
  return m;
}

static V base_color(const Material &m) { return V(m.p[0], m.p[1], m.p[2]); }

// ---- Disney lobes (disneyDiffuse/Metal/Glass/Sheen/Clearcoat.hpp)
static V dis_diffuse_f(const Material &m, V wow, V wiw, V n) {
  Onb b(n);
  V wo = b.local(wow), wi = b.local(wiw);
  float ci = std::fabs(wi.z), co = std::fabs(wo.z);
  const float rough = m.p[7], ss = m.p[5];
  V wh = (wo + wi).normalize();
  float whwi = dot(wh, wi);
  float fd90 = 0.5f + 2.f * rough * std::pow(std::fabs(whwi), 2.f);
  V base = base_color(m);
  V bd = base * (float)(1.f / PI);
  bd = bd * (hacked_schlick(ci, fd90) * hacked_schlick(co, fd90));
  float fss90 = rough * std::pow(std::fabs(whwi), 2.f);
  V bs = (1.25f * base) * (float)(1.f / PI);
  bs = bs * (hacked_schlick(ci, fss90) * hacked_schlick(co, fss90) * (1.f / (ci + co) - 0.5f) + 0.5f);
  return (1.f - ss) * bd + bs * ss;
}
static V dis_metal_f(const Material &m, V wow, V wiw, V n, bool variant) {
  Onb b(n);
  V wo = b.local(wow), wi = b.local(wiw);
  V wh = (wo + wi).normalize();
  if (wi.z <= 0 || wo.z <= 0 || m.tr.smooth()) return V(0.f);
  float dhi = std::fabs(dot(wh, wi));
  V base = base_color(m);
  V F0 = base;
  if (variant) {  // f_variant with its default arguments (disneyMetal.hpp:98-124)
    const float st = 0.5f, eta = 1.0f, specular = 0.5f, metallic = 0.5f;
    V Ks = V(1 - st) + st * base;
    float R0 = sqr((eta - 1) / (eta + 1));
    F0 = specular * R0 * (1 - metallic) * Ks + metallic * base;
  }
  V F = fresnel_schlick(dhi, F0);
  float D = m.tr.D(wh), G = m.tr.G(wo, wi);
  return F * D * G / std::fabs(4.f * wi.z * wo.z);
}
static V dis_sheen_f(const Material &m, V wow, V wiw, V n) {
  Onb b(n);
  V wo = b.local(wow), wi = b.local(wiw);
  V wh = (wo + wi).normalize();
  float a = std::fabs(dot(wh, wi));
  V base = base_color(m);
  float lum = dot(base, V(0.2126f, 0.7152f, 0.0722f));
  V tint = lum > 0.0f ? base / lum : V(1.0f);
  const float st = m.p[11];
  V cs = V(1.f + st * (tint.x - 1.f), 1.f + st * (tint.y - 1.f), 1.f + st * (tint.z - 1.f));
  return cs * std::pow((1 - a), 5.f);
}
static V dis_clearcoat_f(const Material &m, V wow, V wiw, V n) {
  Onb b(n);
  V wo = b.local(wow), wi = b.local(wiw);
  V wh = (wo + wi).normalize();
  if (wi.z <= 0 || wo.z <= 0) return V(0.f);
  float a = std::fabs(dot(wh, wi));
  V F = fresnel_schlick(a, V(sqr((1.5f - 1) / (1.5f + 1))));
  return F * m.cc.D(wh) * m.cc.G(wo, wi) / std::fabs(4.f * wi.z * wo.z);
}
static float eta_of(const Material &m) { return m.type == PT_MAT_DISNEY ? m.p[14] : m.p[0]; }
static V glass_f(const Material &m, V wo, V wi, V n, bool tinted) {
  Onb b(n);
  return mfd_f(m.tr, eta_of(m), b.local(wo.normalize()), b.local(wi.normalize()), base_color(m), tinted);
}
static float glass_pdf(const Material &m, V wo, V wi, V n) {
  if (eta_of(m) == 1 || m.tr.smooth()) return 0.f;
  Onb b(n);
  return mfd_at(m.tr, eta_of(m), b.local(wo.normalize()), b.local(wi.normalize()));
}
// MFDielectric::scatter / DisneyGlass::scatter (dielectric.hpp:19-98)
static bool glass_scatter(const Material &m, V wo, V n, Scatter &s, float uc, float u0, float u1, bool tinted) {
  const float eta = eta_of(m);
  if (eta == 1 || m.tr.smooth()) {
    float R = fresnel_dielectric(dot(n, wo), eta), T = 1 - R;
    if (R == 0 && T == 0) return false;
    if (uc < R / (R + T)) {
      s.dir = reflect_p(wo, n).normalize();
      s.type = SPEC | REFL;
      s.att = V(1.0f);
      s.pdf_val = R;
      return true;
    }
    V wt;
    float etap;
    if (!refract_p(wo, n, eta, etap, wt)) return false;
    s.dir = wt;
    s.type = SPEC | TRANS;
    s.pdf_val = T;
    s.att = V(1.0f);  // TransportMode::Importance (config.hpp:23)
    return true;
  }
  Onb b(n);
  V wol = b.local(wo);
  V wi = mfd_get(m.tr, eta, b, wol, uc, u0, u1);
  if (wi.near_zero()) return false;
  s.dir = wi;
  bool is_refl = dot(b.local(wi), b.local(wo)) > 0;
  s.type = is_refl ? (GLOSSY | REFL) : (GLOSSY | TRANS);
  s.att = glass_f(m, wo, wi, n, tinted);
  s.pdf_val = mfd_at(m.tr, eta, wol, b.local(wi.normalize()));
  return true;
}

// ---- hair (hairMarsch.hpp, hairMarsch.cpp, hairPDF.cpp)
static float hair_Mp(float ci, float co, float si, float so, float v) {
  float a = ci * co / v, b = si * so / v;
  return (v <= .1) ? (fast_exp(log_i0f(a) - b - 1 / v + 0.6931f + std::log(1 / (2 * v))))
                   : (fast_exp(-b) * i0f(a)) / (std::sinh(1 / v) * 2 * v);
}
static float hair_Phi(int p, float go, float gt) { return (float)(2 * p * gt - 2 * go + p * PI); }
static float logistic(float x, float s) {
  x = std::abs(x);
  return std::exp(-x / s) / (s * sqr(1 + std::exp(-x / s)));
}
static float logistic_cdf(float x, float s) { return 1 / (1 + std::exp(-x / s)); }
static float hair_Np(float phi, int p, float s, float go, float gt) {
  float dphi = phi - hair_Phi(p, go, gt);
  while (dphi > PI) dphi -= (float)(2 * PI);
  while (dphi < -PI) dphi += (float)(2 * PI);
  return logistic(dphi, s) / (logistic_cdf((float)PI, s) - logistic_cdf((float)-PI, s));
}
static void hair_Ap(float co, float eta, float h, V T, V ap[4]) {
  float cgo = safe_sqrt(1 - sqr(h));
  float f = fresnel_dielectric(co * cgo, eta);
  ap[0] = V(f);
  ap[1] = sqr(1 - f) * T;
  ap[2] = ap[1] * T * f;
  V d = V(1.f) - T * f;
  ap[3] = d.near_zero() ? V(0.f) : ap[2] * f * T / d;
}
static void hair_ApPDF(const Material &m, float co, float out[4]) {
  const float eta = m.p[4], h = m.p[3];
  float so = safe_sqrt(1 - sqr(co));
  float ct = safe_sqrt(1 - sqr(so / eta));
  float etap = safe_sqrt(sqr(eta) - sqr(so)) / co;
  float cgt = safe_sqrt(1 - sqr(h / etap));
  float k = 2 * cgt / ct;
  V T(std::exp(-m.sigma_a.x * k), std::exp(-m.sigma_a.y * k), std::exp(-m.sigma_a.z * k));
  V ap[4];
  hair_Ap(co, eta, h, T, ap);
  float sumY = 0.f;
  for (auto &a : ap) sumY += (a.x + a.y + a.z) / 3.f;
  for (int i = 0; i < 4; ++i) out[i] = ((ap[i].x + ap[i].y + ap[i].z) / 3.f) / sumY;
}
static void hair_rot(const Material &m, int p, float so, float co, float &sp, float &cp) {
  if (p == 0) {
    sp = so * m.c2k[1] - co * m.s2k[1];
    cp = co * m.c2k[1] + so * m.s2k[1];
  } else if (p == 1) {
    sp = so * m.c2k[0] + co * m.s2k[0];
    cp = co * m.c2k[0] - so * m.s2k[0];
  } else if (p == 2) {
    sp = so * m.c2k[2] + co * m.s2k[2];
    cp = co * m.c2k[2] - so * m.s2k[2];
  } else {
    sp = so;
    cp = co;
  }
  cp = std::abs(cp);
}
static V hair_eval(const Material &m, V wi, V wo) {  // hairMarsch.cpp:28-97
  const float eta = m.p[4], h = m.p[3];
  float so = wo.x, co = safe_sqrt(1 - so * so), phio = std::atan2(wo.z, wo.y);
  float go = std::asin(std::clamp(so, -1.f, 1.f));
  float si = wi.x, ci = safe_sqrt(1 - si * si), phii = std::atan2(wi.z, wi.y);
  float ct = safe_sqrt(1 - sqr(so / eta));
  float etap = safe_sqrt(sqr(eta) - sqr(so));
  float sgt = h / etap, cgt = safe_sqrt(1 - sgt * sgt);
  float gt = std::asin(std::clamp(sgt, -1.f, 1.f));
  float k = 2 * cgt / ct;
  V T(fast_exp(-m.sigma_a.x * k), fast_exp(-m.sigma_a.y * k), fast_exp(-m.sigma_a.z * k));
  float phi = phii - phio;
  V ap[4];
  hair_Ap(co, eta, h, T, ap);
  V bsdf(0.f);
  for (int p = 0; p < 3; ++p) bsdf += ap[p] * (hair_Mp(ci, co, si, so, m.v[p]) * hair_Np(phi, p, m.s, go, gt));
  bsdf += hair_Mp(ci, co, si, so, m.v[3]) * ap[3] / (float)(2 * PI);
  if (std::abs(wi.z) > 0.f) bsdf = bsdf / std::abs(wi.z);
  return bsdf;
}
static float hair_at(const Material &m, V wol, V wil) {  // hairPDF.cpp:101-152
  const float eta = m.p[4], h = m.p[3];
  float si = wil.x, ci = safe_sqrt(1 - si * si), phii = std::atan2(wil.z, wil.y);
  float so = wol.x, co = safe_sqrt(1 - so * so), phio = std::atan2(wol.z, wol.y);
  float go = std::asin(std::clamp(so, -1.f, 1.f));
  float etap = safe_sqrt(sqr(eta) - sqr(so)) / co;
  float gt = std::asin(std::clamp(h / etap, -1.f, 1.f));
  float dphi = phii - phio;
  if (dphi < -PI)
    dphi += (float)(2 * PI);
  else if (dphi > PI)
    dphi -= (float)(2 * PI);
  float ap[4];
  hair_ApPDF(m, co, ap);
  float pdf = 0.f;
  for (int p = 0; p < 3; ++p) {
    float sp, cp;
    hair_rot(m, p, so, co, sp, cp);
    pdf += ap[p] * hair_Mp(ci, cp, si, sp, m.v[p]) * hair_Np(dphi, p, m.s, go, gt);
  }
  return pdf;
}

bool mat_scatter(const Material &m, V ray_dir, const Hit &rec, Scatter &s, float uc, float u0, float u1) {
  // HairMarschner::scatter samples in the hair tangent's frame when set
  // (hairMarsch.cpp:12-24); its attenuation is mat_f, framed by the normal
  const V n = (m.type == PT_MAT_HAIR && rec.has_tangent) ? rec.tangent : rec.normal;
  const V wo = -ray_dir.normalize();
  switch (m.type) {
  case PT_MAT_LAMBERTIAN: {  // material.hpp:88-105
    s.type = DIFF | REFL;
    s.att = base_color(m) * (float)(1.0f / PI);
    Onb b(n);
    s.dir = b.at(cosine_sample(u0, u1)).normalize();
    s.pdf_val = cosine_pdf_at(n, s.dir);
    return true;
  }
  case PT_MAT_CONDUCTOR: {  // conductor.hpp:11-63, mfPDF.hpp:19-45 (BIASED_SAMPLING)
    if (m.tr.smooth()) {
      V wi = reflect_p(wo, n).normalize();
      if (dot(n, wi) <= 0) return false;
      s.dir = wi;
      s.att = fresnel_complex(std::fabs(dot(n, wi)), V(m.p[0], m.p[1], m.p[2]), V(m.p[3], m.p[4], m.p[5]));
      s.type = SPEC | REFL;
      s.pdf_val = 0.f;
      return true;
    }
    Onb b(n);
    V wol = b.local(wo.normalize());
    V mm = m.tr.sample_wm(wol, u0, u1);
    V wil = reflect_p(wol, mm);
    if (!same_hemi(wol, wil)) wil.z = -wol.z;
    V wi = b.at(wil).normalize();
    if (wi.near_zero()) return false;
    if (dot(n, wi) <= 0) return false;
    s.dir = wi;
    s.type = GLOSSY | REFL;
    s.att = mat_f(m, wo, wi, rec);
    s.pdf_val = mf_at(m.tr, b, wol, wi);
    return true;
  }
  case PT_MAT_MF_DIELECTRIC:
    return glass_scatter(m, wo, n, s, uc, u0, u1, false);
  case PT_MAT_THIN_DIELECTRIC: {  // thinDielectric.hpp:14-68
    float R = fresnel_dielectric(std::fabs(dot(n, wo)), m.p[0]), T = 1 - R;
    if (R < 1) {
      R += sqr(T) * R / (1 - sqr(R));
      T = 1 - R;
    }
    if (R == 0 && T == 0) return false;
    if (m.flags & PT_MAT_FLAG_SPLIT_RAY) {
      s.type = (SPEC | REFL) | (SPEC | TRANS);
      s.pdf_val = R;
      return true;
    }
    if (uc < R / (R + T)) {
      s.dir = reflect_p(wo, n).normalize();
      s.type = SPEC | REFL;
      s.pdf_val = R;
    } else {
      s.dir = -wo.normalize();
      s.type = SPEC | TRANS;
      s.pdf_val = T;
    }
    s.att = V(1.0f);
    return true;
  }
  case PT_MAT_PHONG: {
    // The build's consistent form of Phong::scatter (material.hpp:320-366):
    // lobe picked with uc, attenuation = f, pdf_val = scatter_pdf.
    float si = (m.p[3] + m.p[4] + m.p[5]) / 3.0f, di = (m.p[0] + m.p[1] + m.p[2]) / 3.0f;
    float sp = si / (si + di);
    if (uc < sp) {
      V R = reflect_gl(-wo, n);
      Onb b(R);
      float theta = std::acos(std::pow(u0, 1.0f / (m.p[9] + 1.0f)));
      float phi = (float)(2.0f * PI * u1);
      float st = std::sin(theta);
      s.dir = b.at(V(st * std::cos(phi), st * std::sin(phi), std::cos(theta))).normalize();
      s.type = GLOSSY | REFL;
    } else {
      Onb b(n);
      s.dir = b.at(cosine_sample(u0, u1));
      s.type = DIFF | REFL;
    }
    s.att = mat_f(m, wo, s.dir, rec);
    s.pdf_val = mat_pdf(m, wo, s.dir, rec);
    return s.pdf_val > 0.f;
  }
  case PT_MAT_DISNEY: {  // disneyPrincipledBSDF.cpp:3-80
    if (rec.is_inside) return glass_scatter(m, wo, n, s, uc, u0, u1, true);
    float pmf, ur;
    int lobe = sample_discrete(m.w, 4, uc, &pmf, &ur);
    if (lobe == -1 || pmf <= 1e-6f) return false;
    const float v0 = ur, v1 = u1;
    if (lobe == 0) {
      Onb b(n);
      V wi = b.at(cosine_sample(v0, v1));
      s.dir = wi.normalize();
      s.pdf_val = cosine_pdf_at(n, wi);
      s.type = DIFF | REFL;
    } else if (lobe == 1) {
      if (m.tr.smooth()) {
        V wi = reflect_p(wo, n).normalize();
        if (dot(n, wi) <= 0) return false;
        s.dir = wi;
        s.att = fresnel_schlick(std::fabs(dot(n, wi)), base_color(m));
        s.type = SPEC | REFL;
        s.pdf_val = 0.f;
        return true;
      }
      Onb b(n);
      V wol = b.local(wo.normalize());
      V mm = m.tr.sample_wm(wol, v0, v1);
      V wil = reflect_p(wol, mm);
      if (!same_hemi(wol, wil)) wil.z = -wol.z;
      V wi = b.at(wil).normalize();
      if (wi.near_zero() || dot(n, wi) <= 0) return false;
      s.dir = wi;
      s.pdf_val = mf_at(m.tr, b, wol, wi);
      s.type = GLOSSY | REFL;
    } else if (lobe == 2) {
      if (!glass_scatter(m, wo, n, s, ur, v0, v1, true)) return false;
      if (s.type & SPEC) return true;
    } else {
      Onb b(n);
      V wol = b.local(wo.normalize());
      V h = m.cc.sample_h(v0, v1);
      V wil = reflect_p(wol, h);
      if (!same_hemi(wol, wil)) wil.z = -wol.z;
      V wi = b.at(wil).normalize();
      if (dot(n, wi) <= 0) return false;
      s.dir = wi;
      s.pdf_val = m.cc.at(b, wol, wi);
      s.type = GLOSSY | REFL;
    }
    if (s.pdf_val <= 1e-6f) return false;
    V wi = s.dir.normalize();
    Hit r2 = rec;
    r2.is_inside = false;
    s.att = mat_f(m, wo, wi, r2);
    s.pdf_val = mat_pdf(m, wo, wi, r2);
    if (s.pdf_val <= 1e-7f) return false;
    return true;
  }
  case PT_MAT_HAIR: {  // hairMarsch.cpp:4-26 + hairPDF.cpp:14-99
    const float eta = m.p[4], h = m.p[3];
    Onb b(n);
    V wol = b.local(wo);
    float so = wol.x, co = safe_sqrt(1 - so * so), phio = std::atan2(wol.z, wol.y);
    float go = std::asin(std::clamp(so, -1.f, 1.f));
    float apd[4];
    hair_ApPDF(m, co, apd);
    int p = sample_discrete(apd, 4, uc, nullptr, nullptr);
    float sp, cp;
    hair_rot(m, p, so, co, sp, cp);
    float ct = 1 + m.v[p] * std::log(std::max(u0, (float)1e-5) + (1.f - u0) * fast_exp(-2.f / m.v[p]));
    float st = safe_sqrt(1 - sqr(ct));
    float cphi_ = (float)std::cos(2 * PI * u1);
    float si = -ct * sp + st * cphi_ * cp;
    float ci = safe_sqrt(1 - sqr(si));
    float etap = safe_sqrt(sqr(eta) - sqr(so)) / co;
    float gt = std::asin(std::clamp(h / etap, -1.f, 1.f));
    float dphi;
    if (p < 3) {
      float lo = logistic_cdf((float)-PI, m.s), hi = logistic_cdf((float)PI, m.s);
      float uu = lo + uc * (hi - lo);
      float x = -m.s * std::log(1 / uu - 1);
      dphi = hair_Phi(p, go, gt) + std::clamp(x, (float)-PI, (float)PI);
    } else {
      dphi = (float)(2 * PI * uc);
    }
    float phii = dphi + phio;
    V wil(si, ci * std::cos(phii), ci * std::sin(phii));
    V wi = b.at(wil).normalize();
    s.att = mat_f(m, wo, wi, rec);
    s.pdf_val = hair_at(m, wol, b.local(wi));
    s.dir = wi;
    s.type = GLOSSY | REFL;
    return true;
  }
  default:
    return false;  // DiffuseEmitter::scatter (material.hpp:475-481)
  }
}

V mat_f(const Material &m, V wo, V wi, const Hit &rec) {
  // every BSDF in the normal's frame: HairMarschner::f and scatter_pdf too,
  // on a curve as well (hairMarsch.hpp:49, hairMarsch.cpp:115)
  const V n = rec.normal;
  switch (m.type) {
  case PT_MAT_LAMBERTIAN:
    return base_color(m) * (float)(1.0f / PI);
  case PT_MAT_CONDUCTOR: {  // conductor.hpp:109-139
    Onb b(n);
    V wol = b.local(wo.normalize()), wil = b.local(wi.normalize());
    if (wil.z <= 0 || wol.z <= 0) return V(0.f);
    if (m.tr.smooth()) return V(0.f);
    V ml = (wol + wil).normalize();
    float D = m.tr.D(ml), G = m.tr.G(wol, wil);
    V F = fresnel_complex(std::fabs(dot(wol, ml)), V(m.p[0], m.p[1], m.p[2]), V(m.p[3], m.p[4], m.p[5]));
    return D * F * G / (4.f * std::abs(wol.z) * std::abs(wil.z));
  }
  case PT_MAT_MF_DIELECTRIC:
    return glass_f(m, wo, wi, n, false);
  case PT_MAT_PHONG: {  // material.hpp:369-411
    V o = wo.normalize(), i = wi.normalize();
    float ci = dot(n, i);
    if (ci <= 0) return V(0.f);
    float si = (m.p[3] + m.p[4] + m.p[5]) / 3.0f, di = (m.p[0] + m.p[1] + m.p[2]) / 3.0f;
    float sp = si / (si + di);
    V diff = base_color(m) * (float)(1.0f / PI);
    V R = reflect_p(o, n);
    float ca = std::max(dot(i, R), 0.0f);
    float pt = std::pow(ca, m.p[9]);
    float norm = (float)((m.p[9] + 2.0f) / (2.0f * PI));
    V spec = V(m.p[3], m.p[4], m.p[5]) * (norm * pt);
    return sp * spec + (1.0f - sp) * diff;
  }
  case PT_MAT_DISNEY: {  // disneyPrincipledBSDF.hpp:72-91
    if (rec.is_inside) return glass_f(m, wo, wi, n, true);
    V r(0.f);
    r += dis_diffuse_f(m, wo, wi, n) * m.w[0];
    r += dis_metal_f(m, wo, wi, n, true) * m.w[1];
    r += glass_f(m, wo, wi, n, true) * m.w[2];
    r += dis_clearcoat_f(m, wo, wi, n) * m.w[3];
    r += dis_sheen_f(m, wo, wi, n) * m.w[4];
    return r;
  }
  case PT_MAT_HAIR: {
    Onb b(n);
    return hair_eval(m, b.local(wi.normalize()), b.local(wo.normalize()));
  }
  default:
    return V(0.f);
  }
}

float mat_pdf(const Material &m, V wo, V wi, const Hit &rec) {
  // every BSDF in the normal's frame: HairMarschner::f and scatter_pdf too,
  // on a curve as well (hairMarsch.hpp:49, hairMarsch.cpp:115)
  const V n = rec.normal;
  switch (m.type) {
  case PT_MAT_LAMBERTIAN:
    return cosine_pdf_at(n, wi);
  case PT_MAT_CONDUCTOR: {  // conductor.hpp:81-99
    if (m.tr.smooth()) return 0.f;
    Onb b(n);
    if (dot(n, wi) <= 0) return 0.0f;
    return mf_at(m.tr, b, b.local(wo.normalize()), wi);
  }
  case PT_MAT_MF_DIELECTRIC:
    return glass_pdf(m, wo, wi, n);
  case PT_MAT_PHONG: {  // material.hpp:414-463
    V o = wo.normalize(), i = wi.normalize();
    float si = (m.p[3] + m.p[4] + m.p[5]) / 3.0f, di = (m.p[0] + m.p[1] + m.p[2]) / 3.0f;
    float tot = si + di;
    if (tot == 0.f) return 0.f;
    float ps = si / tot, pd = di / tot;
    float pls = 0.f, pld = 0.f;
    if (ps > 0) {
      V R = reflect_gl(-o, n.normalize()).normalize();
      float c = std::max(dot(i.normalize(), R), 0.0f);
      pls = (float)((m.p[9] + 1.0f) / (2.0f * PI) * std::pow(c, m.p[9]));
    }
    if (pd > 0) {
      float c = dot(i, n.normalize());
      if (c > 0) pld = (float)(c / PI);
    }
    return ps * pls + pd * pld;
  }
  case PT_MAT_DISNEY: {  // disneyPrincipledBSDF.cpp:82-113
    if (rec.is_inside) return glass_pdf(m, wo, wi, n);
    float sw = m.w[0] + m.w[1] + m.w[2] + m.w[3];
    float p = 0.f;
    p += (m.w[0] / sw) * cosine_pdf_at(n, wi);
    float pm = 0.f;
    if (!m.tr.smooth()) {
      Onb b(n);
      pm = mf_at(m.tr, b, b.local(wo.normalize()), wi);
    }
    p += (m.w[1] / sw) * pm;
    p += (m.w[2] / sw) * glass_pdf(m, wo, wi, n);
    Onb b(n);
    p += (m.w[3] / sw) * m.cc.at(b, b.local(wo.normalize()), wi);
    return p;
  }
  case PT_MAT_HAIR: {
    Onb b(n);
    return hair_at(m, b.local(wo), b.local(wi.normalize()));
  }
  default:
    return 0.f;
  }
}

V mat_emit(const Material &m, V ray_dir, const Hit &rec) {  // material.hpp:483-488
  if (m.type != PT_MAT_DIFFUSE_EMITTER) return V(0.f);
  if (dot(rec.normal, -ray_dir) > 0) return V(m.p[0], m.p[1], m.p[2]) * m.p[3];
  return V(0.0f);
}

// ==================================================================== scene
struct Box {
  V lo, hi;
  // AABB::intersect (aabb.hpp:21-42)
  bool hit(V o, V d, float tmin, float tmax) const {
    for (int i = 0; i < 3; i++) {
      float inv = 1.0f / d[i];
      float t0 = (lo[i] - o[i]) * inv;
      float t1 = (hi[i] - o[i]) * inv;
      if (inv < 0.0f) std::swap(t0, t1);
      tmin = t0 > tmin ? t0 : tmin;
      tmax = t1 < tmax ? t1 : tmax;
      if (tmax <= tmin) return false;
    }
    return true;
  }
};
static Box merge(const Box &a, const Box &b) {
  return Box{V(std::min(a.lo.x, b.lo.x), std::min(a.lo.y, b.lo.y), std::min(a.lo.z, b.lo.z)),
             V(std::max(a.hi.x, b.hi.x), std::max(a.hi.y, b.hi.y), std::max(a.hi.z, b.hi.z))};
}

struct MeshO {
  std::vector<V> pos, nrm;
  std::vector<std::array<int, 3>> tri, ntri, uvtri;
  std::vector<std::array<float, 2>> uv;
  int mat = 0, prim_base = 0;
  Box aabb;
  struct Node {
    Box box;
    int left = -1, right = -1;
    std::vector<int> ids;
  };
  std::vector<Node> nodes;
  int build(std::vector<int> ids) {  // MeshBVHNode ctor (meshBVH.cpp:6-55)
    V mn(INFINITY), mx(-INFINITY);
    for (int id : ids)
      for (int k : tri[id]) {
        mn = V(std::min(mn.x, pos[k].x), std::min(mn.y, pos[k].y), std::min(mn.z, pos[k].z));
        mx = V(std::max(mx.x, pos[k].x), std::max(mx.y, pos[k].y), std::max(mx.z, pos[k].z));
      }
    int me = (int)nodes.size();
    nodes.emplace_back();
    nodes[me].box = Box{mn - V(1e-3f), mx + V(1e-3f)};
    int count = (int)ids.size();
    if (count <= 4) {
      nodes[me].ids = ids;
      return me;
    }
    V ext = mx - mn;
    int axis = ext.x > ext.y && ext.x > ext.z ? 0 : ext.y > ext.z ? 1 : 2;
    std::sort(ids.begin(), ids.end(), [&](int a, int b) {
      V ca = (pos[tri[a][0]] + pos[tri[a][1]] + pos[tri[a][2]]) / 3.0f;
      V cb = (pos[tri[b][0]] + pos[tri[b][1]] + pos[tri[b][2]]) / 3.0f;
      return ca[axis] < cb[axis];
    });
    int mid = count / 2;
    int l = build(std::vector<int>(ids.begin(), ids.begin() + mid));
    int r = build(std::vector<int>(ids.begin() + mid, ids.end()));
    nodes[me].left = l;
    nodes[me].right = r;
    return me;
  }
  // hitTriangle (meshBVH.cpp:85-143)
  bool hit_tri(int id, V o, V d, float tmin, float tmax, Hit &rec) const {
    const V &p0 = pos[tri[id][0]], &p1 = pos[tri[id][1]], &p2 = pos[tri[id][2]];
    V e1 = p1 - p0, e2 = p2 - p0;
    V P = cross(d, e2);
    float det = dot(e1, P);
    if (std::fabs(det) < 1e-8f) return false;
    float inv = 1.0f / det;
    V T = o - p0;
    float u = dot(T, P) * inv;
    if (u < 0 || u > 1) return false;
    V Q = cross(T, e1);
    float v = dot(d, Q) * inv;
    if (v < 0 || u + v > 1) return false;
    float t = dot(e2, Q) * inv;
    if (t < tmin || t > tmax) return false;
    V n;
    if (!nrm.empty()) {
      const auto &ni = ntri[id];
      n = normalize((1 - u - v) * nrm[ni[0]] + u * nrm[ni[1]] + v * nrm[ni[2]]);
    } else {
      n = normalize(cross(e1, e2));
    }
    V Ng = normalize(cross(e1, e2));
    if (dot(n, Ng) < 0.f) n = -n;
    rec.normal = n;
    rec.t = t;
    rec.position = o + t * d;
    rec.prim = prim_base + id;
    rec.bu = u;
    rec.bv = v;
    return true;
  }
  bool hit_node(int ni, V o, V d, float tmin, float tmax, Hit &rec) const {  // meshBVH.cpp:57-83
    const Node &N = nodes[ni];
    if (!N.box.hit(o, d, tmin, tmax)) return false;
    bool hit = false;
    float closest = tmax;
    if (N.left < 0) {
      for (int id : N.ids)
        if (hit_tri(id, o, d, tmin, closest, rec)) {
          hit = true;
          closest = rec.t;
        }
    } else {
      if (hit_node(N.left, o, d, tmin, closest, rec)) {
        hit = true;
        closest = rec.t;
      }
      if (hit_node(N.right, o, d, tmin, closest, rec)) hit = true;
    }
    return hit;
  }
};

struct Obj {
  int kind, index;
  V cps[4];            // curve control points
  float w0 = 0, w1 = 0;  // curve widths
  V vel;               // motion blur (extension): position + vel * time
  bool moving = false;
  Box box;
  int mat, flip, prim;
  int face = 0;  // pt_object_desc.face: 0 as hit, 1 is_inside always true, 2 always false
  int light = -1;
  // quad
  int axis;
  float k, d0min, d0max, d1min, d1max;
  // sphere
  V c;
  float r;
};

struct Light {
  int type;  // 0 quad, 1 sphere, 2 env
  V v0, e1, e2, normal, c, color;
  V v2;  // quad: vertices[2]
  V vel;
  bool moving = false;
  int texture = 0;  // texture index + 1 of the colour (0: color)
  float radius = 0, area = 0, intensity = 0;
};

// Surface textures (texture.hpp:20-95, texture.cpp:95-193, pattern.hpp:8-114).
struct Tex {
  int kind = 0, fractal = 1, w = 0, h = 0;
  V c1, c2;
  float scale = 10.f;
  std::vector<V> texels;  // [y][x]
};

static const unsigned char kPerlin[256] = {  // Ken Perlin, "Improving Noise" (2002)
    151, 160, 137, 91,  90,  15,  131, 13,  201, 95,  96,  53,  194, 233, 7,   225, 140, 36,  103, 30,  69,  142,
    8,   99,  37,  240, 21,  10,  23,  190, 6,   148, 247, 120, 234, 75,  0,   26,  197, 62,  94,  252, 219, 203,
    117, 35,  11,  32,  57,  177, 33,  88,  237, 149, 56,  87,  174, 20,  125, 136, 171, 168, 68,  175, 74,  165,
    71,  134, 139, 48,  27,  166, 77,  146, 158, 231, 83,  111, 229, 122, 60,  211, 133, 230, 220, 105, 92,  41,
    55,  46,  245, 40,  244, 102, 143, 54,  65,  25,  63,  161, 1,   216, 80,  73,  209, 76,  132, 187, 208, 89,
    18,  169, 200, 196, 135, 130, 116, 188, 159, 86,  164, 100, 109, 198, 173, 186, 3,   64,  52,  217, 226, 250,
    124, 123, 5,   202, 38,  147, 118, 126, 255, 82,  85,  212, 207, 206, 59,  227, 47,  16,  58,  17,  182, 189,
    28,  42,  223, 183, 170, 213, 119, 248, 152, 2,   44,  154, 163, 70,  221, 153, 101, 155, 167, 43,  172, 9,
    129, 22,  39,  253, 19,  98,  108, 110, 79,  113, 224, 232, 178, 185, 112, 104, 218, 246, 97,  228, 251, 34,
    242, 193, 238, 210, 144, 12,  191, 179, 162, 241, 81,  51,  145, 235, 249, 14,  239, 107, 49,  192, 214, 31,
    181, 199, 106, 157, 184, 84,  204, 176, 115, 121, 50,  45,  127, 4,   150, 254, 138, 236, 205, 93,  222, 114,
    67,  29,  24,  72,  243, 141, 128, 195, 78,  66,  215, 61,  156, 180};

static float perlin_grad(int hash, float x, float y) {  // pattern.hpp:43-66
  switch (hash & 7) {
  case 0: return x + y;
  case 1: return -x + y;
  case 2: return x - y;
  case 3: return -x - y;
  case 4: return x;
  case 5: return -x;
  case 6: return y;
  default: return -y;
  }
}
static float perlin_2d(float ux, float uy) {  // perlin_noise_2D, pattern.hpp:72-98
  float x = std::fmod(ux, 256.f), y = std::fmod(uy, 256.f);
  const int X = (int)std::floor(x) & 255, Y = (int)std::floor(y) & 255;
  x = x - std::floor(x);
  y = y - std::floor(y);
  auto smooth = [](float t) {
    t = std::clamp(t, 0.f, 1.f);
    return t * t * t * (t * (t * 6.f - 15.f) + 10.f);
  };
  const float u = smooth(x), v = smooth(y);
  auto P = [](int i) { return (int)kPerlin[i & 255]; };
  const int X1 = (X + 1) % 256, Y1 = (Y + 1) % 256;
  const int aa = P(P(X) + Y), ab = P(P(X) + Y1), ba = P(P(X1) + Y), bb = P(P(X1) + Y1);
  auto lerp = [](float a, float b, float t) { return a + t * (b - a); };
  const float x1 = lerp(perlin_grad(aa, x, y), perlin_grad(ba, x - 1.f, y), u);
  const float x2 = lerp(perlin_grad(ab, x, y - 1.f), perlin_grad(bb, x - 1.f, y - 1.f), u);
  return (lerp(x1, x2, v) + 1.f) * 0.5f;
}
static V tex_eval(const Tex &T, float u, float v) {
  switch (T.kind) {
  case PT_TEX_CHECKER: {  // texture.cpp:164-181
    const float s = std::sin(u * T.scale) * std::sin(v * T.scale);
    return s < 0.f ? T.c1 : T.c2;
  }
  case PT_TEX_NOISE: {  // fractal_perlin_2D, pattern.hpp:100-114
    float total = 0.f, amp = 1.f, freq = 1.f;
    for (int i = 0; i < T.fractal && i < 32; ++i) {
      total += amp * perlin_2d(u * T.scale * freq, v * T.scale * freq);
      amp *= 0.5f;
      freq *= 2.f;
    }
    return V(std::clamp(std::fabs(total), 0.f, 1.f));
  }
  case PT_TEX_IMAGE: {  // ImageTexture::getTexelColor, bilinear (texture.cpp:112-143)
    unsigned x = (unsigned)(u * T.w), y = (unsigned)(v * T.h);
    float x1 = (u * T.w) - x, y1 = (v * T.h) - y;
    x = std::min(x, (unsigned)T.w - 2);
    y = std::min(y, (unsigned)T.h - 2);
    float x2 = 1.0f - x1, y2 = 1.0f - y1;
    V a = T.texels[y * T.w + x], b = T.texels[y * T.w + x + 1];
    V c = T.texels[(y + 1) * T.w + x], e = T.texels[(y + 1) * T.w + x + 1];
    V ab = a * x2 + b * x1, ce = c * x2 + e * x1;
    return ab * y2 + ce * y1;
  }
  default: return T.c1;
  }
}

struct Scene {
  std::vector<Material> mats;
  std::vector<Tex> texs;
  std::vector<struct Obj> box_faces;  // six rectangles per Box object
  // The material at a hit, with a textured colour (ColorVariant, Lambertian
  // albedo / DiffuseEmitter colour) looked up at the hit's texCoords.
  Material shade_mat(const Hit &rec) const {
    Material m = mats[rec.mat];
    const int ti = (int)((uint32_t)m.flags >> PT_MAT_TEXTURE_SHIFT);
    if (ti && (m.type == PT_MAT_LAMBERTIAN || m.type == PT_MAT_DIFFUSE_EMITTER)) {
      V c = tex_eval(texs[ti - 1], rec.tu, rec.tv);
      m.p[0] = c.x;
      m.p[1] = c.y;
      m.p[2] = c.z;
    }
    return m;
  }
  std::vector<MeshO> meshes;
  std::vector<Obj> objs;
  struct TNode {
    Box box;
    int left = -1, right = -1;  // node ids (>= 0) or ~object
  };
  std::vector<TNode> top;
  int root = 0;
  std::vector<Light> lights;
  bool has_env = false;
  int env_w = 0, env_h = 0;
  float env_intensity = 1.f;
  std::vector<V> texels;  // [y][x]
  std::vector<float> env_pdf, alias_prob;
  std::vector<int> alias_idx;
  V bg;
  bool medium = false;
  V sig_a, sig_s;
  float sig_t_max = 0.f;

  // HitRecord::texCoords of a triangle hit: the interpolated uvs
  // (meshBVH.cpp:134-138) or, for a mesh without uvs, the planar fallback of
  // TriangleMesh::intersect over the mesh's box (triangleMesh.cpp:39-51);
  // p is the hit point in the mesh's frame.
  static void mesh_uv(const MeshO &M, Hit &rec, V p) {
    const int id = rec.prim - M.prim_base;
    if (!M.uv.empty()) {
      const auto &ui = M.uvtri[id];
      if (ui[0] < 0 || ui[1] < 0 || ui[2] < 0) return;  // (0, 0)
      const float w = 1.f - rec.bu - rec.bv;
      rec.tu = w * M.uv[ui[0]][0] + rec.bu * M.uv[ui[1]][0] + rec.bv * M.uv[ui[2]][0];
      rec.tv = w * M.uv[ui[0]][1] + rec.bu * M.uv[ui[1]][1] + rec.bv * M.uv[ui[2]][1];
      return;
    }
    const V n(std::fabs(rec.normal.x), std::fabs(rec.normal.y), std::fabs(rec.normal.z));
    const int au = (n.x > n.y && n.x > n.z) ? 1 : 0;
    const int av = (au == 1) ? 2 : (n.y > n.z ? 2 : 1);
    const float u = (p[au] - M.aabb.lo[au]) / (M.aabb.hi[au] - M.aabb.lo[au]);
    const float v = (p[av] - M.aabb.lo[av]) / (M.aabb.hi[av] - M.aabb.lo[av]);
    rec.tu = std::clamp(u, 0.f, 1.f);
    rec.tv = std::clamp(v, 0.f, 1.f);
  }

  // Sphere / AARectangle / TriangleMesh intersect (+ FlipFace, set_normal).
  // A moving object (extension) is intersected in its own frame at the ray's
  // time: origin o - vel * time; the hit position is then taken on the world
  // ray.
  // pt_object_desc.face: a decorated object's fixed is_inside (set_normal
  // given a ray-facing normal by Translate / Rotate / Scale, toggled by an
  // outer FlipFace: objectTransform.hpp:5-181, objectTransform.cpp:95-213).
  bool hit_obj(int oi, V o_w, V d, float tmin, float tmax, Hit &rec, float time) const {
    if (!hit_obj_as_hit(oi, o_w, d, tmin, tmax, rec, time)) return false;
    if (objs[oi].face) rec.is_inside = objs[oi].face == PT_FACE_FRONT;
    return true;
  }
  bool hit_obj_as_hit(int oi, V o_w, V d, float tmin, float tmax, Hit &rec, float time) const {
    const Obj &ob = objs[oi];
    if (ob.kind == PT_OBJ_CURVE) return hit_curve(ob, o_w, d, tmin, tmax, rec, time);
    if (ob.kind == PT_OBJ_BOX) {  // Box::intersect: its ObjectList, closest face (objectList.hpp:84-105)
      bool hit = false;
      float closest = tmax;
      for (int k = 0; k < 6; ++k) {
        Hit tmp;
        if (hit_objref(box_faces[ob.index * 6 + k], o_w, d, tmin, closest, tmp, time)) {
          hit = true;
          closest = tmp.t;
          rec = tmp;
        }
      }
      return hit;
    }
    return hit_objref(ob, o_w, d, tmin, tmax, rec, time);
  }
  static V bezier(const V *c, float u) {  // bezier.hpp:10-18
    float u1 = 1.0f - u;
    float b0 = u1 * u1 * u1, b1 = 3.0f * u * u1 * u1, b2 = 3.0f * u * u * u1, b3 = u * u * u;
    return c[0] * b0 + c[1] * b1 + c[2] * b2 + c[3] * b3;
  }
  static V bezier_d(const V *c, float u) {  // bezier.hpp:24-36
    V d0 = 3.0f * (c[1] - c[0]), d1 = 3.0f * (c[2] - c[1]), d2 = 3.0f * (c[3] - c[2]);
    float u1 = 1.0f - u;
    return d0 * (u1 * u1) + d1 * (2.0f * u * u1) + d2 * (u * u);
  }
  // Curve::intersect (curve.hpp:48-129), in the curve's frame at the ray's time
  bool hit_curve(const Obj &ob, V o_w, V d, float tmin, float tmax, Hit &rec, float time) const {
    const V o = ob.moving ? V(o_w.x - ob.vel.x * time, o_w.y - ob.vel.y * time, o_w.z - ob.vel.z * time) : o_w;
    const int N = 8;
    float bestT = tmax;
    bool found = false;
    V bestP, bestN, bestT3;
    for (int i = 0; i < N; ++i) {
      const V pa = bezier(ob.cps, float(i) / N), pb = bezier(ob.cps, float(i + 1) / N);
      const float u0 = float(i) / N, u1 = float(i + 1) / N;
      const float r0 = ob.w0 + (ob.w1 - ob.w0) * u0, r1 = ob.w0 + (ob.w1 - ob.w0) * u1;
      const float radius = 0.5f * (r0 + r1);
      const float segLen = (pb - pa).length();
      const V axis = (pb - pa) / segLen;
      const V d_perp = d - dot(d, axis) * axis;
      const V delta = o - pa;
      const V o_perp = delta - dot(delta, axis) * axis;
      const float A = dot(d_perp, d_perp), B = 2.0f * dot(d_perp, o_perp);
      const float C = dot(o_perp, o_perp) - radius * radius;
      const float disc = B * B - 4 * A * C;  // gl::solveQuadratic (utility.hpp:112-124)
      if (disc < 0) continue;
      const float sq = std::sqrt(disc);
      const float q = B < 0 ? -0.5f * (B - sq) : -0.5f * (B + sq);
      float roots[2] = {q / A, C / q};
      if (roots[0] > roots[1]) std::swap(roots[0], roots[1]);
      const int nr = roots[0] == roots[1] ? 1 : 2;
      for (int r = 0; r < nr; ++r) {
        const float t = roots[r];
        if (t < tmin || t > bestT) continue;
        const V hp = o + t * d;
        const float proj = dot(hp - pa, axis);
        if (proj < 0.0f || proj > segLen) continue;
        bestT = t;
        bestP = hp;
        const float uu = proj / segLen;
        const V d0 = bezier_d(ob.cps, u0), d1 = bezier_d(ob.cps, u1);
        bestT3 = (d0 + (d1 - d0) * uu).normalize();
        const V v = hp - (pa + axis * proj);
        bestN = (v - dot(v, bestT3) * bestT3).normalize();
        found = true;
      }
    }
    if (!found) return false;
    rec.t = bestT;
    rec.position = o_w + bestT * d;
    rec.tangent = bestT3;
    rec.has_tangent = true;
    rec.set_normal(d, bestN);
    rec.mat = ob.mat;
    rec.prim = ob.prim;
    rec.light = -1;
    return true;
  }

  bool hit_objref(const Obj &ob, V o_w, V d, float tmin, float tmax, Hit &rec, float time) const {
    const V o = ob.moving ? V(o_w.x - ob.vel.x * time, o_w.y - ob.vel.y * time, o_w.z - ob.vel.z * time) : o_w;
    if (ob.kind == PT_OBJ_MESH) {
      const MeshO &M = meshes[ob.index];
      if (!M.hit_node(0, o, d, tmin, tmax, rec)) return false;
      const V p_obj = rec.position;
      if (ob.moving) rec.position = o_w + rec.t * d;
      rec.set_normal(d, rec.normal);
      mesh_uv(M, rec, p_obj);
      rec.mat = M.mat;
      rec.light = -1;
      return true;
    }
    V dn = d.normalize();
    if (ob.kind == PT_OBJ_QUAD) {  // primitive.cpp:31-122
      int a = ob.axis, a0 = a == 0 ? 1 : 0, a1 = a == 2 ? 1 : 2;
      float t = (ob.k - o[a]) / dn[a];
      if (t < tmin || t > tmax) return false;
      float q0 = o[a0] + t * dn[a0], q1 = o[a1] + t * dn[a1];
      if (q0 < ob.d0min || q0 > ob.d0max || q1 < ob.d1min || q1 > ob.d1max) return false;
      rec.t = t;
      rec.position = o_w + t * dn;
      // AARectangle texCoords (primitive.cpp:55-57)
      rec.tu = (q0 - ob.d0min) / (ob.d0max - ob.d0min);
      rec.tv = (q1 - ob.d1min) / (ob.d1max - ob.d1min);
      V nn(a == 0 ? 1.f : 0.f, a == 1 ? 1.f : 0.f, a == 2 ? 1.f : 0.f);
      rec.set_normal(d, nn);
    } else {  // primitive.hpp:124-170
      V oc = o - ob.c;
      float A = dot(dn, dn), B = 2 * dot(dn, oc), Cc = dot(oc, oc) - ob.r * ob.r;
      float disc = B * B - 4 * A * Cc;
      if (disc < 0) return false;
      float delta = std::sqrt(disc);
      float t = (-B - delta) / (2 * A);
      if (t < tmin || t > tmax) {
        t = (-B + delta) / (2 * A);
        if (t < tmin || t > tmax) return false;
      }
      rec.t = t;
      rec.position = o_w + t * dn;
      const V c = ob.moving ? V(ob.c.x + ob.vel.x * time, ob.c.y + ob.vel.y * time, ob.c.z + ob.vel.z * time)
                            : ob.c;
      rec.set_normal(d, (rec.position - c).normalize());
      // Sphere texCoords (primitive.hpp:158-164), in the object's frame
      const V q = ((o + t * dn) - ob.c).normalize();
      const float phi = std::atan2(q.z, q.x), theta = std::asin(std::clamp(q.y, -1.f, 1.f));
      rec.tu = std::fmod(1.f - (phi + (float)PI) / (2.f * (float)PI) + 0.75f, 1.0f);
      rec.tv = (theta + (float)(PI / 2)) / (float)PI;
    }
    if (ob.flip) rec.is_inside = !rec.is_inside;
    rec.mat = ob.mat;
    rec.prim = ob.prim;
    rec.light = ob.light;
    return true;
  }
  bool hit_ref(int ref, V o, V d, float tmin, float tmax, Hit &rec, float time) const {
    if (ref < 0) return hit_obj(~ref, o, d, tmin, tmax, rec, time);
    // BVHNode::intersect (bvh.hpp:27-41): left, then right with tmax = left.t
    const TNode &N = top[ref];
    if (!N.box.hit(o, d, tmin, tmax)) return false;
    bool lh = hit_ref(N.left, o, d, tmin, tmax, rec, time);
    bool rh = hit_ref(N.right, o, d, tmin, lh ? rec.t : tmax, rec, time);
    return lh || rh;
  }
  bool intersect(V o, V d, Hit &rec, float tmin = 0.0001f, float tmax = 1e5f, float time = 0.f) const {
    return hit_ref(root, o, d, tmin, tmax, rec, time);
  }
  Box ref_box(int ref) const { return ref < 0 ? objs[~ref].box : top[ref].box; }
  // BVHNode ctor (bvh.hpp:46-102): halves of the insertion order, rand()
  // axis per node, the axis ordering only the 2-object case.
  int build_top(int i, int j) {
    int axis = std::rand() % 3;
    TNode N;
    if (j - i == 1) {
      N.left = N.right = ~i;
    } else if (j - i == 2) {
      const Box &a = objs[i].box, &b = objs[i + 1].box;
      bool lt = (a.lo[axis] + a.hi[axis]) * 0.5f < (b.lo[axis] + b.hi[axis]) * 0.5f;
      N.left = lt ? ~i : ~(i + 1);
      N.right = lt ? ~(i + 1) : ~i;
    } else {
      int mid = i + (j - i) / 2;
      N.left = build_top(i, mid);
      N.right = build_top(mid, j);
    }
    N.box = merge(ref_box(N.left), ref_box(N.right));
    top.push_back(N);
    return (int)top.size() - 1;
  }

  // HDRITexture::getTexelColor(dir) (texture.hpp:105-115, texture.cpp:112-143)
  V env_le(V dir) const {
    V dn = dir.normalize();
    float theta = std::acos(-dn.y);
    float phi = (float)(std::atan2(-dn.z, dn.x) + PI);
    float u = (float)(phi / (2.0f * PI)), v = (float)(theta / PI);
    unsigned x = (unsigned)(u * env_w), y = (unsigned)(v * env_h);
    float x1 = (u * env_w) - x, y1 = (v * env_h) - y;
    x = std::clamp(x, 0u, (unsigned)env_w - 2);
    y = std::clamp(y, 0u, (unsigned)env_h - 2);
    float x2 = (float)(1.0 - x1), y2 = (float)(1.0 - y1);
    V c1 = texels[y * env_w + x], c2 = texels[y * env_w + x + 1];
    V c3 = texels[(y + 1) * env_w + x], c4 = texels[(y + 1) * env_w + x + 1];
    V c12 = c1 * x2 + c2 * x1, c34 = c3 * x2 + c4 * x1;
    return (c12 * y2 + c34 * y1) * env_intensity;
  }
  float env_alias_pdf(V dir) const {
    V dn = dir.normalize();
    float theta = std::acos(std::clamp(-dn.y, -1.f, 1.f));
    float phi = (float)(std::atan2(-dn.z, dn.x) + PI);
    float u = (float)(phi / (2 * PI)), v = (float)(theta / PI);
    int cx = std::min((int)(u * env_w), env_w - 1), cy = std::min((int)(v * env_h), env_h - 1);
    float st = std::sin(theta);
    if (st <= 0) return 0.f;
    return (float)(env_pdf[cy * env_w + cx] * (double)(env_w * env_h) / (2 * PI * PI * st));
  }
  V env_alias_sample(float u0, float u1, float u2, float &pdf) const {
    const int N = env_w * env_h;
    float f = u0 * N;
    int i = std::min((int)f, N - 1);
    int cell = (f - i < alias_prob[i]) ? i : alias_idx[i];
    int cx = cell % env_w, cy = cell / env_w;
    float u = (cx + u1) / env_w, v = (cy + u2) / env_h;
    float st = (float)std::sin(PI * v), ct = (float)std::cos(PI * v);
    float sp = (float)std::sin(2 * PI * u), cp = (float)std::cos(2 * PI * u);
    pdf = st > 0 ? (float)(env_pdf[cell] * (double)N / (2 * PI * PI * st)) : 0.f;
    return V(-st * cp, -ct, st * sp);
  }
};

Scene *build_scene(const pt_scene_desc *d) {
  auto *S = new Scene();
  for (int i = 0; i < d->n_materials; ++i)
    S->mats.push_back(make_material(d->materials[i].type, d->materials[i].flags, d->materials[i].p));
  int n_tris = 0;
  std::vector<int> tri_base;
  for (int m = 0; m < d->n_meshes; ++m) {
    tri_base.push_back(n_tris);
    n_tris += d->meshes[m].n_triangles;
  }
  S->meshes.resize(d->n_meshes);
  for (int m = 0; m < d->n_meshes; ++m) {
    const pt_mesh_desc &md = d->meshes[m];
    MeshO &M = S->meshes[m];
    for (int i = 0; i < md.n_positions; ++i)
      M.pos.emplace_back(md.positions[3 * i], md.positions[3 * i + 1], md.positions[3 * i + 2]);
    if (md.normals)
      for (int i = 0; i < md.n_normals; ++i)
        M.nrm.emplace_back(md.normals[3 * i], md.normals[3 * i + 1], md.normals[3 * i + 2]);
    const int32_t *ni = md.normal_indices ? md.normal_indices : md.indices;
    for (int t = 0; t < md.n_triangles; ++t) {
      M.tri.push_back({md.indices[3 * t], md.indices[3 * t + 1], md.indices[3 * t + 2]});
      M.ntri.push_back({ni[3 * t], ni[3 * t + 1], ni[3 * t + 2]});
    }
    M.mat = md.material;
    if (md.uvs && md.n_uvs > 0) {
      for (int i = 0; i < md.n_uvs; ++i) M.uv.push_back({md.uvs[2 * i], md.uvs[2 * i + 1]});
      const int32_t *ui = md.uv_indices ? md.uv_indices : md.indices;
      for (int t = 0; t < md.n_triangles; ++t) {
        std::array<int, 3> u3 = {ui[3 * t], ui[3 * t + 1], ui[3 * t + 2]};
        for (int k = 0; k < 3; ++k)
          if (u3[k] >= md.n_uvs) u3[k] = -1;
        M.uvtri.push_back(u3);
      }
    }
    M.prim_base = tri_base[m];
    V mn(INFINITY), mx(-INFINITY);
    for (auto &p : M.pos) {
      mn = V(std::min(mn.x, p.x), std::min(mn.y, p.y), std::min(mn.z, p.z));
      mx = V(std::max(mx.x, p.x), std::max(mx.y, p.y), std::max(mx.z, p.z));
    }
    M.aabb = Box{mn - V(1e-3f), mx + V(1e-3f)};
    std::vector<int> ids(md.n_triangles);
    std::iota(ids.begin(), ids.end(), 0);
    M.build(ids);
  }
  for (int o = 0; o < d->n_objects; ++o) {
    const pt_object_desc &od = d->objects[o];
    Obj ob{};
    ob.kind = od.kind;
    ob.index = od.index;
    ob.vel = V(od.velocity[0], od.velocity[1], od.velocity[2]);
    ob.moving = od.velocity[0] != 0.f || od.velocity[1] != 0.f || od.velocity[2] != 0.f;
    ob.face = od.face;
    if (od.kind == PT_OBJ_MESH) {
      ob.box = S->meshes[od.index].aabb;
      ob.mat = d->meshes[od.index].material;
    } else if (od.kind == PT_OBJ_QUAD) {
      const pt_quad_desc &q = d->quads[od.index];
      ob.axis = q.axis;
      ob.k = q.k;
      ob.d0min = q.d0_min;
      ob.d0max = q.d0_max;
      ob.d1min = q.d1_min;
      ob.d1max = q.d1_max;
      ob.mat = q.material;
      ob.flip = q.flip_face;
      ob.prim = n_tris + od.index;
      int a0 = q.axis == 0 ? 1 : 0, a1 = q.axis == 2 ? 1 : 2;
      V lo, hi;
      lo[q.axis] = q.k - 1e-3f;
      hi[q.axis] = q.k + 1e-3f;
      lo[a0] = q.d0_min;
      hi[a0] = q.d0_max;
      lo[a1] = q.d1_min;
      hi[a1] = q.d1_max;
      ob.box = Box{lo, hi};
    } else if (od.kind == PT_OBJ_CURVE) {  // Curve (curve.hpp:13-46)
      const pt_curve_desc &cv = d->curves[od.index];
      V mn(INFINITY), mx(-INFINITY);
      for (int k = 0; k < 4; ++k) {
        ob.cps[k] = V(cv.cps[k][0], cv.cps[k][1], cv.cps[k][2]);
        mn = V(std::min(mn.x, ob.cps[k].x), std::min(mn.y, ob.cps[k].y), std::min(mn.z, ob.cps[k].z));
        mx = V(std::max(mx.x, ob.cps[k].x), std::max(mx.y, ob.cps[k].y), std::max(mx.z, ob.cps[k].z));
      }
      ob.w0 = cv.width0;
      ob.w1 = cv.width1;
      ob.mat = cv.material;
      const float r = std::max(cv.width0, cv.width1);
      ob.box = Box{mn - V(r), mx + V(r)};
      ob.prim = n_tris + d->n_quads + 6 * (d->boxes ? d->n_boxes : 0) + d->n_spheres + od.index;
    } else if (od.kind == PT_OBJ_BOX) {  // Box (box.hpp:5-53): six faces x1, x0, y1, y0, z1, z0
      const pt_box_desc &bx = d->boxes[od.index];
      const float *lo = bx.min_xyz, *hi = bx.max_xyz;
      const float f[6][6] = {{0, hi[0], lo[1], hi[1], lo[2], hi[2]}, {0, lo[0], lo[1], hi[1], lo[2], hi[2]},
                             {1, hi[1], lo[0], hi[0], lo[2], hi[2]}, {1, lo[1], lo[0], hi[0], lo[2], hi[2]},
                             {2, hi[2], lo[0], hi[0], lo[1], hi[1]}, {2, lo[2], lo[0], hi[0], lo[1], hi[1]}};
      ob.mat = bx.material;
      ob.box = Box{V(lo[0], lo[1], lo[2]), V(hi[0], hi[1], hi[2])};
      if ((int)S->box_faces.size() < 6 * (od.index + 1)) S->box_faces.resize(6 * (od.index + 1));
      for (int k = 0; k < 6; ++k) {
        Obj q{};
        q.kind = PT_OBJ_QUAD;
        q.axis = (int)f[k][0];
        q.k = f[k][1];
        q.d0min = f[k][2];
        q.d0max = f[k][3];
        q.d1min = f[k][4];
        q.d1max = f[k][5];
        q.mat = bx.material;
        q.prim = n_tris + d->n_quads + 6 * od.index + k;
        q.vel = ob.vel;
        q.moving = ob.moving;
        S->box_faces[6 * od.index + k] = q;
      }
    } else {
      const pt_sphere_desc &s = d->spheres[od.index];
      ob.c = V(s.center[0], s.center[1], s.center[2]);
      ob.r = s.radius;
      ob.mat = s.material;
      ob.flip = s.flip_face;
      ob.prim = n_tris + d->n_quads + 6 * (d->boxes ? d->n_boxes : 0) + od.index;
      ob.box = Box{ob.c - V(s.radius), ob.c + V(s.radius)};
    }
    if (ob.moving) {  // the box covers the motion over [0, shutter_max]
      const V sw = ob.vel * std::max(0.f, d->shutter_max);
      ob.box = merge(ob.box, Box{ob.box.lo + sw, ob.box.hi + sw});
    }
    S->objs.push_back(ob);
  }
  std::srand(1);
  S->root = S->build_top(0, (int)S->objs.size());
  // lights (lightDiscovery.hpp:5-81, light.hpp:55-306)
  for (auto &ob : S->objs) {
    if (ob.kind == PT_OBJ_MESH || ob.kind == PT_OBJ_BOX || ob.kind == PT_OBJ_CURVE) continue;
    const Material &m = S->mats[ob.mat];
    if (m.type != PT_MAT_DIFFUSE_EMITTER || m.p[3] <= 0.f) continue;
    Light L{};
    L.intensity = m.p[3];
    L.texture = (int)((uint32_t)m.flags >> PT_MAT_TEXTURE_SHIFT);
    L.color = V(m.p[0], m.p[1], m.p[2]);
    L.vel = ob.vel;
    L.moving = ob.moving;
    if (ob.kind == PT_OBJ_QUAD) {
      auto put = [&](float a, float b) {
        V v;
        v[ob.axis] = ob.k;
        v[ob.axis == 0 ? 1 : 0] = a;
        v[ob.axis == 2 ? 1 : 2] = b;
        return v;
      };
      V v0 = put(ob.d0min, ob.d1min), v1 = put(ob.d0max, ob.d1min), v3 = put(ob.d0min, ob.d1max);
      L.type = 0;
      L.v0 = v0;
      L.v2 = put(ob.d0max, ob.d1max);
      L.e1 = v1 - v0;
      L.e2 = v3 - v0;
      L.normal = cross(L.e1, L.e2).normalize();
      L.area = cross(L.e1, L.e2).length();
    } else {
      L.type = 1;
      L.c = ob.c;
      L.radius = ob.r;
      L.area = (float)(4 * PI * ob.r * ob.r);
    }
    ob.light = (int)S->lights.size();
    S->lights.push_back(L);
  }
  if (d->env) {
    S->has_env = true;
    S->env_w = d->env->width;
    S->env_h = d->env->height;
    S->env_intensity = d->env->intensity;
    const int W = S->env_w, H = S->env_h, N = W * H;
    for (int i = 0; i < N; ++i)
      S->texels.emplace_back(d->env->texels[3 * i], d->env->texels[3 * i + 1], d->env->texels[3 * i + 2]);
    // luminance alias table over texel cells (extension)
    std::vector<double> w(N);
    double sum = 0;
    for (int y = 0; y < H; ++y)
      for (int x = 0; x < W; ++x) {
        double l = 0;
        for (int dy = 0; dy < 2; ++dy)
          for (int dx = 0; dx < 2; ++dx) {
            const V &t = S->texels[std::min(y + dy, H - 1) * W + std::min(x + dx, W - 1)];
            l += 0.2126 * t.x + 0.7152 * t.y + 0.0722 * t.z;
          }
        w[y * W + x] = std::max(0.0, l * 0.25) * std::sin(PI * (y + 0.5) / H);
        sum += w[y * W + x];
      }
    double fl = (sum > 0 ? sum / N : 1.0) * 1e-3;
    sum = 0;
    for (int y = 0; y < H; ++y)
      for (int x = 0; x < W; ++x) {
        w[y * W + x] += fl * std::sin(PI * (y + 0.5) / H);
        sum += w[y * W + x];
      }
    S->env_pdf.resize(N);
    for (int i = 0; i < N; ++i) S->env_pdf[i] = (float)(w[i] / sum);
    S->alias_prob.assign(N, 1.f);
    S->alias_idx.resize(N);
    std::vector<double> sc(N);
    std::vector<int> sm, lg;
    for (int i = 0; i < N; ++i) {
      sc[i] = w[i] / sum * N;
      S->alias_idx[i] = i;
      (sc[i] < 1.0 ? sm : lg).push_back(i);
    }
    while (!sm.empty() && !lg.empty()) {
      int s = sm.back(), l = lg.back();
      sm.pop_back();
      lg.pop_back();
      S->alias_prob[s] = (float)sc[s];
      S->alias_idx[s] = l;
      sc[l] = (sc[l] + sc[s]) - 1.0;
      (sc[l] < 1.0 ? sm : lg).push_back(l);
    }
    Light L{};
    L.type = 2;
    L.intensity = d->env->intensity;
    S->lights.push_back(L);
  }
  for (int k = 0; d->textures && k < d->n_textures; ++k) {
    const pt_texture_desc &t = d->textures[k];
    Tex T;
    T.kind = t.kind;
    T.fractal = t.fractal;
    T.scale = t.scale;
    T.c1 = V(t.color1[0], t.color1[1], t.color1[2]);
    T.c2 = V(t.color2[0], t.color2[1], t.color2[2]);
    if (t.kind == PT_TEX_IMAGE) {
      T.w = t.width;
      T.h = t.height;
      for (int i = 0; i < t.width * t.height; ++i)
        T.texels.emplace_back(t.texels[3 * i], t.texels[3 * i + 1], t.texels[3 * i + 2]);
    }
    S->texs.push_back(T);
  }
  S->bg = V(d->bg_color[0], d->bg_color[1], d->bg_color[2]);
  if (d->medium) {
    S->medium = true;
    S->sig_a = V(d->medium->sigma_a[0], d->medium->sigma_a[1], d->medium->sigma_a[2]);
    S->sig_s = V(d->medium->sigma_s[0], d->medium->sigma_s[1], d->medium->sigma_s[2]);
    S->sig_t_max = max_component(S->sig_a + S->sig_s);
  }
  return S;
}

// ================================================================ integrator
struct PathCtx {
  const Scene *S;
  const pt_job_desc *job;
  uint64_t key;
  uint32_t halton_index;
  int pixel, k;
  float time = 0.f;  // motion blur (extension): the path's time
};

static float dim_value(const PathCtx &P, int dim) {
  const pt_job_desc &j = *P.job;
  if (j.sampler == PT_SAMPLER_STRATIFIED) {
    const uint32_t Sn = (uint32_t)(j.spp_x * j.spp_y);
    uint32_t h = (uint32_t)mix_bits(((uint64_t)P.pixel << 20) ^ ((uint64_t)dim << 8) ^ j.seed);
    uint32_t stratum = (uint32_t)permutation_element((uint32_t)P.k, Sn, h);
    float jit = rand01(P.key, 4096u + (uint32_t)dim);
    return std::min(((float)stratum + jit) / (float)Sn, (float)0x1.fffffep-1);
  }
  return halton_sample(j.sampler, j.sampler_seed, dim, P.halton_index);
}

static float power_heuristic(float nf, float fpdf, float ng, float gpdf) {  // maxdepth_mis.hpp:10-15
  float f = nf * fpdf, g = ng * gpdf;
  if (std::isinf(f)) return 1.f;
  float f2 = f * f, g2 = g * g;
  return (f2 + g2) > 0.f ? f2 / (f2 + g2) : 0.f;
}

struct LightSample {
  bool valid = false;
  V wl, Le;
  float tmax = 0, pdf = 0, G = 0, NoI = 0, NoL = 0, d2 = 0;
  bool env = false;
};

// Light-point offsets of light sample ls at a vertex of bounce `bounce`: the
// per-vertex getOffsets(light_samples_x, light_samples_y) grid
// (random.hpp:47-63, drawn at maxdepth_nee.hpp:91), stratum (ls / y, ls % y).
static std::pair<float, float> light_offset(const PathCtx &P, int bounce, int ls) {
  const pt_job_desc &j = *P.job;
  const uint32_t rbase = 64u + 32u * (uint32_t)bounce;
  const int si = ls / j.light_samples_y, sj = ls % j.light_samples_y;
  return {((float)si + rand01(P.key, rbase + 2u * ls)) / (float)j.light_samples_x,
          ((float)sj + rand01(P.key, rbase + 2u * ls + 1u)) / (float)j.light_samples_y};
}

// A point of light L seen from x: get_sample(ox, oy) (light.hpp:131-137,
// 254-264; envLight.hpp:20-36 over the uniform sphere), get_normal_at there,
// the direction and distance from x, L_emit towards x (texCoords (ox, oy)).
struct LightPointO {
  V p, n, w, Le;
  float len;
};
static LightPointO light_point(const Scene &S, const Light &L, float ox, float oy, V x, float tm) {
  LightPointO r;
  if (L.type == 2) {  // uniformSampleSphere * 1e5 (random.hpp:7-15, envLight.hpp:26-43)
    float z = 1.0f - 2.0f * ox;
    float rr = std::sqrt(std::max(0.f, 1.f - z * z));
    float phi = (float)(2.0f * PI * oy);
    r.p = V(rr * std::cos(phi), rr * std::sin(phi), z) * 1e5f;
    r.w = (r.p - x).normalize();
    r.len = (r.p - x).length();
    r.n = -r.p.normalize();
    r.Le = S.env_le(r.w);
    return r;
  }
  if (L.type == 0) {  // QuadLight::get_sample / get_normal_at
    r.p = L.v0 + ox * L.e1 + oy * L.e2;
    if (L.moving) r.p = V(r.p.x + L.vel.x * tm, r.p.y + L.vel.y * tm, r.p.z + L.vel.z * tm);
    r.n = L.normal;
  } else {  // SphereLight::get_sample
    float theta = (float)(2 * PI * ox);
    float phi = std::acos(2 * oy - 1);
    const V c = L.moving ? V(L.c.x + L.vel.x * tm, L.c.y + L.vel.y * tm, L.c.z + L.vel.z * tm) : L.c;
    r.p = c + L.radius * V(std::sin(phi) * std::cos(theta), std::sin(phi) * std::sin(theta), std::cos(phi));
    r.n = (r.p - c).normalize();
  }
  V ld = r.p - x;
  r.len = ld.length();
  r.w = ld.normalize();
  // L_emit (light.hpp:157-165, 296-303); a textured light at the sample's
  // offsets (maxdepth_nee.hpp:175-176)
  const V lcol = L.texture ? tex_eval(S.texs[L.texture - 1], ox, oy) : L.color;
  r.Le = (dot(r.n, -r.w) > 0.0f) ? lcol * L.intensity : V(0.f);
  return r;
}

// Light::pdf_value(origin, dir): QuadLight light.hpp:164-205 (plane hit,
// the two triangles' edge tests as the reference writes them, dist^2 /
// (area |cos|)), SphereLight :279-294 (1 / visible cap solid angle),
// EnvironmentLight envLight.hpp:58-70 (HDRITexture::pdf_direction, 1 / 4 pi).
static float light_pdf_value(const Light &L, V origin, V dir) {
  if (L.type == 2) return (float)(1.f / (4.f * PI));
  if (L.type == 1) {
    V wc = L.c - origin;
    float dc2 = dot(wc, wc), r2 = L.radius * L.radius;
    if (dc2 <= r2) return (float)(1.f / (4.f * PI));
    float cos_max = std::sqrt(1.f - r2 / dc2);
    float omega = (float)(2.f * PI * (1.f - cos_max));
    return 1.f / omega;
  }
  const V v0 = L.v0, v1 = L.v0 + L.e1, v3 = L.v0 + L.e2, N = L.normal;
  float denom = dot(N, dir);
  if (std::fabs(denom) < 1e-6f) return 0.f;
  float t = dot(v0 - origin, N) / denom;
  if (t <= 0) return 0.f;
  V P = origin + dir * t;
  auto in_tri = [&](V A, V B, V C) {
    if (dot(cross(B - A, C - A), N) < 0) return false;
    if (dot(cross(C - B, P - B), N) < 0) return false;
    if (dot(cross(A - C, P - C), N) < 0) return false;
    return true;
  };
  if (!in_tri(v0, v1, L.v2) && !in_tri(v0, L.v2, v3)) return 0.f;
  float dist2 = dot(P - origin, P - origin);
  float cos_t = std::fabs(dot(N, -dir));
  return dist2 / (L.area * cos_t);
}

// One NEE light sample (maxdepth_nee.hpp:94-210) at shading point x with
// normal n.  surface: NoI weights G; in a medium (surface=false) G = NoL/d2.
static LightSample sample_light(const PathCtx &P, V x, V n, int bounce, int ls, bool surface) {
  const Scene &S = *P.S;
  const pt_job_desc &j = *P.job;
  const uint32_t rbase = 64u + 32u * (uint32_t)bounce;
  const auto lo = light_offset(P, bounce, ls);
  const float ox = lo.first, oy = lo.second;
  const int nl = (int)S.lights.size();
  int li = (int)(rand01(P.key, rbase + 20u + ls) * nl) % nl;
  const Light &L = S.lights[li];
  LightSample r;
  if (L.type == 2) {
    float pdir;
    if (j.env_sampling == PT_ENV_ALIAS) {
      r.wl = S.env_alias_sample(ox, oy, rand01(P.key, rbase + 28u + ls), pdir);
    } else {
      r.wl = light_point(S, L, ox, oy, x, P.time).w;
      pdir = (float)(1.f / (4.f * PI));
    }
    r.env = true;
    r.tmax = std::numeric_limits<float>::max();
    r.pdf = pdir / (float)nl;
    r.NoI = surface ? std::max(0.f, dot(n, r.wl)) : 1.f;
    r.G = r.NoI;
    r.Le = S.env_le(r.wl);
    r.valid = r.pdf > 1e-7f;
    return r;
  }
  const LightPointO lp = light_point(S, L, ox, oy, x, P.time);
  const V ln = lp.n;
  const float len = lp.len;
  r.wl = lp.w;
  r.valid = len >= 0.001f;
  r.tmax = len - 0.001f;
  r.pdf = (L.area <= 1e-7f) ? 0.f : 1.f / (L.area * (float)nl);
  r.NoI = surface ? std::max(0.f, dot(n, r.wl)) : 1.f;
  r.NoL = std::max(0.f, dot(ln, -r.wl));
  r.d2 = len * len;
  r.G = (r.d2 < 1e-7f) ? 0.f : r.NoL * r.NoI / r.d2;
  r.Le = lp.Le;
  if (!(r.pdf > 1e-7f)) r.valid = false;
  return r;
}

// REF_NEE: getRayColor of maxdepth_nee.hpp:9-256, recursive, for scenes
// without a medium.
static V ray_color_ref(const PathCtx &P, V o, V d, int depth, int bounce) {
  const Scene &S = *P.S;
  const pt_job_desc &j = *P.job;
  if (depth == 0) return V(0.f);
  Hit rec;
  if (!S.intersect(o, d, rec, 0.0001f, 1e5f, P.time)) {
    if (S.has_env) return S.env_le(d.normalize());
    return S.bg;
  }
  const Material M = S.shade_mat(rec);
  const int dim0 = 3 * bounce;
  float uc = dim_value(P, dim0), u0 = dim_value(P, dim0 + 1), u1 = dim_value(P, dim0 + 2);
  Scatter s;
  if (!mat_scatter(M, d, rec, s, uc, u0, u1)) return mat_emit(M, d, rec);
  bool hr = s.spec_r(), ht = s.spec_t();
  if (hr && ht) {  // split ray: both children weighted R and T
    float R = s.pdf_val, T = 1.0f - R;
    V wo = -d.normalize();
    V sum(0.0f);
    for (int b = 0; b < 2; ++b) {
      V wi = b == 0 ? reflect_p(wo, rec.normal) : -wo;
      sum += (b == 0 ? R : T) * ray_color_ref(P, rec.position, wi, depth - 1, bounce + 1);
    }
    return mat_emit(M, d, rec) + sum;
  }
  if (hr || ht) return mat_emit(M, d, rec) + s.att * ray_color_ref(P, rec.position, s.dir, depth - 1, bounce + 1);
  V wo = -d.normalize();
  V wi = s.dir.normalize();
  float cos_t = std::abs(dot(rec.normal, wi));
  V light_term(0.f);
  const int LN = j.light_samples_x * j.light_samples_y;
  if (!S.lights.empty() && LN > 0) {
    for (int ls = 0; ls < LN; ++ls) {
      LightSample L = sample_light(P, rec.position, rec.normal, bounce, ls, true);
      float V_ = 0.f;
      if (L.valid) {
        Hit sh;
        V_ = S.intersect(rec.position, L.wl, sh, 0.001f, L.tmax, P.time) ? 0.f : 1.f;
      }
      if (V_ > 0.f && L.pdf > 1e-7f) light_term += mat_f(M, wo, L.wl, rec) * L.Le * L.G / L.pdf;
    }
    light_term = light_term / (float)LN;
  }
  if (depth - 1 == 0) return mat_emit(M, d, rec) + light_term;
  Hit next;
  bool nh = S.intersect(rec.position, wi, next, 0.0001f, 1e5f, P.time);
  if (nh && S.mats[next.mat].type == PT_MAT_DIFFUSE_EMITTER) return mat_emit(M, d, rec) + light_term;
  V att = s.att;
  if (j.rr_start >= 0 && bounce >= j.rr_start) {  // roulette_naive.hpp:35-38 on the continuation
    float q = std::clamp(max_component(s.att), 0.5f, 1.0f);
    if (rand01(P.key, 64u + 32u * (uint32_t)bounce + 31u) > q) return mat_emit(M, d, rec) + light_term;
    att = att / q;
  }
  return mat_emit(M, d, rec) + light_term +
         att * ray_color_ref(P, rec.position, wi, depth - 1, bounce + 1) * cos_t / s.pdf_val;
}

// The build's iterative estimator: REF_NEE semantics or NEE+MIS, with the
// homogeneous medium and Russian roulette extensions.
static V ray_color_iter(const PathCtx &P, V o, V d) {
  const Scene &S = *P.S;
  const pt_job_desc &j = *P.job;
  const bool mis = j.estimator == PT_EST_NEE_MIS;
  const int LN = j.light_samples_x * j.light_samples_y;
  const int limit = mis ? j.max_depth + 1 : j.max_depth;
  V L(0.f), beta(1.f);
  float prev_pdf = -1.f;
  const int dpb = S.medium ? 4 : 3;
  for (int bounce = 0; bounce < limit; ++bounce) {
    Hit rec;
    bool hit = S.intersect(o, d, rec, 0.0001f, 1e5f, P.time);
    const uint32_t rbase = 64u + 32u * (uint32_t)bounce;
    bool in_medium = false;
    float t_s = 0.f;
    if (S.medium && bounce < j.max_depth) {
      float uf = dim_value(P, dpb * bounce);
      t_s = -std::log(1 - uf) / S.sig_t_max;
      in_medium = t_s < (hit ? rec.t : std::numeric_limits<float>::infinity());
    } else if (S.medium && bounce >= j.max_depth) {
      // the extra MIS bounce only looks for emission along the segment: the
      // medium transmittance weights it
      float tt = hit ? rec.t : std::numeric_limits<float>::infinity();
      beta = beta * V(std::exp(-S.sig_t_max * tt));
    }
    if (in_medium) {
      // medium scattering vertex (extension): weight sigma_s / sigma_t
      V x = o + t_s * d.normalize();
      beta = beta * (S.sig_s / (S.sig_a + S.sig_s));
      const float phase = (float)(1.0 / (4.0 * PI));
      for (int ls = 0; ls < LN && !S.lights.empty(); ++ls) {
        LightSample Ls = sample_light(P, x, V(0, 0, 1), bounce, ls, false);
        if (!Ls.valid || Ls.env) continue;
        float pl = Ls.pdf;
        float G = Ls.G;
        if (mis && Ls.NoL > 0.f) {
          pl = Ls.pdf * Ls.d2 / Ls.NoL;
          G = 1.f;
        }
        if (G <= 0.f) continue;
        Hit sh;
        if (S.intersect(x, Ls.wl, sh, 0.001f, Ls.tmax, P.time)) continue;
        float w = mis ? power_heuristic((float)LN, pl, 1.f, phase) : 1.f;
        float tr = std::exp(-S.sig_t_max * std::sqrt(Ls.d2));
        L += beta * Ls.Le * (phase * G / pl * w * tr / (float)LN);
      }
      float u0 = dim_value(P, dpb * bounce + 2), u1 = dim_value(P, dpb * bounce + 3);
      float z = 1.f - 2.f * u0, rr = std::sqrt(std::max(0.f, 1.f - z * z));
      float ph = (float)(2 * PI * u1);
      o = x;
      d = V(rr * std::cos(ph), rr * std::sin(ph), z);
      prev_pdf = phase;
      if (bounce + 1 >= limit) break;
      continue;
    }
    if (!hit) {
      if (S.has_env) {
        float w = 1.f;
        if (mis && prev_pdf >= 0.f) {
          float pl = j.env_sampling == PT_ENV_ALIAS ? S.env_alias_pdf(d) : (float)(1.0 / (4.0 * PI));
          w = power_heuristic(1.f, prev_pdf, (float)LN, pl / (float)S.lights.size());
        }
        L += beta * S.env_le(d.normalize()) * w;
      } else {
        L += beta * S.bg;
      }
      break;
    }
    const Material M = S.shade_mat(rec);
    if (M.type == PT_MAT_DIFFUSE_EMITTER) {
      if (prev_pdf < 0.f) {
        L += beta * mat_emit(M, d, rec);
      } else if (mis) {
        if (rec.light >= 0) {
          const Light &Lt = S.lights[rec.light];
          const V lc = Lt.moving ? V(Lt.c.x + Lt.vel.x * P.time, Lt.c.y + Lt.vel.y * P.time, Lt.c.z + Lt.vel.z * P.time)
                                 : Lt.c;
          V ln = Lt.type == 0 ? Lt.normal : (rec.position - lc).normalize();
          float cl = dot(ln, -d.normalize());
          if (cl > 0.f) {
            float pl = rec.t * rec.t / (cl * Lt.area * (float)S.lights.size());
            const V lcol = Lt.texture ? tex_eval(S.texs[Lt.texture - 1], rec.tu, rec.tv) : Lt.color;
            L += beta * lcol * Lt.intensity * power_heuristic(1.f, prev_pdf, (float)LN, pl);
          }
        } else {
          L += beta * mat_emit(M, d, rec);
        }
      }
      break;
    }
    if (bounce >= j.max_depth) break;
    const int dim0 = dpb * bounce + (S.medium ? 1 : 0);
    float uc = dim_value(P, dim0), u0 = dim_value(P, dim0 + 1), u1 = dim_value(P, dim0 + 2);
    Scatter s;
    V wo = -d.normalize();
    bool ok = mat_scatter(M, d, rec, s, uc, u0, u1);
    const bool hr = s.spec_r(), ht = s.spec_t();
    if (ok && (hr || ht)) {
      if (bounce + 1 >= limit) break;
      V wi = s.dir;
      if (hr && ht) wi = (uc < s.pdf_val) ? reflect_p(wo, rec.normal).normalize() : -wo;
      beta = beta * ((hr && ht) ? V(1.f) : s.att);
      prev_pdf = -1.f;
      o = rec.position;
      d = wi;
      continue;
    }
    if (!ok && !mis) break;
    if (!S.lights.empty()) {
      V lt(0.f);
      for (int ls = 0; ls < LN; ++ls) {
        LightSample Ls = sample_light(P, rec.position, rec.normal, bounce, ls, true);
        if (!Ls.valid) continue;
        float pl = Ls.pdf, G = Ls.G;
        if (mis && !Ls.env && Ls.NoL > 0.f) {
          pl = Ls.pdf * Ls.d2 / Ls.NoL;
          G = Ls.NoI;
        }
        if (G <= 0.f) continue;
        V f = mat_f(M, wo, Ls.wl, rec);
        float w = mis ? power_heuristic((float)LN, pl, 1.f, mat_pdf(M, wo, Ls.wl, rec)) : 1.f;
        V c = f * Ls.Le * (G / pl * w / (float)LN);
        if (c.x == 0.f && c.y == 0.f && c.z == 0.f) continue;
        Hit sh;
        if (S.intersect(rec.position, Ls.wl, sh, 0.001f, Ls.tmax, P.time)) continue;
        float tr = S.medium ? (Ls.env ? 0.f : std::exp(-S.sig_t_max * std::sqrt(Ls.d2))) : 1.f;
        lt += beta * c * tr;
      }
      L += lt;
    }
    if (!ok || bounce + 1 >= limit) break;
    V wi = s.dir.normalize();
    float c = std::abs(dot(rec.normal, wi));
    V nb = beta * s.att * (c / s.pdf_val);
    if (j.rr_start >= 0 && bounce >= j.rr_start) {
      float q = std::clamp(max_component(s.att), 0.5f, 1.0f);
      if (rand01(P.key, rbase + 31u) > q) break;
      nb = nb / q;
    }
    beta = nb;
    prev_pdf = s.pdf_val;
    o = rec.position;
    d = wi;
  }
  return L;
}

// Camera + pixel offsets: PerspectiveCamera (camera.cpp:7-56) and
// FrameBuffer::setOffsets (framebuffer.cpp:131-145) with the build's RNG.
struct Camera {
  V pos, bl, hor, ver, hv, vv;
  float r;
  explicit Camera(const pt_camera_desc &c) {
    float h = std::tan(c.fov / 2.f);
    float ph = 1.0f * h * 2.0f, pw = ph * c.aspect;
    V up(c.up[0], c.up[1], c.up[2]), front(c.front[0], c.front[1], c.front[2]);
    pos = V(c.position[0], c.position[1], c.position[2]);
    V lookat = -front.normalize();
    hv = cross(up, lookat).normalize();
    vv = cross(lookat, hv).normalize();
    hor = hv * pw * c.focal_dist;
    ver = vv * ph * c.focal_dist;
    bl = pos - hor / 2.0f - ver / 2.0f;
    bl = bl - lookat * c.focal_dist;
    r = c.focal_dist / c.aperture * 0.5f;
  }
};

static std::vector<std::pair<float, float>> offsets(const pt_job_desc &j) {
  std::vector<std::pair<float, float>> off;
  const uint64_t key = path_key(j.seed ^ 0x5bd1e995u, 0xffffffffffull);
  for (int i = 0; i < j.spp_x; ++i)
    for (int k = 0; k < j.spp_y; ++k) {
      const uint32_t s = (uint32_t)(i * j.spp_y + k);
      float a = (float)i / (float)j.spp_x, b = (float)(i + 1) / (float)j.spp_x;
      float c = (float)k / (float)j.spp_y, d = (float)(k + 1) / (float)j.spp_y;
      off.push_back({a + (b - a) * rand01(key, 2 * s), c + (d - c) * rand01(key, 2 * s + 1)});
    }
  return off;
}

}  // namespace orc

using namespace orc;

extern "C" {

void *or_scene_create(const pt_scene_desc *d) { return build_scene(d); }
void or_scene_destroy(void *s) { delete static_cast<Scene *>(s); }
int or_scene_num_lights(void *s) { return (int)static_cast<Scene *>(s)->lights.size(); }

void or_sampler_eval(int strategy, uint32_t seed, uint32_t first, int n, int dims, float *out) {
  for (int i = 0; i < n; ++i)
    for (int d = 0; d < dims; ++d) out[(size_t)i * dims + d] = halton_sample(strategy, seed, d, first + (uint32_t)i);
}

// The sample values of paths [first, first + n) of a job in render order
// (pixel q = g % (W * H), grid sample k = spp_begin + g / (W * H)): pixel-grid
// offsets (2n), sampler dimensions (n * dims), light-point offsets
// (n * bounces * LN * 2) -- the values or_render's paths draw.
void or_path_samples(const pt_job_desc *job, int64_t first, int n, int dims, int bounces, float *pix, float *dv,
                     float *lo) {
  const pt_job_desc &j = *job;
  const auto off = offsets(j);
  const bool win = j.full_width > 0 || j.full_height > 0;
  const int X0 = win ? j.crop_x : 0, Y0 = win ? j.crop_y : 0;
  const int FW = win ? j.full_width : j.width, FH = win ? j.full_height : j.height;
  const int Sn = j.spp_x * j.spp_y, LN = j.light_samples_x * j.light_samples_y;
  const int64_t npix = (int64_t)j.width * j.height;
  for (int s = 0; s < n; ++s) {
    const int64_t g = first + s;
    const int q = (int)(g % npix), k = j.spp_begin + (int)(g / npix);
    const int gi = X0 + q % j.width, gj = Y0 + q / j.width;
    const uint64_t lin = ((uint64_t)gi * FH + gj) * (uint64_t)Sn + k;
    PathCtx P{nullptr, &j, path_key(j.seed, lin), (uint32_t)(lin + 1u), gj * FW + gi, k};
    pix[2 * s] = off[k].first;
    pix[2 * s + 1] = off[k].second;
    for (int d = 0; d < dims; ++d) dv[(size_t)s * dims + d] = dim_value(P, d);
    for (int b = 0; b < bounces; ++b)
      for (int ls = 0; ls < LN; ++ls) {
        const auto o = light_offset(P, b, ls);
        const size_t i = (((size_t)s * bounces + b) * LN + ls) * 2;
        lo[i] = o.first;
        lo[i + 1] = o.second;
      }
  }
}

void or_trace_closest(void *s, const float *rays, int n, float tmin, float tmax, float *t, int *prim) {
  const Scene &S = *static_cast<Scene *>(s);
  for (int i = 0; i < n; ++i) {
    Hit rec;
    V o(rays[6 * i], rays[6 * i + 1], rays[6 * i + 2]), d(rays[6 * i + 3], rays[6 * i + 4], rays[6 * i + 5]);
    bool h = S.intersect(o, d, rec, tmin, tmax);
    t[i] = h ? rec.t : std::numeric_limits<float>::max();
    prim[i] = h ? rec.prim : -1;
  }
}

// The Light methods of light `light` at n items (u, v, x): get_sample,
// get_normal_at, direction from x, L_emit towards x, pdf_value(x, dir);
// *area = get_area(); pdf_dir (may be NULL): pdf_value(x, pdf_dir[i]).
// Returns -1 for a bad light index.
int or_light_eval(void *s, int light, int n, const float *uv, const float *x, const float *pdf_dir, float *point,
                  float *normal, float *dir, float *le, float *pdf, float *area) {
  const Scene &S = *static_cast<Scene *>(s);
  if (light < 0 || light >= (int)S.lights.size()) return -1;
  const Light &L = S.lights[light];
  *area = L.type == 2 ? INFINITY : L.area;
  for (int i = 0; i < n; ++i) {
    const V xi(x[3 * i], x[3 * i + 1], x[3 * i + 2]);
    const LightPointO lp = light_point(S, L, uv[2 * i], uv[2 * i + 1], xi, 0.f);
    const V out[4] = {lp.p, lp.n, lp.w, lp.Le};
    float *dst[4] = {point, normal, dir, le};
    for (int k = 0; k < 4; ++k)
      for (int c = 0; c < 3; ++c) dst[k][3 * i + c] = out[k][c];
    pdf[i] = light_pdf_value(L, xi, pdf_dir ? V(pdf_dir[3 * i], pdf_dir[3 * i + 1], pdf_dir[3 * i + 2]) : lp.w);
  }
  return 0;
}

// The HitRecord of each ray's closest hit: t, prim, position, normal (turned
// towards the ray) and is_inside.
void or_intersect(void *s, const float *rays, int n, float tmin, float tmax, float *t, int *prim, float *pos,
                  float *nrm, uint8_t *inside) {
  const Scene &S = *static_cast<Scene *>(s);
  for (int i = 0; i < n; ++i) {
    Hit rec;
    V o(rays[6 * i], rays[6 * i + 1], rays[6 * i + 2]), d(rays[6 * i + 3], rays[6 * i + 4], rays[6 * i + 5]);
    const bool h = S.intersect(o, d, rec, tmin, tmax);
    t[i] = h ? rec.t : std::numeric_limits<float>::max();
    prim[i] = h ? rec.prim : -1;
    for (int c = 0; c < 3; ++c) {
      pos[3 * i + c] = h ? rec.position[c] : 0.f;
      nrm[3 * i + c] = h ? rec.normal[c] : 0.f;
    }
    inside[i] = (h && rec.is_inside) ? 1 : 0;
  }
}

void or_bsdf_eval(const pt_material_desc *md, int n, const float *wo, const float *wi, const float *nrm,
                  const uint8_t *front, float *f, float *pdf) {
  Material m = make_material(md->type, md->flags, md->p);
  for (int i = 0; i < n; ++i) {
    Hit rec;
    rec.normal = V(nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]);
    rec.is_inside = front[i] != 0;
    V o(wo[3 * i], wo[3 * i + 1], wo[3 * i + 2]), w(wi[3 * i], wi[3 * i + 1], wi[3 * i + 2]);
    V fv = mat_f(m, o, w, rec);
    f[3 * i] = fv.x;
    f[3 * i + 1] = fv.y;
    f[3 * i + 2] = fv.z;
    pdf[i] = mat_pdf(m, o, w, rec);
  }
}

void or_bsdf_sample(const pt_material_desc *md, int n, const float *wo, const float *nrm, const uint8_t *front,
                    const float *uc, const float *u, uint8_t *ok, float *wi, float *att, float *pdf, uint32_t *ty) {
  Material m = make_material(md->type, md->flags, md->p);
  for (int i = 0; i < n; ++i) {
    Hit rec;
    rec.normal = V(nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]);
    rec.is_inside = front[i] != 0;
    Scatter s;
    V o(wo[3 * i], wo[3 * i + 1], wo[3 * i + 2]);
    bool r = mat_scatter(m, -o, rec, s, uc[i], u[2 * i], u[2 * i + 1]);
    ok[i] = r;
    for (int c = 0; c < 3; ++c) {
      wi[3 * i + c] = r ? s.dir[c] : 0.f;
      att[3 * i + c] = r ? s.att[c] : 0.f;
    }
    pdf[i] = r ? s.pdf_val : 0.f;
    ty[i] = r ? s.type : 0u;
  }
}

// Renders the job; mean/var are width*height*3, [j][i][c].  recursive != 0
// selects the recursive REF_NEE restatement (scenes without a medium).
// FrameBuffer::gaussianBlur (framebuffer.cpp:60-129) over a film laid out
// [row][column][rgb] (row 0 = bottom, as pixel_color[j][i]).  Returns 0 when
// it blurred, 1 when the reference would refuse the arguments (film copied).
// A texture (pt_texture_desc) evaluated at n points (u, v) as the kernels'
// ColorVariant lookups do.
int or_tex_eval(const pt_texture_desc *d, int n, const float *uv, float *rgb) {
  Tex T;
  T.kind = d->kind;
  T.c1 = V(d->color1[0], d->color1[1], d->color1[2]);
  T.c2 = V(d->color2[0], d->color2[1], d->color2[2]);
  T.scale = d->scale;
  T.fractal = d->fractal;
  if (d->kind == PT_TEX_IMAGE) {
    if (!d->texels || d->width < 2 || d->height < 2) return -1;
    T.w = d->width;
    T.h = d->height;
    T.texels.resize((size_t)T.w * T.h);
    for (size_t i = 0; i < T.texels.size(); ++i)
      T.texels[i] = V(d->texels[3 * i], d->texels[3 * i + 1], d->texels[3 * i + 2]);
  }
  for (int k = 0; k < n; ++k) {
    const V c = tex_eval(T, uv[2 * k], uv[2 * k + 1]);
    rgb[3 * k] = c.x;
    rgb[3 * k + 1] = c.y;
    rgb[3 * k + 2] = c.z;
  }
  return 0;
}

int or_gaussian_blur(const float *in, float *out, int W, int H, int kernel, float sigma) {
  if (kernel % 2 == 0 || kernel < 3 || !(sigma > 0.0f)) {
    std::memcpy(out, in, sizeof(float) * 3 * (size_t)W * H);
    return 1;
  }
  std::vector<std::vector<float>> k2(kernel, std::vector<float>(kernel));
  float sum = 0.0f;
  for (int x = -kernel / 2; x <= kernel / 2; x++)
    for (int y = -kernel / 2; y <= kernel / 2; y++) {
      float r = (float)std::sqrt((double)(x * x + y * y));
      float e = std::exp(-(r * r) / (2 * sigma * sigma));
      k2[x + kernel / 2][y + kernel / 2] = (float)((double)e / (2 * M_PI * sigma * sigma));
      sum += k2[x + kernel / 2][y + kernel / 2];
    }
  for (auto &row : k2)
    for (float &v : row) v /= sum;
  for (int i = 0; i < H; i++)
    for (int j = 0; j < W; j++) {
      float c[3] = {0.f, 0.f, 0.f};
      for (int s = 0; s < kernel; s++)
        for (int t = 0; t < kernel; t++) {
          int ix = std::min(std::max(i - kernel / 2 + s, 0), H - 1);
          int iy = std::min(std::max(j - kernel / 2 + t, 0), W - 1);
          for (int ch = 0; ch < 3; ++ch) c[ch] += in[3 * ((size_t)ix * W + iy) + ch] * k2[s][t];
        }
      for (int ch = 0; ch < 3; ++ch) out[3 * ((size_t)i * W + j) + ch] = c[ch];
    }
  return 0;
}

// getRayColor for n given primary rays (pt_ray_color's contract): path i is
// frame pixel (first_index - 1 + i, 0) of a one-row frame at 1 spp, Halton
// index first_index + i; its direction is normalised.  recursive: the
// REF_NEE recursion when the job's estimator is REF_NEE and there is no medium.
void or_ray_color(void *s, const pt_job_desc *job, const float *rays, int n, uint32_t first_index, float *out,
                  int recursive) {
  const Scene &S = *static_cast<Scene *>(s);
  pt_job_desc j = *job;
  j.width = n;
  j.height = 1;
  j.spp_x = j.spp_y = 1;
  j.spp_begin = j.spp_end = 0;
  j.crop_x = (int32_t)(first_index - 1u);
  j.crop_y = 0;
  j.full_width = (int32_t)(first_index - 1u) + n;
  j.full_height = 1;
  const bool use_rec = recursive && !S.medium && j.estimator == PT_EST_REF_NEE;
  for (int i = 0; i < n; ++i) {
    const uint64_t lin = (uint64_t)(first_index - 1u) + i;
    PathCtx P{&S, &j, path_key(j.seed, lin), (uint32_t)(lin + 1u), (int)lin, 0};
    P.time = j.camera.shutter > 0.f ? j.camera.shutter * rand01(P.key, 3u) : 0.f;
    const V o(rays[6 * i], rays[6 * i + 1], rays[6 * i + 2]);
    const V d = V(rays[6 * i + 3], rays[6 * i + 4], rays[6 * i + 5]).normalize();
    const V c = use_rec ? ray_color_ref(P, o, d, j.max_depth, 0) : ray_color_iter(P, o, d);
    for (int ch = 0; ch < 3; ++ch) out[3 * i + ch] = c[ch];
  }
}

int or_render(void *s, const pt_job_desc *job, float *mean, float *var, int threads, int recursive) {
  const Scene &S = *static_cast<Scene *>(s);
  const pt_job_desc &j = *job;
  Camera cam(j.camera);
  auto off = offsets(j);
  const int W = j.width, H = j.height, Sn = j.spp_x * j.spp_y;
  // window of a larger frame (pt_job_desc crop fields): frame coordinates
  // drive the camera and the sample streams
  const bool win = j.full_width > 0 || j.full_height > 0;
  const int X0 = win ? j.crop_x : 0, Y0 = win ? j.crop_y : 0;
  const int FW = win ? j.full_width : W, FH = win ? j.full_height : H;
  const int b = j.spp_begin, e = j.spp_end ? j.spp_end : Sn;
  if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
  const bool use_rec = recursive && !S.medium && j.estimator == PT_EST_REF_NEE;
  std::atomic<int> next_col{0};
  auto worker = [&]() {
    for (int i = next_col++; i < W; i = next_col++) {
      for (int jj = 0; jj < H; ++jj) {
        double sum[3] = {0, 0, 0}, sq[3] = {0, 0, 0};
        const int gi = X0 + i, gj = Y0 + jj;
        for (int k = b; k < e; ++k) {
          uint64_t lin = ((uint64_t)gi * FH + gj) * (uint64_t)Sn + k;
          PathCtx P{&S, &j, path_key(j.seed, lin), (uint32_t)(lin + 1u), gj * FW + gi, k};
          P.time = j.camera.shutter > 0.f ? j.camera.shutter * rand01(P.key, 3u) : 0.f;
          float u = ((float)gi + off[k].first) / (float)FW, v = ((float)gj + off[k].second) / (float)FH;
          float lx = -cam.r + (cam.r - -cam.r) * rand01(P.key, 1u);
          float ly = -cam.r + (cam.r - -cam.r) * rand01(P.key, 2u);
          V ps = cam.pos + (cam.hv * lx + cam.vv * ly);
          V dir = (cam.bl + u * cam.hor + v * cam.ver - ps).normalize();
          V c = use_rec ? ray_color_ref(P, ps, dir, j.max_depth, 0) : ray_color_iter(P, ps, dir);
          for (int ch = 0; ch < 3; ++ch) {
            sum[ch] += c[ch];
            sq[ch] += (double)c[ch] * c[ch];
          }
        }
        const int n = e - b;
        for (int ch = 0; ch < 3; ++ch) {
          double m = sum[ch] / n;
          mean[(jj * W + i) * 3 + ch] = (float)m;
          if (var) var[(jj * W + i) * 3 + ch] = (float)(n > 1 ? (sq[ch] - n * m * m) / (n - 1) : 0.0);
        }
      }
    }
  };
  std::vector<std::thread> pool;
  for (int t = 0; t < threads; ++t) pool.emplace_back(worker);
  for (auto &t : pool) t.join();
  return 0;
}

}  // extern "C"
