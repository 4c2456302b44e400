// pt_bsdf_disney.cuh -- DisneyPrincipledBSDF and its lobes.
//
// Restates include/material/disneyPrincipledBSDF.hpp:8-99,
// src/material/disneyPrincipledBSDF.cpp:3-114 and the lobes
// disneyDiffuse.hpp, disneyMetal.hpp, disneyGlass.hpp, disneySheen.hpp,
// disneyClearcoat.hpp (+ ClearcoatTRD, materialMath.hpp:216-279 and
// ClearcoatPDF, PDF/clearcoatPDF.hpp:6-61), including the reference's
// behaviour that a FRONT-face hit (HitRecord::is_inside == true) routes to
// the glass lobe alone, that the metal lobe of the mixture is evaluated with
// f_variant's default arguments (disneyPrincipledBSDF.hpp:85), and that the
// chosen lobe receives u = {uc_remapped, u[1]}.
//
// MatRec.p: see pt_material_desc.  MatRec.d (host-derived):
//   d[0..4] diffuse, metal, glass, clearcoat, sheen weights
//   d[5], d[6] alpha_x, alpha_y (fromRoughnessAnisotropic)
//   d[7] clearcoat alpha
#pragma once

namespace pt {

PT_HD float schlick_w(float c) {  // pow(1 - c, 5) as the reference evaluates it in double
  double x = 1.0 - (double)c;
  double x2 = x * x;
  return (float)(x2 * x2 * x);
}
PT_HD V3 fresnel_schlick(float c, V3 F0) {  // materialMath.hpp:55-58
  float w = schlick_w(c);
  return F0 + (v3(1.f) - F0) * w;
}
PT_HD float hacked_schlick(float c, float F90) {  // materialMath.hpp:60-63
  return 1.f + (F90 - 1.f) * powf(1.f - c, 5.f);
}

PT_HD V3 dis_base(const MatRec &m) { return v3(m.p[0], m.p[1], m.p[2]); }
PT_HD TR dis_tr(const MatRec &m) { return TR{m.d[5], m.d[6]}; }

// DisneyDiffuse::f (disneyDiffuse.hpp:43-64)
PT_HD V3 dis_diffuse_f(const MatRec &m, V3 wo_w, V3 wi_w, V3 n) {
  Onb b = make_onb(n);
  V3 wo = to_local(b, wo_w), wi = to_local(b, wi_w);
  float ci = fabsf(wi.z), co = fabsf(wo.z);
  const float rough = m.p[7], ss = m.p[5];
  V3 wh = normalize(wo + wi);
  float whwi = dot(wh, wi);
  float fd90 = 0.5f + 2.f * rough * powf(fabsf(whwi), 2.f);
  V3 base = dis_base(m);
  V3 bd = base * PT_INV_PI_F;
  bd = bd * (hacked_schlick(ci, fd90) * hacked_schlick(co, fd90));
  float fss90 = rough * powf(fabsf(whwi), 2.f);
  V3 bs = (base * 1.25f) * PT_INV_PI_F;
  bs = bs * (hacked_schlick(ci, fss90) * hacked_schlick(co, fss90) * (1.f / (ci + co) - 0.5f) + 0.5f);
  return (1.f - ss) * bd + bs * ss;
}

// DisneyMetal::f / f_variant (disneyMetal.hpp:74-124); F0 = base (f) or
// the default-argument C0 = 0.5 * base (f_variant with specular_tint 0.5,
// eta 1, specular 0.5, metallic 0.5).
PT_HD V3 dis_metal_f(const MatRec &m, V3 wo_w, V3 wi_w, V3 n, bool variant) {
  Onb b = make_onb(n);
  V3 wo = to_local(b, wo_w), wi = to_local(b, wi_w);
  V3 wh = normalize(wo + wi);
  TR d = dis_tr(m);
  if (wi.z <= 0.f || wo.z <= 0.f || tr_smooth(d)) return v3(0.f);
  float dhi = fabsf(dot(wh, wi));
  V3 base = dis_base(m);
  V3 F0 = variant ? base * 0.5f : base;
  V3 F = fresnel_schlick(dhi, F0);
  float D = tr_D(d, wh), G = tr_G(d, wo, wi);
  return F * (D * G / fabsf(4.f * wi.z * wo.z));
}
PT_HD float dis_metal_pdf(const MatRec &m, V3 wo_w, V3 wi_w, V3 n) {
  TR d = dis_tr(m);
  if (tr_smooth(d)) return 0.f;
  Onb b = make_onb(n);
  return mf_pdf_at(d, b, to_local(b, normalize(wo_w)), wi_w);
}

// DisneyGlass (disneyGlass.hpp): MFDielectric with a base-colour tint.
PT_HD bool dis_glass_smooth(const MatRec &m) { return m.p[14] == 1.f || tr_smooth(dis_tr(m)); }
PT_HD V3 dis_glass_f(const MatRec &m, V3 wo_w, V3 wi_w, V3 n) {
  if (dis_glass_smooth(m)) return v3(0.f);
  const float eta = m.p[14];
  TR d = dis_tr(m);
  Onb b = make_onb(n);
  V3 wol = to_local(b, normalize(wo_w)), wil = to_local(b, normalize(wi_w));
  float co = wol.z, ci = wil.z;
  bool refl = ci * co > 0.f;
  float etap = 1.f;
  if (!refl) etap = co > 0.f ? eta : (1.f / eta);
  V3 wm = wil * etap + wol;
  if (ci == 0.f || co == 0.f || length(wm) == 0.f) return v3(0.f);
  wm = face_forward(normalize(wm), v3(0.f, 0.f, 1.f));
  if (dot(wm, wil) * ci < 0.f || dot(wm, wol) * co < 0.f) return v3(0.f);
  float F = fresnel_dielectric(dot(wol, wm), eta);
  V3 color = dis_base(m);
  if (refl) return color * (tr_D(d, wm) * tr_G(d, wol, wil) * F / fabsf(4.f * ci * co));
  float den = sqr(dot(wil, wm) + dot(wol, wm) / etap) * ci * co;
  V3 sc = v3(safe_sqrt(color.x), safe_sqrt(color.y), safe_sqrt(color.z));
  return sc * (tr_D(d, wm) * (1.f - F) * tr_G(d, wol, wil) * fabsf(dot(wil, wm) * dot(wol, wm) / den));
}
PT_HD float dis_glass_pdf(const MatRec &m, V3 wo_w, V3 wi_w, V3 n) {
  if (dis_glass_smooth(m)) return 0.f;
  Onb b = make_onb(n);
  return mfd_pdf_local(m.p[14], dis_tr(m), to_local(b, normalize(wo_w)), to_local(b, normalize(wi_w)));
}
PT_HD BsdfSample dis_glass_sample(const MatRec &m, V3 wo, V3 n, float uc, float u0, float u1) {
  BsdfSample s;
  s.ok = false;
  s.pdf = 0.f;
  s.type = 0;
  s.att = v3(0.f);
  s.wi = v3(0.f);
  const float eta = m.p[14];
  V3 won = normalize(wo);
  if (dis_glass_smooth(m)) {
    float R = fresnel_dielectric(dot(n, won), eta), T = 1.f - R;
    if (R == 0.f && T == 0.f) return s;
    if (uc < R / (R + T)) {
      s.wi = normalize(reflect_pbrt(won, n));
      s.type = BX_SPECULAR_R;
      s.att = v3(1.f);
      s.pdf = R;
      s.ok = true;
      return s;
    }
    float etap;
    V3 wt;
    if (!refract_pbrt(won, n, eta, etap, wt)) return s;
    s.wi = wt;
    s.type = BX_SPECULAR_T;
    s.att = v3(1.f);
    s.pdf = T;
    s.ok = true;
    return s;
  }
  TR d = dis_tr(m);
  Onb b = make_onb(n);
  V3 wol = to_local(b, won);
  V3 mm = tr_sample_wm(d, wol, u0, u1);
  float R = fresnel_dielectric(dot(wol, mm), eta), T = 1.f - R;
  if (R + T == 0.f) return s;
  V3 wil;
  if (uc < R / (R + T)) {
    wil = reflect_pbrt(wol, mm);
    if (!same_hemi(wol, wil)) wil.z = -wil.z;
  } else {
    float es;
    bool valid = refract_pbrt(wol, mm, eta, es, wil);
    if (!valid || same_hemi(wol, wil)) wil = reflect_pbrt(wol, mm);
  }
  V3 wi = to_world(b, wil);
  if (near_zero(wi)) return s;
  s.wi = wi;
  s.type = dot(to_local(b, wi), to_local(b, won)) > 0.f ? BX_GLOSSY_R : BX_GLOSSY_T;
  s.att = dis_glass_f(m, won, wi, n);
  s.pdf = mfd_pdf_local(eta, d, wol, to_local(b, normalize(wi)));
  s.ok = true;
  return s;
}

// DisneySheen::f (disneySheen.hpp:41-71)
PT_HD V3 dis_sheen_f(const MatRec &m, V3 wo_w, V3 wi_w, V3 n) {
  Onb b = make_onb(n);
  V3 wo = to_local(b, wo_w), wi = to_local(b, wi_w);
  V3 wh = normalize(wo + wi);
  float a = fabsf(dot(wh, wi));
  V3 base = dis_base(m);
  float lum = base.x * 0.2126f + base.y * 0.7152f + base.z * 0.0722f;  // colors.hpp:42-46
  V3 tint = lum > 0.f ? base / lum : v3(1.f);
  const float st = m.p[11];
  V3 cs = v3(1.f + st * (tint.x - 1.f), 1.f + st * (tint.y - 1.f), 1.f + st * (tint.z - 1.f));
  return cs * powf(1.f - a, 5.f);
}

// ClearcoatTRD (materialMath.hpp:216-279)
PT_HD float cc_D(float alpha, V3 h) {
  float up = alpha * alpha - 1.f;
  float lo = (float)(PT_PI * (double)logf(sqr(alpha)));
  float term = 1.f + (sqr(alpha) - 1.f) * sqr(h.z);
  return up / (lo * term);
}
PT_HD float cc_lambda(V3 w) {
  float t2 = tan2t(w);
  if (isinf(t2)) return 0.f;
  float a2 = sqr(cos_phi(w) * 0.25f) + sqr(sin_phi(w) * 0.25f);
  return (sqrtf(1.f + a2 * t2) - 1.f) * 0.5f;
}
PT_HD V3 dis_clearcoat_f(const MatRec &m, V3 wo_w, V3 wi_w, V3 n) {
  Onb b = make_onb(n);
  V3 wo = to_local(b, wo_w), wi = to_local(b, wi_w);
  V3 wh = normalize(wo + wi);
  if (wi.z <= 0.f || wo.z <= 0.f) return v3(0.f);
  float a = fabsf(dot(wh, wi));
  const float R0 = sqr((1.5f - 1.f) / (1.5f + 1.f));
  V3 F = fresnel_schlick(a, v3(R0));
  float D = cc_D(m.d[7], wh);
  float G = 1.f / (1.f + cc_lambda(wo) + cc_lambda(wi));
  return F * (D * G / fabsf(4.f * wi.z * wo.z));
}
PT_HD float cc_pdf_at(float alpha, const Onb &b, V3 wol, V3 wi_w) {  // ClearcoatPDF::at
  V3 wi = to_local(b, normalize(wi_w));
  if (wi.z <= 0.f) return 0.f;
  V3 h = normalize(wol + wi);
  float den = 4.f * fabsf(dot(wi, h));
  if (den < 1e-6f) return 0.f;
  return cc_D(alpha, h) * fabsf(h.z) / den;
}
PT_HD float dis_clearcoat_pdf(const MatRec &m, V3 wo_w, V3 wi_w, V3 n) {
  Onb b = make_onb(n);
  return cc_pdf_at(m.d[7], b, to_local(b, normalize(wo_w)), wi_w);
}

// DisneyPrincipledBSDF::f (disneyPrincipledBSDF.hpp:72-91)
PT_HD V3 disney_f(const MatRec &m, V3 wo, V3 wi, V3 n, bool front) {
  if (front) return dis_glass_f(m, wo, wi, n);
  V3 r = v3(0.f);
  r += dis_diffuse_f(m, wo, wi, n) * m.d[0];
  r += dis_metal_f(m, wo, wi, n, true) * m.d[1];
  r += dis_glass_f(m, wo, wi, n) * m.d[2];
  r += dis_clearcoat_f(m, wo, wi, n) * m.d[3];
  r += dis_sheen_f(m, wo, wi, n) * m.d[4];
  return r;
}
// DisneyPrincipledBSDF::scatter_pdf (disneyPrincipledBSDF.cpp:82-113)
PT_HD float disney_pdf(const MatRec &m, V3 wo, V3 wi, V3 n, bool front) {
  if (front) return dis_glass_pdf(m, wo, wi, n);
  float sw = m.d[0] + m.d[1] + m.d[2] + m.d[3];
  float p = 0.f;
  p += (m.d[0] / sw) * cosine_pdf(n, wi);
  p += (m.d[1] / sw) * dis_metal_pdf(m, wo, wi, n);
  p += (m.d[2] / sw) * dis_glass_pdf(m, wo, wi, n);
  p += (m.d[3] / sw) * dis_clearcoat_pdf(m, wo, wi, n);
  return p;
}

// gl::sampleDiscrete (utility.hpp:155-190) over up to 4 weights.
PT_HD int sample_discrete(const float *w, int n, float u, float *pmf, float *u_remap) {
  float sw = 0.f;
  for (int i = 0; i < n; ++i) sw += w[i];
  float up = u * sw;
  if (up == sw) up = nextafterf(up, -INFINITY);
  int off = 0;
  float sum = 0.f;
  while (off < n - 1 && sum + w[off] <= up) {
    sum += w[off];
    ++off;
  }
  if (pmf) *pmf = w[off] / sw;
  if (u_remap) *u_remap = fminf((up - sum) / w[off], 0x1.fffffep-1f);
  return off;
}

// DisneyPrincipledBSDF::scatter (disneyPrincipledBSDF.cpp:3-80)
PT_HD BsdfSample disney_sample(const MatRec &m, V3 wo, V3 n, bool front, float uc, float u0,
                               float u1) {
  if (front) return dis_glass_sample(m, wo, n, uc, u0, u1);
  BsdfSample s;
  s.ok = false;
  s.pdf = 0.f;
  s.type = 0;
  s.att = v3(0.f);
  s.wi = v3(0.f);
  float w[4] = {m.d[0], m.d[1], m.d[2], m.d[3]};
  float pmf, ur;
  int lobe = sample_discrete(w, 4, uc, &pmf, &ur);
  if (pmf <= 1e-6f) return s;
  V3 won = normalize(wo);
  const float v0 = ur, v1 = u1;  // the chosen lobe gets u = {uc_remapped, u[1]}
  if (lobe == 0) {               // DisneyDiffuse::scatter
    Onb b = make_onb(n);
    V3 wi = to_world(b, cosine_hemisphere(v0, v1));
    s.wi = normalize(wi);
    s.pdf = fmaxf(dot(normalize(wi), b.w), 0.f) * (float)(1.0 / PT_PI);
    s.type = BX_DIFFUSE_R;
    s.ok = true;
  } else if (lobe == 1) {  // DisneyMetal::scatter
    TR d = dis_tr(m);
    if (tr_smooth(d)) {
      V3 wi = normalize(reflect_pbrt(won, n));
      if (dot(n, wi) <= 0.f) return s;
      s.wi = wi;
      s.att = fresnel_schlick(fabsf(dot(n, wi)), dis_base(m));
      s.type = BX_SPECULAR_R;
      s.ok = true;
      return s;
    }
    Onb b = make_onb(n);
    V3 wol = to_local(b, won);
    V3 mm = tr_sample_wm(d, wol, v0, v1);
    V3 wil = reflect_pbrt(wol, mm);
    if (!same_hemi(wol, wil)) wil.z = -wol.z;
    V3 wi = normalize(to_world(b, wil));
    if (near_zero(wi) || dot(n, wi) <= 0.f) return s;
    s.wi = wi;
    s.pdf = mf_pdf_at(d, b, wol, wi);
    s.type = BX_GLOSSY_R;
    s.ok = true;
  } else if (lobe == 2) {  // DisneyGlass::scatter
    s = dis_glass_sample(m, won, n, ur, v0, v1);
    if (!s.ok) return s;
    if (s.type & BX_SPECULAR) return s;
  } else {  // DisneyClearcoat::scatter
    Onb b = make_onb(n);
    V3 wol = to_local(b, won);
    const float alpha = m.d[7];
    float upv = 1.f - powf(sqr(alpha), 1.f - v0);
    float lov = 1.f - sqr(alpha);
    float ch = safe_sqrt(upv / lov);
    float sh = safe_sqrt(1.f - sqr(ch));
    float sp, cp;
    sincospi_(2.f * v1, &sp, &cp);
    V3 hl = v3(sh * cp, sh * sp, ch);
    V3 wil = reflect_pbrt(wol, hl);
    if (!same_hemi(wol, wil)) wil.z = -wol.z;
    V3 wi = normalize(to_world(b, wil));
    if (dot(n, wi) <= 0.f) return s;
    s.wi = wi;
    s.pdf = cc_pdf_at(alpha, b, wol, wi);
    s.type = BX_GLOSSY_R;
    s.ok = true;
  }
  if (s.pdf <= 1e-6f) {
    s.ok = false;
    return s;
  }
  V3 wi = normalize(s.wi);
  s.att = disney_f(m, won, wi, n, false);
  s.pdf = disney_pdf(m, won, wi, n, false);
  if (s.pdf <= 1e-7f) s.ok = false;
  return s;
}

}  // namespace pt
