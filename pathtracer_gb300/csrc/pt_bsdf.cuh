// pt_bsdf.cuh -- per-material sample / eval / pdf device functions.
//
// Each family restates one reference Material subclass (file:line at the
// function).  Directions are world-space; `n` is the shading normal turned
// towards the incoming ray and `front` is HitRecord::is_inside
// (materialBase.hpp:47-52: true when the ray hit the front face).
// TransportMode is Importance throughout, as config.hpp:23 sets it.
#pragma once
#include "pt_scene.cuh"

namespace pt {

// BxDFFlags (material/materialFlags.hpp:3-17)
enum : uint32_t {
  BX_REFLECTION = 1u,
  BX_TRANSMISSION = 2u,
  BX_DIFFUSE = 4u,
  BX_GLOSSY = 8u,
  BX_SPECULAR = 16u,
  BX_DIFFUSE_R = 5u,
  BX_GLOSSY_R = 9u,
  BX_GLOSSY_T = 10u,
  BX_SPECULAR_R = 17u,
  BX_SPECULAR_T = 18u
};

struct BsdfSample {
  bool ok;
  V3 wi;         // sampled direction (not normalised, as the reference stores it)
  V3 att;        // ScatterRecord::attenuation
  float pdf;     // ScatterRecord::pdf_val
  uint32_t type; // ScatterRecord::sampled_type
};

PT_HD float sqr(float x) { return x * x; }
PT_HD float clampf(float x, float a, float b) { return fminf(fmaxf(x, a), b); }
PT_HD float safe_sqrt(float x) { return sqrtf(fmaxf(0.f, x)); }

// pbrt helpers (utility.hpp:741-812)
PT_HD V3 reflect_pbrt(V3 wo, V3 n) { return -wo + 2.f * dot(wo, n) * n; }
PT_HD bool same_hemi(V3 a, V3 b) { return a.z * b.z > 0.f; }
PT_HD float cos2t(V3 w) { return w.z * w.z; }
PT_HD float sin2t(V3 w) { return fmaxf(0.f, 1.f - cos2t(w)); }
PT_HD float tan2t(V3 w) { return sin2t(w) / cos2t(w); }
PT_HD float cos_phi(V3 w) {
  float s = sqrtf(sin2t(w));
  return (s == 0.f) ? 1.f : clampf(w.x / s, -1.f, 1.f);
}
PT_HD float sin_phi(V3 w) {
  float s = sqrtf(sin2t(w));
  return (s == 0.f) ? 0.f : clampf(w.y / s, -1.f, 1.f);
}
PT_HD V3 face_forward(V3 n, V3 v) { return (dot(n, v) < 0.f) ? -n : n; }

// pbrt::refract (utility.hpp:746-770)
PT_HD bool refract_pbrt(V3 wi, V3 n, float eta, float &etap, V3 &wt) {
  float c = dot(n, wi);
  if (c < 0.f) {
    eta = 1.f / eta;
    c = -c;
    n = -n;
  }
  float s2i = fmaxf(0.f, 1.f - c * c);
  float s2t = s2i / (eta * eta);
  if (s2t >= 1.f) return false;
  float ct = safe_sqrt(1.f - s2t);
  wt = -wi / eta + (c / eta - ct) * n;
  wt = normalize(wt);
  etap = eta;
  return true;
}

// gl::fresnelDielectric (materialMath.hpp:6-28)
PT_HD float fresnel_dielectric(float ci, float eta) {
  ci = clampf(ci, -1.f, 1.f);
  if (ci < 0.f) {
    eta = 1.f / eta;
    ci = -ci;
  }
  float s2i = 1.f - ci * ci;
  float s2t = s2i / (eta * eta);
  if (s2t >= 1.f) return 1.f;
  float ct = safe_sqrt(1.f - s2t);
  float rpa = (eta * ci - ct) / (eta * ci + ct);
  float rpe = (ci - eta * ct) / (ci + eta * ct);
  return (rpa * rpa + rpe * rpe) * 0.5f;
}

// gl::fresnelComplex (materialMath.hpp:30-53), complex float arithmetic.
struct Cx {
  float re, im;
};
PT_HD Cx cmul(Cx a, Cx b) { return Cx{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
PT_HD Cx cdiv(Cx a, Cx b) {
  // Smith's algorithm (CACM 1962) for a stable complex quotient.
  if (fabsf(b.re) >= fabsf(b.im)) {
    float r = b.im / b.re, d = b.re + b.im * r;
    return Cx{(a.re + a.im * r) / d, (a.im - a.re * r) / d};
  }
  float r = b.re / b.im, d = b.re * r + b.im;
  return Cx{(a.re * r + a.im) / d, (a.im * r - a.re) / d};
}
PT_HD Cx csqrt_(Cx z) {
  // principal root: |w| = sqrt((|z| + |re|)/2), chosen to avoid cancellation
  float m = hypotf(z.re, z.im);
  if (m == 0.f) return Cx{0.f, 0.f};
  float t = sqrtf(0.5f * (m + fabsf(z.re)));
  if (z.re >= 0.f) return Cx{t, z.im / (2.f * t)};
  return Cx{fabsf(z.im) / (2.f * t), copysignf(t, z.im)};
}
PT_HD float cnorm(Cx z) { return z.re * z.re + z.im * z.im; }
PT_HD float fresnel_complex1(float ci, float eta, float k) {
  ci = clampf(ci, 0.f, 1.f);
  float s2i = 1.f - ci * ci;
  Cx e{eta, k};
  Cx s2t = cdiv(Cx{s2i, 0.f}, cmul(e, e));
  Cx ct = csqrt_(Cx{1.f - s2t.re, -s2t.im});
  Cx eci{e.re * ci, e.im * ci};
  Cx rpa = cdiv(Cx{eci.re - ct.re, eci.im - ct.im}, Cx{eci.re + ct.re, eci.im + ct.im});
  Cx ect = cmul(e, ct);
  Cx rpe = cdiv(Cx{ci - ect.re, -ect.im}, Cx{ci + ect.re, ect.im});
  return (cnorm(rpa) + cnorm(rpe)) * 0.5f;
}
PT_HD V3 fresnel_complex(float ci, const float *eta, const float *k) {
  return V3{fresnel_complex1(ci, eta[0], k[0]), fresnel_complex1(ci, eta[1], k[1]),
            fresnel_complex1(ci, eta[2], k[2])};
}

// ------------------------------------------- Trowbridge-Reitz (GGX)
// TrowbridgeReitzDistribution (materialMath.hpp:109-214)
struct TR {
  float ax, ay;
};
PT_HD bool tr_smooth(TR d) { return fmaxf(d.ax, d.ay) < 1e-3f; }
PT_HD float tr_D(TR d, V3 wm) {
  float t2 = tan2t(wm);
  if (isinf(t2)) return 0.f;
  float c4 = sqr(cos2t(wm));
  float e = t2 * (sqr(cos_phi(wm) / d.ax) + sqr(sin_phi(wm) / d.ay));
  return 1.f / ((float)PT_PI * d.ax * d.ay * c4 * sqr(1.f + e));
}
PT_HD float tr_lambda(TR d, V3 w) {
  float t2 = tan2t(w);
  if (isinf(t2)) return 0.f;
  float a2 = sqr(cos_phi(w) * d.ax) + sqr(sin_phi(w) * d.ay);
  return (sqrtf(1.f + a2 * t2) - 1.f) * 0.5f;
}
PT_HD float tr_G1(TR d, V3 w) { return 1.f / (1.f + tr_lambda(d, w)); }
PT_HD float tr_G(TR d, V3 wo, V3 wi) { return 1.f / (1.f + tr_lambda(d, wo) + tr_lambda(d, wi)); }
PT_HD float tr_Dw(TR d, V3 w, V3 wm) { return tr_G1(d, w) / fabsf(w.z) * tr_D(d, wm) * fabsf(dot(w, wm)); }
// visible-normal sampling, sample_wm (materialMath.hpp:178-200)
PT_HD V3 tr_sample_wm(TR d, V3 w, float u0, float u1) {
  V3 wh = normalize(v3(d.ax * w.x, d.ay * w.y, w.z));
  if (wh.z < 0.f) wh = -wh;
  V3 t1 = (wh.z < 0.99999f) ? normalize(cross(v3(0.f, 0.f, 1.f), wh)) : v3(1.f, 0.f, 0.f);
  V3 t2 = cross(wh, t1);
  // sampleUniformDiskPolar (utility.hpp:589-594)
  float r = sqrtf(u0);
  float s, c;
  sincospi_(2.f * u1, &s, &c);
  float px = r * c, py = r * s;
  float h = sqrtf(1.f - px * px);
  float tt = (1.f + wh.z) * 0.5f;
  py = h + tt * (py - h);
  float pz = sqrtf(fmaxf(0.f, 1.f - (px * px + py * py)));
  V3 nh = px * t1 + py * t2 + pz * wh;
  return normalize(v3(d.ax * nh.x, d.ay * nh.y, fmaxf(1e-6f, nh.z)));
}

// fromRoughnessAnisotropic (materialMath.hpp:119-132)
PT_HD TR tr_from_roughness(float roughness, float aniso) {
  aniso = fmaxf(0.f, fminf(aniso, 1.0f / 0.9f - 0.00001f));
  float aspect = safe_sqrt(1.f - 0.9f * aniso);
  if (aspect == 0.f) aspect = 0.0001f;
  return TR{fmaxf(0.0001f, sqr(roughness) / aspect), fmaxf(0.0001f, sqr(roughness) * aspect)};
}

// ------------------------------------------------------------ Lambertian
// Lambertian (material.hpp:79-137), CosinePDF (PDF/pdf.hpp:19-37)
PT_HD V3 cosine_hemisphere(float r1, float r2) {  // random.hpp:25-31
  float s, c;
  sincospi_(2.f * r1, &s, &c);
  float sr = sqrtf(r2);
  return V3{c * sr, s * sr, sqrtf(1.f - r2)};
}
PT_HD float cosine_pdf(V3 n, V3 wi) {
  float c = dot(normalize(wi), normalize(n));
  return fmaxf(c, 0.f) * (float)(1.0 / PT_PI);
}
PT_HD V3 lam_f(const MatRec &m) { return v3(m.p[0], m.p[1], m.p[2]) * PT_INV_PI_F; }
PT_HD BsdfSample lam_sample(const MatRec &m, V3 n, float u0, float u1) {
  BsdfSample s;
  Onb b = make_onb(n);
  s.wi = normalize(to_world(b, cosine_hemisphere(u0, u1)));
  s.type = BX_DIFFUSE_R;
  s.att = lam_f(m);
  s.pdf = fmaxf(dot(normalize(s.wi), b.w), 0.f) * (float)(1.0 / PT_PI);
  s.ok = true;
  return s;
}

// ------------------------------------------------------------- Conductor
// Conductor (conductor.hpp:4-145) + MicrofacetPDF (PDF/mfPDF.hpp:6-62)
PT_HD TR cond_tr(const MatRec &m) { return TR{m.p[6], m.p[7]}; }
PT_HD V3 cond_f(const MatRec &m, V3 wo, V3 wi, V3 n) {
  Onb b = make_onb(n);
  V3 wol = to_local(b, normalize(wo)), wil = to_local(b, normalize(wi));
  if (wil.z <= 0.f || wol.z <= 0.f) return v3(0.f);
  TR d = cond_tr(m);
  if (tr_smooth(d)) return v3(0.f);
  V3 ml = normalize(wol + wil);
  float D = tr_D(d, ml), G = tr_G(d, wol, wil);
  V3 F = fresnel_complex(fabsf(dot(wol, ml)), m.p, m.p + 3);
  return F * (D * G / (4.f * fabsf(wol.z) * fabsf(wil.z)));
}
PT_HD float mf_pdf_at(TR d, const Onb &b, V3 wol, V3 wi_world) {
  V3 wi = to_local(b, normalize(wi_world));
  if (wi.z <= 0.f) return 0.f;
  V3 mm = normalize(wol + wi);
  float den = 4.f * fabsf(dot(wol, mm));
  if (den < 1e-6f) return 0.f;
  return tr_Dw(d, wol, mm) / den;
}
PT_HD float cond_pdf(const MatRec &m, V3 wo, V3 wi, V3 n) {
  TR d = cond_tr(m);
  if (tr_smooth(d)) return 0.f;
  Onb b = make_onb(n);
  if (dot(n, wi) <= 0.f) return 0.f;
  return mf_pdf_at(d, b, to_local(b, normalize(wo)), wi);
}
PT_HD BsdfSample cond_sample(const MatRec &m, V3 wo, V3 n, float u0, float u1) {
  BsdfSample s;
  s.ok = false;
  s.pdf = 0.f;
  s.type = 0;
  s.att = v3(0.f);
  s.wi = v3(0.f);
  V3 won = normalize(wo);
  TR d = cond_tr(m);
  if (tr_smooth(d)) {
    V3 wi = normalize(reflect_pbrt(won, n));
    if (dot(n, wi) <= 0.f) return s;
    s.wi = wi;
    s.att = fresnel_complex(fabsf(dot(n, wi)), m.p, m.p + 3);
    s.type = BX_SPECULAR_R;
    s.ok = true;
    return s;
  }
  Onb b = make_onb(n);
  V3 wol = to_local(b, won);
  V3 mm = tr_sample_wm(d, wol, u0, u1);
  V3 wil = reflect_pbrt(wol, mm);
  if (!same_hemi(wol, wil)) wil.z = -wol.z;  // BIASED_SAMPLING branch (mfPDF.hpp:29-30)
  V3 wi = normalize(to_world(b, wil));
  if (near_zero(wi)) return s;
  if (dot(n, wi) <= 0.f) return s;
  s.wi = wi;
  s.type = BX_GLOSSY_R;
  s.att = cond_f(m, won, wi, n);
  s.pdf = mf_pdf_at(d, b, wol, wi);
  s.ok = true;
  return s;
}

// ---------------------------------------------------------- MFDielectric
// MFDielectric (dielectric.hpp:5-167) + MFDielectricPDF
// (PDF/mfDielectricPDF.hpp:7-147), TransportMode::Importance.
PT_HD bool mfd_smooth(const MatRec &m) { return m.p[0] == 1.f || tr_smooth(TR{m.p[1], m.p[2]}); }
PT_HD V3 mfd_f(const MatRec &m, V3 wo, V3 wi, V3 n) {
  if (mfd_smooth(m)) return v3(0.f);
  const float eta = m.p[0];
  TR d{m.p[1], m.p[2]};
  Onb b = make_onb(n);
  V3 wol = to_local(b, normalize(wo)), wil = to_local(b, normalize(wi));
  float co = wol.z, ci = wil.z;
  bool refl = ci * co > 0.f;
  float etap = 1.f;
  if (!refl) etap = co > 0.f ? eta : (1.f / eta);
  V3 wm = wil * etap + wol;
  if (ci == 0.f || co == 0.f || length(wm) == 0.f) return v3(0.f);
  wm = face_forward(normalize(wm), v3(0.f, 0.f, 1.f));
  if (dot(wm, wil) * ci < 0.f || dot(wm, wol) * co < 0.f) return v3(0.f);
  float F = fresnel_dielectric(dot(wol, wm), eta);
  if (refl) return v3(tr_D(d, wm) * tr_G(d, wol, wil) * F / fabsf(4.f * ci * co));
  float den = sqr(dot(wil, wm) + dot(wol, wm) / etap) * ci * co;
  float ft = tr_D(d, wm) * (1.f - F) * tr_G(d, wol, wil) * fabsf(dot(wil, wm) * dot(wol, wm) / den);
  return v3(ft);
}
PT_HD float mfd_pdf_local(float eta, TR d, V3 wol, V3 wil) {
  if (wil.z == 0.f) return 0.f;
  float co = wol.z, ci = wil.z;
  bool refl = ci * co > 0.f;
  float etap = 1.f;
  if (!refl) etap = co > 0.f ? eta : (1.f / eta);
  V3 wm = wil * etap + wol;
  if (ci == 0.f || co == 0.f || length(wm) == 0.f) return 0.f;
  wm = face_forward(normalize(wm), v3(0.f, 0.f, 1.f));
  if (dot(wm, wil) * ci < 0.f || dot(wm, wol) * wol.z < 0.f) return 0.f;
  float R = fresnel_dielectric(dot(wol, wm), eta), T = 1.f - R;
  if (R + T == 0.f) return 0.f;
  if (refl) return tr_Dw(d, wol, wm) / (4.f * fabsf(dot(wol, wm))) * R / (R + T);
  float den = sqr(dot(wil, wm) + dot(wol, wm) / etap);
  float dwm = fabsf(dot(wil, wm)) / den;
  return tr_Dw(d, wol, wm) * dwm * T / (R + T);
}
PT_HD float mfd_pdf(const MatRec &m, V3 wo, V3 wi, V3 n) {
  if (mfd_smooth(m)) return 0.f;
  Onb b = make_onb(n);
  return mfd_pdf_local(m.p[0], TR{m.p[1], m.p[2]}, to_local(b, normalize(wo)),
                       to_local(b, normalize(wi)));
}
PT_HD BsdfSample mfd_sample(const MatRec &m, V3 wo, V3 n, float uc, float u0, float u1) {
  BsdfSample s;
  s.ok = false;
  s.pdf = 0.f;
  s.type = 0;
  s.att = v3(0.f);
  s.wi = v3(0.f);
  const float eta = m.p[0];
  V3 won = normalize(wo);
  if (mfd_smooth(m)) {
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
  TR d{m.p[1], m.p[2]};
  Onb b = make_onb(n);
  V3 wol = to_local(b, won);
  V3 mm = tr_sample_wm(d, wol, u0, u1);
  float R = fresnel_dielectric(dot(wol, mm), eta), T = 1.f - R;
  if (R + T == 0.f) return s;
  V3 wil;
  if (uc < R / (R + T)) {
    wil = reflect_pbrt(wol, mm);
    if (!same_hemi(wol, wil)) wil.z = -wil.z;  // BIASED_SAMPLING (mfDielectricPDF.hpp:39-40)
  } else {
    float es;
    bool valid = refract_pbrt(wol, mm, eta, es, wil);
    if (!valid || same_hemi(wol, wil)) wil = reflect_pbrt(wol, mm);  // (:61-62)
  }
  V3 wi = to_world(b, wil);
  if (near_zero(wi)) return s;
  s.wi = wi;
  bool is_refl = dot(to_local(b, wi), to_local(b, won)) > 0.f;
  s.type = is_refl ? BX_GLOSSY_R : BX_GLOSSY_T;
  s.att = mfd_f(m, won, wi, n);
  s.pdf = mfd_pdf_local(eta, d, wol, to_local(b, normalize(wi)));
  s.ok = true;
  return s;
}

// --------------------------------------------------------- ThinDielectric
// ThinDielectric (thinDielectric.hpp:3-70).  The split-ray mode returns both
// specular flags; the integrator then follows one child chosen with
// probability R (same expectation as the two-child recursion).
PT_HD BsdfSample thin_sample(const MatRec &m, V3 wo, V3 n, float uc) {
  BsdfSample s;
  s.ok = false;
  s.att = v3(1.f);
  s.wi = v3(0.f);
  V3 won = normalize(wo);
  float R = fresnel_dielectric(fabsf(dot(n, won)), m.p[0]), T = 1.f - R;
  if (R < 1.f) {
    R += sqr(T) * R / (1.f - sqr(R));
    T = 1.f - R;
  }
  if (R == 0.f && T == 0.f) {
    s.pdf = 0.f;
    s.type = 0;
    return s;
  }
  s.ok = true;
  if (m.flags & 1) {  // use_split_ray
    s.type = BX_SPECULAR_R | BX_SPECULAR_T;
    s.pdf = R;
    // the child direction is chosen by the integrator
    s.wi = (uc < R) ? normalize(reflect_pbrt(won, n)) : -won;
    return s;
  }
  if (uc < R / (R + T)) {
    s.wi = normalize(reflect_pbrt(won, n));
    s.type = BX_SPECULAR_R;
    s.pdf = R;
  } else {
    s.wi = -won;
    s.type = BX_SPECULAR_T;
    s.pdf = T;
  }
  return s;
}

// ------------------------------------------------------------------ Phong
// Phong (material.hpp:303-465): f and scatter_pdf as the reference.  The
// reference's scatter() picks the lobe with a fresh rand_num, returns the
// specular colour as attenuation and leaves pdf_val = 0 on the diffuse
// branch; this build picks the lobe with uc and returns attenuation = f and
// pdf_val = scatter_pdf, a consistent estimator of the same f.
PT_HD float phong_spec_prob(const MatRec &m) {
  float si = (m.p[3] + m.p[4] + m.p[5]) / 3.f;
  float di = (m.p[0] + m.p[1] + m.p[2]) / 3.f;
  return si / (si + di);
}
PT_HD V3 reflect_gl(V3 v, V3 n) {  // gl::reflect (utility.hpp:38-44)
  V3 a = normalize(v), b = normalize(n);
  return normalize(a - 2.f * dot(a, b) * b);
}
PT_HD V3 phong_f(const MatRec &m, V3 wo, V3 wi, V3 n) {
  V3 o = normalize(wo), i = normalize(wi);
  float ci = dot(n, i);
  if (ci <= 0.f) return v3(0.f);
  float sp = phong_spec_prob(m);
  const float sh = m.p[9];
  V3 diff = v3(m.p[0], m.p[1], m.p[2]) * (float)(1.0 / PT_PI);
  V3 R = reflect_pbrt(o, n);
  float ca = fmaxf(dot(i, R), 0.f);
  float pt_ = powf(ca, sh);
  float norm = (sh + 2.f) / (2.f * (float)PT_PI);
  V3 spec = v3(m.p[3], m.p[4], m.p[5]) * (norm * pt_);
  return sp * spec + (1.f - sp) * diff;
}
PT_HD float phong_lobe_pdf(V3 R, float sh, V3 dir) {  // PhongLobePDF::at (pdf.hpp:66-70)
  float c = fmaxf(dot(normalize(dir), normalize(R)), 0.f);
  return (sh + 1.f) / (2.f * (float)PT_PI) * powf(c, sh);
}
PT_HD float phong_pdf(const MatRec &m, V3 wo, V3 wi, V3 n) {
  float si = (m.p[3] + m.p[4] + m.p[5]) / 3.f;
  float di = (m.p[0] + m.p[1] + m.p[2]) / 3.f;
  float tot = si + di;
  if (tot == 0.f) return 0.f;
  float ps = si / tot, pd = di / tot;
  V3 o = normalize(wo), i = normalize(wi);
  float pls = 0.f;
  if (ps > 0.f) pls = phong_lobe_pdf(reflect_gl(-o, normalize(n)), m.p[9], i);
  float pld = 0.f;
  if (pd > 0.f) {
    float c = dot(i, normalize(n));
    if (c > 0.f) pld = c / (float)PT_PI;
  }
  return ps * pls + pd * pld;
}
PT_HD BsdfSample phong_sample(const MatRec &m, V3 wo, V3 n, float uc, float u0, float u1) {
  BsdfSample s;
  V3 o = normalize(wo);
  float sp = phong_spec_prob(m);
  if (uc < sp) {
    V3 R = reflect_gl(-o, n);
    Onb b = make_onb(R);
    float theta = acosf(powf(u0, 1.f / (m.p[9] + 1.f)));
    float st, ct, sphi, cphi;
    sincos_(theta, &st, &ct);
    sincospi_(2.f * u1, &sphi, &cphi);
    s.wi = normalize(to_world(b, v3(st * cphi, st * sphi, ct)));
    s.type = BX_GLOSSY_R;
  } else {
    Onb b = make_onb(n);
    s.wi = to_world(b, cosine_hemisphere(u0, u1));
    s.type = BX_DIFFUSE_R;
  }
  s.att = phong_f(m, o, s.wi, n);
  s.pdf = phong_pdf(m, o, s.wi, n);
  s.ok = s.pdf > 0.f;
  return s;
}

}  // namespace pt

#include "pt_bsdf_disney.cuh"
#include "pt_bsdf_hair.cuh"

namespace pt {

// ------------------------------------------------------------- dispatch
PT_HD bool mat_is_emitter(const MatRec &m) { return m.type == 7; }
PT_HD bool mat_is_delta_only(const MatRec &m) {
  return (m.type == 3) || (m.type == 2 && mfd_smooth(m)) || (m.type == 1 && tr_smooth(cond_tr(m)));
}
// DiffuseEmitter::emit (material.hpp:483-488)
PT_HD V3 mat_emit(const MatRec &m, V3 n, V3 ray_dir) {
  if (m.type != 7) return v3(0.f);
  if (dot(n, -ray_dir) > 0.f) return v3(m.p[0], m.p[1], m.p[2]) * m.p[3];
  return v3(0.f);
}

PT_HD V3 bsdf_f(const MatRec &m, V3 wo, V3 wi, V3 n, bool front) {
  switch (m.type) {
  case 0: return lam_f(m);
  case 1: return cond_f(m, wo, wi, n);
  case 2: return mfd_f(m, wo, wi, n);
  case 4: return phong_f(m, wo, wi, n);
  case 5: return disney_f(m, wo, wi, n, front);
  case 6: return hair_f(m, wo, wi, n);
  default: return v3(0.f);
  }
}
PT_HD float bsdf_pdf(const MatRec &m, V3 wo, V3 wi, V3 n, bool front) {
  switch (m.type) {
  case 0: return cosine_pdf(n, wi);
  case 1: return cond_pdf(m, wo, wi, n);
  case 2: return mfd_pdf(m, wo, wi, n);
  case 4: return phong_pdf(m, wo, wi, n);
  case 5: return disney_pdf(m, wo, wi, n, front);
  case 6: return hair_pdf(m, wo, wi, n);
  default: return 0.f;
  }
}
// ---------------------------------------------------- fused f + pdf (NEE)
// The same values as bsdf_f / bsdf_pdf, sharing the frame, half vector,
// D, G and Fresnel terms between the two.
PT_HD void cond_eval(const MatRec &m, V3 wo, V3 wi, V3 n, V3 &f, float &pdf) {
  f = v3(0.f);
  pdf = 0.f;
  TR d = cond_tr(m);
  if (tr_smooth(d)) return;
  Onb b = make_onb(n);
  V3 wol = to_local(b, normalize(wo)), wil = to_local(b, normalize(wi));
  if (wil.z <= 0.f) return;
  V3 ml = normalize(wol + wil);
  float D = tr_D(d, ml);
  float c = fabsf(dot(wol, ml));
  float den = 4.f * c;
  if (den >= 1e-6f) pdf = tr_G1(d, wol) / fabsf(wol.z) * D * c / den;
  if (wol.z <= 0.f) return;
  float G = tr_G(d, wol, wil);
  V3 F = fresnel_complex(c, m.p, m.p + 3);
  f = F * (D * G / (4.f * fabsf(wol.z) * fabsf(wil.z)));
}
PT_HD void mfd_eval_local(float eta, TR d, V3 wol, V3 wil, V3 tint, bool tinted, V3 &f, float &pdf) {
  f = v3(0.f);
  pdf = 0.f;
  float co = wol.z, ci = wil.z;
  if (ci == 0.f || co == 0.f) return;
  bool refl = ci * co > 0.f;
  float etap = 1.f;
  if (!refl) etap = co > 0.f ? eta : (1.f / eta);
  V3 wm = wil * etap + wol;
  if (length(wm) == 0.f) return;
  wm = face_forward(normalize(wm), v3(0.f, 0.f, 1.f));
  const float dwi = dot(wm, wil), dwo = dot(wm, wol);
  if (dwi * ci < 0.f || dwo * co < 0.f) return;
  const float F = fresnel_dielectric(dwo, eta), R = F, T = 1.f - F;
  const float D = tr_D(d, wm), G = tr_G(d, wol, wil);
  const float Dw = tr_G1(d, wol) / fabsf(wol.z) * D * fabsf(dwo);
  if (refl) {
    float v = D * G * F / fabsf(4.f * ci * co);
    f = tinted ? tint * v : v3(v);
    pdf = Dw / (4.f * fabsf(dwo)) * R / (R + T);
  } else {
    float s = sqr(dwi + dwo / etap);
    float ft = D * (1.f - F) * G * fabsf(dwi * dwo / (s * ci * co));
    f = tinted ? v3(safe_sqrt(tint.x), safe_sqrt(tint.y), safe_sqrt(tint.z)) * ft : v3(ft);
    pdf = Dw * (fabsf(dwi) / s) * T / (R + T);
  }
}

// Compile-time material dispatch for the per-family shade kernels; T < 0
// dispatches at run time.
template <int T>
PT_HD void bsdf_eval_t(const MatRec &m, V3 wo, V3 wi, V3 n, bool front, V3 &f, float &pdf);
template <int T>
PT_HD BsdfSample bsdf_sample_t(const MatRec &m, V3 wo, V3 n, bool front, float uc, float u0, float u1);

PT_HD BsdfSample bsdf_sample(const MatRec &m, V3 wo, V3 n, bool front, float uc, float u0,
                             float u1) {
  switch (m.type) {
  case 0: return lam_sample(m, n, u0, u1);
  case 1: return cond_sample(m, wo, n, u0, u1);
  case 2: return mfd_sample(m, wo, n, uc, u0, u1);
  case 3: return thin_sample(m, wo, n, uc);
  case 4: return phong_sample(m, wo, n, uc, u0, u1);
  case 5: return disney_sample(m, wo, n, front, uc, u0, u1);
  case 6: return hair_sample(m, wo, n, uc, u0, u1);
  default: {
    BsdfSample s;
    s.ok = false;
    s.wi = v3(0.f);
    s.att = v3(0.f);
    s.pdf = 0.f;
    s.type = 0;
    return s;
  }
  }
}

template <int T>
PT_HD void bsdf_eval_t(const MatRec &m, V3 wo, V3 wi, V3 n, bool front, V3 &f, float &pdf) {
  if constexpr (T == 0) {
    f = lam_f(m);
    pdf = cosine_pdf(n, wi);
  } else if constexpr (T == 1) {
    cond_eval(m, wo, wi, n, f, pdf);
  } else if constexpr (T == 2) {
    if (mfd_smooth(m)) {
      f = v3(0.f);
      pdf = 0.f;
    } else {
      Onb b = make_onb(n);
      mfd_eval_local(m.p[0], TR{m.p[1], m.p[2]}, to_local(b, normalize(wo)), to_local(b, normalize(wi)),
                     v3(1.f), false, f, pdf);
    }
  } else if constexpr (T == 3) {
    f = v3(0.f);
    pdf = 0.f;
  } else if constexpr (T == 4) {
    f = phong_f(m, wo, wi, n);
    pdf = phong_pdf(m, wo, wi, n);
  } else if constexpr (T == 5) {
    if (front && !dis_glass_smooth(m)) {
      Onb b = make_onb(n);
      mfd_eval_local(m.p[14], dis_tr(m), to_local(b, normalize(wo)), to_local(b, normalize(wi)), dis_base(m),
                     true, f, pdf);
    } else {
      f = disney_f(m, wo, wi, n, front);
      pdf = disney_pdf(m, wo, wi, n, front);
    }
  } else if constexpr (T == 6) {
    f = hair_f(m, wo, wi, n);
    pdf = hair_pdf(m, wo, wi, n);
  } else {
    f = bsdf_f(m, wo, wi, n, front);
    pdf = bsdf_pdf(m, wo, wi, n, front);
  }
}

template <int T>
PT_HD BsdfSample bsdf_sample_t(const MatRec &m, V3 wo, V3 n, bool front, float uc, float u0, float u1) {
  if constexpr (T == 0) return lam_sample(m, n, u0, u1);
  else if constexpr (T == 1) return cond_sample(m, wo, n, u0, u1);
  else if constexpr (T == 2) return mfd_sample(m, wo, n, uc, u0, u1);
  else if constexpr (T == 3) return thin_sample(m, wo, n, uc);
  else if constexpr (T == 4) return phong_sample(m, wo, n, uc, u0, u1);
  else if constexpr (T == 5) return disney_sample(m, wo, n, front, uc, u0, u1);
  else if constexpr (T == 6) return hair_sample(m, wo, n, uc, u0, u1);
  else return bsdf_sample(m, wo, n, front, uc, u0, u1);
}

}  // namespace pt
