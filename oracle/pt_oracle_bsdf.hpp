// pt_oracle_bsdf.hpp -- materials of the CPU oracle, restating
// include/material/*.hpp, src/material/*.cpp and include/PDF/*.hpp of the
// reference one class at a time (file:line at each).  ORACLE ONLY.
#pragma once
#include <vector>

#include "pt_oracle_math.hpp"

namespace orc {

enum : uint32_t { REFL = 1, TRANS = 2, DIFF = 4, GLOSSY = 8, SPEC = 16 };

struct Hit {  // HitRecord (materialBase.hpp:32-53)
  float t = std::numeric_limits<float>::max();
  V normal, position;
  bool is_inside = false;  // front-face flag
  int mat = -1;
  int prim = -1;
  int light = -1;
  float bu = 0.f, bv = 0.f;  // triangle barycentrics of the hit
  bool has_tangent = false;  // a curve hit: HitRecord::hair_tangent
  V tangent;
  float tu = 0.f, tv = 0.f;  // HitRecord::texCoords
  void set_normal(V dir, V n) {
    is_inside = dot(dir, n) < 0;
    normal = is_inside ? n : -n;
  }
};

struct Scatter {  // ScatterRecord (materialBase.hpp:11-30)
  V dir;
  uint32_t type = ~0u;
  float pdf_val = 0.f;
  V att;
  bool spec_r() const { return (type & (SPEC | REFL)) == (SPEC | REFL); }
  bool spec_t() const { return (type & (SPEC | TRANS)) == (SPEC | TRANS); }
};

// pbrt helpers (utility.hpp:741-812)
inline V reflect_p(V wo, V n) { return -wo + 2 * dot(wo, n) * n; }
inline bool same_hemi(V a, V b) { return a.z * b.z > 0; }
inline float cos2(V w) { return sqr(w.z); }
inline float sin2(V w) { return std::max<float>(0, 1 - cos2(w)); }
inline float tan2(V w) { return sin2(w) / cos2(w); }
inline float cphi(V w) {
  float s = std::sqrt(sin2(w));
  return (s == 0) ? 1 : std::clamp(w.x / s, -1.f, 1.f);
}
inline float sphi(V w) {
  float s = std::sqrt(sin2(w));
  return (s == 0) ? 0 : std::clamp(w.y / s, -1.f, 1.f);
}
inline V face_fwd(V n, V v) { return (dot(n, v) < 0.f) ? -n : n; }
inline bool refract_p(V wi, V n, float eta, float &etap, V &wt) {
  float c = dot(n, wi);
  if (c < 0) {
    eta = 1 / eta;
    c = -c;
    n = -n;
  }
  float s2i = std::max<float>(0, 1 - sqr(c));
  float s2t = s2i / sqr(eta);
  if (s2t >= 1) return false;
  float ct = safe_sqrt(1 - s2t);
  wt = -wi / eta + (c / eta - ct) * n;
  wt = wt.normalize();
  etap = eta;
  return true;
}
inline V reflect_gl(V v, V n) {  // gl::reflect (utility.hpp:38-44)
  V a = v.normalize(), b = n.normalize();
  float d = dot(a, b);
  return (a - 2 * d * b).normalize();
}

inline float fresnel_dielectric(float ci, float eta) {  // materialMath.hpp:6-28
  ci = std::clamp(ci, -1.f, 1.f);
  if (ci < 0) {
    eta = 1 / eta;
    ci = -ci;
  }
  float s2i = 1 - sqr(ci);
  float s2t = s2i / sqr(eta);
  if (s2t >= 1) return 1.f;
  float ct = safe_sqrt(1 - s2t);
  float rpa = (eta * ci - ct) / (eta * ci + ct);
  float rpe = (ci - eta * ct) / (ci + eta * ct);
  return (sqr(rpa) + sqr(rpe)) / 2;
}
inline float fresnel_complex1(float ci, std::complex<float> eta) {  // materialMath.hpp:30-45
  using Cx = std::complex<float>;
  ci = std::clamp(ci, 0.f, 1.f);
  float s2i = 1 - sqr(ci);
  Cx s2t = s2i / (eta * eta);
  Cx ct = std::sqrt(Cx(1.0f, 0.0f) - s2t);
  Cx rpa = (eta * ci - ct) / (eta * ci + ct);
  Cx rpe = (ci - eta * ct) / (ci + eta * ct);
  return (std::norm(rpa) + std::norm(rpe)) / 2.f;
}
inline V fresnel_complex(float ci, V eta, V k) {
  return V(fresnel_complex1(ci, {eta.x, k.x}), fresnel_complex1(ci, {eta.y, k.y}),
           fresnel_complex1(ci, {eta.z, k.z}));
}
inline V fresnel_schlick(float c, V F0) {  // materialMath.hpp:55-58
  double w = std::pow(1.0 - c, 5.0);
  return V((float)(F0.x + (1.0 - F0.x) * w), (float)(F0.y + (1.0 - F0.y) * w), (float)(F0.z + (1.0 - F0.z) * w));
}
inline float hacked_schlick(float c, float F90) { return 1.f + (F90 - 1.f) * std::pow(1.f - c, 5.f); }

// TrowbridgeReitzDistribution (materialMath.hpp:109-214)
struct TR {
  float ax, ay;
  static TR from_rough(float r, float aniso) {
    aniso = std::max(0.0f, std::min(aniso, 1.0f / 0.9f - 0.00001f));
    float aspect = safe_sqrt(1.0f - 0.9f * aniso);
    if (aspect == 0.0f) aspect = 0.0001f;
    return TR{std::max(0.0001f, sqr(r) / aspect), std::max(0.0001f, sqr(r) * aspect)};
  }
  bool smooth() const { return std::max(ax, ay) < 1e-3f; }
  float D(V wm) const {
    float t2 = tan2(wm);
    if (std::isinf(t2)) return 0;
    float c4 = sqr(cos2(wm));
    float e = t2 * (sqr(cphi(wm) / ax) + sqr(sphi(wm) / ay));
    return (float)(1 / (PI * ax * ay * c4 * sqr(1 + e)));
  }
  float lambda(V w) const {
    float t2 = tan2(w);
    if (std::isinf(t2)) return 0;
    float a2 = sqr(cphi(w) * ax) + sqr(sphi(w) * ay);
    return (std::sqrt(1 + a2 * t2) - 1) / 2;
  }
  float G1(V w) const { return 1 / (1 + lambda(w)); }
  float G(V wo, V wi) const { return 1 / (1 + lambda(wo) + lambda(wi)); }
  float D(V w, V wm) const { return G1(w) / std::abs(w.z) * D(wm) * std::fabs(dot(w, wm)); }
  V sample_wm(V w, float u0, float u1) const {
    V wh = V(ax * w.x, ay * w.y, w.z).normalize();
    if (wh.z < 0) wh = -wh;
    V T1 = (wh.z < 0.99999f) ? cross(V(0, 0, 1), wh).normalize() : V(1, 0, 0);
    V T2 = cross(wh, T1);
    float r = std::sqrt(u0);
    float theta = (float)(2 * PI * u1);
    float px = r * std::cos(theta), py = r * std::sin(theta);
    float h = std::sqrt(1 - sqr(px));
    py = h + ((1 + wh.z) / 2) * (py - h);
    float pz = std::sqrt(std::max<float>(0, 1 - (sqr(px) + sqr(py))));
    V nh = px * T1 + py * T2 + pz * wh;
    return V(ax * nh.x, ay * nh.y, std::max<float>(1e-6f, nh.z)).normalize();
  }
};

// CosinePDF (PDF/pdf.hpp:19-37), cosineSampleHemiSphere (random.hpp:25-31)
inline V cosine_sample(float r1, float r2) {
  return V((float)(std::cos(2.f * PI * r1) * std::sqrt(r2)), (float)(std::sin(2.f * PI * r1) * std::sqrt(r2)),
           std::sqrt(1 - r2));
}
inline float cosine_pdf_at(V n, V wi) { return (float)(std::max(dot(wi.normalize(), n.normalize()), 0.f) / PI); }

// MicrofacetPDF::at (mfPDF.hpp:48-61)
inline float mf_at(const TR &d, const Onb &b, V wol, V wi_w) {
  V wi = b.local(wi_w.normalize());
  if (wi.z <= 0) return 0.f;
  V m = (wol + wi).normalize();
  float den = 4 * std::abs(dot(wol, m));
  if (den < 1e-6) return 0.f;
  return d.D(wol, m) / den;
}

// MFDielectricPDF::at (mfDielectricPDF.hpp:97-145)
inline float mfd_at(const TR &d, float eta, V wo, V wi) {
  if (eta == 1 || d.smooth()) return 0.f;
  if (wi.z == 0) return 0;
  float co = wo.z, ci = wi.z;
  bool refl = ci * co > 0;
  float etap = 1;
  if (!refl) etap = co > 0 ? eta : (1 / eta);
  V wm = wi * etap + wo;
  if (ci == 0 || co == 0 || wm.length() == 0) return 0.f;
  wm = face_fwd(wm.normalize(), V(0, 0, 1));
  if (dot(wm, wi) * ci < 0 || dot(wm, wo) * wo.z < 0) return 0.f;
  float R = fresnel_dielectric(dot(wo, wm), eta), T = 1 - R;
  if (R + T == 0) return 0.f;
  if (refl) return d.D(wo, wm) / (4.f * std::fabs(dot(wo, wm))) * R / (R + T);
  float den = sqr(dot(wi, wm) + dot(wo, wm) / etap);
  return d.D(wo, wm) * (std::fabs(dot(wi, wm)) / den) * T / (R + T);
}
// MFDielectricPDF::get with BIASED_SAMPLING (mfDielectricPDF.hpp:25-95)
inline V mfd_get(const TR &d, float eta, const Onb &b, V wo, float uc, float u0, float u1) {
  V m = d.sample_wm(wo, u0, u1);
  float R = fresnel_dielectric(dot(wo, m), eta), T = 1 - R;
  if (R + T == 0) return V();
  V wil;
  if (uc < R / (R + T)) {
    wil = reflect_p(wo, m);
    if (!same_hemi(wo, wil)) wil.z = -wil.z;
  } else {
    float es;
    bool valid = refract_p(wo, m, eta, es, wil);
    if (!valid || same_hemi(wo, wil)) wil = reflect_p(wo, m);
  }
  return b.at(wil);
}
// MFDielectric::f / DisneyGlass::f (dielectric.hpp:120-166, disneyGlass.hpp)
inline V mfd_f(const TR &d, float eta, V wol, V wil, V tint, bool tinted) {
  if (eta == 1 || d.smooth()) return V(0.f);
  float co = wol.z, ci = wil.z;
  bool refl = ci * co > 0;
  float etap = 1;
  if (!refl) etap = co > 0 ? eta : (1 / eta);
  V wm = wil * etap + wol;
  if (ci == 0 || co == 0 || wm.length() == 0) return V(0.f);
  wm = face_fwd(wm.normalize(), V(0, 0, 1));
  if (dot(wm, wil) * ci < 0 || dot(wm, wol) * co < 0) return V(0.f);
  float F = fresnel_dielectric(dot(wol, wm), eta);
  if (refl) {
    float v = d.D(wm) * d.G(wol, wil) * F / std::abs(4 * ci * co);
    return tinted ? tint * V(v) : V(v);
  }
  float den = sqr(dot(wil, wm) + dot(wol, wm) / etap) * ci * co;
  float ft = d.D(wm) * (1 - F) * d.G(wol, wil) * std::abs(dot(wil, wm) * dot(wol, wm) / den);
  if (tinted) return V(safe_sqrt(tint.x), safe_sqrt(tint.y), safe_sqrt(tint.z)) * ft;
  return V(ft);
}

// ClearcoatTRD (materialMath.hpp:216-279), ClearcoatPDF (clearcoatPDF.hpp)
struct CC {
  float alpha;
  float D(V h) const {
    float up = alpha * alpha - 1;
    float lo = (float)(PI * std::log(sqr(alpha)));
    float term = 1 + (sqr(alpha) - 1) * sqr(h.z);
    return up / (lo * term);
  }
  float lambda(V w) const {
    float t2 = tan2(w);
    if (std::isinf(t2)) return 0;
    float a2 = sqr(cphi(w) * 0.25f) + sqr(sphi(w) * 0.25f);
    return (std::sqrt(1 + a2 * t2) - 1) / 2;
  }
  float G(V wo, V wi) const { return 1.f / (1.f + lambda(wo) + lambda(wi)); }
  V sample_h(float u0, float u1) const {
    float up = 1 - std::pow(sqr(alpha), 1 - u0);
    float lo = 1 - sqr(alpha);
    float ch = safe_sqrt(up / lo), sh = safe_sqrt(1 - sqr(ch));
    float az = (float)(2 * PI * u1);
    return V(sh * std::cos(az), sh * std::sin(az), ch);
  }
  float at(const Onb &b, V wol, V wi_w) const {
    V wi = b.local(wi_w.normalize());
    if (wi.z <= 0) return 0.f;
    V h = (wol + wi).normalize();
    float den = 4 * std::abs(dot(wi, h));
    if (den < 1e-6) return 0.f;
    return D(h) * std::abs(h.z) / den;
  }
};

inline int sample_discrete(const float *w, int n, float u, float *pmf, float *ur) {  // utility.hpp:155-190
  if (n == 0) {
    if (pmf) *pmf = 0;
    return -1;
  }
  float sw = 0.f;
  for (int i = 0; i < n; ++i) sw += w[i];
  float up = u * sw;
  if (up == sw) up = std::nextafter(up, -std::numeric_limits<float>::infinity());
  int off = 0;
  float sum = 0.f;
  while (sum + w[off] <= up) {
    sum += w[off];
    ++off;
  }
  if (pmf) *pmf = w[off] / sw;
  if (ur) *ur = std::min((up - sum) / w[off], (float)0x1.fffffep-1);
  return off;
}

// gl::fastExp, I0f, logI0f (utility.hpp:192-237)
inline float fast_exp(float x) {
  float xp = x * 1.442695041f;
  float fxp = std::floor(xp), f = xp - fxp;
  int i = (int)fxp;
  float two_f = std::fma(f, std::fma(f, std::fma(f, 0.0781455737f, 0.226173572f), 0.695556856f), 1.f);
  uint32_t bits;
  std::memcpy(&bits, &two_f, 4);
  int e = (int)(bits >> 23) - 127 + i;
  if (e < -126) return 0;
  if (e > 127) return std::numeric_limits<float>::infinity();
  bits &= 0x807fffffu;
  bits |= (uint32_t)(e + 127) << 23;
  float r;
  std::memcpy(&r, &bits, 4);
  return r;
}
inline float i0f(float x) {
  float term = 1.0f, sum = term, x2 = x * x;
  for (int k = 1; k < 500; ++k) {
    term *= x2 / (4.0f * k * k);
    sum += term;
    if (term < 1e-6f * sum) break;
    if (sum > 3.402823466e+38f * 0.5f) break;
  }
  return sum;
}
inline float log_i0f(float x) {
  if (x > 12.0f) return x - 0.5f * std::log(2.0f * 3.14159265358979323846f * x);
  return std::log(i0f(x));
}

// ------------------------------------------------------------- materials
struct Material {
  int type = 0, flags = 0;
  float p[30] = {0};
  // derived
  TR tr{0, 0};
  CC cc{0};
  float w[5] = {0};       // Disney lobe weights
  float v[4] = {0}, s = 0, s2k[3] = {0}, c2k[3] = {0};  // hair
  V sigma_a;
};

Material make_material(int type, int flags, const float *p);
bool mat_scatter(const Material &m, V ray_dir, const Hit &rec, Scatter &s, float uc, float u0, float u1);
V mat_f(const Material &m, V wo, V wi, const Hit &rec);
float mat_pdf(const Material &m, V wo, V wi, const Hit &rec);
V mat_emit(const Material &m, V ray_dir, const Hit &rec);

}  // namespace orc
