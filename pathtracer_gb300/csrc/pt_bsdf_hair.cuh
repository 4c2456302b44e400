// pt_bsdf_hair.cuh -- HairMarschner (include/material/hairMarsch.hpp:3-158,
// src/material/hairMarsch.cpp:4-117) and HairPDF (src/PDF/hairPDF.cpp:9-153).
//
// The reference's own formulas are kept, including its choices that differ
// from pbrt-v4: evalMarschner passes the unrotated (cos, sin) theta_o to Mp
// and its etap omits the 1/cos(theta_o) factor; HairPDF::at sums only the
// p < pMax lobes; HairPDF::get reuses uc for the azimuthal sample.  The
// frame is OrthoBasis(normal) (the hair tangent defaults to the normal,
// hairMarsch.cpp:13-16).
//
// MatRec.p: sigma_a (3), h, eta, beta_m, beta_n, alpha, [eumelanin,
// pheomelanin].  MatRec.d (host-derived): d[0..3] v[p], d[4] s,
// d[5..7] sin2kAlpha, d[8..10] cos2kAlpha, d[11..13] sigma_a actually used.
#pragma once

namespace pt {

// gl::fastExp (utility.hpp:213-237): pbrt-v4's polynomial 2^f with exponent
// re-insertion.  The reference throws for exponents above 127; this build
// returns +inf there.
PT_HD float fast_exp(float x) {
  float xp = x * 1.442695041f;
  float fxp = floorf(xp);
  float f = xp - fxp;
  int i = (int)fxp;
  float two_f = fmaf(f, fmaf(f, fmaf(f, 0.0781455737f, 0.226173572f), 0.695556856f), 1.f);
  uint32_t bits = f2u(two_f);
  int e = (int)(bits >> 23) - 127 + i;
  if (e < -126) return 0.f;
  if (e > 127) return INFINITY;
  bits &= 0x807fffffu;
  bits |= (uint32_t)(e + 127) << 23;
  return u2f(bits);
}
// gl::I0f / gl::logI0f (utility.hpp:192-211)
PT_HD float i0f(float x) {
  float term = 1.f, sum = term, x2 = x * x;
  for (int k = 1; k < 500; ++k) {
    term *= x2 / (4.f * k * k);
    sum += term;
    if (term < 1e-6f * sum) break;
    if (sum > FLT_MAX * 0.5f) break;
  }
  return sum;
}
PT_HD float log_i0f(float x) {
  if (x > 12.f) return x - 0.5f * logf(2.f * 3.14159265358979323846f * x);
  return logf(i0f(x));
}
PT_HD float safe_asin(float x) { return asinf(clampf(x, -1.f, 1.f)); }

PT_HD float hair_Mp(float ci, float co, float si, float so, float v) {
  float a = ci * co / v, b = si * so / v;
  if (v <= 0.1f) return fast_exp(log_i0f(a) - b - 1.f / v + 0.6931f + logf(1.f / (2.f * v)));
  return (fast_exp(-b) * i0f(a)) / (sinhf(1.f / v) * 2.f * v);
}
PT_HD float hair_Phi(int p, float go, float gt) { return 2.f * p * gt - 2.f * go + p * (float)PT_PI; }
PT_HD float logistic_(float x, float s) {
  x = fabsf(x);
  float e = expf(-x / s);
  return e / (s * sqr(1.f + e));
}
PT_HD float logistic_cdf(float x, float s) { return 1.f / (1.f + expf(-x / s)); }
PT_HD float hair_Np(float phi, int p, float s, float go, float gt) {
  float dphi = phi - hair_Phi(p, go, gt);
  if (!(fabsf(dphi) < 1e4f)) return 0.f;  // bounds the wrap loops below
  while (dphi > (float)PT_PI) dphi -= 2.f * (float)PT_PI;
  while (dphi < -(float)PT_PI) dphi += 2.f * (float)PT_PI;
  const float a = -(float)PT_PI, b = (float)PT_PI;
  return logistic_(dphi, s) / (logistic_cdf(b, s) - logistic_cdf(a, s));
}

// HairMarschner::Ap (hairMarsch.hpp:92-109)
PT_HD void hair_Ap(float co, float eta, float h, V3 T, V3 ap[4]) {
  float cgo = safe_sqrt(1.f - h * h);
  float ct = co * cgo;
  float f = fresnel_dielectric(ct, eta);
  ap[0] = v3(f);
  ap[1] = sqr(1.f - f) * T;
  ap[2] = ap[1] * T * f;
  V3 d = v3(1.f) - T * f;
  if (!near_zero(d))
    ap[3] = ap[2] * f * T / d;
  else
    ap[3] = v3(0.f);  // left default-constructed (zero) in the reference
}

// HairMarschner::ApPDF (hairMarsch.hpp:126-157)
PT_HD void hair_ApPDF(const MatRec &m, float co, float pdf[4]) {
  const float eta = m.p[4], h = m.p[3];
  float so = safe_sqrt(1.f - sqr(co));
  float st = so / eta;
  float ct = safe_sqrt(1.f - sqr(st));
  float etap = safe_sqrt(sqr(eta) - sqr(so)) / co;
  float sgt = h / etap;
  float cgt = safe_sqrt(1.f - sqr(sgt));
  float k = 2.f * cgt / ct;
  V3 T = v3(expf(-m.d[11] * k), expf(-m.d[12] * k), expf(-m.d[13] * k));
  V3 ap[4];
  hair_Ap(co, eta, h, T, ap);
  float sumY = 0.f;
  for (int i = 0; i < 4; ++i) sumY += (ap[i].x + ap[i].y + ap[i].z) / 3.f;
  for (int i = 0; i < 4; ++i) pdf[i] = ((ap[i].x + ap[i].y + ap[i].z) / 3.f) / sumY;
}

PT_HD void hair_rot(const MatRec &m, int p, float so, float co, float &sp, float &cp) {
  const float *s2k = m.d + 5, *c2k = m.d + 8;
  if (p == 0) {
    sp = so * c2k[1] - co * s2k[1];
    cp = co * c2k[1] + so * s2k[1];
  } else if (p == 1) {
    sp = so * c2k[0] + co * s2k[0];
    cp = co * c2k[0] - so * s2k[0];
  } else if (p == 2) {
    sp = so * c2k[2] + co * s2k[2];
    cp = co * c2k[2] - so * s2k[2];
  } else {
    sp = so;
    cp = co;
  }
  cp = fabsf(cp);
}

// HairMarschner::evalMarschner (hairMarsch.cpp:28-97), local frame.
PT_HD V3 hair_eval(const MatRec &m, V3 wi, V3 wo) {
  const float eta = m.p[4], h = m.p[3];
  float so = wo.x, co = safe_sqrt(1.f - so * so);
  float phio = atan2f(wo.z, wo.y);
  float go = safe_asin(so);
  float si = wi.x, ci = safe_sqrt(1.f - si * si);
  float phii = atan2f(wi.z, wi.y);
  float st = so / eta, ct = safe_sqrt(1.f - st * st);
  float etap = safe_sqrt(sqr(eta) - sqr(so));
  float sgt = h / etap, cgt = safe_sqrt(1.f - sgt * sgt);
  float gt = safe_asin(sgt);
  float k = 2.f * cgt / ct;
  V3 T = v3(fast_exp(-m.d[11] * k), fast_exp(-m.d[12] * k), fast_exp(-m.d[13] * k));
  float phi = phii - phio;
  V3 ap[4];
  hair_Ap(co, eta, h, T, ap);
  V3 bsdf = v3(0.f);
  for (int p = 0; p < 3; ++p) {
    float mp = hair_Mp(ci, co, si, so, m.d[p]);
    float np = hair_Np(phi, p, m.d[4], go, gt);
    bsdf += ap[p] * (mp * np);
  }
  bsdf += hair_Mp(ci, co, si, so, m.d[3]) * ap[3] / (2.f * (float)PT_PI);
  if (fabsf(wi.z) > 0.f) bsdf = bsdf / fabsf(wi.z);
  return bsdf;
}

PT_HD V3 hair_f(const MatRec &m, V3 wo, V3 wi, V3 n) {
  Onb b = make_onb(n);
  return hair_eval(m, to_local(b, normalize(wi)), to_local(b, normalize(wo)));
}

// HairPDF::at (hairPDF.cpp:101-152)
PT_HD float hair_pdf_local(const MatRec &m, V3 wol, V3 wil) {
  const float eta = m.p[4], h = m.p[3];
  float si = wil.x, ci = safe_sqrt(1.f - si * si);
  float phii = atan2f(wil.z, wil.y);
  float so = wol.x, co = safe_sqrt(1.f - so * so);
  float phio = atan2f(wol.z, wol.y);
  float go = safe_asin(so);
  float etap = safe_sqrt(sqr(eta) - sqr(so)) / co;
  float sgt = h / etap;
  float gt = safe_asin(sgt);
  float dphi = phii - phio;
  if (dphi < -(float)PT_PI)
    dphi += 2.f * (float)PT_PI;
  else if (dphi > (float)PT_PI)
    dphi -= 2.f * (float)PT_PI;
  float ap[4];
  hair_ApPDF(m, co, ap);
  float pdf = 0.f;
  for (int p = 0; p < 3; ++p) {
    float sp, cp;
    hair_rot(m, p, so, co, sp, cp);
    pdf += ap[p] * hair_Mp(ci, cp, si, sp, m.d[p]) * hair_Np(dphi, p, m.d[4], go, gt);
  }
  return pdf;
}
PT_HD float hair_pdf(const MatRec &m, V3 wo, V3 wi, V3 n) {
  Onb b = make_onb(n);
  return hair_pdf_local(m, to_local(b, wo), to_local(b, normalize(wi)));
}

// HairMarschner::scatter + HairPDF::get (hairMarsch.cpp:4-26, hairPDF.cpp:14-99)
PT_HD BsdfSample hair_sample(const MatRec &m, V3 wo, V3 n, float uc, float u0, float u1) {
  BsdfSample s;
  const float eta = m.p[4], h = m.p[3];
  V3 won = normalize(wo);
  Onb b = make_onb(n);
  V3 wol = to_local(b, won);
  float so = wol.x, co = safe_sqrt(1.f - so * so);
  float phio = atan2f(wol.z, wol.y);
  float go = safe_asin(so);
  float apd[4];
  hair_ApPDF(m, co, apd);
  int p = sample_discrete(apd, 4, uc, nullptr, nullptr);
  float sp, cp;
  hair_rot(m, p, so, co, sp, cp);
  const float vp = m.d[p];
  float ct = 1.f + vp * logf(fmaxf(u0, 1e-5f) + (1.f - u0) * fast_exp(-2.f / vp));
  float st = safe_sqrt(1.f - sqr(ct));
  float sphi, cphi;
  sincospi_(2.f * u1, &sphi, &cphi);
  float si = -ct * sp + st * cphi * cp;
  float ci = safe_sqrt(1.f - sqr(si));
  float etap = safe_sqrt(sqr(eta) - sqr(so)) / co;
  float sgt = h / etap;
  float gt = safe_asin(sgt);
  float dphi;
  if (p < 3) {
    // sampleTrimmedLogistic (utility.hpp:279-285)
    const float a = -(float)PT_PI, bb = (float)PT_PI, sc = m.d[4];
    float uu = logistic_cdf(a, sc) + uc * (logistic_cdf(bb, sc) - logistic_cdf(a, sc));
    float x = -sc * logf(1.f / uu - 1.f);
    dphi = hair_Phi(p, go, gt) + clampf(x, a, bb);
  } else {
    dphi = 2.f * (float)PT_PI * uc;
  }
  float phii = dphi + phio;
  float sphii, cphii;
  sincos_(phii, &sphii, &cphii);
  V3 wil = v3(si, ci * cphii, ci * sphii);
  V3 wi = normalize(to_world(b, wil));
  s.wi = wi;
  s.att = hair_f(m, won, wi, n);
  s.pdf = hair_pdf_local(m, wol, to_local(b, wi));
  s.type = BX_GLOSSY_R;
  s.ok = true;
  return s;
}

}  // namespace pt
