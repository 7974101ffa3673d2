// Event sampling: (y, m) from the nuclear cross section, z = cos(theta) from
// the elementary one, pair transverse momentum from the photon pT spectra,
// two-body kinematics and the pT / eta cuts.
//
// Reference: UpcGenerator::generateEvent / generateEvents
// (src/UpcGenerator.cpp:715-889), pairProduction (:388-423),
// twoPartDecayUniform (:526-561), checkKinCuts (:563-587),
// UpcCrossSection::getPairMomentum / getPhotonPt (src/UpcCrossSection.cpp:1021-1074),
// UpcSampler1D/2D (include/UpcSampler.h:37-142).
//
// Random numbers: Philox4x32-10 (Salmon et al., SC'11) keyed by SEED, one
// counter per candidate event, so candidate i is the same whatever the launch
// shape.  Accepted events keep candidate order: pass 1 marks accepted
// candidates in a bit mask and counts them per 256-candidate tile, a scan of
// the tile counts gives each tile its output offset, and pass 2 regenerates
// only the accepted candidates of each tile into their slots.  The first N
// accepted candidates are kept and the rejected ones before the N-th are
// counted, which is the reference's generateEvents loop.
//
// Kinematics are FP32; the (y, m) and z CDFs and their inversion are FP64.
#include "upcg_internal.h"

namespace upcg {

namespace {

__device__ __forceinline__ uint4 philox_round(uint4 c, uint2 k) {
  const uint32_t lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
  const uint32_t lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
  return make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
}

__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    if (r > 0) {
      k.x += 0x9E3779B9u;
      k.y += 0xBB67AE85u;
    }
    c = philox_round(c, k);
  }
  return c;
}

__device__ __forceinline__ double u53(uint32_t a, uint32_t b) {  // [0, 1)
  const uint64_t x = ((uint64_t)a << 21) ^ (uint64_t)(b >> 11);
  return (double)(x & ((1ull << 53) - 1)) * (1.0 / 9007199254740992.0);
}

__device__ __forceinline__ float u24(uint32_t a) {  // [0, 1)
  return (float)(a >> 8) * (1.0f / 16777216.0f);
}

constexpr float kTwoPiF = 6.28318530717958647692f;

// num / den in FP32 for 0 <= num <= den (a CDF difference and its bin's
// width): the fraction of the way through a bin, in [0, 1); 0 for an empty
// bin.  Widths below 2^-100 are scaled up first (exact in FP64).
__device__ __forceinline__ float frac_in_bin(double num, double den) {
  if (!(den > 0.)) return 0.f;
  if (den < 0x1p-100) {
    num *= 0x1p100;
    den *= 0x1p100;
  }
  const float f = (float)num / (float)den;
  return f < 0.f ? 0.f : (f < 0x1.fffffep-1f ? f : 0x1.fffffep-1f);
}

// The (y, m) and z CDFs are also held in 64-bit fixed point (value * 2^64,
// 1 saturating to 2^64 - 1) and searched with a 64-bit uniform r: integer
// compares instead of FP64 ones, which on this part run at 1/64 of the FP32
// rate.  The bin is the largest k with cdf[k] <= r, as before.
__device__ __forceinline__ int cdf_find_from_fx(const uint64_t* __restrict__ cdf, int n, int k,
                                                uint64_t r) {
#pragma unroll 1
  for (int s = 0; s < 8; ++s) {
    if (k + 1 >= n || __ldg(cdf + k + 1) > r) return k;
    ++k;
  }
  int hi = n;
  while (hi - k > 1) {
    const int mid = (k + hi) >> 1;
    if (r >= __ldg(cdf + mid)) k = mid; else hi = mid;
  }
  return k;
}

__device__ __forceinline__ int cdf_find_fx(const uint64_t* __restrict__ cdf, int n, uint64_t r) {
  int lo = 0, hi = n;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (r >= __ldg(cdf + mid)) lo = mid; else hi = mid;
  }
  return lo;
}

// num / den for fixed-point num <= den: both scaled so that den has its top
// bit set, then their top 32 bits divided in FP32; [0, 1), 0 for den = 0
__device__ __forceinline__ float frac_fx(uint64_t num, uint64_t den) {
  if (den == 0) return 0.f;
  if (num >= den) return 0x1.fffffep-1f;
  const int s = __clzll((long long)den);
  const float f = (float)(uint32_t)((num << s) >> 32) / (float)(uint32_t)((den << s) >> 32);
  return f < 0x1.fffffep-1f ? f : 0x1.fffffep-1f;
}

// cdf[k] <= r < cdf[k+1] over n bins (the last non-empty bin if r >= cdf[n]).
__device__ __forceinline__ int cdf_find(const double* __restrict__ cdf, int n, double r) {
  int lo = 0, hi = n;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (r >= __ldg(cdf + mid)) lo = mid; else hi = mid;
  }
  return lo;
}

__device__ __forceinline__ int cdf_find_f(const float* __restrict__ cdf, int n, float r) {
  int lo = 0, hi = n;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (r >= __ldg(cdf + mid)) lo = mid; else hi = mid;
  }
  return lo;
}

// The same answers as cdf_find / cdf_find_f (the largest k < n with
// cdf[k] <= r), started from a guide-table entry k0 <= answer: a few forward
// steps, or a binary search over [k, n) through a run of empty bins.
__device__ __forceinline__ int cdf_find_from(const double* __restrict__ cdf, int n, int k,
                                             double r) {
#pragma unroll 1
  for (int s = 0; s < 8; ++s) {
    if (k + 1 >= n || __ldg(cdf + k + 1) > r) return k;
    ++k;
  }
  int hi = n;
  while (hi - k > 1) {
    const int mid = (k + hi) >> 1;
    if (r >= __ldg(cdf + mid)) k = mid; else hi = mid;
  }
  return k;
}

__device__ __forceinline__ int cdf_find_from_f(const float* __restrict__ cdf, int n, int k,
                                               float r) {
#pragma unroll 1
  for (int s = 0; s < 8; ++s) {
    if (k + 1 >= n || __ldg(cdf + k + 1) > r) return k;
    ++k;
  }
  int hi = n;
  while (hi - k > 1) {
    const int mid = (k + hi) >> 1;
    if (r >= __ldg(cdf + mid)) k = mid; else hi = mid;
  }
  return k;
}

// Photon pT from the tabulated spectrum closest in ln(k^2/gtot^2): the table
// at grid point i or i+1, chosen with the interpolation weight.
__device__ float photon_pt(const EventParams& e, const float* __restrict__ tabs, float lnk,
                           float u, float usel) {
  float t = (2.f * lnk - e.pt_c0) * e.pt_inv_dlne;
  t = t < 0.f ? 0.f : (t > (float)(e.pt_ne - 1) ? (float)(e.pt_ne - 1) : t);
  int i = (int)t;
  if (i > e.pt_ne - 2) i = e.pt_ne - 2;
  const float fr = t - (float)i;
  if (usel < fr) ++i;
  const float* I = tabs + (size_t)i * (e.pt_nbins + 1);
  const int ib = cdf_find_from_f(I, e.pt_nbins,
                                 __ldg(e.gpt + (size_t)i * e.gpt_n + (int)(u * (float)e.gpt_n)), u);
  const float lo = __ldg(I + ib), hi = __ldg(I + ib + 1);
  const float w = e.f_ptw;
  float x = ib * w;
  if (hi > lo) x += w * (u - lo) / (hi - lo);
  return x;
}

struct Cand {
  double m;  // FP64 for getBinY; y and z are drawn in FP32 (the record's type)
  float y, z;
  float sign;
  float p0[4], p1[4];
  int mbin;
};

__device__ __forceinline__ float eta_f(float px, float py, float pz) {
  const float pt = sqrtf(px * px + py * py);
  if (pt > 0.f) return asinhf(pz / pt);
  if (pz == 0.f) return 0.f;
  return pz > 0.f ? 10e10f : -10e10f;
}

// Boost a rest-frame momentum v (energy ev) by the frame of the 4-vector
// (px, py, pz, E) of invariant mass M: p' = v + P [ (P.v)/(M (E + M)) + ev/M ].
__device__ __forceinline__ void boost_by(float vx, float vy, float vz, float ev, float px,
                                         float py, float pz, float E, float M, float* out) {
  const float pv = px * vx + py * vy + pz * vz;
  const float f = pv / (M * (E + M)) + ev / M;
  out[0] = vx + f * px;
  out[1] = vy + f * py;
  out[2] = vz + f * pz;
  out[3] = (E * ev + pv) / M;
}

// TVector3::RotateUz: v from the frame whose z axis is the direction of p
__device__ __forceinline__ void rotate_uz_f(float& vx, float& vy, float& vz, float px, float py,
                                            float pz) {
  const float pm = sqrtf(px * px + py * py + pz * pz);
  if (!(pm > 0.f)) return;
  const float u1 = px / pm, u2 = py / pm, u3 = pz / pm;
  float up = u1 * u1 + u2 * u2;
  if (up > 0.f) {
    up = sqrtf(up);
    const float x = (u1 * u3 * vx - u2 * vy + u1 * up * vz) / up;
    const float yy = (u2 * u3 * vx + u1 * vy + u2 * up * vz) / up;
    const float z = (u3 * u3 * vx - vx + u3 * up * vz) / up;
    vx = x;
    vy = yy;
    vz = z;
  } else if (u3 < 0.f) {
    vx = -vx;
    vz = -vz;
  }
}

// Vector meson (src/UpcGenerator.cpp:761-764, 425-472; getMomentumVM,
// src/UpcCrossSection.cpp:1076-1104): the emitter picked with the reference's
// test Uniform(0,1) < ratio[yBin] (a ratio of the two emitters' dsigma/dy, not
// a fraction), the photon pT from its spectrum, the pomeron pT by inverting
// the F^2 table between tmin and the end, cuts on the meson, then the decay
// angle theta with density min(sin theta (1 + c cos^2 theta), 1) on [0, pi]
// (the reference's rejection test against a unit envelope).  Philox blocks:
// 1 (azimuths), 2 (photon pT), 3 (decay azimuth, charges), 4 (emitter,
// pomeron), 5.. (decay-angle tries, two per block).
__device__ bool gen_vm(const EventParams& e, const float* __restrict__ pttab, Cand& c,
                       uint32_t clo, uint32_t chi, uint2 key, uint4 r1, uint4 r2) {
  const double yedge_hi = e.ymin + e.dy * e.ny;
  int yb = (int)((double)(int)(e.ny * (c.y - e.ymin)) / (yedge_hi - e.ymin));
  yb = yb < 0 ? 0 : (yb > e.ny - 1 ? e.ny - 1 : yb);
  const uint4 r4 = philox4x32_10(make_uint4(clo, chi, 4u, 0x55504347u), key);
  const bool target = u53(r4.x, r4.y) < __ldg(e.vm_ratio + yb);
  const double sgn = target ? 1. : -1.;
  const float m = (float)c.m, y = c.y;
  const float ptPhot = photon_pt(e, pttab, logf(0.5f * m) + (float)sgn * y, u24(r2.x), u24(r2.y));
  // pomeron: t = tmin + ptPom^2 with density F(t)^2 on [tmin, end of table]
  const double ePom = c.m / 2. * exp(-sgn * c.y);
  const double tmin = (ePom * ePom) / (e.vm_g1 * e.vm_g1);
  const double dq = kPomQmax / kPomN;
  const double* __restrict__ G = e.pom_cdf;
  int jm = (int)(sqrt(tmin) / dq);
  jm = jm > kPomN - 1 ? kPomN - 1 : jm;
  double ta = (jm * dq) * (jm * dq), tb = ((jm + 1) * dq) * ((jm + 1) * dq);
  const double g0 = __ldg(G + jm), g1 = __ldg(G + jm + 1);
  double gmin = g0 + (g1 - g0) * (tmin - ta) / (tb - ta);
  gmin = gmin < 0. ? 0. : (gmin > 1. ? 1. : gmin);
  const double u = gmin + u53(r4.z, r4.w) * (1. - gmin);
  int lo = jm, hi = kPomN;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (u >= __ldg(G + mid)) lo = mid; else hi = mid;
  }
  const double c0 = __ldg(G + lo), c1 = __ldg(G + lo + 1);
  ta = (lo * dq) * (lo * dq);
  tb = ((lo + 1) * dq) * ((lo + 1) * dq);
  double t = c1 > c0 ? ta + (u - c0) / (c1 - c0) * (tb - ta) : ta;
  t = t < tmin ? tmin : t;
  const float ptPom = (float)sqrt(t - tmin);
  float s1, c1f, s2, c2f;
  sincosf(kTwoPiF * u24(r1.z), &s1, &c1f);
  sincosf(kTwoPiF * u24(r1.w), &s2, &c2f);
  const float ppx = ptPhot * c1f + ptPom * c2f;
  const float ppy = ptPhot * s1 + ptPom * s2;
  const float mt = sqrtf(m * m + ppx * ppx + ppy * ppy);
  const float ppz = mt * sinhf(y), pE = mt * coshf(y);
  // checkKinCuts on the meson (the decay follows the cuts)
  if (e.doPtCut && sqrtf(ppx * ppx + ppy * ppy) < e.f_minPt) return false;
  if (e.doEtaCut) {
    const float et = eta_f(ppx, ppy, ppz);
    if (et < e.f_minEta || et > e.f_maxEta) return false;
  }
  // twoPartDecayVM's angle: at most 32 tries (acceptance above 0.8 per try)
  const float cc = e.dght_law ? 0.605f : 1.f;
  float theta = 0.25f * kTwoPiF;
  bool ok = false;
  for (int blk = 0; blk < 16 && !ok; ++blk) {
    const uint4 rr = philox4x32_10(make_uint4(clo, chi, 5u + (uint32_t)blk, 0x55504347u), key);
    for (int tr = 0; tr < 2 && !ok; ++tr) {
      const float th = 0.5f * kTwoPiF * u24(tr ? rr.z : rr.x);
      const float test = u24(tr ? rr.w : rr.y);
      float sth, cth;
      sincosf(th, &sth, &cth);
      if (test < sth * (1.f + cc * cth * cth)) {
        theta = th;
        ok = true;
      }
    }
  }
  if (!ok) atomicAdd(e.vm_err, 1u);
  const uint4 r3 = philox4x32_10(make_uint4(clo, chi, 3u, 0x55504347u), key);
  c.sign = (r3.y & 1u) ? 1.f : -1.f;
  const float md = e.mDght;
  const float pmag = sqrtf(fmaxf(m * m * 0.25f - md * md, 0.f));
  float sp, cp, sth, cth;
  sincosf(kTwoPiF * u24(r3.x), &sp, &cp);
  sincosf(theta, &sth, &cth);
  float vx = pmag * sth * cp, vy = pmag * sth * sp, vz = pmag * cth;
  rotate_uz_f(vx, vy, vz, ppx, ppy, ppz);
  const float ev = sqrtf(pmag * pmag + md * md);
  boost_by(-vx, -vy, -vz, ev, ppx, ppy, ppz, pE, m, c.p0);
  boost_by(vx, vy, vz, ev, ppx, ppy, ppz, pE, m, c.p1);
  return true;
}

// getBinY of the (y, m) sampler (include/UpcSampler.h:130-133) for the mass:
// int(nBinsY (m - lo)) / (hi - lo), the int() truncating the numerator, then
// the return's truncation.  The quotient comes from a table made on the host
// with that FP64 division for every integer numerator (no FP64 division per
// candidate); clamped to the mass bins.
__device__ __forceinline__ int sampler_mbin(const EventParams& e, double m) {
  const int nnum = (int)(e.nm_d * (m - e.mmin));
  const int mb = (nnum >= 0 && nnum < e.mbin_lut_n) ? __ldg(e.mbin_lut + nnum)
                                                    : (int)((double)nnum / (e.medge_hi - e.mmin));
  return mb < 0 ? 0 : (mb > e.nm - 1 ? e.nm - 1 : mb);
}

// getBinX of the (y, m) sampler for the rapidity (include/UpcSampler.h:124-128),
// clamped to the rapidity bins
__device__ __forceinline__ int sampler_ybin(const EventParams& e, double y) {
  const double yedge_hi = e.ymin + e.dy * e.ny;
  const int yb = (int)((double)(int)(e.ny * (y - e.ymin)) / (yedge_hi - e.ymin));
  return yb < 0 ? 0 : (yb > e.ny - 1 ? e.ny - 1 : yb);
}

__device__ bool gen_candidate(const EventParams& e, const double* __restrict__ cdf2,
                              const double* __restrict__ cdfz, const float* __restrict__ pttab,
                              uint64_t idx, Cand& c) {
  const uint2 key = make_uint2((uint32_t)e.seed, (uint32_t)(e.seed >> 32));
  const uint32_t clo = (uint32_t)idx, chi = (uint32_t)(idx >> 32);
  const uint4 r0 = philox4x32_10(make_uint4(clo, chi, 0u, 0x55504347u), key);
  const uint4 r1 = philox4x32_10(make_uint4(clo, chi, 1u, 0x55504347u), key);
  const uint4 r2 = philox4x32_10(make_uint4(clo, chi, 2u, 0x55504347u), key);
  // (y, m): gsl_histogram2d_pdf_sample with r1 for the bin and y, r2 for m
  const int n2 = e.ny * e.nm;
  const uint64_t ra = ((uint64_t)r0.x << 32) | r0.y;
  const double rb = u53(r0.z, r0.w);
  const int k = cdf_find_from_fx(e.cdf2fx, n2, __ldg(e.g2 + (int)(ra >> (64 - e.g2_bits))), ra);
  const int iy = k / e.nm, im = k - iy * e.nm;
  // the position inside the bin, (r - c0) / (c1 - c0), in FP32 (the event
  // stores y in FP32); m in FP64, for getBinY
  const float delta = frac_fx(ra - __ldg(e.cdf2fx + k), __ldg(e.cdf2fx + k + 1) - __ldg(e.cdf2fx + k));
  c.y = fmaf((float)iy + delta, e.f_dy, e.f_ymin);
  double mlo, mw;  // the mass bin's lower edge and width
  if (e.medges) {
    const double2 me = __ldg(e.medges + im);
    mlo = me.x;
    mw = me.y;
  } else {
    mlo = e.mmin + e.dm * im;
    mw = (e.mmin + e.dm * (im + 1)) - mlo;
  }
  c.m = mlo + rb * mw;
  (void)cdf2;
  const int mb = sampler_mbin(e, c.m);
  c.mbin = mb;
  // z = cos(theta)
  if (!e.ignoreCSZ && !e.polarized) {
    const uint64_t rz = ((uint64_t)r1.x << 32) | r1.y;
    const uint64_t* cz = e.cdfzfx + (size_t)mb * (e.nz + 1);
    const int iz = cdf_find_from_fx(
        cz, e.nz, __ldg(e.gz + (size_t)mb * e.gz_n + (int)(rz >> (64 - e.gz_bits))), rz);
    const float dl = frac_fx(rz - __ldg(cz + iz), __ldg(cz + iz + 1) - __ldg(cz + iz));
    c.z = fmaf(e.f_dz, (float)iz + dl, e.f_zmin);
  } else if (!e.ignoreCSZ) {
    // polarized: the scalar or pseudoscalar z sampler of this mass bin; the
    // reference draws Uniform(0, 1) < polCSRatio[yBin][mBin] (getBinX of y, as getBinY)
    const double rz = u53(r1.x, r1.y);
    const double* cz = cdfz + (size_t)mb * (e.nz + 1);
    const int yb = sampler_ybin(e, (double)c.y);
    const uint4 r4 = philox4x32_10(make_uint4(clo, chi, 4u, 0x55504347u), key);
    if (!(u53(r4.x, r4.y) < __ldg(e.ratio + (size_t)yb * e.nm + mb)))
      cz = e.cdfz_ps + (size_t)mb * (e.nz + 1);
    const int iz = cdf_find(cz, e.nz, rz);
    const double z0 = __ldg(cz + iz), z1 = __ldg(cz + iz + 1);
    const float dl = frac_in_bin(rz - z0, z1 - z0);
    c.z = fmaf(e.f_dz, (float)iz + dl, e.f_zmin);
  } else {
    c.z = -1.f + 2.f * u24(r1.x);
  }
  if (e.vm) return gen_vm(e, pttab, c, clo, chi, key, r1, r2);
  // pair momentum (getPairMomentum)
  const float m = (float)c.m, y = c.y;
  float ppx = 0.f, ppy = 0.f, mt = m;
  if (e.useNonzeroGamPt) {
    // ln k1,2 = ln(m/2) +- y
    const float lnm2 = logf(0.5f * m);
    const float a1 = kTwoPiF * u24(r1.z), a2 = kTwoPiF * u24(r1.w);
    const float pt1 = photon_pt(e, pttab, lnm2 + y, u24(r2.x), u24(r2.y));
    const float pt2 = photon_pt(e, pttab, lnm2 - y, u24(r2.z), u24(r2.w));
    float s1, c1f, s2, c2f;
    sincosf(a1, &s1, &c1f);
    sincosf(a2, &s2, &c2f);
    ppx = pt1 * c1f + pt2 * c2f;
    ppy = pt1 * s1 + pt2 * s2;
    mt = sqrtf(m * m + ppx * ppx + ppy * ppy);
  }
  const float ppz = mt * sinhf(y), pE = mt * coshf(y);
  const uint4 r3 = philox4x32_10(make_uint4(clo, chi, 3u, 0x55504347u), key);
  if (e.procID != 51) {
    // pairProduction: back-to-back leptons, |p| = sqrt(M^2/4 - m_l^2), boosted
    const float pmag = sqrtf(fmaxf(m * m * 0.25f - e.mPart * e.mPart, 0.f));
    const float cz = c.z;
    const float sz = sqrtf(fmaxf(1.f - cz * cz, 0.f));
    float sp, cp;
    sincosf(kTwoPiF * u24(r3.x), &sp, &cp);
    const float vx = pmag * sz * cp, vy = pmag * sz * sp, vz = pmag * cz;
    const float ev = sqrtf(pmag * pmag + e.mPart * e.mPart);
    boost_by(vx, vy, vz, ev, ppx, ppy, ppz, pE, m, c.p0);
    boost_by(-vx, -vy, -vz, ev, ppx, ppy, ppz, pE, m, c.p1);
    c.sign = (r3.y & 1u) ? 1.f : -1.f;
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const float* pp = q ? c.p1 : c.p0;
      if (e.doPtCut && sqrtf(pp[0] * pp[0] + pp[1] * pp[1]) < e.f_minPt) return false;
      if (e.doEtaCut) {
        const float et = eta_f(pp[0], pp[1], pp[2]);
        if (et < e.f_minEta || et > e.f_maxEta) return false;
      }
    }
    return true;
  }
  // ALP: cuts on the ALP, then the isotropic two-photon decay
  if (e.doPtCut && sqrtf(ppx * ppx + ppy * ppy) < e.f_minPt) return false;
  if (e.doEtaCut) {
    const float et = eta_f(ppx, ppy, ppz);
    if (et < e.f_minEta || et > e.f_maxEta) return false;
  }
  const float eph = 0.5f * m;
  float sp, cp;
  sincosf(kTwoPiF * u24(r3.x), &sp, &cp);
  const float ct = -1.f + 2.f * u24(r3.z);
  const float st = sqrtf(fmaxf(1.f - ct * ct, 0.f));
  float vx = eph * st * cp, vy = eph * st * sp, vz = eph * ct;
  // RotateUz onto the ALP direction (a rotation of an isotropic decay)
  rotate_uz_f(vx, vy, vz, ppx, ppy, ppz);
  boost_by(-vx, -vy, -vz, eph, ppx, ppy, ppz, pE, m, c.p0);
  boost_by(vx, vy, vz, eph, ppx, ppy, ppz, pE, m, c.p1);
  c.sign = 1.f;
  return true;
}

constexpr int kTile = 256;

__device__ __forceinline__ EventRecord to_record(const Cand& c) {
  EventRecord rec;
  rec.m = (float)c.m;
  rec.y = c.y;
  rec.z = c.z;
  rec.sign = c.sign;
  for (int q = 0; q < 4; ++q) {
    rec.p0[q] = c.p0[q];
    rec.p1[q] = c.p1[q];
  }
  return rec;
}

// Pass 1, persistent: warp-tile wt (32 candidates; wt = 8 t + w is warp w
// of the 256-candidate tile t) -> its accept word mask[wt]; with stage, its
// accepted records to stage[32 wt + rank] in candidate order.  Every warp
// runs its warp-tiles on its own (no block barrier), so warps that draw cheap
// candidates never wait for the slow ones of their block.
__global__ void __launch_bounds__(kTile, 4) k_events_flags(EventParams e, const double* __restrict__ cdf2,
                                                        const double* __restrict__ cdfz,
                                                        const float* __restrict__ pttab,
                                                        uint64_t cand0, int64_t ncand, int64_t nwt,
                                                        uint32_t* __restrict__ mask,
                                                        EventRecord* __restrict__ stage,
                                                        int32_t* __restrict__ stage_mbin) {
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = (int64_t)gridDim.x * (kTile / 32);
  for (int64_t wt = (int64_t)blockIdx.x * (kTile / 32) + (threadIdx.x >> 5); wt < nwt; wt += nwarps) {
    const int64_t local = wt * 32 + lane;
    bool ok = false;
    Cand c;
    if (local < ncand) ok = gen_candidate(e, cdf2, cdfz, pttab, cand0 + (uint64_t)local, c);
    const unsigned bal = __ballot_sync(0xffffffffu, ok);
    if (lane == 0) mask[wt] = bal;
    if (stage && ok) {
      const size_t slot = (size_t)wt * 32 + __popc(bal & ((1u << lane) - 1u));
      stage[slot] = to_record(c);
      if (stage_mbin) stage_mbin[slot] = c.mbin;
    }
  }
}

// Pass 2 from the staging slots: tile t's accepted records to out_base +
// tile_off[t] + r (below nmax), r counted over the tile's 8 warp-tiles in
// order; one thread per record (3 float4 when out is 16-byte aligned).
__global__ void k_events_copy(const EventRecord* __restrict__ stage,
                              const int32_t* __restrict__ stage_mbin,
                              const uint32_t* __restrict__ mask,
                              const int64_t* __restrict__ tile_off, int64_t out_base,
                              int64_t nmax, EventRecord* __restrict__ out,
                              int32_t* __restrict__ mbin) {
  const int64_t tile = blockIdx.x;
  const int64_t base = out_base + tile_off[tile];
  if (base >= nmax) return;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int before = 0;
  for (int q = 0; q < w; ++q) before += __popc(__ldg(mask + tile * (kTile / 32) + q));
  const int cnt = __popc(__ldg(mask + tile * (kTile / 32) + w));
  if (lane >= cnt) return;
  const int64_t slot = base + before + lane;
  if (slot >= nmax) return;
  const size_t src = (size_t)(tile * (kTile / 32) + w) * 32 + lane;
  if ((reinterpret_cast<uintptr_t>(out) & 15) == 0) {  // 48-byte records: 3 float4 each
    const float4* a = reinterpret_cast<const float4*>(stage + src);
    float4* b = reinterpret_cast<float4*>(out + slot);
    b[0] = __ldg(a);
    b[1] = __ldg(a + 1);
    b[2] = __ldg(a + 2);
  } else {
    out[slot] = stage[src];
  }
  if (mbin) mbin[slot] = __ldg(stage_mbin + src);
}

__global__ void __launch_bounds__(kTile, 5) k_events_write(EventParams e, const double* __restrict__ cdf2,
                                                        const double* __restrict__ cdfz,
                                                        const float* __restrict__ pttab,
                                                        uint64_t cand0, int64_t ncand,
                                                        const uint32_t* __restrict__ mask,
                                                        const int64_t* __restrict__ tile_off,
                                                        int64_t out_base, int64_t nmax,
                                                        EventRecord* __restrict__ out,
                                                        int32_t* __restrict__ mbin) {
  __shared__ uint32_t sm[kTile / 32];
  __shared__ int pre[kTile / 32 + 1];
  const int tile = blockIdx.x;
  const int64_t base = tile_off ? tile_off[tile] : (int64_t)tile * kTile;
  if (out_base + base >= nmax) return;
  if (threadIdx.x < kTile / 32)
    sm[threadIdx.x] = mask ? mask[(size_t)tile * (kTile / 32) + threadIdx.x] : 0xffffffffu;
  __syncthreads();
  if (threadIdx.x == 0) {
    pre[0] = 0;
    for (int w = 0; w < kTile / 32; ++w) pre[w + 1] = pre[w] + __popc(sm[w]);
  }
  __syncthreads();
  const int total = pre[kTile / 32];
  const int r = threadIdx.x;  // r-th accepted candidate of the tile
  if (r >= total) return;
  int w = 0;
  while (pre[w + 1] <= r) ++w;
  int rem = r - pre[w];
  uint32_t bits = sm[w];
  int lane = 0;
  for (;;) {
    const int b = __ffs(bits) - 1;
    if (rem == 0) { lane = b; break; }
    bits &= bits - 1;
    --rem;
  }
  const int64_t local = (int64_t)tile * kTile + w * 32 + lane;
  if (local >= ncand) return;
  const int64_t slot = out_base + base + r;
  if (slot >= nmax) return;
  Cand c;
  gen_candidate(e, cdf2, cdfz, pttab, cand0 + (uint64_t)local, c);
  out[slot] = to_record(c);
  if (mbin) mbin[slot] = c.mbin;
}

// Exclusive scan of the tile counts (one CTA; tiles per chunk <= 2^20) and the
// total, the counts given or taken from the accept words: 8192 counts per round, loaded coalesced into shared memory; each
// thread sums 8 consecutive ones, a warp-shuffle scan and a scan of the 32
// warp totals give the thread's offset, and a carry runs across rounds.
constexpr int kScanThreads = 1024, kScanPer = 8;

__global__ void __launch_bounds__(kScanThreads) k_scan_tiles(const int* __restrict__ cnt,
                                                            const uint32_t* __restrict__ mask,
                                                            int64_t* __restrict__ off, int n,
                                                            int64_t* __restrict__ total) {
  __shared__ int s_cnt[kScanThreads * kScanPer];
  __shared__ int64_t s_warp[kScanThreads / 32];
  __shared__ int64_t s_carry;
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  if (t == 0) s_carry = 0;
  for (int base = 0; base < n; base += kScanThreads * kScanPer) {
    if (mask) {  // a tile's count: the set bits of its 8 accept words (32 bytes)
      for (int j = t; j < kScanThreads * kScanPer; j += kScanThreads) {
        int v = 0;
        if (base + j < n) {
          const uint4* m4 = reinterpret_cast<const uint4*>(mask + (size_t)(base + j) * 8);
          const uint4 a = __ldg(m4), b = __ldg(m4 + 1);
          v = __popc(a.x) + __popc(a.y) + __popc(a.z) + __popc(a.w) + __popc(b.x) + __popc(b.y) +
              __popc(b.z) + __popc(b.w);
        }
        s_cnt[j] = v;
      }
    } else {
      for (int j = t; j < kScanThreads * kScanPer; j += kScanThreads)
        s_cnt[j] = base + j < n ? __ldg(cnt + base + j) : 0;
    }
    __syncthreads();
    int64_t mine = 0;
#pragma unroll
    for (int i = 0; i < kScanPer; ++i) mine += s_cnt[t * kScanPer + i];
    int64_t inc = mine;  // inclusive scan within the warp
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int64_t v = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += v;
    }
    if (lane == 31) s_warp[w] = inc;
    __syncthreads();
    if (w == 0) {  // scan of the warp totals
      int64_t x = s_warp[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int64_t v = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += v;
      }
      s_warp[lane] = x;  // inclusive
    }
    __syncthreads();
    int64_t run = s_carry + (w > 0 ? s_warp[w - 1] : 0) + inc - mine;
#pragma unroll
    for (int i = 0; i < kScanPer; ++i) {
      const int j = base + t * kScanPer + i;
      if (j < n) off[j] = run;
      run += s_cnt[t * kScanPer + i];
    }
    __syncthreads();
    if (t == 0) s_carry += s_warp[31];
    __syncthreads();
  }
  if (t == 0) *total = s_carry;
}

// Photon pT spectra: dN/dpT ~ F(pT^2 + e)^2 pT^3 / (pT^2 + e)^2 on 5000 bins of
// [0, 6 hc / R] (content at the upper bin edge), for e = k^2/gtot^2 on a log
// grid.  FP32 throughout (the tables are FP32), from an FP32 copy of the
// form-factor spline.
__global__ void k_pt_tables(EventParams e, SplineF ff, float* __restrict__ out,
                            uint16_t* __restrict__ guide) {
  extern __shared__ float sdf[];
  const int ie = blockIdx.x;
  const float ered = expf((float)e.pt_lne0 + (float)e.pt_dlne * ie);
  const int nb = e.pt_nbins;
  const float inv_pi2x4 = (float)(1. / (4 * kPi * kPi));
  const float w = (float)e.pt_width;
#pragma unroll 4
  for (int b = threadIdx.x; b < nb; b += blockDim.x) {  // independent bins: loads overlap
    const float pt = w * (b + 1);
    const float arg = pt * pt + ered;
    const float f = spline_eval_f(ff, ff.coef, arg);
    sdf[b] = (f * f) * pt * pt * pt * inv_pi2x4 / (arg * arg);
  }
  __syncthreads();
  {  // cumulative sum: contiguous runs per thread, block scan of the run sums
    __shared__ float sw[32];
    const int t = threadIdx.x, nt = blockDim.x, lane = t & 31, wid = t >> 5;
    const int per = (nb + nt - 1) / nt;
    const int lo = t * per, hi = lo + per < nb ? lo + per : nb;
    float run = 0.f;
    for (int b = lo; b < hi; ++b) run += sdf[b];
    float incl = run;  // inclusive scan of the run sums: warps, then warp totals
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const float y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    if (lane == 31) sw[wid] = incl;
    __syncthreads();
    if (wid == 0) {
      float v = lane < nt / 32 ? sw[lane] : 0.f;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const float y = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += y;
      }
      sw[lane] = v;
    }
    __syncthreads();
    float acc = (wid > 0 ? sw[wid - 1] : 0.f) + incl - run;
    for (int b = lo; b < hi; ++b) {
      acc += sdf[b];
      sdf[b] = acc;
    }
  }
  __syncthreads();
  const float inv_tot = 1.f / sdf[nb - 1];
  float* o = out + (size_t)ie * (nb + 1);
  if (threadIdx.x == 0) o[0] = 0.f;
  __syncthreads();  // every thread has read sdf[nb - 1]
  for (int b = threadIdx.x; b < nb; b += blockDim.x) {
    const float c = sdf[b] * inv_tot;
    o[b + 1] = c;
    sdf[b] = c;
  }
  if (!guide) return;
  // the row's guide table: entry j = the bin of u = j / K in the CDF
  // {0, sdf[0], ..., sdf[len - 2]} (cdf_find_f's answer: the largest k < len
  // with cdf[k] <= u, or 0), from shared memory.  Each thread takes a run of
  // consecutive points: a binary search for the first, then a forward walk
  // of at most 8 bins per point, finished by a binary search above the
  // walk's bin where the CDF is flat (its tail); the CDF is nondecreasing
  // (a running sum of non-negative terms), so each step keeps the answer.
  __syncthreads();
  const int K = e.gpt_n, len = nb;
  auto cdf_at = [&](int k) { return k == 0 ? 0.f : sdf[k - 1]; };
  uint16_t* g = guide + (size_t)ie * K;
  const int per = (K + blockDim.x - 1) / blockDim.x;
  const int j0 = threadIdx.x * per, j1 = min(K, j0 + per);
  int lo = 0;
  for (int j = j0; j < j1; ++j) {
    const float u = (float)j / (float)K;
    int steps = 0;
    while (steps < 8 && lo + 1 < len && u >= cdf_at(lo + 1)) {
      ++lo;
      ++steps;
    }
    if (lo + 1 < len && u >= cdf_at(lo + 1)) {  // cdf[lo] <= u still holds
      int hi = len;
      while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (u >= cdf_at(mid)) lo = mid; else hi = mid;
      }
    }
    g[j] = (uint16_t)lo;
  }
}

// Guide tables: bucket j of K starts at the answer of the plain search for
// r = j / K (exact in floating point for K a power of two).
__global__ void k_guide_rows_d(const double* __restrict__ cdf, int rows, int len, int K,
                               int* __restrict__ guide) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)rows * K) return;
  const int r = (int)(t / K), j = (int)(t - (int64_t)r * K);
  guide[t] = cdf_find(cdf + (size_t)r * (len + 1), len, (double)j / (double)K);
}

// fixed-point copy of a CDF (see cdf_find_from_fx)
__global__ void k_cdf_fixed(const double* __restrict__ cdf, int64_t n, uint64_t* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = cdf_to_fx(cdf[i]);
}

// guide[r][j]: the bin of r_j = j 2^(64 - bits) in fixed-point CDF row r
__global__ void k_guide_rows_fx(const uint64_t* __restrict__ cdf, int rows, int len, int bits,
                                int* __restrict__ guide) {
  const int64_t K = (int64_t)1 << bits;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)rows * K) return;
  const int r = (int)(t >> bits);
  const uint64_t j = (uint64_t)(t - ((int64_t)r << bits));
  guide[t] = cdf_find_fx(cdf + (size_t)r * (len + 1), len, j << (64 - bits));
}

// Every candidate of [cand0, cand0 + n) with its accept flag (single-event API).
__global__ void k_events_all(EventParams e, const double* __restrict__ cdf2,
                             const double* __restrict__ cdfz, const float* __restrict__ pttab,
                             uint64_t cand0, int64_t n, EventRecord* __restrict__ out,
                             uint8_t* __restrict__ flag) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  Cand c;
  const bool ok = gen_candidate(e, cdf2, cdfz, pttab, cand0 + (uint64_t)i, c);
  EventRecord rec;
  rec.m = (float)c.m;
  rec.y = c.y;
  rec.z = c.z;
  rec.sign = c.sign;
  for (int q = 0; q < 4; ++q) { rec.p0[q] = c.p0[q]; rec.p1[q] = c.p1[q]; }
  out[i] = rec;
  flag[i] = ok ? 1 : 0;
}

__global__ void k_philox_dump(uint64_t seed, uint64_t c0, int64_t n, uint32_t* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint64_t c = c0 + (uint64_t)i;
  const uint4 r = philox4x32_10(make_uint4((uint32_t)c, (uint32_t)(c >> 32), 0u, 0u),
                                make_uint2((uint32_t)seed, (uint32_t)(seed >> 32)));
  out[4 * i + 0] = r.x;
  out[4 * i + 1] = r.y;
  out[4 * i + 2] = r.z;
  out[4 * i + 3] = r.w;
}

}  // namespace

cudaError_t launch_events_all(const EventParams& e, const double* d_cdf2, const double* d_cdfz,
                              const float* d_ptcdf, uint64_t cand0, int64_t n, EventRecord* d_out,
                              uint8_t* d_flag, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  note_launch();
  k_events_all<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(e, d_cdf2, d_cdfz, d_ptcdf, cand0, n,
                                                           d_out, d_flag);
  return cudaGetLastError();
}

cudaError_t launch_philox_dump(uint64_t seed, uint64_t c0, int64_t n, uint32_t* d_out,
                               cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  note_launch();
  k_philox_dump<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(seed, c0, n, d_out);
  return cudaGetLastError();
}

cudaError_t launch_guide2_fx(const EventParams& e, const uint64_t* d_cdf2fx, int* d_g2,
                             cudaStream_t st) {
  if (e.g2_n != (1 << e.g2_bits)) return cudaErrorInvalidValue;
  note_launch();
  k_guide_rows_fx<<<(e.g2_n + 255) / 256, 256, 0, st>>>(d_cdf2fx, 1, e.nm * e.ny, e.g2_bits, d_g2);
  return cudaGetLastError();
}

cudaError_t launch_guides(const EventParams& e, const double* d_cdf2, const double* d_cdfz,
                          int* d_g2, int* d_gz, cudaStream_t st, uint64_t* d_cdf2fx,
                          uint64_t* d_cdfzfx) {
  if (e.g2_n != (1 << e.g2_bits) || e.gz_n != (1 << e.gz_bits)) return cudaErrorInvalidValue;
  // each guide set is built when its buffer is given (null: skipped), with
  // the fixed-point copy of its CDF
  const int n2 = e.nm * e.ny;
  if (d_g2) {
    if (!d_cdf2fx) return cudaErrorInvalidValue;
    note_launch();
    k_cdf_fixed<<<(unsigned)((n2 + 1 + 255) / 256), 256, 0, st>>>(d_cdf2, n2 + 1, d_cdf2fx);
    note_launch();
    k_guide_rows_fx<<<(e.g2_n + 255) / 256, 256, 0, st>>>(d_cdf2fx, 1, n2, e.g2_bits, d_g2);
  }
  if (d_gz && !e.ignoreCSZ && !e.polarized) {  // polarized z: plain searches on two CDF sets
    if (!d_cdfzfx) return cudaErrorInvalidValue;
    const int64_t nzc = (int64_t)e.nm * (e.nz + 1);
    note_launch();
    carveout_max_shared<k_cdf_fixed>();
    k_cdf_fixed<<<(unsigned)((nzc + 255) / 256), 256, 0, st>>>(d_cdfz, nzc, d_cdfzfx);
    const int64_t nz = (int64_t)e.nm * e.gz_n;
    note_launch();
    carveout_max_shared<k_guide_rows_fx>();
    k_guide_rows_fx<<<(unsigned)((nz + 255) / 256), 256, 0, st>>>(d_cdfzfx, e.nm, e.nz, e.gz_bits,
                                                                  d_gz);
  }
  return cudaGetLastError();
}

cudaError_t launch_photon_pt_tables(const EventParams& e, const SplineU& ff, float4* d_ff32,
                                    float* d_cdf, cudaStream_t st, uint16_t* d_gpt) {
  const size_t smem = sizeof(float) * e.pt_nbins;
  if (smem > 48 * 1024) return cudaErrorInvalidValue;
  if (d_gpt && e.pt_nbins > 65535) return cudaErrorInvalidValue;
  note_launch();
  carveout_max_shared<k_coef_f32>();
  k_coef_f32<<<(ff.n - 1 + 255) / 256, 256, 0, st>>>(ff.coef, d_ff32, ff.n - 1);
  const SplineF f32{d_ff32, (float)ff.x0, (float)ff.h, (float)ff.inv_h, ff.n};
  note_launch();
  carveout_max_shared<k_pt_tables>();
  k_pt_tables<<<e.pt_ne, 256, smem, st>>>(e, f32, d_cdf, d_gpt);
  return cudaGetLastError();
}

cudaError_t launch_events_flags(const EventParams& e, const double* d_cdf2, const double* d_cdfz,
                                const float* d_ptcdf, uint64_t cand0, int64_t ncand,
                                uint32_t* d_mask, cudaStream_t st, EventRecord* d_stage,
                                int32_t* d_stage_mbin) {
  // one resident wave: SMs x the blocks of k_events_flags an SM holds
  static std::atomic<int> waves[64] = {};  // per device id, 0 until measured
  int dev = 0;
  cudaError_t err = cudaGetDevice(&dev);
  if (err != cudaSuccess) return err;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  int wave = waves[dev].load(std::memory_order_relaxed);
  if (!wave) {
    int sms = 0, per = 0;
    err = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (err != cudaSuccess) return err;
    err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_events_flags, kTile, 0);
    if (err != cudaSuccess) return err;
    wave = std::max(1, sms * std::max(1, per));
    waves[dev].store(wave, std::memory_order_relaxed);
  }
  const int64_t tiles = (ncand + kTile - 1) / kTile;
  const int64_t nwt = tiles * (kTile / 32);
  const int64_t grid = std::min<int64_t>(tiles, wave);
  if (grid <= 0) return cudaSuccess;
  note_launch();
  k_events_flags<<<(unsigned)grid, kTile, 0, st>>>(e, d_cdf2, d_cdfz, d_ptcdf, cand0, ncand, nwt,
                                                  d_mask, d_stage, d_stage_mbin);
  return cudaGetLastError();
}

cudaError_t launch_events_copy(const EventRecord* d_stage, const int32_t* d_stage_mbin,
                               const uint32_t* d_mask, const int64_t* d_tile_off, int64_t tiles,
                               int64_t out_base, int64_t nmax, EventRecord* d_out, int32_t* d_mbin,
                               cudaStream_t st) {
  if (tiles <= 0) return cudaSuccess;
  note_launch();
  k_events_copy<<<(unsigned)tiles, kTile, 0, st>>>(d_stage, d_stage_mbin, d_mask, d_tile_off,
                                                   out_base, nmax, d_out, d_mbin);
  return cudaGetLastError();
}

cudaError_t launch_events_write(const EventParams& e, const double* d_cdf2, const double* d_cdfz,
                                const float* d_ptcdf, uint64_t cand0, int64_t ncand,
                                const uint32_t* d_mask, const int64_t* d_tile_off,
                                int64_t out_base, int64_t nmax, EventRecord* d_out,
                                int32_t* d_mbin, cudaStream_t st) {
  const int64_t tiles = (ncand + kTile - 1) / kTile;
  note_launch();
  k_events_write<<<(unsigned)tiles, kTile, 0, st>>>(e, d_cdf2, d_cdfz, d_ptcdf, cand0, ncand,
                                                   d_mask, d_tile_off, out_base, nmax, d_out,
                                                   d_mbin);
  return cudaGetLastError();
}

cudaError_t launch_scan_tiles(const int* d_count, const uint32_t* d_mask, int64_t* d_off, int n,
                              int64_t* d_total, cudaStream_t st) {
  note_launch();
  k_scan_tiles<<<1, kScanThreads, 0, st>>>(d_count, d_mask, d_off, n, d_total);
  return cudaGetLastError();
}

// The event kernels' bin functions on given values (axis 0: sampler_mbin of
// m, axis 1: sampler_ybin of y), for bit-exact checks against getBinY/getBinX.
namespace {
__global__ void k_sampler_bins(EventParams e, const double* __restrict__ x, int n, int axis,
                               int* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = axis == 0 ? sampler_mbin(e, x[i]) : sampler_ybin(e, x[i]);
}
}  // namespace

cudaError_t launch_sampler_bins(const EventParams& e, const double* d_x, int n, int axis,
                                int* d_out, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  note_launch();
  k_sampler_bins<<<(n + 255) / 256, 256, 0, st>>>(e, d_x, n, axis, d_out);
  return cudaGetLastError();
}

}  // namespace upcg
