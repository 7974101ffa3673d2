// CPU oracle -- samplers and event loop (TEST INFRASTRUCTURE ONLY).
//
// Restates include/UpcSampler.h:37-142 (GSL histogram PDFs),
// src/UpcGenerator.cpp:715-889 (generateEvent / generateEvents),
// src/UpcCrossSection.cpp:1021-1074 (getPhotonPt / getPairMomentum) and the
// ROOT vector algebra they use (TLorentzVector boosts, TVector3::RotateUz).
// The random streams follow the reference's engines: GSL's mt19937
// (std::mt19937, same initialisation; gsl_rng_uniform = x / 2^32) for the
// samplers -- one engine per sampler, all seeded with SEED as in
// src/UpcGenerator.cpp:688-700 -- and ROOT's TRandomMT64 (std::mt19937_64,
// x / 2^64) for gRandom.  The two uniforms of the 2-D sampler are drawn in
// argument order (r1 first); the reference leaves that order to the compiler.
#include <cmath>
#include <cstdint>
#include <random>
#include <unordered_map>
#include <vector>

#include "oracle_ctx.hpp"
#include "upcg_oracle.h"

namespace uo {

namespace {

struct GslUniform {  // gsl_rng_default (mt19937) + gsl_rng_uniform
  std::mt19937 e;
  explicit GslUniform(unsigned long s) : e((uint32_t)(s == 0 ? 4357 : s)) {}
  double operator()() { return e() / 4294967296.0; }
};

struct RootMT64 {  // TRandomMT64::Rndm / Uniform
  std::mt19937_64 e;
  explicit RootMT64(uint64_t s) : e(s) {}
  double rndm() {
    for (;;) {
      uint64_t x = e();
      if (x != 0) return x * (1.0 / 18446744073709551616.0);
    }
  }
  double uniform(double lo, double hi) { return lo + (hi - lo) * rndm(); }
};

// gsl_histogram_pdf_init: running mean, then cumulative (bin/mean)/n.
std::vector<double> gsl_cdf(const double* bins, size_t n) {
  std::vector<double> sum(n + 1);
  double mean = 0;
  for (size_t i = 0; i < n; i++) mean += (bins[i] - mean) / ((double)(i + 1));
  double s = 0;
  sum[0] = 0;
  for (size_t i = 0; i < n; i++) {
    s += (bins[i] / mean) / n;
    sum[i + 1] = s;
  }
  return sum;
}

// find(): i with sum[i] <= r < sum[i+1]; -1 when r is outside [sum[0], sum[n]).
long gsl_find(const std::vector<double>& sum, double r) {
  const size_t n = sum.size() - 1;
  if (r < sum[0] || r >= sum[n]) return -1;
  size_t lo = 0, hi = n;
  while (hi - lo > 1) {
    size_t mid = (hi + lo) / 2;
    if (r >= sum[mid]) lo = mid; else hi = mid;
  }
  return (long)lo;
}

struct Vec4 { double x, y, z, t; };

void boost(Vec4& p, double bx, double by, double bz) {  // TLorentzVector::Boost
  double b2 = bx * bx + by * by + bz * bz;
  double gamma = 1.0 / std::sqrt(1.0 - b2);
  double bp = bx * p.x + by * p.y + bz * p.z;
  double gamma2 = b2 > 0 ? (gamma - 1.0) / b2 : 0.0;
  double x = p.x + gamma2 * bp * bx + gamma * bx * p.t;
  double y = p.y + gamma2 * bp * by + gamma * by * p.t;
  double z = p.z + gamma2 * bp * bz + gamma * bz * p.t;
  p.t = gamma * (p.t + bp);
  p.x = x; p.y = y; p.z = z;
}

void rotate_uz(Vec4& p, double u1, double u2, double u3) {  // TVector3::RotateUz
  double up = u1 * u1 + u2 * u2;
  if (up) {
    up = std::sqrt(up);
    double px = p.x, py = p.y, pz = p.z;
    p.x = (u1 * u3 * px - u2 * py + u1 * up * pz) / up;
    p.y = (u2 * u3 * px + u1 * py + u2 * up * pz) / up;
    p.z = (u3 * u3 * px - px + u3 * up * pz) / up;
  } else if (u3 < 0.) {
    p.x = -p.x;
    p.z = -p.z;
  }
}

double pt_of(const Vec4& p) { return std::sqrt(p.x * p.x + p.y * p.y); }

double eta_of(const Vec4& p) {  // TVector3::PseudoRapidity
  double mag = std::sqrt(p.x * p.x + p.y * p.y + p.z * p.z);
  double ct = mag == 0.0 ? 1.0 : p.z / mag;
  if (ct * ct < 1) return -0.5 * std::log((1.0 - ct) / (1.0 + ct));
  if (p.z == 0) return 0;
  return p.z > 0 ? 10e10 : -10e10;
}

Vec4 set_vect_m(double x, double y, double z, double m) {
  return Vec4{x, y, z, std::sqrt(x * x + y * y + z * z + m * m)};
}

// getPhotonPt's cached 5000-bin TH1D + TH1::GetRandom (src/UpcCrossSection.cpp:1021-1051).
struct PhotonPt {
  const Ctx& c;
  std::unordered_map<int, std::vector<double>> cache;
  explicit PhotonPt(const Ctx& cc) : c(cc) {}
  double sample(double ePhot, RootMT64& rng) {
    const double pi2x4 = 4 * M_PI * M_PI;
    const double hc = 0.1973269718;
    const int nbins = 5000;
    const double hi = 6. * hc / c.R;
    int key = ePhot * 1e3;
    auto it = cache.find(key);
    if (it == cache.end()) {
      double ereds = (ePhot * ePhot) / (c.gtot * c.gtot);
      std::vector<double> integ(nbins + 1, 0.0);
      for (int bin = 1; bin <= nbins; bin++) {
        double pt = 6. * hc / c.R / nbins * bin;
        double arg = pt * pt + ereds;
        double ff = c.formfac.eval(arg);
        double prob = (ff * ff) * pt * pt * pt / (pi2x4 * arg * arg);
        integ[bin] = integ[bin - 1] + prob;
      }
      const double tot = integ[nbins];
      for (int bin = 1; bin <= nbins; bin++) integ[bin] /= tot;
      it = cache.emplace(key, std::move(integ)).first;
    }
    const std::vector<double>& I = it->second;
    double r1 = rng.rndm();
    // TMath::BinarySearch over I[0..nbins-1]
    long ib = (long)(std::lower_bound(I.begin(), I.begin() + nbins, r1) - I.begin());
    if (!(ib != nbins && I[ib] == r1)) ib -= 1;
    const double w = hi / nbins;
    double x = ib * w;
    if (r1 > I[ib]) x += w * (r1 - I[ib]) / (I[ib + 1] - I[ib]);
    if (cache.size() > 30000) cache.clear();
    return x;
  }
};

}  // namespace

}  // namespace uo

extern "C" int uo_generate(uo_ctx* h, const double* cs_ym, const double* cs_zm,
                           const double* ratio, int64_t nevents, uint64_t seed,
                           double* rec, int64_t* rejected, int32_t* mbin_out) {
  using namespace uo;
  const Ctx& c = h->c;
  // polarized (src/UpcGenerator.cpp:686-692, 744-751): cs_zm holds the scalar
  // [nm][nz] then the pseudoscalar [nm][nz] tables, ratio the nuccs_s / nuccs_p
  // [ny][nm]; each mass bin has a scalar and a pseudoscalar z sampler
  const bool pol = c.usePolarizedCS;
  if (pol && !ratio) return -3;
  // vector mesons: cs_ym is [ny][1], ratio the emitter ratio [ny] of nuc_cs_y
  if (c.isVM && !ratio) return -3;
  const int nm = c.nm, ny = c.ny, nz = c.nz;
  const double dm = (c.mmax - c.mmin) / nm, dz = (c.zmax - c.zmin) / nz,
               dy = (c.ymax - c.ymin) / ny;
  std::vector<double> em(nm + 1), ez(nz + 1), ey(ny + 1);
  for (int i = 0; i < nm + 1; ++i) em[i] = c.mmin + dm * i;
  for (int i = 0; i < nz + 1; ++i) ez[i] = c.zmin + dz * i;
  for (int i = 0; i < ny + 1; ++i) ey[i] = c.ymin + dy * i;
  // 2-D sampler over [ny][nm] (x = y-edges, y = m-edges), src/UpcGenerator.cpp:700
  std::vector<double> sum2 = gsl_cdf(cs_ym, (size_t)ny * nm);
  GslUniform rng2(seed);
  std::vector<std::vector<double>> sumz, sumz2;
  std::vector<GslUniform> rngz, rngz2;
  if (!c.ignoreCSZ) {
    sumz.reserve(nm);
    rngz.reserve(nm);
    for (int i = 0; i < nm; ++i) {
      sumz.push_back(gsl_cdf(cs_zm + (size_t)i * nz, nz));
      rngz.emplace_back(seed);
    }
    if (pol) {
      sumz2.reserve(nm);
      rngz2.reserve(nm);
      for (int i = 0; i < nm; ++i) {
        sumz2.push_back(gsl_cdf(cs_zm + (size_t)(nm + i) * nz, nz));
        rngz2.emplace_back(seed);
      }
    }
  }
  RootMT64 groot(seed);
  PhotonPt ptgen(c);
  int64_t evt = 0, rej = 0;
  while (evt < nevents) {
    // (y, m) from the 2-D pdf (gsl_histogram2d_pdf_sample)
    double r1 = rng2(), r2 = rng2();
    if (r2 == 1.0) r2 = 0.0;
    if (r1 == 1.0) r1 = 0.0;
    long k = gsl_find(sum2, r1);
    if (k < 0) return -4;
    long i = k / nm, j = k - i * nm;
    double delta = (r1 - sum2[k]) / (sum2[k + 1] - sum2[k]);
    double yPair = ey[i] + delta * (ey[i + 1] - ey[i]);
    double mPair = em[j] + r2 * (em[j + 1] - em[j]);
    int mBin = uo_sampler_bin(nm, em.front(), em.back(), mPair);
    double cost;
    if (!c.ignoreCSZ) {
      bool scalar = true;
      if (pol) {
        const int yBin = uo_sampler_bin(ny, ey.front(), ey.back(), yPair);
        scalar = groot.uniform(0, 1) < ratio[(size_t)yBin * nm + mBin];
      }
      std::vector<double>& S = scalar ? sumz[mBin] : sumz2[mBin];
      double r = scalar ? rngz[mBin]() : rngz2[mBin]();
      if (r == 1.0) r = 0.0;
      long iz = gsl_find(S, r);
      if (iz < 0) return -4;
      double dl = (r - S[iz]) / (S[iz + 1] - S[iz]);
      cost = ez[iz] + dl * (ez[iz + 1] - ez[iz]);
    } else {
      cost = groot.uniform(-1., 1.);
    }
    Vec4 pp;
    if (c.isVM) {
      // target pick (src/UpcGenerator.cpp:761-764): Uniform(0,1) < the y-bin's
      // emitter ratio; getMomentumVM (src/UpcCrossSection.cpp:1076-1104)
      const int yBin = uo_sampler_bin(ny, ey.front(), ey.back(), yPair);
      const bool target = groot.uniform(0, 1) < ratio[yBin];
      const double sign = target ? 1 : -1;
      const double ePhot = mPair / 2 * std::exp(sign * yPair);
      const double ePom = mPair / 2 * std::exp(-sign * yPair);
      const double ptPhot = ptgen.sample(ePhot, groot);
      const double phi1 = groot.uniform(0, 2 * M_PI);
      const double phi2 = groot.uniform(0, 2 * M_PI);
      const double tmin = (ePom * ePom) / (c.g1 * c.g1);
      double ptPom;
      while (true) {
        ptPom = 32. * groot.uniform(0., 1.) * 0.1973269718 * c.R;
        const double t2 = tmin + ptPom * ptPom;
        const double ff = c.calc_form_fac(t2) / c.A;
        const double test = groot.uniform(0., 1.);
        if (test < ff * ff * ptPom) break;
      }
      const double px = ptPhot * std::cos(phi1) + ptPom * std::cos(phi2);
      const double py = ptPhot * std::sin(phi1) + ptPom * std::sin(phi2);
      const double pt = std::sqrt(px * px + py * py);
      const double mt = std::sqrt(mPair * mPair + pt * pt);
      pp = Vec4{px, py, mt * std::sinh(yPair), mt * std::cosh(yPair)};
    } else if (!c.useNonzeroGamPt) {
      // getPairMomentum (src/UpcCrossSection.cpp:1053-1074)
      double mt = mPair;
      pp = Vec4{0., 0., mt * std::sinh(yPair), mt * std::cosh(yPair)};
    } else {
      double k1 = mPair / 2 * std::exp(yPair);
      double k2 = mPair / 2 * std::exp(-yPair);
      double a1 = groot.uniform(0, 2 * M_PI);
      double a2 = groot.uniform(0, 2 * M_PI);
      double pt1 = ptgen.sample(k1, groot);
      double pt2 = ptgen.sample(k2, groot);
      double px = pt1 * std::cos(a1) + pt2 * std::cos(a2);
      double py = pt1 * std::sin(a1) + pt2 * std::sin(a2);
      double pt = std::sqrt(px * px + py * py);
      double mt = std::sqrt(mPair * mPair + pt * pt);
      pp = Vec4{px, py, mt * std::sinh(yPair), mt * std::cosh(yPair)};
    }
    Vec4 d0, d1;
    double sign0 = 1;
    bool pass = true;
    const double bx = pp.x / pp.t, by = pp.y / pp.t, bz = pp.z / pp.t;
    if (c.isVM) {
      // cuts on the meson (the decay comes after checkKinCuts), then
      // twoPartDecayVM (src/UpcGenerator.cpp:425-472)
      if (c.doPtCut && pt_of(pp) < c.minPt) pass = false;
      if (pass && c.doEtaCut) {
        double e = eta_of(pp);
        if (e < c.minEta || e > c.maxEta) pass = false;
      }
      if (pass) {
        double theta, dndtheta = 0;
        while (true) {
          theta = M_PI * groot.uniform(0., 1.);
          double test = groot.uniform(0., 1.);
          const double ct = std::cos(theta);
          if (c.dghtPDG == 11 || c.dghtPDG == 13) dndtheta = std::sin(theta) * (1. + ct * ct);
          else if (c.dghtPDG == 2212) dndtheta = std::sin(theta) * (1. + 0.605 * ct * ct);
          if (test < dndtheta) break;
        }
        sign0 = groot.uniform(-1, 1) > 0 ? 1 : -1;
        double mag2 = pp.t * pp.t - (pp.x * pp.x + pp.y * pp.y + pp.z * pp.z);
        double pMag = std::sqrt(mag2 / 4. - c.mDght * c.mDght);
        double phi = groot.uniform(0., 2. * M_PI);
        double vx = pMag * std::sin(theta) * std::cos(phi);
        double vy = pMag * std::sin(theta) * std::sin(phi);
        double vz = pMag * std::cos(theta);
        d0 = set_vect_m(-vx, -vy, -vz, c.mDght);
        d1 = set_vect_m(vx, vy, vz, c.mDght);
        double pm = std::sqrt(pp.x * pp.x + pp.y * pp.y + pp.z * pp.z);
        double u1 = pm > 0 ? pp.x / pm : 0, u2 = pm > 0 ? pp.y / pm : 0, u3 = pm > 0 ? pp.z / pm : 0;
        rotate_uz(d0, u1, u2, u3);
        rotate_uz(d1, u1, u2, u3);
        boost(d0, bx, by, bz);
        boost(d1, bx, by, bz);
      }
    } else if (c.procID != 51) {
      // pair production (src/UpcGenerator.cpp:769-776, 388-423)
      double mag2 = pp.t * pp.t - (pp.x * pp.x + pp.y * pp.y + pp.z * pp.z);
      double pMag = std::sqrt(mag2 / 4 - c.mPart * c.mPart);
      double theta = std::acos(cost);
      double phi = groot.uniform(0., 2. * M_PI);
      double vx = pMag * std::sin(theta) * std::cos(phi);
      double vy = pMag * std::sin(theta) * std::sin(phi);
      double vz = pMag * std::cos(theta);
      d0 = set_vect_m(vx, vy, vz, c.mPart);
      d1 = set_vect_m(-vx, -vy, -vz, c.mPart);
      boost(d0, bx, by, bz);
      boost(d1, bx, by, bz);
      sign0 = groot.uniform(-1, 1) > 0 ? 1 : -1;
      for (const Vec4* p : {&d0, &d1}) {
        if (c.doPtCut && pt_of(*p) < c.minPt) { pass = false; break; }
        if (c.doEtaCut) {
          double e = eta_of(*p);
          if (e < c.minEta || e > c.maxEta) { pass = false; break; }
        }
      }
    } else {
      // single ALP: cuts on the ALP itself, then the uniform two-photon decay
      if (c.doPtCut && pt_of(pp) < c.minPt) pass = false;
      if (pass && c.doEtaCut) {
        double e = eta_of(pp);
        if (e < c.minEta || e > c.maxEta) pass = false;
      }
      if (pass) {  // twoPartDecayUniform (src/UpcGenerator.cpp:526-561)
        double mag = std::sqrt(std::max(0.0, pp.t * pp.t - (pp.x * pp.x + pp.y * pp.y + pp.z * pp.z)));
        double e1 = mag / 2.;
        double p1 = std::sqrt(e1 * e1);
        double phi1 = groot.uniform(0., 2. * M_PI);
        double cost1 = groot.uniform(-1., 1.);
        double th1 = std::acos(cost1);
        double vx = p1 * std::sin(th1) * std::cos(phi1);
        double vy = p1 * std::sin(th1) * std::sin(phi1);
        double vz = p1 * std::cos(th1);
        d0 = set_vect_m(-vx, -vy, -vz, 0.);
        d1 = set_vect_m(vx, vy, vz, 0.);
        double pm = std::sqrt(pp.x * pp.x + pp.y * pp.y + pp.z * pp.z);
        double u1 = pm > 0 ? pp.x / pm : 0, u2 = pm > 0 ? pp.y / pm : 0, u3 = pm > 0 ? pp.z / pm : 0;
        rotate_uz(d0, u1, u2, u3);
        rotate_uz(d1, u1, u2, u3);
        boost(d0, bx, by, bz);
        boost(d1, bx, by, bz);
      }
    }
    if (!pass) { ++rej; continue; }
    double* r = rec + 12 * evt;
    r[0] = mPair; r[1] = yPair; r[2] = cost; r[3] = sign0;
    r[4] = d0.x; r[5] = d0.y; r[6] = d0.z; r[7] = d0.t;
    r[8] = d1.x; r[9] = d1.y; r[10] = d1.z; r[11] = d1.t;
    if (mbin_out) mbin_out[evt] = mBin;
    ++evt;
  }
  (void)ratio;
  *rejected = rej;
  return 0;
}
