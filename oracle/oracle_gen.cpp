// CPU oracle -- samplers and event loop (TEST INFRASTRUCTURE ONLY).
//
// Restates include/UpcSampler.h:37-142 (GSL histogram PDFs),
// src/UpcGenerator.cpp:715-889 (generateEvent / generateEvents),
// src/UpcCrossSection.cpp:1021-1074 (getPhotonPt / getPairMomentum) and the
// ROOT vector algebra they use (TLorentzVector boosts, TVector3::RotateUz),
// on the engines and primitives of oracle_gen_prims.hpp.  The random streams
// follow the reference's engines: GSL's mt19937 for the samplers -- one
// engine per sampler, all seeded with SEED as in
// src/UpcGenerator.cpp:688-700 -- and ROOT's TRandomMT64 for gRandom.  The
// two uniforms of the 2-D sampler are drawn as GCC orders the reference's two
// argument calls (right to left).  The event stream is bit-exact with the
// reference's own src/UpcGenerator.cpp compiled here (ref_gen_shim.cpp,
// tests/test_oracle_pins.py).
#include <cmath>
#include <cstdint>
#include <random>
#include <unordered_map>
#include <vector>

#include "oracle_ctx.hpp"
#include "oracle_gen_prims.hpp"
#include "upcg_oracle.h"

namespace uo {

namespace {

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
      std::vector<double> prob(nbins);
      for (int bin = 1; bin <= nbins; bin++) {
        double pt = 6. * hc / c.R / nbins * bin;
        double arg = pt * pt + ereds;
        double ff = c.formfac.eval(arg);
        prob[bin - 1] = (ff * ff) * pt * pt * pt / (pi2x4 * arg * arg);
      }
      it = cache.emplace(key, th1_integral(prob.data(), nbins)).first;
    }
    const double x = th1_sample(it->second, nbins, 0., hi, rng.rndm());
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
    // gsl_histogram2d_pdf_sample(hpdf, gsl_rng_uniform(rng), gsl_rng_uniform(rng), ...)
    // (include/UpcSampler.h:120): C++ leaves the order of the two draws to
    // the compiler; GCC evaluates the arguments right to left, so r2 (the
    // position inside the mass bin) is drawn first
    double r2 = rng2();
    double r1 = rng2();
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
        double u[3];
        unit3(pp.x, pp.y, pp.z, u);
        rotate_uz(d0, u[0], u[1], u[2]);
        rotate_uz(d1, u[0], u[1], u[2]);
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
        double e1 = mag_of(pp) / 2.;
        double p1 = std::sqrt(e1 * e1);
        double phi1 = groot.uniform(0., 2. * M_PI);
        double cost1 = groot.uniform(-1., 1.);
        double th1 = std::acos(cost1);
        double vx = p1 * std::sin(th1) * std::cos(phi1);
        double vy = p1 * std::sin(th1) * std::sin(phi1);
        double vz = p1 * std::cos(th1);
        d0 = set_vect_m(-vx, -vy, -vz, 0.);
        d1 = set_vect_m(vx, vy, vz, 0.);
        double u[3];
        unit3(pp.x, pp.y, pp.z, u);
        rotate_uz(d0, u[0], u[1], u[2]);
        rotate_uz(d1, u[0], u[1], u[2]);
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
