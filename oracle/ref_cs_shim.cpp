// C entry points around the reference's own UpcCrossSection
// (src/UpcCrossSection.cpp and the process classes it news), compiled from the
// reference sources where they lie by oracle/build.py into oracle/_ref/, with
// the GSL / ROOT stand-ins of oracle/refshim/ (TEST INFRASTRUCTURE ONLY).
//
// uref_cs_init repeats UpcCrossSection::init (src/UpcCrossSection.cpp:116-137)
// without prepareTwoPhotonLumi (its file cache needs ROOT): the statics and
// grid of one configuration, rho0 by calcWSRho, prepareGAA, prepareFormFac
// and, for BREAKUP_MODE > 1, prepareBreakupProb.  The other entries call the
// reference's member functions one point at a time.  Like the reference, one
// configuration per process at a time (its splines and nucleus are globals).
#include <pthread.h>

#include <functional>
#include <memory>

#include "UpcCrossSection.h"

extern gsl_interp_accel* gslInterpAccGAA;
extern gsl_spline* gslSplineGAA;
extern gsl_interp_accel* gslInterpAccBreakP;
extern gsl_spline* gslSplineBreakP;

namespace {
std::unique_ptr<UpcCrossSection> g_cs;

// prepareBreakupProb keeps two arrays of 10^6 doubles on the stack
// (src/UpcCrossSection.cpp:422-423, 16 MB): the set-up runs on a thread with a
// 256 MB stack instead of the caller's.
int on_big_stack(std::function<void()> fn) {
  pthread_attr_t attr;
  pthread_attr_init(&attr);
  pthread_attr_setstacksize(&attr, (size_t)256 << 20);
  pthread_t th;
  auto body = [](void* p) -> void* {
    (*static_cast<std::function<void()>*>(p))();
    return nullptr;
  };
  const int rc = pthread_create(&th, &attr, body, &fn);
  pthread_attr_destroy(&attr);
  if (rc != 0) return -1;
  pthread_join(th, nullptr);
  return 0;
}
}

extern "C" {

int uref_cs_init(int Z, int A, double R, double a, double sqrts, int is_point, int breakup_mode,
                 int proc_id, double alp_mass, double alp_width, double mmin, double mmax, int nm,
                 double ymin, double ymax, int ny, int use_polarized) {
  g_cs.reset();  // frees the previous configuration's splines
  UpcCrossSection::Z = Z;
  UpcCrossSection::A = A;
  UpcCrossSection::R = R;
  UpcCrossSection::a = a;
  UpcCrossSection::sqrts = sqrts;
  // the beam Lorentz factors as UpcGenerator sets them (src/UpcGenerator.cpp:188-192, 307-311)
  UpcCrossSection::g1 = sqrts / (2. * phys_consts::mProt);
  UpcCrossSection::g2 = sqrts / (2. * phys_consts::mProt);
  g_cs = std::make_unique<UpcCrossSection>();
  UpcCrossSection& c = *g_cs;
  c.isPoint = is_point != 0;
  c.breakupMode = breakup_mode;
  c.usePolarizedCS = use_polarized != 0;
  c.alpMass = alp_mass;
  c.alpWidth = alp_width;
  c.mmin = mmin;
  c.mmax = mmax;
  c.nm = nm;
  c.ymin = ymin;
  c.ymax = ymax;
  c.ny = ny;
  c.setElemProcess(proc_id);
  // UpcCrossSection::init up to prepareTwoPhotonLumi
  return on_big_stack([&c] {
    c.factor = UpcCrossSection::Z * UpcCrossSection::Z * phys_consts::alpha / M_PI / M_PI /
               phys_consts::hc / phys_consts::hc;
    UpcCrossSection::mNucl = (UpcCrossSection::Z * phys_consts::mProt +
                              (UpcCrossSection::A - UpcCrossSection::Z) * phys_consts::mNeut) /
                             UpcCrossSection::A;
    UpcCrossSection::rho0 = c.calcWSRho();
    c.prepareGAA();
    c.prepareFormFac();
    if (c.breakupMode > 1) c.prepareBreakupProb();
  });
}

double uref_cs_rho0() { return UpcCrossSection::rho0; }
double uref_cs_flux_point(double b, double k) { return g_cs->fluxPoint(b, k); }
double uref_cs_flux_form(double b, double k) { return g_cs->fluxForm(b, k); }
double uref_cs_form_factor(double q2) { return UpcCrossSection::calcFormFac(q2); }
double uref_cs_breakup_prob(double b, int mode) { return g_cs->calcBreakupProb(b, mode); }
double uref_cs_gaa_spline(double b) { return gsl_spline_eval(gslSplineGAA, b, gslInterpAccGAA); }
double uref_cs_breakup_spline(double b) {
  return gsl_spline_eval(gslSplineBreakP, b, gslInterpAccBreakP);
}
double uref_cs_lumi(double m, double y) { return g_cs->calcTwoPhotonLumi(m, y); }
void uref_cs_lumi_pol(double m, double y, double* s, double* p) {
  g_cs->calcTwoPhotonLumiPol(*s, *p, m, y);
}
double uref_cs_photon_flux(double m, double y) { return g_cs->calcPhotonFlux(m, y); }
}
