// CPU oracle -- configuration and tables of one generator instance
// (TEST INFRASTRUCTURE ONLY).  Field defaults are the reference's:
// include/UpcCrossSection.h:73-172, include/UpcGenerator.h:62-73.
#pragma once

#include <string>
#include <vector>

#include "oracle_num.hpp"

namespace uo {

struct Ctx {
  Ctx();
  // nucleus / beam
  double R = 6.68, a = 0.447, rho0 = 0.;
  int Z = 82, A = 208;
  double sqrts = 5020., g1 = 0, g2 = 0, gtot = 0;
  // process
  int procID = 15;
  double aLep = 0, alpMass = 1., alpWidth = 0.010;
  double mPart = 0;
  int partPDG = 0;
  bool isCharged = true, ignoreCSZ = false;
  // vector-meson photoproduction (src/UpcPhotoNuclearVM.cpp:55-93): the
  // reference's SHADOWING and DECAY_PDG keys, the meson's dsdt constants
  bool isVM = false;
  int shadowing = 0, dghtPDG = 0;
  double mDght = 0, vm_c0 = 0, vm_pw = 0.4, vm_mu2 = 0, mNucl = 0;
  // grid
  double zmin = -1, zmax = 1, mmin = 3.56, mmax = 50., ymin = -6., ymax = 6.;
  int nz = 100, nm = 1001, ny = 121;
  const int nb1 = 120, nb2 = 120;
  // flags
  bool isPoint = true, useNonzeroGamPt = true, usePolarizedCS = false;
  int breakupMode = 1;
  // generator
  bool doPtCut = false, doEtaCut = false;
  double minPt = 0, minEta = 0, maxEta = 0;
  long seed = 0, nEvents = 1000;
  int numThreads = 1;
  // Tolerance of the form-factor flux QAGS (epsabs = epsrel).  The reference
  // fixes 1e-4 (src/UpcCrossSection.cpp:209); the key ORACLE_FLUX_EPS, which
  // the reference does not have, tightens it so that tests can tell the
  // reference's quadrature noise from the error of an approximation.
  double fluxEps = 1e-4;
  // derived
  double factor = 0, cs_nn = 0;
  bool initialized = false;
  NaturalSpline gaa, formfac, breakup;
  // breakup tables (per context; the reference keeps them in function statics)
  std::vector<double> bu_ee, bu_se;
  double bu_zcon = 0, bu_o0 = 0, bu_omaxx = 0, bu_gammatarg = 0;
  int bu_n = 0;

  void set_collision(float s, int z, int a);
  int set_param(const std::string& k, const std::string& v);
  int setup_process();
  double cs_m(double m, int flag) const;
  double cs_zm(double z, double m, int flag) const;
  double calc_ws_rho() const;
  void prepare_gaa();
  double calc_form_fac(double q2) const;
  void prepare_form_fac();
  void prepare_breakup_tables();
  double breakup_prob(double b, int mode) const;
  void prepare_breakup();
  double flux_point(double b, double k) const;
  double flux_form(double b, double k, QagsResult* info) const;
  double two_photon_lumi(double m, double y) const;
  void two_photon_lumi_pol(double m, double y, double* ns, double* np) const;
  int init_tables();
  int lumi_table(double* out, double* out2, int im_lo, int im_hi) const;
  void cs_zm_table(int flag, double* out) const;
  void nuc_cs_ym(const double* lumi, const double* lumi2, double* cs, double* ratio,
                 double* tot) const;
  // photonuclear path (oracle_vm.cpp)
  double photon_flux(double m, double y) const;
  double vm_cs_y(double y) const;
  void nuc_cs_y(double* cs, double* ratio, double* tot) const;
};

}  // namespace uo

// Opaque handle of the C interface (upcg_oracle.h).
struct uo_ctx {
  uo::Ctx c;
};
