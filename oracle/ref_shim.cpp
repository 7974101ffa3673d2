// C entry points around the reference's own elementary gamma-gamma cross
// sections, compiled from the reference sources by oracle/build.py into
// oracle/_ref/ (TEST INFRASTRUCTURE ONLY).  Only these two translation units of
// the reference build without ROOT/GSL (src/UpcTwoPhotonDilep.cpp,
// src/UpcTwoPhotonALP.cpp); they pin the oracle's restatement bit for bit.
#include "UpcTwoPhotonALP.h"
#include "UpcTwoPhotonDilep.h"

extern "C" {

// flag: 0 unpolarized, 1 scalar, 2 pseudoscalar (as fillCrossSectionZM's flag)
double uref_dilep_cs_m(int pdg, double alep, double m, int flag) {
  UpcTwoPhotonDilep p(pdg);
  p.aLep = alep;
  if (flag == 1) return p.calcCrossSectionMPolS(m);
  if (flag == 2) return p.calcCrossSectionMPolPS(m);
  return p.calcCrossSectionM(m);
}

double uref_dilep_cs_zm(int pdg, double alep, double z, double m, int flag) {
  UpcTwoPhotonDilep p(pdg);
  p.aLep = alep;
  if (flag == 1) return p.calcCrossSectionZMPolS(z, m);
  if (flag == 2) return p.calcCrossSectionZMPolPS(z, m);
  return p.calcCrossSectionZM(z, m);
}

double uref_dilep_mass(int pdg) {
  UpcTwoPhotonDilep p(pdg);
  return p.mPart;
}

double uref_alp_cs_m(double mass, double width, double m) {
  UpcTwoPhotonALP p(mass, width);
  return p.calcCrossSectionM(m);
}
}
