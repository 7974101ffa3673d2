/* CPU oracle -- C interface for the tests and the CPU-baseline leg of bench.py.
 *
 * TEST INFRASTRUCTURE ONLY: an FP64 C++/OpenMP restatement of upcgen's
 * two-photon luminosity, nuclear cross-section and (m,y,z) sampling path
 * (src/UpcCrossSection.cpp, src/UpcGenerator.cpp, include/UpcSampler.h,
 * src/UpcTwoPhotonDilep.cpp, src/UpcTwoPhotonALP.cpp of the reference).  It is
 * the checker for the CUDA library, never part of it.
 *
 * Parity status: the reference needs ROOT and GSL, neither of which is
 * available, so its CMake project cannot be built here.  The restatement is
 * pinned (a) bit for bit against the reference's own src/UpcCrossSection.cpp
 * and the process classes it creates, compiled from their sources against
 * stand-in GSL / ROOT headers (oracle/refshim/) whose luminosity-path calls
 * run this oracle's restated primitives (oracle/ref_cs_shim.cpp; fixture
 * tests/golden/ref_cs.json): rho0, G_AA, the form factor, both fluxes, the
 * breakup probability, luminosity cells and calcPhotonFlux on 8
 * configurations; (b) the event loop, bit for bit against the reference's
 * own src/UpcGenerator.cpp compiled the same way (oracle/ref_gen_shim.cpp;
 * fixture tests/golden/ref_gen.npz): every 4-momentum, pdg code, rejected
 * count and totNuclX of five configurations, with the random engines,
 * histogram samplers and vector algebra of oracle_gen_prims.hpp behind the
 * stand-ins; (c) for the elementary gamma-gamma cross sections, bit for bit
 * against UpcTwoPhotonDilep.cpp / UpcTwoPhotonALP.cpp compiled as they are;
 * (d) the primitives themselves (K0/K1/J1, QAGS, natural cubic splines)
 * against scipy's independent implementations, not against GSL / ROOT,
 * which are absent.
 */
#ifndef UPCG_ORACLE_H_
#define UPCG_ORACLE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct uo_ctx uo_ctx;

uo_ctx* uo_create(void);
void uo_destroy(uo_ctx* h);
/* parameters.in keys, UpcGenerator::setParameterValue (src/UpcGenerator.cpp:183-305) */
int uo_set_param(uo_ctx* h, const char* key, const char* value);
void uo_set_num_threads(uo_ctx* h, int n);
/* UpcGenerator::init process overrides (src/UpcGenerator.cpp:66-142) followed by
 * UpcCrossSection::init tables (src/UpcCrossSection.cpp:116-131), without the
 * luminosity table. */
int uo_init_tables(uo_ctx* h);
/* Effective grid after the process overrides. */
void uo_grid(const uo_ctx* h, double* mmin, double* mmax, int* nm, double* ymin,
             double* ymax, int* ny, double* zmin, double* zmax, int* nz);
double uo_rho0(const uo_ctx* h);
double uo_gamma(const uo_ctx* h);

/* primitives */
void uo_bessel_k01(double x, double* k0, double* k1);
double uo_bessel_k1_as(double x);
double uo_simpson(int n, const double* v, double h);
/* QAGS over one of the test integrands (id) -- see oracle_cs.cpp */
int uo_qags_test(int id, double p0, double p1, double a, double b, double epsabs,
                 double epsrel, int limit, double* result, double* abserr,
                 int* neval, int* nint);
void uo_spline_natural(int n, const double* x, const double* y, int m,
                       const double* xe, double* ye);

/* per-point quantities, UpcCrossSection methods */
double uo_flux_point(const uo_ctx* h, double b, double k);
double uo_flux_form(const uo_ctx* h, double b, double k, int* status,
                    int* neval, int* nint);
double uo_form_factor(const uo_ctx* h, double q2);        /* calcFormFac */
double uo_form_factor_spline(const uo_ctx* h, double q2); /* gslSplineFormFac */
double uo_gaa(const uo_ctx* h, double b);                 /* gslSplineGAA */
double uo_breakup_prob(const uo_ctx* h, double b, int mode); /* calcBreakupProb */
double uo_breakup_spline(const uo_ctx* h, double b);     /* gslSplineBreakP */
double uo_two_photon_lumi(const uo_ctx* h, double m, double y);
void uo_two_photon_lumi_pol(const uo_ctx* h, double m, double y, double* ls,
                            double* lp);
/* Elementary cross sections of the configured process. */
double uo_cs_m(const uo_ctx* h, double m, int flag);
double uo_cs_zm(const uo_ctx* h, double z, double m, int flag);

/* Tables.  lumi[im*ny+iy] = L(m_im, y_iy)*dm*dy (hD2LDMDY bin (im+1,iy+1));
 * for the polarized form lumi holds the scalar and lumi2 the pseudoscalar part. */
int uo_lumi_table(uo_ctx* h, double* lumi, double* lumi2, int im_lo, int im_hi);
/* csZM[im*nz+iz] (fillCrossSectionZM, flag 0/1/2) */
int uo_cs_zm_table(const uo_ctx* h, int flag, double* out);
/* cs[iy*nm+im] and total (mb), calcNucCrossSectionYM; ratio may be NULL */
int uo_nuc_cs_ym(const uo_ctx* h, const double* lumi, const double* lumi2,
                 double* cs, double* ratio, double* tot_mb);

/* Event generation: UpcGenerator::generateEvent loop (src/UpcGenerator.cpp:715-889).
 * rec[i*12 + ...] = m, y, z, charge-sign of particle 0, then px,py,pz,E of
 * the two final-state particles (ALP: the two decay photons).  Needs the cs
 * tables from uo_nuc_cs_ym / uo_cs_zm_table. */
double uo_photon_flux(const uo_ctx* h, double m, double y);
double uo_vm_cs_y(const uo_ctx* h, double y);
int uo_nuc_cs_y(const uo_ctx* h, double* cs, double* ratio, double* tot);
int uo_generate(uo_ctx* h, const double* cs_ym, const double* cs_zm,
                const double* ratio, int64_t nevents, uint64_t seed,
                double* rec, int64_t* rejected, int32_t* mbin);
/* getBinX / getBinY of UpcSampler2D (include/UpcSampler.h:124-134) */
int uo_sampler_bin(int nbins, double lo, double hi, double x);

#ifdef __cplusplus
}
#endif
#endif
