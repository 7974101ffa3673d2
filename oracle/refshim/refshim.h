// Stand-in declarations of the GSL and ROOT interfaces that the reference's
// src/UpcCrossSection.cpp and its process classes include (TEST
// INFRASTRUCTURE ONLY: used by oracle/build.py to compile those reference
// sources, where they lie, into oracle/_ref/ for parity pins).
//
// ROOT and GSL are not installed here.  The calls on the luminosity path get
// real implementations backed by the oracle's own restated primitives
// (oracle/oracle_num.hpp): GSL's natural cubic spline (gsl_interp_cspline),
// QAGS (gsl_integration_qags), the Bessel functions K0, K1 (gsl_sf_bessel_*)
// and J1 (the C library's j1, as the oracle), and TMath::BesselK1 (the
// Abramowitz & Stegun 9.8.7/9.8.8 polynomials the oracle restates).  So a pin
// built on them checks the reference's own code around those calls -- node
// layouts, loops, clamps, branch conditions -- against the oracle's
// restatement of it.  Everything else (histograms, files, graphs, TF1, 2-D
// splines, random numbers) only has to compile: calling it stops the process
// with a message, and no pin calls it.
#pragma once

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "../oracle_num.hpp"

namespace refshim {
[[noreturn]] inline void unavailable(const char* what) {
  std::fprintf(stderr, "refshim: %s is not available without ROOT/GSL\n", what);
  std::abort();
}
}  // namespace refshim

// ------------------------------------------------------------------ GSL --
#ifndef GSL_EDOM
#define GSL_EDOM 1
#endif

struct gsl_interp_type {
  const char* name;
};
inline const gsl_interp_type gsl_interp_cspline_type{"cspline"};
inline const gsl_interp_type* gsl_interp_cspline = &gsl_interp_cspline_type;

struct gsl_interp_accel {
  int unused = 0;
};
inline gsl_interp_accel* gsl_interp_accel_alloc() { return new gsl_interp_accel(); }
inline void gsl_interp_accel_free(gsl_interp_accel* a) { delete a; }

struct gsl_spline {
  uo::NaturalSpline s;
  size_t n = 0;
};
inline gsl_spline* gsl_spline_alloc(const gsl_interp_type* t, size_t n) {
  if (t != gsl_interp_cspline) refshim::unavailable("a GSL spline other than cspline");
  auto* sp = new gsl_spline();
  sp->n = n;
  return sp;
}
inline int gsl_spline_init(gsl_spline* sp, const double* x, const double* y, size_t n) {
  sp->s.build(x, y, (int)n);
  return 0;
}
inline double gsl_spline_eval(const gsl_spline* sp, double x, gsl_interp_accel*) {
  return sp->s.eval(x);
}
inline void gsl_spline_free(gsl_spline* sp) { delete sp; }

struct gsl_function {
  double (*function)(double x, void* params);
  void* params;
};
struct gsl_integration_workspace {
  size_t limit;
};
inline gsl_integration_workspace* gsl_integration_workspace_alloc(size_t n) {
  return new gsl_integration_workspace{n};
}
inline void gsl_integration_workspace_free(gsl_integration_workspace* w) { delete w; }
inline int gsl_integration_qags(const gsl_function* f, double a, double b, double epsabs,
                                double epsrel, size_t limit, gsl_integration_workspace* w,
                                double* result, double* abserr) {
  if (limit > w->limit) limit = w->limit;
  auto fn = [f](double x) { return f->function(x, f->params); };
  const uo::QagsResult r = uo::qags(fn, a, b, epsabs, epsrel, (int)limit);
  *result = r.result;
  *abserr = r.abserr;
  return r.status;
}

inline double gsl_sf_bessel_K0(double x) {
  double k0, k1;
  uo::bessel_k01(x, &k0, &k1);
  return k0;
}
inline double gsl_sf_bessel_K1(double x) {
  double k0, k1;
  uo::bessel_k01(x, &k0, &k1);
  return k1;
}
inline double gsl_sf_bessel_J1(double x) { return ::j1(x); }

struct gsl_interp2d_type {
  const char* name;
};
inline const gsl_interp2d_type gsl_interp2d_bicubic_type{"bicubic"};
inline const gsl_interp2d_type* gsl_interp2d_bicubic = &gsl_interp2d_bicubic_type;
struct gsl_spline2d {
  int unused = 0;
};
inline gsl_spline2d* gsl_spline2d_alloc(const gsl_interp2d_type*, size_t, size_t) {
  refshim::unavailable("gsl_spline2d");
}
inline int gsl_spline2d_init(gsl_spline2d*, const double*, const double*, const double*, size_t,
                             size_t) {
  refshim::unavailable("gsl_spline2d");
}
inline double gsl_spline2d_eval(const gsl_spline2d*, double, double, gsl_interp_accel*,
                                gsl_interp_accel*) {
  refshim::unavailable("gsl_spline2d");
}
inline void gsl_spline2d_free(gsl_spline2d*) {}

// ----------------------------------------------------------------- ROOT --
typedef int Int_t;
typedef double Double_t;
typedef float Float_t;
typedef bool Bool_t;
typedef unsigned int UInt_t;
typedef long Long64_t;
typedef const char Option_t;

class TString {
 public:
  TString() = default;
  TString(const char* s) : s_(s ? s : "") {}
  TString(const std::string& s) : s_(s) {}
  const char* Data() const { return s_.c_str(); }
  operator const char*() const { return s_.c_str(); }
  TString& operator+=(const char* o) {
    s_ += o;
    return *this;
  }
  TString& operator+=(const TString& o) {
    s_ += o.s_;
    return *this;
  }
  friend TString operator+(const TString& a, const char* b) { return TString(a.s_ + b); }
  friend TString operator+(const TString& a, const TString& b) { return TString(a.s_ + b.s_); }
  friend TString operator+(const char* a, const TString& b) { return TString(a + b.s_); }
  friend TString operator+(const TString& a, const std::string& b) { return TString(a.s_ + b); }

 private:
  std::string s_;
};

inline const char* Form(const char* fmt, ...) {
  static thread_local char buf[4096];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  return buf;
}

namespace TMath {
inline double Pi() { return M_PI; }
inline double Sqrt(double x) { return std::sqrt(x); }
inline double Cos(double x) { return std::cos(x); }
inline double Sin(double x) { return std::sin(x); }
inline double Tan(double x) { return std::tan(x); }
inline double Exp(double x) { return std::exp(x); }
inline double Log(double x) { return std::log(x); }
inline double Abs(double x) { return std::fabs(x); }
inline double Power(double x, double y) { return std::pow(x, y); }
inline double CosH(double x) { return std::cosh(x); }
inline double SinH(double x) { return std::sinh(x); }
inline double TanH(double x) { return std::tanh(x); }
inline double ACosH(double x) { return std::acosh(x); }
inline double ASinH(double x) { return std::asinh(x); }
inline double ATan2(double y, double x) { return std::atan2(y, x); }
template <class T>
inline T Max(T a, T b) { return a > b ? a : b; }
template <class T>
inline T Min(T a, T b) { return a < b ? a : b; }
inline double BesselK1(double x) { return uo::bessel_k1_as(x); }
}  // namespace TMath

class TObject {
 public:
  virtual ~TObject() = default;
  enum { kIsSortedX = 1 };
  void SetBit(unsigned, bool = true) {}
  virtual int Write(const char* = nullptr, int = 0, int = 0) { refshim::unavailable("Write"); }
};

class TAxis {
 public:
  double GetBinCenter(int) const { refshim::unavailable("TAxis"); }
  double GetBinLowEdge(int) const { refshim::unavailable("TAxis"); }
  double GetBinUpEdge(int) const { refshim::unavailable("TAxis"); }
  double GetBinWidth(int) const { refshim::unavailable("TAxis"); }
  double GetXmin() const { refshim::unavailable("TAxis"); }
  double GetXmax() const { refshim::unavailable("TAxis"); }
  int FindBin(double) const { refshim::unavailable("TAxis"); }
  int FindFixBin(double) const { refshim::unavailable("TAxis"); }
  int GetNbins() const { refshim::unavailable("TAxis"); }
};

class TDirectory;
class TH1 : public TObject {
 public:
  TH1() = default;
  void SetDirectory(TDirectory*) {}
  int GetNbinsX() const { refshim::unavailable("histograms"); }
  int GetNbinsY() const { refshim::unavailable("histograms"); }
  TAxis* GetXaxis() { refshim::unavailable("histograms"); }
  TAxis* GetYaxis() { refshim::unavailable("histograms"); }
  double GetBinContent(int) const { refshim::unavailable("histograms"); }
  double GetBinContent(int, int) const { refshim::unavailable("histograms"); }
  void SetBinContent(int, double) { refshim::unavailable("histograms"); }
  void SetBinContent(int, int, double) { refshim::unavailable("histograms"); }
  double GetRandom() { refshim::unavailable("histograms"); }
  double Interpolate(double) { refshim::unavailable("histograms"); }
  double Interpolate(double, double) { refshim::unavailable("histograms"); }
  int FindBin(double) { refshim::unavailable("histograms"); }
  int FindBin(double, double) { refshim::unavailable("histograms"); }
  int Fill(double) { refshim::unavailable("histograms"); }
  int Fill(double, double) { refshim::unavailable("histograms"); }
  TObject* Clone(const char* = "") const { refshim::unavailable("histograms"); }
  void Scale(double) { refshim::unavailable("histograms"); }
};
class TH1D : public TH1 {
 public:
  TH1D() = default;
  TH1D(const char*, const char*, int, double, double) {}
  TH1D(const char*, const char*, int, const double*) {}
};
class TH2D : public TH1 {
 public:
  TH2D() = default;
  TH2D(const char*, const char*, int, double, double, int, double, double) {}
  TH2D(const char*, const char*, int, const double*, int, const double*) {}
  TH1D* ProjectionX(const char* = "_px") { refshim::unavailable("histograms"); }
  TH1D* ProjectionY(const char* = "_py") { refshim::unavailable("histograms"); }
};

class TDirectory : public TObject {};
class TFile : public TDirectory {
 public:
  TFile() = default;
  TFile(const char*, const char* = "", const char* = "", int = 0) {
    refshim::unavailable("TFile");
  }
  TObject* Get(const char*) { refshim::unavailable("TFile"); }
  bool IsOpen() const { return false; }
  bool IsZombie() const { return true; }
  void Close(const char* = "") {}
  int Write(const char* = nullptr, int = 0, int = 0) override { refshim::unavailable("TFile"); }
};

class TTree : public TObject {
 public:
  TTree() = default;
  TTree(const char*, const char*) { refshim::unavailable("TTree"); }
  template <class... A>
  void Branch(A...) { refshim::unavailable("TTree"); }
  int Fill() { refshim::unavailable("TTree"); }
  void SetAutoSave(long) {}
};

class TGraph : public TObject {
 public:
  TGraph() = default;
  TGraph(int, const double*, const double*) {}
  void SetPoint(int, double, double) { refshim::unavailable("TGraph"); }
  double Eval(double, void* = nullptr, const char* = "") const { refshim::unavailable("TGraph"); }
};
class TGraph2D : public TObject {
 public:
  TGraph2D() = default;
  double Interpolate(double, double) { refshim::unavailable("TGraph2D"); }
  void SetPoint(int, double, double, double) { refshim::unavailable("TGraph2D"); }
};
class TSpline3 : public TObject {
 public:
  TSpline3() = default;
  TSpline3(const char*, TGraph*) {}
  double Eval(double) const { refshim::unavailable("TSpline3"); }
};

class TF1 : public TObject {
 public:
  TF1() = default;
  template <class F>
  TF1(const char*, F, double, double, int = 0) {}
  void SetParameter(int, double) {}
  void SetParameters(const double*) {}
  void FixParameter(int, double) {}
  void SetNpx(int) {}
  double Eval(double, double = 0, double = 0, double = 0) const { refshim::unavailable("TF1"); }
  double Integral(double, double, double = 1e-12) { refshim::unavailable("TF1"); }
};

class TVector3 {
 public:
  TVector3() = default;
  TVector3(double x, double y, double z) : x_(x), y_(y), z_(z) {}
  double X() const { return x_; }
  double Y() const { return y_; }
  double Z() const { return z_; }

 private:
  double x_ = 0, y_ = 0, z_ = 0;
};
class TLorentzVector {
 public:
  TLorentzVector() = default;
  TLorentzVector(double px, double py, double pz, double e) : p_{px, py, pz, e} {}
  void SetPxPyPzE(double px, double py, double pz, double e) { p_[0] = px, p_[1] = py, p_[2] = pz, p_[3] = e; }
  void SetXYZM(double, double, double, double) { refshim::unavailable("TLorentzVector"); }
  double Px() const { return p_[0]; }
  double Py() const { return p_[1]; }
  double Pz() const { return p_[2]; }
  double E() const { return p_[3]; }
  double Pt() const { return std::sqrt(p_[0] * p_[0] + p_[1] * p_[1]); }
  double M() const { refshim::unavailable("TLorentzVector"); }
  double Eta() const { refshim::unavailable("TLorentzVector"); }
  double Phi() const { refshim::unavailable("TLorentzVector"); }
  double Rapidity() const { refshim::unavailable("TLorentzVector"); }
  TVector3 BoostVector() const { refshim::unavailable("TLorentzVector"); }
  void Boost(const TVector3&) { refshim::unavailable("TLorentzVector"); }
  void Boost(double, double, double) { refshim::unavailable("TLorentzVector"); }
  TLorentzVector operator+(const TLorentzVector& o) const {
    return TLorentzVector(p_[0] + o.p_[0], p_[1] + o.p_[1], p_[2] + o.p_[2], p_[3] + o.p_[3]);
  }

 private:
  double p_[4] = {0, 0, 0, 0};
};

class TParticle : public TObject {
 public:
  TParticle() = default;
  template <class... A>
  TParticle(A...) {}
};
class TClonesArray : public TObject {};

class TRandom : public TObject {
 public:
  double Uniform(double = 1.) { refshim::unavailable("gRandom"); }
  double Uniform(double, double) { refshim::unavailable("gRandom"); }
  double Rndm() { refshim::unavailable("gRandom"); }
  void SetSeed(unsigned long) {}
};
template <class T>
class TRandomGen : public TRandom {};
class TRandomMT64 : public TRandom {};
inline TRandom* gRandom = nullptr;

class TSystem : public TObject {
 public:
  bool AccessPathName(const char*) { refshim::unavailable("gSystem"); }
  int Exec(const char*) { refshim::unavailable("gSystem"); }
  int Unlink(const char*) { refshim::unavailable("gSystem"); }
};
inline TSystem* gSystem = nullptr;
class TROOT : public TObject {};
inline TROOT* gROOT = nullptr;
namespace ROOT {
inline void EnableThreadSafety() {}
}  // namespace ROOT
