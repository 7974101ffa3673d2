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
// restatement of it.
//
// For the generator pin (src/UpcGenerator.cpp with ref_gen_shim.cpp) the
// event loop's calls are real too, backed by oracle_gen_prims.hpp: GSL's
// mt19937 and histogram PDFs (gsl_rng, gsl_histogram[2d]_pdf), ROOT's
// TRandomMT64 behind gRandom, TLorentzVector / TVector3 algebra, TH1D with
// GetRandom, and TH2D histograms kept in an in-memory stand-in of the
// luminosity's ROOT file (TFile, gSystem->AccessPathName), so that
// UpcCrossSection::prepareTwoPhotonLumi / calcNucCrossSectionYM run as
// written.  Everything else (graphs, TF1, 2-D splines, trees) only has to
// compile: calling it stops the process with a message, and no pin calls it.
#pragma once

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../oracle_gen_prims.hpp"
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

// GSL random numbers (gsl_rng_default = mt19937) and histogram PDFs
struct gsl_rng_type {
  const char* name;
};
inline const gsl_rng_type gsl_rng_mt19937_type{"mt19937"};
inline const gsl_rng_type* gsl_rng_default = &gsl_rng_mt19937_type;
struct gsl_rng {
  uo::GslUniform u;
};
inline gsl_rng* gsl_rng_alloc(const gsl_rng_type* t) {
  if (t != gsl_rng_default) refshim::unavailable("a GSL generator other than mt19937");
  return new gsl_rng();
}
inline void gsl_rng_set(gsl_rng* r, unsigned long seed) { r->u = uo::GslUniform(seed); }
inline double gsl_rng_uniform(gsl_rng* r) { return r->u(); }
inline void gsl_rng_free(gsl_rng* r) { delete r; }

struct gsl_histogram {
  size_t n;
  double* range;
  double* bin;
};
inline gsl_histogram* gsl_histogram_alloc(size_t n) {
  auto* h = new gsl_histogram{n, new double[n + 1](), new double[n]()};
  return h;
}
inline int gsl_histogram_set_ranges(gsl_histogram* h, const double* range, size_t size) {
  if (size != h->n + 1) refshim::unavailable("gsl_histogram_set_ranges of another size");
  for (size_t i = 0; i < size; ++i) h->range[i] = range[i];
  return 0;
}
inline void gsl_histogram_free(gsl_histogram* h) {
  delete[] h->range;
  delete[] h->bin;
  delete h;
}
struct gsl_histogram_pdf {
  size_t n;
  std::vector<double> range, sum;
};
inline gsl_histogram_pdf* gsl_histogram_pdf_alloc(size_t n) { return new gsl_histogram_pdf{n, {}, {}}; }
inline int gsl_histogram_pdf_init(gsl_histogram_pdf* p, const gsl_histogram* h) {
  for (size_t i = 0; i < h->n; ++i)
    if (h->bin[i] < 0) return GSL_EDOM;
  p->range.assign(h->range, h->range + h->n + 1);
  p->sum = uo::gsl_cdf(h->bin, h->n);
  return 0;
}
inline double gsl_histogram_pdf_sample(const gsl_histogram_pdf* p, double r) {
  if (r == 1.0) r = 0.0;
  const long i = uo::gsl_find(p->sum, r);
  if (i < 0) refshim::unavailable("gsl_histogram_pdf_sample outside the pdf");
  const double delta = (r - p->sum[i]) / (p->sum[i + 1] - p->sum[i]);
  return p->range[i] + delta * (p->range[i + 1] - p->range[i]);
}
inline void gsl_histogram_pdf_free(gsl_histogram_pdf* p) { delete p; }

struct gsl_histogram2d {
  size_t nx, ny;
  double* xrange;
  double* yrange;
  double* bin;
};
inline gsl_histogram2d* gsl_histogram2d_alloc(size_t nx, size_t ny) {
  return new gsl_histogram2d{nx, ny, new double[nx + 1](), new double[ny + 1](),
                             new double[nx * ny]()};
}
inline int gsl_histogram2d_set_ranges(gsl_histogram2d* h, const double* xr, size_t xs,
                                      const double* yr, size_t ys) {
  if (xs != h->nx + 1 || ys != h->ny + 1)
    refshim::unavailable("gsl_histogram2d_set_ranges of another size");
  for (size_t i = 0; i < xs; ++i) h->xrange[i] = xr[i];
  for (size_t i = 0; i < ys; ++i) h->yrange[i] = yr[i];
  return 0;
}
inline void gsl_histogram2d_free(gsl_histogram2d* h) {
  delete[] h->xrange;
  delete[] h->yrange;
  delete[] h->bin;
  delete h;
}
struct gsl_histogram2d_pdf {
  size_t nx, ny;
  std::vector<double> xrange, yrange, sum;
};
inline gsl_histogram2d_pdf* gsl_histogram2d_pdf_alloc(size_t nx, size_t ny) {
  return new gsl_histogram2d_pdf{nx, ny, {}, {}, {}};
}
inline int gsl_histogram2d_pdf_init(gsl_histogram2d_pdf* p, const gsl_histogram2d* h) {
  const size_t n = h->nx * h->ny;
  for (size_t i = 0; i < n; ++i)
    if (h->bin[i] < 0) return GSL_EDOM;
  p->xrange.assign(h->xrange, h->xrange + h->nx + 1);
  p->yrange.assign(h->yrange, h->yrange + h->ny + 1);
  p->sum = uo::gsl_cdf(h->bin, n);
  return 0;
}
inline int gsl_histogram2d_pdf_sample(const gsl_histogram2d_pdf* p, double r1, double r2,
                                      double* x, double* y) {
  if (r2 == 1.0) r2 = 0.0;
  if (r1 == 1.0) r1 = 0.0;
  const long k = uo::gsl_find(p->sum, r1);
  if (k < 0) refshim::unavailable("gsl_histogram2d_pdf_sample outside the pdf");
  const long i = k / (long)p->ny, j = k - i * (long)p->ny;
  const double delta = (r1 - p->sum[k]) / (p->sum[k + 1] - p->sum[k]);
  *x = p->xrange[i] + delta * (p->xrange[i + 1] - p->xrange[i]);
  *y = p->yrange[j] + r2 * (p->yrange[j + 1] - p->yrange[j]);
  return 0;
}
inline void gsl_histogram2d_pdf_free(gsl_histogram2d_pdf* p) { delete p; }

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
  virtual TObject* Clone(const char* = "") const { refshim::unavailable("Clone"); }
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
inline double refshim_rndm();  // gRandom->Rndm(), defined with TRandom below

// Histograms on uniform bins with ROOT's bin numbering (0 underflow, n + 1
// overflow; 2-D global bin = bx + (nx + 2) by).  What the luminosity path and
// the event loop call is real: contents, Clone, Write into the current
// stand-in file, and the 1-D GetRandom (TH1::ComputeIntegral + GetRandom on
// gRandom, oracle_gen_prims.hpp).
class TH1 : public TObject {
 public:
  TH1() = default;
  static void AddDirectory(bool = true) {}
  void SetDirectory(TDirectory*) {}
  const char* GetName() const { return name_.c_str(); }
  int GetNbinsX() const { return nx_; }
  int GetNbinsY() const { return ny_; }
  TAxis* GetXaxis() { refshim::unavailable("histogram axes"); }
  TAxis* GetYaxis() { refshim::unavailable("histogram axes"); }
  double GetBinContent(int bin) const { return a_.at(bin); }
  double GetBinContent(int bx, int by) const { return a_.at(bx + (nx_ + 2) * by); }
  void SetBinContent(int bin, double v) {
    a_.at(bin) = v;
    integral_.clear();
  }
  void SetBinContent(int bx, int by, double v) {
    a_.at(bx + (nx_ + 2) * by) = v;
    integral_.clear();
  }
  double GetRandom() {
    if (ny_ != 0) refshim::unavailable("GetRandom of a 2-D histogram");
    if (integral_.empty()) integral_ = uo::th1_integral(a_.data() + 1, nx_);
    return uo::th1_sample(integral_, nx_, xmin_, xmax_, refshim_rndm());
  }
  double Interpolate(double) { refshim::unavailable("histograms"); }
  double Interpolate(double, double) { refshim::unavailable("histograms"); }
  int FindBin(double) { refshim::unavailable("histograms"); }
  int FindBin(double, double) { refshim::unavailable("histograms"); }
  int Fill(double) { refshim::unavailable("histograms"); }
  int Fill(double, double) { refshim::unavailable("histograms"); }
  void Scale(double) { refshim::unavailable("histograms"); }
  int Write(const char* = nullptr, int = 0, int = 0) override;

 protected:
  void book(const char* name, int nx, double x0, double x1, int ny, double y0, double y1) {
    name_ = name ? name : "";
    nx_ = nx, ny_ = ny, xmin_ = x0, xmax_ = x1, ymin_ = y0, ymax_ = y1;
    a_.assign(ny == 0 ? nx + 2 : (size_t)(nx + 2) * (ny + 2), 0.0);
  }
  std::string name_;
  int nx_ = 0, ny_ = 0;  // ny_ = 0: 1-D
  double xmin_ = 0, xmax_ = 0, ymin_ = 0, ymax_ = 0;
  std::vector<double> a_;
  std::vector<double> integral_;
};
class TH1D : public TH1 {
 public:
  TH1D() = default;
  TH1D(const char* name, const char*, int n, double x0, double x1) { book(name, n, x0, x1, 0, 0, 0); }
  TH1D(const char*, const char*, int, const double*) { refshim::unavailable("variable bins"); }
  TObject* Clone(const char* name = "") const override {
    auto* c = new TH1D(*this);
    if (name && *name) c->name_ = name;
    return c;
  }
};
class TH2D : public TH1 {
 public:
  TH2D() = default;
  TH2D(const char* name, const char*, int nx, double x0, double x1, int ny, double y0, double y1) {
    book(name, nx, x0, x1, ny, y0, y1);
  }
  TH2D(const char*, const char*, int, const double*, int, const double*) {}
  TH1D* ProjectionX(const char* = "_px") { refshim::unavailable("histograms"); }
  TH1D* ProjectionY(const char* = "_py") { refshim::unavailable("histograms"); }
  TObject* Clone(const char* name = "") const override {
    auto* c = new TH2D(*this);
    if (name && *name) c->name_ = name;
    return c;
  }
};

// The luminosity's ROOT file, in memory: TFile(name, "recreate") opens an
// empty file and makes it current, an object's Write() stores a copy of it
// there, TFile(name) opens it again and Get() returns a copy.
namespace refshim {
struct FileStore {
  std::mutex mu;
  std::map<std::string, std::map<std::string, std::shared_ptr<TObject>>> files;
  std::string current;
};
inline FileStore& files() {
  static FileStore st;
  return st;
}
}  // namespace refshim

inline int TH1::Write(const char*, int, int) {
  auto& st = refshim::files();
  std::lock_guard<std::mutex> lock(st.mu);
  if (st.current.empty()) refshim::unavailable("TH1::Write without an open file");
  st.files[st.current][name_] = std::shared_ptr<TObject>(Clone());
  return 1;
}

class TDirectory : public TObject {};
class TFile : public TDirectory {
 public:
  TFile() = default;
  TFile(const char* name, const char* opt = "", const char* = "", int = 0) : name_(name) {
    const std::string o = opt ? opt : "";
    auto& st = refshim::files();
    std::lock_guard<std::mutex> lock(st.mu);
    if (o == "recreate" || o == "RECREATE" || o == "new" || o == "NEW" || o == "create" ||
        o == "CREATE") {
      st.files[name_].clear();
    } else if (!st.files.count(name_)) {
      zombie_ = true;
      return;
    }
    st.current = name_;
  }
  TObject* Get(const char* key) {
    auto& st = refshim::files();
    std::lock_guard<std::mutex> lock(st.mu);
    auto f = st.files.find(name_);
    if (f == st.files.end()) return nullptr;
    auto o = f->second.find(key);
    return o == f->second.end() ? nullptr : o->second->Clone();
  }
  bool IsOpen() const { return !zombie_; }
  bool IsZombie() const { return zombie_; }
  void Close(const char* = "") {
    auto& st = refshim::files();
    std::lock_guard<std::mutex> lock(st.mu);
    if (st.current == name_) st.current.clear();
  }
  int Write(const char* = nullptr, int = 0, int = 0) override { return 0; }

 private:
  std::string name_;
  bool zombie_ = false;
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
  double Mag2() const { return x_ * x_ + y_ * y_ + z_ * z_; }
  double Mag() const { return std::sqrt(Mag2()); }
  void SetMagThetaPhi(double mag, double theta, double phi) {
    const double amag = std::fabs(mag);
    x_ = amag * std::sin(theta) * std::cos(phi);
    y_ = amag * std::sin(theta) * std::sin(phi);
    z_ = amag * std::cos(theta);
  }
  TVector3 operator-() const { return TVector3(-x_, -y_, -z_); }
  TVector3 Unit() const {
    double u[3];
    uo::unit3(x_, y_, z_, u);
    return TVector3(u[0], u[1], u[2]);
  }
  void RotateUz(const TVector3& u) {
    uo::Vec4 p{x_, y_, z_, 0.};
    uo::rotate_uz(p, u.x_, u.y_, u.z_);
    x_ = p.x, y_ = p.y, z_ = p.z;
  }

 private:
  double x_ = 0, y_ = 0, z_ = 0;
};
class TLorentzVector {
 public:
  TLorentzVector() = default;
  TLorentzVector(double px, double py, double pz, double e) : p_{px, py, pz, e} {}
  void SetPxPyPzE(double px, double py, double pz, double e) { p_ = uo::Vec4{px, py, pz, e}; }
  void SetXYZM(double x, double y, double z, double m) { p_ = uo::set_vect_m(x, y, z, m); }
  void SetVectM(const TVector3& v, double m) { SetXYZM(v.X(), v.Y(), v.Z(), m); }
  double Px() const { return p_.x; }
  double Py() const { return p_.y; }
  double Pz() const { return p_.z; }
  double E() const { return p_.t; }
  double Pt() const { return uo::pt_of(p_); }
  double Mag2() const { return uo::mag2_of(p_); }
  double Mag() const { return uo::mag_of(p_); }
  double M() const { return uo::mag_of(p_); }
  double Eta() const { return uo::eta_of(p_); }
  double Phi() const { refshim::unavailable("TLorentzVector::Phi"); }
  double Rapidity() const { refshim::unavailable("TLorentzVector::Rapidity"); }
  TVector3 Vect() const { return TVector3(p_.x, p_.y, p_.z); }
  TVector3 BoostVector() const { return TVector3(p_.x / p_.t, p_.y / p_.t, p_.z / p_.t); }
  void Boost(const TVector3& b) { Boost(b.X(), b.Y(), b.Z()); }
  void Boost(double bx, double by, double bz) { uo::boost(p_, bx, by, bz); }
  void RotateUz(const TVector3& u) { uo::rotate_uz(p_, u.X(), u.Y(), u.Z()); }
  TLorentzVector operator+(const TLorentzVector& o) const {
    return TLorentzVector(p_.x + o.p_.x, p_.y + o.p_.y, p_.z + o.p_.z, p_.t + o.p_.t);
  }

 private:
  uo::Vec4 p_{0, 0, 0, 0};
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
  virtual double Rndm() { refshim::unavailable("TRandom::Rndm"); }
  double Uniform(double x1 = 1.) { return x1 * Rndm(); }
  double Uniform(double x1, double x2) { return x1 + (x2 - x1) * Rndm(); }
  virtual void SetSeed(unsigned long) {}
};
template <class T>
class TRandomGen : public TRandom {};
class TRandomMT64 : public TRandom {  // the 64-bit Mersenne twister (oracle_gen_prims.hpp)
 public:
  double Rndm() override { return g_.rndm(); }
  void SetSeed(unsigned long s) override { g_ = uo::RootMT64(s); }

 private:
  uo::RootMT64 g_;
};
inline TRandom* gRandom = nullptr;
inline double refshim_rndm() {
  if (!gRandom) refshim::unavailable("gRandom before the generator's init");
  return gRandom->Rndm();
}

// AccessPathName follows ROOT's sense: true when the path can NOT be accessed
// (neither a stand-in file written in this process nor a file on disk)
class TSystem : public TObject {
 public:
  bool AccessPathName(const char* path) {
    {
      auto& st = refshim::files();
      std::lock_guard<std::mutex> lock(st.mu);
      if (st.files.count(path)) return false;
    }
    std::FILE* f = std::fopen(path, "r");
    if (!f) return true;
    std::fclose(f);
    return false;
  }
  int Exec(const char*) { refshim::unavailable("gSystem"); }
  int Unlink(const char*) { refshim::unavailable("gSystem"); }
};
inline TSystem refshim_system;
inline TSystem* gSystem = &refshim_system;
class TROOT : public TObject {};
inline TROOT* gROOT = nullptr;
namespace ROOT {
inline void EnableThreadSafety() {}
}  // namespace ROOT
