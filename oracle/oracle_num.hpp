// CPU oracle -- numerical primitives.
//
// TEST INFRASTRUCTURE ONLY.  This file is part of the FP64 CPU restatement of
// upcgen's luminosity / cross-section / sampling path that the tests and the
// CPU-baseline leg of bench.py use as a checker.  Product code never includes,
// links or calls anything under oracle/.
//
// The reference obtains these primitives from GSL and ROOT, which are not
// present here.  Each one is re-derived from its published mathematics:
//   * gsl_sf_bessel_K0/K1 (src/UpcCrossSection.cpp:171-172): any FP64-accurate
//     K0/K1; here the ascending series (A&S 9.6.11/9.6.13) for x<=2 and the
//     trapezoid rule on K_nu(x)=int_0^inf exp(-x cosh t) cosh(nu t) dt
//     (A&S 9.6.24) above, plus the Hankel asymptotic series for x>30.
//   * TMath::BesselK1 (src/UpcCrossSection.cpp:982-999): ROOT documents it as
//     the Abramowitz & Stegun polynomial approximations 9.8.3 / 9.8.7 / 9.8.8;
//     the published coefficients are used verbatim because the breakup
//     probability inherits their ~1e-7 error.
//   * gsl_interp_cspline natural cubic spline (src/UpcCrossSection.cpp:385-387,
//     411-413, 431-433, 458-460): the textbook natural spline (second
//     derivatives from the symmetric tridiagonal system, zero at both ends).
//   * gsl_integration_qags (src/UpcCrossSection.cpp:209): QUADPACK QAGS
//     (Piessens et al. 1983): 21-point Gauss-Kronrod rule, bisection of the
//     interval with the largest error, Wynn epsilon extrapolation.  GSL's
//     variant is followed where it differs from the Fortran original (the
//     epsilon table's result history is updated after, not before, use).
//   * simpson (src/UpcCrossSection.cpp:139-150), restated as written.
#pragma once

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstddef>
#include <vector>

namespace uo {

// ---------------------------------------------------------------- Simpson --
// src/UpcCrossSection.cpp:139-150 (the reference applies it to an even number
// of points as well; the same weights are kept).
inline double simpson(int n, const double* v, double h) {
  double sum = v[0] + v[n - 1];
  for (int i = 1; i < n - 1; i += 2) sum += 4. * v[i];
  for (int i = 2; i < n - 1; i += 2) sum += 2. * v[i];
  return sum * h / 3.;
}

// --------------------------------------------------- natural cubic spline --
// Piecewise cubic S_i(x) = y_i + d (b_i + d (c_i + d e_i)), d = x - x_i, with
// c_i = S''(x_i)/2 solved from the natural-spline tridiagonal system.
struct NaturalSpline {
  std::vector<double> x, y, c;
  void build(const double* xs, const double* ys, int n) {
    x.assign(xs, xs + n);
    y.assign(ys, ys + n);
    c.assign(n, 0.0);
    const int m = n - 2;  // unknowns c_1 .. c_{n-2}
    if (m <= 0) return;
    std::vector<double> diag(m), off(m), rhs(m);
    for (int i = 0; i < m; ++i) {
      const double h0 = x[i + 1] - x[i];
      const double h1 = x[i + 2] - x[i + 1];
      diag[i] = 2.0 * (h0 + h1);
      off[i] = h1;
      rhs[i] = 3.0 * ((y[i + 2] - y[i + 1]) / h1 - (y[i + 1] - y[i]) / h0);
    }
    // Thomas elimination for the symmetric tridiagonal matrix.
    std::vector<double> cp(m), dp(m);
    cp[0] = off[0] / diag[0];
    dp[0] = rhs[0] / diag[0];
    for (int i = 1; i < m; ++i) {
      const double den = diag[i] - off[i - 1] * cp[i - 1];
      cp[i] = off[i] / den;
      dp[i] = (rhs[i] - off[i - 1] * dp[i - 1]) / den;
    }
    c[m] = dp[m - 1];
    for (int i = m - 2; i >= 0; --i) c[i + 1] = dp[i] - cp[i] * c[i + 2];
  }
  // Interval i with x_i <= xx < x_{i+1}; the last knot maps to the last
  // interval; values outside the knot range use the edge polynomial (GSL >= 2
  // would raise GSL_EDOM there instead).
  int interval(double xx) const {
    const int n = (int)x.size();
    int i = (int)(std::upper_bound(x.begin(), x.end(), xx) - x.begin()) - 1;
    if (i < 0) i = 0;
    if (i > n - 2) i = n - 2;
    return i;
  }
  double eval(double xx) const {
    const int i = interval(xx);
    const double h = x[i + 1] - x[i];
    const double dy = y[i + 1] - y[i];
    const double d = xx - x[i];
    const double b = dy / h - h * (c[i + 1] + 2.0 * c[i]) / 3.0;
    const double e = (c[i + 1] - c[i]) / (3.0 * h);
    return y[i] + d * (b + d * (c[i] + d * e));
  }
};

// ---------------------------------------------------- modified Bessel K --
constexpr double kEulerGamma = 0.57721566490153286061;

// Ascending series, valid and accurate for 0 < x <= 2.
inline void bessel_k01_series(double x, double* k0, double* k1) {
  const double t = 0.25 * x * x;
  const double lg = std::log(0.5 * x);
  double i0 = 0, i1s = 0, s0 = 0, s1 = 0;
  double term0 = 1.0;   // t^k / (k!)^2
  double term1 = 1.0;   // t^k / (k! (k+1)!)
  double hk = 0.0;      // harmonic number H_k
  for (int k = 0; k < 40; ++k) {
    if (k > 0) {
      term0 *= t / ((double)k * (double)k);
      term1 *= t / ((double)k * (double)(k + 1));
      hk += 1.0 / k;
    }
    i0 += term0;
    i1s += term1;
    s0 += hk * term0;                               // sum_{k>=1} H_k t^k/(k!)^2
    s1 += (-2.0 * kEulerGamma + 2.0 * hk + 1.0 / (k + 1)) * term1;  // psi(k+1)+psi(k+2)
    if (term0 < 1e-18 * i0 && k > 2) break;
  }
  const double i1 = 0.5 * x * i1s;
  *k0 = -(lg + kEulerGamma) * i0 + s0;
  *k1 = 1.0 / x + lg * i1 - 0.25 * x * s1;
}

// Trapezoid rule on the integral representation, x > 2.
inline void bessel_k01_integral(double x, double* k0, double* k1) {
  const double h = 0.125;
  double s0 = 0.5, s1 = 0.5;
  for (int n = 1; n < 400; ++n) {
    const double t = n * h;
    const double sh = std::sinh(0.5 * t);
    const double cm1 = 2.0 * sh * sh;  // cosh t - 1
    const double e = std::exp(-x * cm1);
    s0 += e;
    s1 += e * (1.0 + cm1);
    if (x * cm1 > 50.0) break;
  }
  const double ex = std::exp(-x) * h;
  *k0 = s0 * ex;
  *k1 = s1 * ex;
}

// Hankel asymptotic series, x > 30 (truncation error below e^{-2x}).
inline void bessel_k01_asym(double x, double* k0, double* k1) {
  const double pre = std::sqrt(M_PI / (2.0 * x)) * std::exp(-x);
  double a0 = 1.0, a1 = 1.0, t0 = 1.0, t1 = 1.0;
  for (int k = 1; k < 30; ++k) {
    const double q = 2.0 * k - 1.0;
    t0 *= (0.0 - q * q) / (k * 8.0 * x);
    t1 *= (4.0 - q * q) / (k * 8.0 * x);
    a0 += t0;
    a1 += t1;
    if (std::fabs(t0) < 1e-18 && std::fabs(t1) < 1e-18) break;
  }
  *k0 = pre * a0;
  *k1 = pre * a1;
}

inline void bessel_k01(double x, double* k0, double* k1) {
  if (x <= 2.0) bessel_k01_series(x, k0, k1);
  else if (x <= 30.0) bessel_k01_integral(x, k0, k1);
  else bessel_k01_asym(x, k0, k1);
}

// Abramowitz & Stegun 9.8.3 (I1, |x| < 3.75) -- the branch K1 needs.
inline double bessel_i1_as(double x) {
  const double y = (x / 3.75) * (x / 3.75);
  return x * (0.5 + y * (0.87890594 + y * (0.51498869 + y * (0.15084934 +
              y * (0.2658733e-1 + y * (0.301532e-2 + y * 0.32411e-3))))));
}

// Abramowitz & Stegun 9.8.7 (x <= 2) and 9.8.8 (x > 2).
inline double bessel_k1_as(double x) {
  if (x <= 0) return 0;
  if (x <= 2) {
    const double y = x * x / 4;
    return std::log(x / 2) * bessel_i1_as(x) +
           (1 / x) * (1. + y * (0.15443144 + y * (-0.67278579 + y * (-0.18156897 +
           y * (-0.1919402e-1 + y * (-0.110404e-2 + y * (-0.4686e-4)))))));
  }
  const double y = 2 / x;
  return (std::exp(-x) / std::sqrt(x)) *
         (1.25331414 + y * (0.23498619 + y * (-0.3655620e-1 + y * (0.1504268e-1 +
          y * (-0.780353e-2 + y * (0.325614e-2 + y * (-0.68245e-3)))))));
}

// -------------------------------------------------------------- QAGS ----
// 21-point Gauss-Kronrod nodes and weights (Kronrod extension of the 10-point
// Gauss rule); these are mathematical constants, checked in the tests for
// exactness on polynomials of degree <= 31 (Kronrod) and <= 19 (Gauss).
struct GK21 {
  static constexpr double xgk[11] = {
      0.995657163025808080735527280689003, 0.973906528517171720077964012084452,
      0.930157491355708226001207180059508, 0.865063366688984510732096688423493,
      0.780817726586416897063717578345042, 0.679409568299024406234327365114874,
      0.562757134668604683339000099272694, 0.433395394129247190799265943165784,
      0.294392862701460198131126603103866, 0.148874338981631210884826001129720,
      0.000000000000000000000000000000000};
  static constexpr double wgk[11] = {
      0.011694638867371874278064396062192, 0.032558162307964727478818972459390,
      0.054755896574351996031381300244580, 0.075039674810919952767043140916190,
      0.093125454583697605535065465083366, 0.109387158802297641899210590325805,
      0.123491976262065851077208980430855, 0.134709217311473325928054001771707,
      0.142775938577060080797094273138717, 0.147739104901338491374841515972068,
      0.149445554002916905664936468389821};
  static constexpr double wg[5] = {
      0.066671344308688137593568809893332, 0.149451349150580593145776339657697,
      0.219086362515982043995534934228163, 0.269266719309996355091226921569469,
      0.295524224714752870173892994651338};
};

inline double qk_rescale_error(double err, double resabs, double resasc) {
  err = std::fabs(err);
  if (resasc != 0 && err != 0) {
    const double scale = std::pow(200 * err / resasc, 1.5);
    err = scale < 1 ? resasc * scale : resasc;
  }
  if (resabs > DBL_MIN / (50 * DBL_EPSILON)) {
    const double floor_err = 50 * DBL_EPSILON * resabs;
    if (floor_err > err) err = floor_err;
  }
  return err;
}

template <class F>
inline void qk21(F& f, double a, double b, double* result, double* abserr,
                 double* resabs, double* resasc) {
  const double center = 0.5 * (a + b);
  const double half = 0.5 * (b - a);
  const double fc = f(center);
  double fv1[10], fv2[10];
  double resg = 0.0;
  double resk = fc * GK21::wgk[10];
  double rabs = std::fabs(resk);
  for (int j = 0; j < 5; ++j) {           // nodes shared with the Gauss rule
    const int n = 2 * j + 1;
    const double dx = half * GK21::xgk[n];
    const double f1 = f(center - dx), f2 = f(center + dx);
    fv1[n] = f1;
    fv2[n] = f2;
    resg += GK21::wg[j] * (f1 + f2);
    resk += GK21::wgk[n] * (f1 + f2);
    rabs += GK21::wgk[n] * (std::fabs(f1) + std::fabs(f2));
  }
  for (int j = 0; j < 5; ++j) {           // Kronrod-only nodes
    const int n = 2 * j;
    const double dx = half * GK21::xgk[n];
    const double f1 = f(center - dx), f2 = f(center + dx);
    fv1[n] = f1;
    fv2[n] = f2;
    resk += GK21::wgk[n] * (f1 + f2);
    rabs += GK21::wgk[n] * (std::fabs(f1) + std::fabs(f2));
  }
  const double mean = 0.5 * resk;
  double rasc = GK21::wgk[10] * std::fabs(fc - mean);
  for (int j = 0; j < 10; ++j)
    rasc += GK21::wgk[j] * (std::fabs(fv1[j] - mean) + std::fabs(fv2[j] - mean));
  const double err = (resk - resg) * half;
  *result = resk * half;
  *resabs = rabs * std::fabs(half);
  *resasc = rasc * std::fabs(half);
  *abserr = qk_rescale_error(err, *resabs, *resasc);
}

// Status codes follow GSL's numbering of QAGS outcomes:
// 0 success, 11 max iterations, 18 roundoff, 21 bad integrand,
// 22 extrapolation-table roundoff, 23 divergent.
struct QagsResult {
  double result = 0, abserr = 0;
  int neval = 0, nintervals = 0, status = 0;
};

// Adaptive bisection workspace: interval list plus an index list kept sorted
// by decreasing error estimate (the QUADPACK "qpsrt" insertion policy).
struct QagsList {
  int limit = 0, size = 0, nrmax = 0, cur = 0, max_level = 0;
  std::vector<double> lo, hi, r, e;
  std::vector<int> order, level;
  explicit QagsList(int lim)
      : limit(lim), lo(lim), hi(lim), r(lim), e(lim), order(lim), level(lim) {}

  void start(double a, double b, double r0, double e0) {
    size = 1; nrmax = 0; cur = 0; max_level = 0;
    lo[0] = a; hi[0] = b; r[0] = r0; e[0] = e0; order[0] = 0; level[0] = 0;
  }
  void keep_sorted() {
    const int last = size - 1;
    int nr = nrmax;
    int imax = order[nr];
    if (last < 2) {
      order[0] = 0; order[1] = 1; cur = imax;
      return;
    }
    const double emax = e[imax];
    while (nr > 0 && emax > e[order[nr - 1]]) {
      order[nr] = order[nr - 1];
      --nr;
    }
    const int top = (last < limit / 2 + 2) ? last : limit - last + 1;
    int i = nr + 1;
    while (i < top && emax < e[order[i]]) {
      order[i - 1] = order[i];
      ++i;
    }
    order[i - 1] = imax;
    const double emin = e[last];
    int k = top - 1;
    while (k > i - 2 && emin >= e[order[k]]) {
      order[k + 1] = order[k];
      --k;
    }
    order[k + 1] = last;
    cur = order[nr];
    nrmax = nr;
  }
  // Replace the bisected interval by its halves (larger error keeps the slot).
  void split(double a1, double b1, double r1, double e1,
             double a2, double b2, double r2, double e2) {
    const int im = cur, in = size;
    const int lv = level[im] + 1;
    if (e2 > e1) {
      lo[im] = a2; r[im] = r2; e[im] = e2; level[im] = lv;
      lo[in] = a1; hi[in] = b1; r[in] = r1; e[in] = e1; level[in] = lv;
    } else {
      hi[im] = b1; r[im] = r1; e[im] = e1; level[im] = lv;
      lo[in] = a2; hi[in] = b2; r[in] = r2; e[in] = e2; level[in] = lv;
    }
    ++size;
    if (lv > max_level) max_level = lv;
    keep_sorted();
  }
  bool cur_is_large() const { return level[cur] < max_level; }
  void reset_to_largest() { nrmax = 0; cur = order[0]; }
  bool advance_to_large() {
    const int last = size - 1;
    const int bound = (last > 1 + limit / 2) ? limit + 1 - last : last;
    for (int k = nrmax; k <= bound; ++k) {
      cur = order[nrmax];
      if (level[cur] < max_level) return true;
      ++nrmax;
    }
    return false;
  }
  double total() const {
    double s = 0;
    for (int k = 0; k < size; ++k) s += r[k];
    return s;
  }
};

// Wynn epsilon table with the 3-result error history.
struct EpsTable {
  int n = 0, nres = 0;
  double tab[52];
  double hist[3];
  void push(double v) {
    if (n < 52) { tab[n] = v; ++n; }
  }
  void extrapolate(double* result, double* abserr) {
    const int n0 = n - 1;
    const double cur = tab[n0];
    *result = cur;
    *abserr = DBL_MAX;
    if (n0 < 2) {
      *abserr = std::max(DBL_MAX, 5 * DBL_EPSILON * std::fabs(cur));
      return;
    }
    tab[n0 + 2] = tab[n0];
    const int newelm = n0 / 2;
    tab[n0] = DBL_MAX;
    int nfin = n0;
    bool converged = false;
    for (int i = 0; i < newelm; ++i) {
      double res = tab[n0 - 2 * i + 2];
      const double e0 = tab[n0 - 2 * i - 2];
      const double e1 = tab[n0 - 2 * i - 1];
      const double e2 = res;
      const double d2 = e2 - e1, a2 = std::fabs(d2);
      const double t2 = std::max(std::fabs(e2), std::fabs(e1)) * DBL_EPSILON;
      const double d3 = e1 - e0, a3 = std::fabs(d3);
      const double t3 = std::max(std::fabs(e1), std::fabs(e0)) * DBL_EPSILON;
      if (a2 < t2 && a3 < t3) {
        *result = res;
        *abserr = std::max(a2 + a3, 5 * DBL_EPSILON * std::fabs(res));
        converged = true;
        break;
      }
      const double e3 = tab[n0 - 2 * i];
      tab[n0 - 2 * i] = e1;
      const double d1 = e1 - e3, a1 = std::fabs(d1);
      const double t1 = std::max(std::fabs(e1), std::fabs(e3)) * DBL_EPSILON;
      if (a1 < t1 || a2 < t2 || a3 < t3) {
        nfin = 2 * i;
        break;
      }
      const double ss = (1 / d1 + 1 / d2) - 1 / d3;
      if (std::fabs(ss * e1) <= 1e-4) {
        nfin = 2 * i;
        break;
      }
      res = e1 + 1 / ss;
      tab[n0 - 2 * i] = res;
      const double err = a2 + std::fabs(res - e2) + a3;
      if (err <= *abserr) {
        *abserr = err;
        *result = res;
      }
    }
    if (converged) return;
    if (nfin == 49) nfin = 2 * (49 / 2);
    if (n0 % 2 == 1) {
      for (int i = 0; i <= newelm; ++i) tab[1 + 2 * i] = tab[2 * i + 3];
    } else {
      for (int i = 0; i <= newelm; ++i) tab[2 * i] = tab[2 * i + 2];
    }
    if (n0 != nfin)
      for (int i = 0; i <= nfin; ++i) tab[i] = tab[n0 - nfin + i];
    n = nfin + 1;
    if (nres < 3) {
      hist[nres] = *result;
      *abserr = DBL_MAX;
    } else {
      *abserr = std::fabs(*result - hist[2]) + std::fabs(*result - hist[1]) +
                std::fabs(*result - hist[0]);
      hist[0] = hist[1];
      hist[1] = hist[2];
      hist[2] = *result;
    }
    ++nres;
    *abserr = std::max(*abserr, 5 * DBL_EPSILON * std::fabs(*result));
  }
};

template <class F>
QagsResult qags(F f, double a, double b, double epsabs, double epsrel, int limit) {
  QagsResult out;
  int neval = 0;
  auto fc = [&](double x) { ++neval; return f(x); };
  double r0, e0, rabs0, rasc0;
  qk21(fc, a, b, &r0, &e0, &rabs0, &rasc0);
  double tol = std::max(epsabs, epsrel * std::fabs(r0));
  out.nintervals = 1;
  if (e0 <= 100 * DBL_EPSILON * rabs0 && e0 > tol) {
    out.result = r0; out.abserr = e0; out.status = 18; out.neval = neval;
    return out;
  }
  if ((e0 <= tol && e0 != rasc0) || e0 == 0.0) {
    out.result = r0; out.abserr = e0; out.neval = neval;
    return out;
  }
  if (limit == 1) {
    out.result = r0; out.abserr = e0; out.status = 11; out.neval = neval;
    return out;
  }
  QagsList ws(limit);
  ws.start(a, b, r0, e0);
  EpsTable tab;
  tab.push(r0);
  double area = r0, errsum = e0, res_ext = r0, err_ext = DBL_MAX;
  double ertest = 0, err_large = 0, correc = 0;
  int ktmin = 0, rt1 = 0, rt2 = 0, rt3 = 0, err_type = 0, err_type2 = 0;
  int iter = 1;
  const bool positive = std::fabs(r0) >= (1 - 50 * DBL_EPSILON) * rabs0;
  bool extrap = false, no_extrap = false;
  bool final_sum = false;  // result = sum over intervals (vs extrapolated)
  bool goto_return = false;

  do {
    const int im = ws.cur;
    const double ai = ws.lo[im], bi = ws.hi[im], ri = ws.r[im], ei = ws.e[im];
    const int lvl = ws.level[im] + 1;
    const double a1 = ai, b1 = 0.5 * (ai + bi), a2 = b1, b2 = bi;
    ++iter;
    double ar1, er1, rb1, rc1, ar2, er2, rb2, rc2;
    qk21(fc, a1, b1, &ar1, &er1, &rb1, &rc1);
    qk21(fc, a2, b2, &ar2, &er2, &rb2, &rc2);
    const double ar12 = ar1 + ar2, er12 = er1 + er2;
    errsum = errsum + er12 - ei;
    area = area + ar12 - ri;
    tol = std::max(epsabs, epsrel * std::fabs(area));
    if (rc1 != er1 && rc2 != er2) {
      const double delta = ri - ar12;
      if (std::fabs(delta) <= 1.0e-5 * std::fabs(ar12) && er12 >= 0.99 * ei) {
        if (!extrap) ++rt1; else ++rt2;
      }
      if (iter > 10 && er12 > ei) ++rt3;
    }
    if (rt1 + rt2 >= 10 || rt3 >= 20) err_type = 2;
    if (rt2 >= 5) err_type2 = 1;
    {
      const double tmp = (1 + 100 * DBL_EPSILON) * (std::fabs(a2) + 1000 * DBL_MIN);
      if (std::fabs(a1) <= tmp && std::fabs(b2) <= tmp) err_type = 4;
    }
    ws.split(a1, b1, ar1, er1, a2, b2, ar2, er2);
    if (errsum <= tol) { final_sum = true; break; }
    if (err_type) break;
    if (iter >= limit - 1) { err_type = 1; break; }
    if (iter == 2) {
      err_large = errsum;
      ertest = tol;
      tab.push(area);
      continue;
    }
    if (no_extrap) continue;
    err_large += -ei;
    if (lvl < ws.max_level) err_large += er12;
    if (!extrap) {
      if (ws.cur_is_large()) continue;
      extrap = true;
      ws.nrmax = 1;
    }
    if (!err_type2 && err_large > ertest) {
      if (ws.advance_to_large()) continue;
    }
    tab.push(area);
    double reseps, abseps;
    tab.extrapolate(&reseps, &abseps);
    ++ktmin;
    if (ktmin > 5 && err_ext < 0.001 * errsum) err_type = 5;
    if (abseps < err_ext) {
      ktmin = 0;
      err_ext = abseps;
      res_ext = reseps;
      correc = err_large;
      ertest = std::max(epsabs, epsrel * std::fabs(reseps));
      if (err_ext <= ertest) break;
    }
    if (tab.n == 1) no_extrap = true;
    if (err_type == 5) break;
    ws.reset_to_largest();
    extrap = false;
    err_large = errsum;
  } while (iter < limit);

  if (!final_sum) {
    out.result = res_ext;
    out.abserr = err_ext;  // reported before the roundoff correction below
    if (err_ext == DBL_MAX) {
      final_sum = true;
    } else {
      if (err_type || err_type2) {
        if (err_type2) err_ext += correc;
        if (err_type == 0) err_type = 3;
        if (res_ext != 0.0 && area != 0.0) {
          if (err_ext / std::fabs(res_ext) > errsum / std::fabs(area)) final_sum = true;
        } else if (err_ext > errsum) {
          final_sum = true;
        } else if (area == 0.0) {
          goto_return = true;
        }
      }
      if (!final_sum && !goto_return) {
        const double max_area = std::max(std::fabs(res_ext), std::fabs(area));
        if (!(!positive && max_area < 0.01 * rabs0)) {
          const double ratio = res_ext / area;
          if (ratio < 0.01 || ratio > 100.0 || errsum > std::fabs(area)) err_type = 6;
        }
      }
    }
  }
  if (final_sum) {
    out.result = ws.total();
    out.abserr = errsum;
  }
  if (err_type > 2) --err_type;
  static const int code[] = {0, 11, 18, 21, 18, 22};
  out.status = code[err_type < 0 ? 0 : (err_type > 5 ? 5 : err_type)];
  out.neval = neval;
  out.nintervals = ws.size;
  return out;
}

}  // namespace uo
