// Device-side numerics shared by the upcgen GB300 kernels.
//
// Special functions the reference takes from GSL / ROOT, written from their
// published mathematics (CUDA has no K0/K1):
//   * K0, K1 (gsl_sf_bessel_K0/K1 in src/UpcCrossSection.cpp:171-172):
//     ascending series (A&S 9.6.11/9.6.13) for x <= 2, trapezoid rule on
//     K_nu(x) = int_0^inf exp(-x cosh t) cosh(nu t) dt (A&S 9.6.24) with step
//     0.15 for 2 < x <= 18.5 (aliasing error below exp(-(2 pi / h)^2 / 2x) <
//     1e-17), Hankel asymptotic series above 18.5 (truncation below e^{-2x}).
//   * K1 of ROOT's TMath::BesselK1 (src/UpcCrossSection.cpp:982-999): the
//     Abramowitz & Stegun polynomials 9.8.3 / 9.8.7 / 9.8.8, whose ~1e-7
//     error the breakup probability inherits.
//   * natural cubic splines (gsl_interp_cspline) as per-interval polynomial
//     coefficients {y_i, b_i, c_i, d_i}; the interval of x is the one a
//     binary search over the knots x_i = x0 + i*h would return.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace upcg {

constexpr double kAlpha = 1.0 / 137.035999074;  // include/UpcPhysConstants.h:26-32
constexpr double kHc = 0.1973269718;
constexpr double kMProt = 0.9382720813;
constexpr double kMNeut = 0.939565346;
constexpr double kMEl = 0.000510998946;
constexpr double kMMu = 0.1056583745;
constexpr double kMTau = 1.77686;
constexpr double kPi = 3.14159265358979323846;
constexpr double kEulerGamma = 0.57721566490153286061;

// cosh(n h) - 1 for h = 0.15, n = 1..40 (2 sinh^2(n h / 2)).
__constant__ static double kCoshM1[40] = {
    0.011271109576670463, 0.045338514128860481, 0.10297016855597102, 0.18546521824226767,
    0.29468328467684468, 0.43308638544877426, 0.60379443358715978, 0.8106555673243746,
    1.0583328956714328, 1.3524096152432474, 1.6995148679003012, 2.1074731763172654,
    2.585480826087903, 3.144313170410316, 3.7965675304601945, 4.5569471669655064,
    5.4425927243320906, 6.4734686188062902, 7.67281308072124, 9.0676619957777636,
    10.689458353904875, 12.574761044029561, 14.766068972562996, 17.31277908306263,
    20.272299872959394, 23.71134550848798, 27.707439710042841, 32.350663308872811,
    37.745684868920648, 44.014120148530033, 51.297273589522334, 59.759323632891935,
    69.591023665202954, 81.014002023233587, 94.28575798851459, 109.70546639256477,
    127.6207216815091, 148.43537346625885, 172.61863018894627, 200.71563612245592};

__device__ __forceinline__ void bessel_k01(double x, double& k0, double& k1) {
  if (x <= 2.0) {
    const double t = 0.25 * x * x;
    const double lg = log(0.5 * x);
    double i0 = 1.0, i1s = 1.0, s0 = 0.0;
    double s1 = -2.0 * kEulerGamma + 1.0;  // k = 0 term of psi(k+1)+psi(k+2)
    double term0 = 1.0, term1 = 1.0, hk = 0.0;
#pragma unroll 1
    for (int k = 1; k < 30; ++k) {
      const double dk = (double)k;
      term0 *= t / (dk * dk);
      term1 *= t / (dk * (dk + 1.0));
      hk += 1.0 / dk;
      i0 += term0;
      i1s += term1;
      s0 += hk * term0;
      s1 += (-2.0 * kEulerGamma + 2.0 * hk + 1.0 / (dk + 1.0)) * term1;
      if (term0 < 1e-18 * i0) break;
    }
    k0 = -(lg + kEulerGamma) * i0 + s0;
    k1 = 1.0 / x + lg * (0.5 * x * i1s) - 0.25 * x * s1;
  } else if (x <= 18.5) {
    double s0 = 0.5, s1 = 0.5;
#pragma unroll 1
    for (int n = 0; n < 40; ++n) {
      const double cm1 = kCoshM1[n];
      const double e = exp(-x * cm1);
      s0 += e;
      s1 += e * (1.0 + cm1);
      if (x * cm1 > 50.0) break;
    }
    const double ex = exp(-x) * 0.15;
    k0 = s0 * ex;
    k1 = s1 * ex;
  } else {
    const double pre = sqrt(kPi / (2.0 * x)) * exp(-x);
    double a0 = 1.0, a1 = 1.0, t0 = 1.0, t1 = 1.0;
#pragma unroll 1
    for (int k = 1; k < 40; ++k) {
      const double q = 2.0 * k - 1.0;
      t0 *= (0.0 - q * q) / (k * 8.0 * x);
      t1 *= (4.0 - q * q) / (k * 8.0 * x);
      a0 += t0;
      a1 += t1;
      if (fabs(t0) < 1e-18 && fabs(t1) < 1e-18) break;
    }
    k0 = pre * a0;
    k1 = pre * a1;
  }
}

// Abramowitz & Stegun 9.8.3 / 9.8.7 / 9.8.8 (TMath::BesselK1).
// calcFormFac (src/UpcCrossSection.cpp:436-445): the Woods-Saxon form factor
// (symmetrised-Fermi closed form), normalised to ~A at Q2 -> 0
__device__ __forceinline__ double calc_form_fac(double Q2, double rho0, double R, double a) {
  const double Q = sqrt(Q2) / kHc;
  const double coshVal = cosh(kPi * Q * a);
  const double sinhVal = sinh(kPi * Q * a);
  double ff = 4 * kPi * kPi * rho0 * a * a * a / (Q * a * Q * a * sinhVal * sinhVal) *
              (kPi * Q * a * coshVal * sin(Q * R) - Q * R * cos(Q * R) * sinhVal);
  ff += 8 * kPi * rho0 * a * a * a * exp(-R / a) / (1 + Q * Q * a * a) / (1 + Q * Q * a * a);
  return ff;
}

__device__ __forceinline__ double bessel_k1_as(double x) {
  if (x <= 0) return 0;
  if (x <= 2) {
    const double y = x * x / 4;
    const double u = (x / 3.75) * (x / 3.75);
    const double i1 = x * (0.5 + u * (0.87890594 + u * (0.51498869 + u * (0.15084934 +
                      u * (0.2658733e-1 + u * (0.301532e-2 + u * 0.32411e-3))))));
    return log(x / 2) * i1 +
           (1 / x) * (1. + y * (0.15443144 + y * (-0.67278579 + y * (-0.18156897 +
           y * (-0.1919402e-1 + y * (-0.110404e-2 + y * (-0.4686e-4)))))));
  }
  const double y = 2 / x;
  return (exp(-x) / sqrt(x)) *
         (1.25331414 + y * (0.23498619 + y * (-0.3655620e-1 + y * (0.1504268e-1 +
          y * (-0.780353e-2 + y * (0.325614e-2 + y * (-0.68245e-3)))))));
}

// Natural cubic spline on uniform knots x_i = x0 + i*h, i < n, stored as one
// double4 {y_i, b_i, c_i, d_i} per interval (n-1 of them).
struct SplineU {
  const double4* coef;
  double x0, h, inv_h;
  int n;
};

__device__ __forceinline__ int spline_interval(const SplineU& s, double x, double& xi) {
  int i = (int)floor((x - s.x0) * s.inv_h);
  i = i < 0 ? 0 : (i > s.n - 2 ? s.n - 2 : i);
  xi = s.x0 + i * s.h;
  if (x < xi && i > 0) {
    --i;
    xi = s.x0 + i * s.h;
  } else if (i < s.n - 2) {
    const double xn = s.x0 + (i + 1) * s.h;
    if (x >= xn) {
      ++i;
      xi = xn;
    }
  }
  return i;
}

__device__ __forceinline__ double4 ldg4(const double4* p) {
  const double2 lo = __ldg(reinterpret_cast<const double2*>(p));
  const double2 hi = __ldg(reinterpret_cast<const double2*>(p) + 1);
  return make_double4(lo.x, lo.y, hi.x, hi.y);
}

__device__ __forceinline__ double spline_eval(const SplineU& s, double x) {
  double xi;
  const int i = spline_interval(s, x, xi);
  const double4 c = ldg4(s.coef + i);
  const double d = x - xi;
  return c.x + d * (c.y + d * (c.z + d * c.w));
}

// Same, with the coefficients staged in shared memory.
__device__ __forceinline__ double spline_eval_smem(const SplineU& s, const double4* sc,
                                                   double x) {
  double xi;
  const int i = spline_interval(s, x, xi);
  const double4 c = sc[i];
  const double d = x - xi;
  return c.x + d * (c.y + d * (c.z + d * c.w));
}

// FP32 copy of a uniform-knot spline (coefficients {y, b, c, d} per interval)
struct SplineF {
  const float4* coef;
  float x0, h, inv_h;
  int n;
};

__device__ __forceinline__ float spline_eval_f(const SplineF& s, const float4* coef, float x) {
  int i = (int)floorf((x - s.x0) * s.inv_h);
  i = i < 0 ? 0 : (i > s.n - 2 ? s.n - 2 : i);
  float xi = s.x0 + i * s.h;
  if (x < xi && i > 0) {
    --i;
    xi = s.x0 + i * s.h;
  }
  const float4 c = coef[i];
  const float d = x - xi;
  return c.x + d * (c.y + d * (c.z + d * c.w));
}

// FP32 copy of n spline intervals
__global__ void k_coef_f32(const double4* __restrict__ in, float4* __restrict__ out, int n);

// 21-point Gauss-Kronrod rule (Kronrod extension of the 10-point Gauss rule).
__constant__ static double kXgk[11] = {
    0.995657163025808080735527280689003, 0.973906528517171720077964012084452,
    0.930157491355708226001207180059508, 0.865063366688984510732096688423493,
    0.780817726586416897063717578345042, 0.679409568299024406234327365114874,
    0.562757134668604683339000099272694, 0.433395394129247190799265943165784,
    0.294392862701460198131126603103866, 0.148874338981631210884826001129720,
    0.000000000000000000000000000000000};
__constant__ static double kWgk[11] = {
    0.011694638867371874278064396062192, 0.032558162307964727478818972459390,
    0.054755896574351996031381300244580, 0.075039674810919952767043140916190,
    0.093125454583697605535065465083366, 0.109387158802297641899210590325805,
    0.123491976262065851077208980430855, 0.134709217311473325928054001771707,
    0.142775938577060080797094273138717, 0.147739104901338491374841515972068,
    0.149445554002916905664936468389821};
__constant__ static double kWg[5] = {
    0.066671344308688137593568809893332, 0.149451349150580593145776339657697,
    0.219086362515982043995534934228163, 0.269266719309996355091226921569469,
    0.295524224714752870173892994651338};

// A CDF value in [0, 1] as 64-bit fixed point (1 and above: all ones)
__device__ __forceinline__ uint64_t cdf_to_fx(double v) {
  return v >= 1. ? ~0ull : (v > 0. ? (uint64_t)(v * 18446744073709551616.0) : 0ull);
}

}  // namespace upcg
