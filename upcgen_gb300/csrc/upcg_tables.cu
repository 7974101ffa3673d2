// Nuclear tables on the GPU: Woods-Saxon form factor, G_AA(b), Coulomb-breakup
// probability, and the natural cubic splines through them.
//
// Reference: src/UpcCrossSection.cpp
//   calcFormFac :436-445, prepareFormFac :447-461     -> k_formfac_values
//   prepareGAA :364-414                               -> k_ta_values, k_gaa_rows
//   calcBreakupProb :752-1019, prepareBreakupProb :416-434
//                                  -> breakup_energy_table (host), k_breakup_values
//   gsl_interp_cspline (natural) construction          -> k_spline_c, k_spline_coef
//
// The natural-spline system on uniform knots is solved by its closed-form
// inverse kernel (see k_spline_c): one independent dot product per knot, the
// same solution as a global tridiagonal solve to 1e-16, with 1e6 knots in
// one launch.
#include <algorithm>
#include <cmath>

#include "upcg_device.cuh"
#include "upcg_internal.h"

namespace upcg {

namespace {

// Natural cubic spline on uniform knots x_i = x0 + i h (gsl_interp_cspline).
// The second-derivative halves c_i solve c_{i-1} + 4 c_i + c_{i+1} = s_i with
// s_i = 3 (y_{i+1} - 2 y_i + y_{i-1}) / h^2 and c_0 = c_{n-1} = 0.  The
// inverse of the (1, 4, 1) operator on the infinite lattice is the kernel
// G_m = (-rho)^|m| / (2 sqrt 3), rho = 2 - sqrt 3, and the natural ends are
// odd reflections of s about knots 0 and n-1 (they make c vanish there), so
//   c_i = sum_j (G_{i-j} - G_{i+j} - G_{i-(2(n-1)-j)}) s_j.
// Terms with |m| > kSplHalf are below rho^27 / (2 sqrt 3) = 8e-17 of the
// largest and are dropped: every c_i is an independent 55-term FP64 dot
// product -- no serial recurrence and no division per knot.
constexpr int kSplHalf = 27;
constexpr int kSplThreads = 256;
struct SplKernel {
  double g[kSplHalf + 1];
};

__device__ __forceinline__ double knot(double x0, double h, int i) { return x0 + i * h; }

__global__ void __launch_bounds__(kSplThreads) k_spline_c(const double* __restrict__ y, int n,
                                                         double s_scale, SplKernel G,
                                                         double* __restrict__ c) {
  __shared__ double ss[kSplThreads + 2 * kSplHalf];
  const int i0 = blockIdx.x * kSplThreads;
  // s_j for j in [i0 - half, i0 + 256 + half), zero outside [1, n-2]
  for (int t = threadIdx.x; t < kSplThreads + 2 * kSplHalf; t += kSplThreads) {
    const int j = i0 - kSplHalf + t;
    ss[t] = (j >= 1 && j <= n - 2) ? s_scale * ((y[j + 1] - y[j]) - (y[j] - y[j - 1])) : 0.;
  }
  __syncthreads();
  const int i = i0 + threadIdx.x;
  if (i >= n) return;
  if (i == 0 || i == n - 1) {
    c[i] = 0.;
    return;
  }
  const double* sc = ss + threadIdx.x + kSplHalf;  // sc[j - i] = s_j
  double v = G.g[0] * sc[0];
#pragma unroll
  for (int m = 1; m <= kSplHalf; ++m) v += G.g[m] * (sc[-m] + sc[m]);
  // left image: s_j at distance m = i + j (j >= 1); right image: j = 2(n-1) - i - m
  for (int m = i + 1; m <= kSplHalf; ++m) v -= G.g[m] * sc[m - 2 * i];
  for (int m = n - i; m <= kSplHalf; ++m) {
    const int j = 2 * (n - 1) - i - m;
    if (j >= 1) v -= G.g[m] * sc[j - i];
  }
  c[i] = v;
}

// {y_i, b_i, c_i, d_i} per interval, as gsl_interp_cspline (the knot spacing
// is the uniform h; 1/h and h/3 from the host)
__global__ void k_spline_coef(const double* __restrict__ y, const double* __restrict__ c, int n,
                              double inv_h, double h3, double inv_3h,
                              double4* __restrict__ coef, float4* __restrict__ coef32) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n - 1) return;
  const double dy = y[i + 1] - y[i];
  const double b = dy * inv_h - h3 * (c[i + 1] + 2.0 * c[i]);
  const double d = (c[i + 1] - c[i]) * inv_3h;
  coef[i] = make_double4(y[i], b, c[i], d);
  if (coef32) coef32[i] = make_float4((float)y[i], (float)b, (float)c[i], (float)d);
}

// calcFormFac (src/UpcCrossSection.cpp:436-445) on Q2 = Q2min + i*dQ2.
__global__ void k_formfac_values(double* __restrict__ out, int n, double x0, double h,
                                 double rho0, double R, double a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = calc_form_fac(x0 + i * h, rho0, R, a);
}

// The same closed form for the fast form's knots with fewer FP64
// transcendentals (GB300's FP64 pipe runs at 1/64 of the FP32 rate): one
// sincos for sin, cos(QR); sinh, cosh(x) from one exp where x = pi Q a >=
// 0.05 (below, the bracket's terms cancel like (QR)^-2 and e^x - e^-x would
// pass its rounding on: the library's sinh, cosh there, the first knots
// only); exp(-R/a) once on the host.  Values move by rounding, not by the
// formula.
__global__ void k_formfac_values_fast(double* __restrict__ out, int n, double x0, double h,
                                      double rho0, double R, double a, double e_ra) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double Q = sqrt(x0 + i * h) / kHc;
  const double x = kPi * Q * a;
  double sinhVal, coshVal;
  if (x < 0.05) {
    sinhVal = sinh(x);
    coshVal = cosh(x);
  } else {
    const double ex = exp(x), emx = 1. / ex;
    sinhVal = 0.5 * (ex - emx);
    coshVal = 0.5 * (ex + emx);
  }
  double sqr, cqr;
  sincos(Q * R, &sqr, &cqr);
  const double qa2 = 1 + Q * Q * a * a;
  double ff = 4 * kPi * kPi * rho0 * a * a * a / (Q * a * Q * a * sinhVal * sinhVal) *
              (x * coshVal * sqr - Q * R * cqr * sinhVal);
  ff += 8 * kPi * rho0 * a * a * a * e_ra / qa2 / qa2;
  out[i] = ff;
}

__device__ __forceinline__ double eval_u(const double4* coef, int n, double h, double x) {
  SplineU s{coef, 0.0, h, 1.0 / h, n};
  return spline_eval_smem(s, coef, x);
}

// prepareGAA (src/UpcCrossSection.cpp:364-414), first part: T_A(b) on 200
// nodes, Simpson over z; one CTA per b, one thread per z node, the weighted
// sum taken in the reference's order by one thread.
__global__ void __launch_bounds__(256) k_ta_values(double rho0, double R, double a,
                                                   double* __restrict__ ta_y) {
  constexpr int nb = 200;
  __shared__ double v[nb];
  const double db = 20. / (nb - 1);
  const double b = blockIdx.x * db;
  const int iz = threadIdx.x;
  if (iz < nb) {
    const double z = iz * db, r = sqrt(b * b + z * z);
    v[iz] = rho0 / (1 + exp((r - R) / a));
  }
  __syncthreads();
  if (iz == 0) {
    double sum = v[0] + v[nb - 1];
    for (int i = 1; i < nb - 1; i += 2) sum += 4. * v[i];
    for (int i = 2; i < nb - 1; i += 2) sum += 2. * v[i];
    ta_y[blockIdx.x] = 2. * (sum * db / 3.);
  }
}

// G_AA(b_ib) = exp(-sigma_NN T_AA(b_ib)): one CTA per b, one thread per s.
__global__ void __launch_bounds__(256) k_gaa_rows(const double4* __restrict__ ta_coef, double csNN,
                                                  GaaConsts k, double* __restrict__ gaa_y) {
  constexpr int nb = 200;
  __shared__ double4 sTAc[nb - 1];
  __shared__ double vs[nb];
  const double bmax = 20.;
  const double db = bmax / (nb - 1);
  for (int i = threadIdx.x; i < nb - 1; i += blockDim.x) sTAc[i] = ta_coef[i];
  __syncthreads();
  const int ib = blockIdx.x, is = threadIdx.x;
  const double b = ib * db;
  if (is < nb) {
    const double s = is * db;
    double sum_phi = 0;
    for (int q = 0; q < 5; ++q) {
      const double r = sqrt(b * b + s * s + 2. * b * s * k.cosk[q]);
      sum_phi += 2. * kPi * k.wk[q] * eval_u(sTAc, nb, db, r < bmax ? r : bmax);
    }
    vs[is] = 2. * s * eval_u(sTAc, nb, db, s < bmax ? s : bmax) * sum_phi;
  }
  __syncthreads();
  if (threadIdx.x == 0) {  // Simpson weights in the reference's order
    double sum = vs[0] + vs[nb - 1];
    for (int i = 1; i < nb - 1; i += 2) sum += 4. * vs[i];
    for (int i = 2; i < nb - 1; i += 2) sum += 2. * vs[i];
    gaa_y[ib] = exp(-csNN * (sum * db / 3.));
  }
}

// The fast form's T_A and G_AA: the nodes, Simpson weights and order of the
// sums of k_ta_values / k_gaa_rows, with the integrands in FP32 and the sums
// in FP64.  The fast form reads only an FP32 copy of the G_AA spline, and
// FP64 is the scarce unit while the table chains run side by side (GB300
// issues FP32 at 64x its FP64 rate); G_AA moves by ~1e-6 (the sums' terms
// carry FP32's 6e-8).
__global__ void __launch_bounds__(256) k_ta_values_f(float rho0, float R, float a,
                                                     double* __restrict__ ta_y) {
  constexpr int nb = 200;
  __shared__ double v[nb];
  const float db = 20.f / (nb - 1);
  const float b = blockIdx.x * db;
  const int iz = threadIdx.x;
  if (iz < nb) {
    const float z = iz * db, r = sqrtf(b * b + z * z);
    v[iz] = (double)(rho0 / (1.f + expf((r - R) / a)));
  }
  __syncthreads();
  if (iz == 0) {
    const double dbd = 20. / (nb - 1);
    double sum = v[0] + v[nb - 1];
    for (int i = 1; i < nb - 1; i += 2) sum += 4. * v[i];
    for (int i = 2; i < nb - 1; i += 2) sum += 2. * v[i];
    ta_y[blockIdx.x] = 2. * (sum * dbd / 3.);
  }
}

__device__ __forceinline__ float eval_uf(const float4* coef, int n, float h, float x) {
  const SplineF s{coef, 0.f, h, 1.f / h, n};
  return spline_eval_f(s, coef, x);
}

__global__ void __launch_bounds__(256) k_gaa_rows_f(const float4* __restrict__ ta_coef,
                                                    double csNN, GaaConsts k,
                                                    double* __restrict__ gaa_y) {
  constexpr int nb = 200;
  __shared__ float4 sTAc[nb - 1];
  __shared__ double vs[nb];
  const float bmax = 20.f;
  const float db = bmax / (nb - 1);
  for (int i = threadIdx.x; i < nb - 1; i += blockDim.x) sTAc[i] = ta_coef[i];
  __syncthreads();
  const int ib = blockIdx.x, is = threadIdx.x;
  const float b = ib * db;
  if (is < nb) {
    const float s = is * db;
    float sum_phi = 0.f;
    for (int q = 0; q < 5; ++q) {
      const float r = sqrtf(b * b + s * s + 2.f * b * s * (float)k.cosk[q]);
      sum_phi += 2.f * (float)kPi * (float)k.wk[q] * eval_uf(sTAc, nb, db, r < bmax ? r : bmax);
    }
    vs[is] = (double)(2.f * s * eval_uf(sTAc, nb, db, s < bmax ? s : bmax) * sum_phi);
  }
  __syncthreads();
  if (threadIdx.x == 0) {  // Simpson weights in the reference's order
    const double dbd = 20. / (nb - 1);
    double sum = vs[0] + vs[nb - 1];
    for (int i = 1; i < nb - 1; i += 2) sum += 4. * vs[i];
    for (int i = 2; i < nb - 1; i += 2) sum += 2. * vs[i];
    gaa_y[ib] = exp(-csNN * (sum * dbd / 3.));
  }
}

// Photo-neutron data of src/UpcCrossSection.cpp:778-851, 1-based (index 0 unused).
const double kE1[23] = {0., 103., 106., 112., 119., 127., 132., 145., 171., 199., 230., 235.,
                               254., 280., 300., 320., 330., 333., 373., 390., 420., 426., 440.};
const double kS1[23] = {0., 12.0, 11.5, 12.0, 12.0, 12.0, 15.0, 17.0, 28.0, 33.0,
                               52.0, 60.0, 70.0, 76.0, 85.0, 86.0, 89.0, 89.0, 75.0, 76.0, 69.0, 59.0, 61.0};
const double kE2[12] = {0., 2000., 3270., 4100., 4810., 6210., 6600.,
                               7790., 8400., 9510., 13600., 16400.};
const double kS2[12] = {0., .1266, .1080, .0805, .1017, .0942, .0844, .0841, .0755, .0827,
                               .0626, .0740};
const double kE3[29] = {0., 26., 28., 30., 32., 34., 36., 38., 40., 44., 46., 48., 50., 52., 55.,
                               57., 62., 64., 66., 69., 72., 74., 76., 79., 82., 86., 92., 98., 103.};
const double kS3[29] = {0., 30., 21.5, 22.5, 18.5, 17.5, 15., 14.5, 19., 17.5, 16., 14.,
                               20., 16.5, 17.5, 17., 15.5, 18., 15.5, 15.5, 15., 13.5, 18., 14.5, 15.5, 12.5, 13.,
                               13., 12.};
const double kSigt[160] = {
    0., .4245, .4870, .5269, .4778, .4066, .3341, .2444, .2245, .2005,
    .1783, .1769, .1869, .1940, .2117, .2226, .2327, .2395, .2646, .2790, .2756,
    .2607, .2447, .2211, .2063, .2137, .2088, .2017, .2050, .2015, .2121, .2175,
    .2152, .1917, .1911, .1747, .1650, .1587, .1622, .1496, .1486, .1438, .1556,
    .1468, .1536, .1544, .1536, .1468, .1535, .1442, .1515, .1559, .1541, .1461,
    .1388, .1565, .1502, .1503, .1454, .1389, .1445, .1425, .1415, .1424, .1432,
    .1486, .1539, .1354, .1480, .1443, .1435, .1491, .1435, .1380, .1317, .1445,
    .1375, .1449, .1359, .1383, .1390, .1361, .1286, .1359, .1395, .1327, .1387,
    .1431, .1403, .1404, .1389, .1410, .1304, .1363, .1241, .1284, .1299, .1325,
    .1343, .1387, .1328, .1444, .1334, .1362, .1302, .1338, .1339, .1304, .1314,
    .1287, .1404, .1383, .1292, .1436, .1280, .1326, .1321, .1268, .1278, .1243,
    .1239, .1271, .1213, .1338, .1287, .1343, .1231, .1317, .1214, .1370, .1232,
    .1301, .1348, .1294, .1278, .1227, .1218, .1198, .1193, .1342, .1323, .1248,
    .1220, .1139, .1271, .1224, .1347, .1249, .1163, .1362, .1236, .1462, .1356,
    .1198, .1419, .1324, .1288, .1336, .1335, .1266};
const double kSigtn[160] = {
    0., .3125, .3930, .4401, .4582, .3774, .3329, .2996, .2715, .2165,
    .2297, .1861, .1551, .2020, .2073, .2064, .2193, .2275, .2384, .2150, .2494,
    .2133, .2023, .1969, .1797, .1693, .1642, .1463, .1280, .1555, .1489, .1435,
    .1398, .1573, .1479, .1493, .1417, .1403, .1258, .1354, .1394, .1420, .1364,
    .1325, .1455, .1326, .1397, .1286, .1260, .1314, .1378, .1353, .1264, .1471,
    .1650, .1311, .1261, .1348, .1277, .1518, .1297, .1452, .1453, .1598, .1323,
    .1234, .1212, .1333, .1434, .1380, .1330, .12, .12, .12, .12, .12, .12, .12, .12,
    .12, .12, .12, .12, .12, .12, .12, .12, .12, .12, .12, .12, .12, .12, .12, .12, .12,
    .12, .12, .12, .12, .12, .12, .12, .12, .12, .12, .12, .12, .12, .12, .12, .12, .12,
    .12, .12, .12, .12, .12, .12, .12, .12, .12, .12, .12, .12, .12, .12, .12, .12, .12,
    .12, .12, .12, .12, .12, .12, .12, .12, .12, .12, .12, .12, .12, .12, .12, .12, .12,
    .12, .12, .12, .12, .12, .12, .12, .12, .12, .12, .12, .12, .12};

}  // namespace

// Energy / cross-section table of calcBreakupProb's first-call set-up
// (src/UpcCrossSection.cpp:893-969); lead values as hard-coded there.  A
// ~650-entry recurrence: built on the host (a serial FP64 chain is the
// slowest thing a GPU can run), then copied.
int breakup_energy_table(double gammatarg, double* ee, double* se) {
  const double zp = 82, ap = 208;
  const double si1 = 640., gg1 = 4.05, o1 = 13.42, o0 = 7.4;
  const double delo = .05;
  const double scon = .1 * gg1 * gg1 * si1;
  const int ne = int((25. - o0) / delo) + 1;
  for (int i = 1; i <= ne; i++) {
    ee[i] = o0 + (i - 1) * delo;
    se[i] = scon * ee[i] * ee[i] /
            (((o1 * o1 - ee[i] * ee[i]) * (o1 * o1 - ee[i] * ee[i])) + ee[i] * ee[i] * gg1 * gg1);
  }
  int ij = ne;
  for (int j = 1; j <= 27; j++) { ij++; ee[ij] = kE3[j]; se[ij] = .1 * ap * kS3[j] / 208.; }
  for (int j = 1; j <= 22; j++) { ij++; ee[ij] = kE1[j]; se[ij] = .1 * ap * kS1[j] / 208.; }
  for (int j = 9; j <= 70; j++) {
    ij++;
    ee[ij] = ee[ij - 1] + 25.;
    se[ij] = .1 * (zp * kSigt[j] + (ap - zp) * kSigtn[j]);
  }
  for (int j = 1; j <= 11; j++) { ij++; ee[ij] = kE2[j]; se[ij] = .1 * ap * kS2[j]; }
  const double x = .0677, y = .129, eps = .0808, eta = .4525, em = .94;
  const double exx = std::pow(10., .05);
  double s = .002 * em * ee[ij];
  const int ictr = gammatarg > (2. * 150. * 150.) ? 150 : 100;
  for (int j = 1; j <= ictr; j++) {
    ij++;
    s = s * exx;
    ee[ij] = 1000. * .5 * (s - em * em) / em;
    se[ij] = .1 * .65 * ap * (x * std::pow(s, eps) + y * std::pow(s, (-eta)));
  }
  ee[0] = se[0] = 0.;
  ee[ij + 1] = 99999999999.;
  se[ij + 1] = 0.;
  return ij + 2;
}

namespace {

// calcBreakupProb (src/UpcCrossSection.cpp:972-1018) on b = bmin + i*db.
// The single-neutron sum p1n of the reference never reaches its result and is
// not computed.  Per (b, E_k) the A&S K1 needs ln(x/2) and 1/x of
// x = E_k b / (hc gamma_t): both come from per-energy tables (ln E_k, 1/E_k)
// and one log and one division per b, so the inner loop is FMAs only.
// One warp per b: lane l takes the energies k = 2 + 32 j + l, the
// trapezoid's left value f_{k-1} comes from the neighbouring lane, and the
// warp sums its terms at the end (the reference sums them in k order; the
// difference is rounding).  A thread per b would be a 650-step serial FP64
// chain, which on this part's narrow FP64 pipe is latency-bound.
__global__ void __launch_bounds__(256) k_breakup_values(const double* __restrict__ tab, int nt,
                                                        int n, double x0, double h, int mode,
                                                        double gammatarg, double omaxx,
                                                        double zcon, double* __restrict__ out) {
  extern __shared__ double s_tab[];  // ee | se | ln ee | 1/ee
  for (int i = threadIdx.x; i < 4 * nt; i += blockDim.x) {
    const int part = i / nt, j = i - part * nt;
    s_tab[i] = tab[part * kBreakupTabMax + j];
  }
  __syncthreads();
  const double* see = s_tab;
  const double* sse = s_tab + nt;
  const double* slne = s_tab + 2 * nt;
  const double* sinv = s_tab + 3 * nt;
  const int lane = threadIdx.x & 31;
  // warps stride over b (whole warps together), so that each block's table
  // load serves several b
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += nwarps) {
  const double b = x0 + i * h;
  const double hbarcmev = 197.3269718, o0 = 7.4;
  const double beta = b / ((hbarcmev) * gammatarg);  // x = E beta
  const double ln_half_beta = log(0.5 * beta);
  const double inv_beta = 1. / beta;
  // f_k = se_k ee_k K1(ee_k beta)^2
  auto f = [&](int k) {
    const double x = see[k] * beta;
    double K1;
    if (x > 2.) {
      K1 = bessel_k1_as(x);
    } else {
      const double y = x * x * 0.25;
      const double u = x * x * (1. / 14.0625);  // (x / 3.75)^2
      const double i1 = x * (0.5 + u * (0.87890594 + u * (0.51498869 + u * (0.15084934 +
                        u * (0.2658733e-1 + u * (0.301532e-2 + u * 0.32411e-3))))));
      K1 = (slne[k] + ln_half_beta) * i1 +
           (sinv[k] * inv_beta) * (1. + y * (0.15443144 + y * (-0.67278579 + y * (-0.18156897 +
           y * (-0.1919402e-1 + y * (-0.110404e-2 + y * (-0.4686e-4)))))));
    }
    return sse[k] * see[k] * K1 * K1;
  };
  const double omax = fmin(omaxx, 4. * gammatarg * (hbarcmev) / b);
  double p = 0.;
  if (!(omax < o0)) {
    double part = 0.;
    double carry = lane == 31 ? f(1) : 0.;  // f_{k-1} of lane 0 in the first round
    for (int k0 = 2; k0 < nt; k0 += 32) {
      const int k = k0 + lane;
      const bool in = k < nt && see[k] < omax;
      const double fk = in ? f(k) : 0.;
      double fm = __shfl_up_sync(0xffffffffu, fk, 1);
      const double c = __shfl_sync(0xffffffffu, carry, 31);
      if (lane == 0) fm = c;
      if (in) part += (see[k] - see[k - 1]) * .5 * (fm + fk);
      carry = fk;
      if (!__any_sync(0xffffffffu, in)) break;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    const double pxn = zcon * part;
    if (mode == 1) p = 1.;
    if (mode == 2) p = (1 - exp(-1 * pxn)) * (1 - exp(-1 * pxn));
    if (mode == 3) p = exp(-2 * pxn);
    if (mode == 4) p = 2. * exp(-pxn) * (1. - exp(-pxn));
  }
  if (lane == 0) out[i] = p;
  }
}

// The same sums in FP32 for the fast form (luminosity methods 1 and 4, whose
// budget is 1e-4): per lane the trapezoid terms of beta^2 f_k (magnitudes
// near se / ee instead of up to 1e35 at b -> 0) in FP32, the warp sum and the
// 1/beta^2 in FP64; relative error ~1e-6, at 1/64 of the FP64 pipe's cost per
// term.
constexpr int kBreakupThreads = 256;

__device__ __forceinline__ float bessel_k1_as_f(float x) {  // bessel_k1_as, x > 2
  const float y = 2.f / x;
  return (expf(-x) * rsqrtf(x)) *
         (1.25331414f + y * (0.23498619f + y * (-0.3655620e-1f + y * (0.1504268e-1f +
          y * (-0.780353e-2f + y * (0.325614e-2f + y * (-0.68245e-3f)))))));
}

// A block takes 32 consecutive b: warp 0 computes their FP64 prologue (beta,
// ln(beta/2), omax) and epilogue (1/beta^2, the mode formula) one b per lane,
// so that each FP64 instruction serves 32 b (a warp FP64 instruction costs the
// same with 1 useful lane as with 32); the 8 warps share the 32 FP32 sums
// over the energy table, 4 b each.  Same arithmetic, in the same order, as
// one warp per b.
__global__ void __launch_bounds__(256) k_breakup_values_f(const double* __restrict__ tab, int nt,
                                                          int n, double x0, double h, int mode,
                                                          double gammatarg, double omaxx,
                                                          double zcon, double* __restrict__ out) {
  extern __shared__ float s_tabf[];  // ee | se | ln ee | 1/ee
  __shared__ float s_beta[32], s_lnhb[32], s_omax[32];
  __shared__ double s_sum[32];
  __shared__ unsigned s_run;
  for (int i = threadIdx.x; i < 4 * nt; i += blockDim.x) {
    const int part = i / nt, j = i - part * nt;
    s_tabf[i] = (float)tab[part * kBreakupTabMax + j];
  }
  const float* see = s_tabf;
  const float* sse = s_tabf + nt;
  const float* slne = s_tabf + 2 * nt;
  const float* sinv = s_tabf + 3 * nt;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const double hbarcmev = 197.3269718, o0 = 7.4;
  for (int i0 = blockIdx.x * 32; i0 < n; i0 += gridDim.x * 32) {
    if (w == 0) {  // FP64 prologue, b = i0 + lane
      const int ib = i0 + lane;
      const double b = x0 + ib * h;
      const double beta_d = b / ((hbarcmev) * gammatarg);
      const double omax = fmin(omaxx, 4. * gammatarg * (hbarcmev) / b);
      s_beta[lane] = (float)beta_d;
      s_lnhb[lane] = (float)log(0.5 * beta_d);
      s_omax[lane] = (float)omax;
      const unsigned run = __ballot_sync(0xffffffffu, ib < n && !(omax < o0));
      if (lane == 0) s_run = run;
    }
    __syncthreads();
    const unsigned run = s_run;
    for (int jb = w; jb < 32; jb += kBreakupThreads / 32) {
      if (!((run >> jb) & 1u)) continue;
      const float beta = s_beta[jb], ln_half_beta = s_lnhb[jb], omaxf = s_omax[jb];
      // g_k = beta^2 f_k = se_k ee_k (beta K1(ee_k beta))^2
      auto g = [&](int k) {
        const float x = see[k] * beta;
        float bk1;  // beta K1(x)
        if (x > 2.f) {
          bk1 = beta * bessel_k1_as_f(x);
        } else {
          const float y = x * x * 0.25f;
          const float u = x * x * (1.f / 14.0625f);
          const float i1 = x * (0.5f + u * (0.87890594f + u * (0.51498869f + u * (0.15084934f +
                           u * (0.2658733e-1f + u * (0.301532e-2f + u * 0.32411e-3f))))));
          bk1 = beta * (slne[k] + ln_half_beta) * i1 +
                sinv[k] * (1.f + y * (0.15443144f + y * (-0.67278579f + y * (-0.18156897f +
                y * (-0.1919402e-1f + y * (-0.110404e-2f + y * (-0.4686e-4f)))))));
        }
        return sse[k] * see[k] * bk1 * bk1;
      };
      float part = 0.f;
      float carry = lane == 31 ? g(1) : 0.f;
      for (int k0 = 2; k0 < nt; k0 += 32) {
        const int k = k0 + lane;
        const bool in = k < nt && see[k] < omaxf;
        const float gk = in ? g(k) : 0.f;
        float gm = __shfl_up_sync(0xffffffffu, gk, 1);
        const float c = __shfl_sync(0xffffffffu, carry, 31);
        if (lane == 0) gm = c;
        if (in) part += (see[k] - see[k - 1]) * .5f * (gm + gk);
        carry = gk;
        if (!__any_sync(0xffffffffu, in)) break;
      }
      double sum = (double)part;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
      if (lane == 0) s_sum[jb] = sum;
    }
    __syncthreads();
    if (w == 0) {  // FP64 epilogue
      const int ib = i0 + lane;
      if (ib < n) {
        double p = 0.;
        if ((run >> lane) & 1u) {
          const double b = x0 + ib * h;
          const double beta_d = b / ((hbarcmev) * gammatarg);
          const double pxn = zcon * s_sum[lane] / (beta_d * beta_d);
          if (mode == 1) p = 1.;
          if (mode == 2) p = (1 - exp(-1 * pxn)) * (1 - exp(-1 * pxn));
          if (mode == 3) p = exp(-2 * pxn);
          if (mode == 4) p = 2. * exp(-pxn) * (1. - exp(-pxn));
        }
        out[ib] = p;
      }
    }
    __syncthreads();  // s_* are rewritten by the next group
  }
}

// calcBreakupProb at arbitrary b (the point entry of the C ABI).
__global__ void k_breakup_pts(const double* __restrict__ ee_g, const double* __restrict__ se_g,
                              const int* __restrict__ n_tab, const double* __restrict__ bv, int n,
                              int mode, double gammatarg, double omaxx, double zcon,
                              double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int nt = *n_tab;
  const double b = bv[i];
  const double hbarcmev = 197.3269718, o0 = 7.4;
  double pxn = 0.;
  const double omax = fmin(omaxx, 4. * gammatarg * (hbarcmev) / b);
  double p = 0.;
  if (!(omax < o0)) {
    double gk1m = bessel_k1_as(ee_g[1] * b / ((hbarcmev) * gammatarg));
    int k = 2;
    while (k < nt && ee_g[k] < omax) {
      const double gk1 = bessel_k1_as(ee_g[k] * b / ((hbarcmev) * gammatarg));
      pxn = pxn + zcon * (ee_g[k] - ee_g[k - 1]) * .5 *
                      (se_g[k - 1] * ee_g[k - 1] * gk1m * gk1m + se_g[k] * ee_g[k] * gk1 * gk1);
      k = k + 1;
      gk1m = gk1;
    }
    if (mode == 1) p = 1.;
    if (mode == 2) p = (1 - exp(-1 * pxn)) * (1 - exp(-1 * pxn));
    if (mode == 3) p = exp(-2 * pxn);
    if (mode == 4) p = 2. * exp(-pxn) * (1. - exp(-pxn));
  }
  out[i] = p;
}

__global__ void k_formfac_pts(const double* __restrict__ q2, double* __restrict__ out, int n,
                              double rho0, double R, double a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = calc_form_fac(q2[i], rho0, R, a);
}

}  // namespace

cudaError_t launch_breakup_points(double gammatarg, double omaxx, double zcon, int mode,
                                  const double* d_ee, const double* d_se, const int* d_ntab,
                                  const double* d_b, double* d_out, int n, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  note_launch();
  k_breakup_pts<<<(n + 127) / 128, 128, 0, st>>>(d_ee, d_se, d_ntab, d_b, n, mode, gammatarg,
                                                 omaxx, zcon, d_out);
  return cudaGetLastError();
}

cudaError_t launch_formfac_points(const double* d_q2, double* d_out, int n, double rho0,
                                  double R, double a, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  note_launch();
  k_formfac_pts<<<(n + 255) / 256, 256, 0, st>>>(d_q2, d_out, n, rho0, R, a);
  return cudaGetLastError();
}

__global__ void k_coef_f32(const double4* __restrict__ in, float4* __restrict__ out, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double4 c = in[i];
  out[i] = make_float4((float)c.x, (float)c.y, (float)c.z, (float)c.w);
}

cudaError_t build_spline_uniform(const double* d_y, int n, double x0, double h, double* d_c,
                                 double4* d_coef, cudaStream_t st, float4* d_coef32) {
  (void)x0;
  if (n < 2 * kSplHalf + 4) return cudaErrorInvalidValue;  // the two end images must not meet
  static SplKernel G = [] {
    SplKernel k{};
    const double rho = 2. - std::sqrt(3.);
    double p = 1. / (2. * std::sqrt(3.));
    for (int m = 0; m <= kSplHalf; ++m) {
      k.g[m] = p;
      p *= -rho;
    }
    return k;
  }();
  note_launch();
  k_spline_c<<<(n + kSplThreads - 1) / kSplThreads, kSplThreads, 0, st>>>(d_y, n, 3. / (h * h), G,
                                                                         d_c);
  note_launch();
  k_spline_coef<<<(n - 1 + 255) / 256, 256, 0, st>>>(d_y, d_c, n, 1. / h, h / 3., 1. / (3. * h),
                                                     d_coef, d_coef32);
  return cudaGetLastError();
}

cudaError_t launch_formfac_values(double* d_out, int n, double x0, double h, double rho0,
                                  double R, double a, cudaStream_t st, int fast) {
  note_launch();
  if (fast)
    k_formfac_values_fast<<<(n + 255) / 256, 256, 0, st>>>(d_out, n, x0, h, rho0, R, a,
                                                           std::exp(-R / a));
  else
    k_formfac_values<<<(n + 255) / 256, 256, 0, st>>>(d_out, n, x0, h, rho0, R, a);
  return cudaGetLastError();
}

cudaError_t launch_gaa(double rho0, double R, double a, double csNN, const GaaConsts& k,
                       double4* d_coef, double4* d_ta_coef, double* d_work, cudaStream_t st,
                       float4* d_coef32, float4* d_ta32) {
  // d_work: T_A values | T_A spline scratch | G_AA values | G_AA spline scratch (200 each)
  constexpr int nb = 200;
  const double db = 20. / (nb - 1);
  double* ta_y = d_work;
  double* ta_c = d_work + nb;
  double* g_y = d_work + 2 * nb;
  double* g_c = d_work + 3 * nb;
  note_launch();
  if (d_ta32)
    k_ta_values_f<<<nb, 256, 0, st>>>((float)rho0, (float)R, (float)a, ta_y);
  else
    k_ta_values<<<nb, 256, 0, st>>>(rho0, R, a, ta_y);
  cudaError_t e = build_spline_uniform(ta_y, nb, 0., db, ta_c, d_ta_coef, st, d_ta32);
  if (e != cudaSuccess) return e;
  note_launch();
  if (d_ta32)
    k_gaa_rows_f<<<nb, 256, 0, st>>>(d_ta32, csNN, k, g_y);
  else
    k_gaa_rows<<<nb, 256, 0, st>>>(d_ta_coef, csNN, k, g_y);
  return build_spline_uniform(g_y, nb, 0., db, g_c, d_coef, st, d_coef32);
}

cudaError_t launch_breakup_values(const double* d_tab, int nt, double gammatarg, double omaxx,
                                  double zcon, int mode, int n, double x0, double h,
                                  double* d_out, cudaStream_t st, int fp32) {
  if (nt > kBreakupTabMax) return cudaErrorInvalidValue;
  // 8 warps per block, each over several b: 4 blocks per SM of 152
  const unsigned blocks = (unsigned)std::min<size_t>(((size_t)n * 32 + 255) / 256, 608);
  if (fp32) {  // 32 b per block
    const unsigned bf = (unsigned)std::min<size_t>(((size_t)n + 31) / 32, 152 * 16);
    note_launch();
    k_breakup_values_f<<<bf, kBreakupThreads, 4 * sizeof(float) * nt, st>>>(
        d_tab, nt, n, x0, h, mode, gammatarg, omaxx, zcon, d_out);
    return cudaGetLastError();
  }
  const size_t smem = 4 * sizeof(double) * nt;
  static std::atomic<uint64_t> attr{0};  // devices with the limit raised
  {
    const cudaError_t ea = smem_attr_once(attr, k_breakup_values, (int)(4 * sizeof(double) * kBreakupTabMax));
    if (ea != cudaSuccess) return ea;
  }
  note_launch();
  k_breakup_values<<<blocks, 256, smem, st>>>(d_tab, nt, n, x0, h, mode, gammatarg, omaxx, zcon,
                                              d_out);
  return cudaGetLastError();
}

}  // namespace upcg
