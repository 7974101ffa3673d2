// Grid (precision) form of the two-photon luminosity for the point-charge flux
// (luminosity method 3): the b-quadrature of calcTwoPhotonLumi
// (src/UpcCrossSection.cpp:221-271) on fixed logarithmic grids shared by all
// cells, so that the whole table is two dense products on the tensor cores:
//
//   N[w][r] = N(w, r) r^2 dln r      (flux x quadrature weight, w on nw points,
//                                      r on nr points in [r0, r1])
//   T = N . G,  Lg = T . N^T          (G[r][s]: the azimuthal survival sum)
//   L(m, y) / (2 pi^2 m) = Lg(k1, k2) + c (F1 (S2 + F2) + S1 F2)
//
// where k1,2 = m/2 e^{+-y} are interpolated on the w grid (4-point Lagrange in
// ln w), S(w) = sum_r N[w][r] and F(w) is the flux integral beyond r1, taken in
// closed form (G = c there: every azimuth has b >= 20 fm).  The quadrature
// differs from the reference's per-cell 120-bin midpoint rule, so the table
// carries a discretisation difference that the tests state.
//
// The radial weights follow the reference's integration range per photon:
// b from R (point flux, :226) to bmax = max(5 g hc / k, 5 R) (:228-229),
// trapezoidal in ln b with the partial end intervals folded into the first and
// last radius inside the range.
#include <cuda_bf16.h>

#include "upcg_device.cuh"
#include "upcg_internal.h"

namespace upcg {

namespace {

// S(ln x) = ln(K1^2 + K0^2/g^2) + 2x by 4-point Lagrange on the FP32 table
__device__ __forceinline__ float s_table(const GridForm& gf, float lnx) {
  float t = (float)((lnx - gf.su0) * gf.sinv_h);
  int p0 = (int)floorf(t) - 1;
  p0 = p0 < 0 ? 0 : (p0 > gf.sn - 4 ? gf.sn - 4 : p0);
  const float s = t - (float)p0;
  const float s1 = s - 1.f, s2 = s - 2.f, s3 = s - 3.f;
  const float* q = gf.s32 + p0;
  return -s1 * s2 * s3 * (1.f / 6.f) * __ldg(q) + s * s2 * s3 * 0.5f * __ldg(q + 1) -
         s * s1 * s3 * 0.5f * __ldg(q + 2) + s * s1 * s2 * (1.f / 6.f) * __ldg(q + 3);
}

// x^2/2 (K1^2 - K0 K2) + x^2/2 (K0^2 - K1^2) / g^2: the antiderivative of
// x (K1^2 + K0^2/g^2) (Lommel's integrals, K2 = K0 + 2 K1 / x)
__device__ double lommel(double x, double g) {
  double K0, K1;
  bessel_k01(x, K0, K1);
  const double K2 = K0 + 2. * K1 / x;
  return 0.5 * x * x * ((K1 * K1 - K0 * K2) + (K0 * K0 - K1 * K1) / (g * g));
}

constexpr int kFluxThreads = 256;

// one CTA per photon-energy row
__global__ void __launch_bounds__(kFluxThreads) k_grid_flux(LumiParams p, GridForm gf,
                                                            __nv_bfloat16* __restrict__ nh,
                                                            __nv_bfloat16* __restrict__ nl,
                                                            double* __restrict__ rowsum,
                                                            double* __restrict__ tail) {
  __shared__ double red[kFluxThreads / 32];
  __shared__ int lim[2];
  __shared__ double cut[2];
  const int iw = blockIdx.x;
  const size_t row = (size_t)iw * gf.nr;
  if (iw >= gf.nw) {  // padding rows of the last 128-row tile
    for (int j = threadIdx.x; j < gf.nr; j += kFluxThreads) {
      nh[row + j] = __float2bfloat16(0.f);
      nl[row + j] = __float2bfloat16(0.f);
    }
    return;
  }
  const double lnk = gf.lw0 + iw * gf.hw;
  const double g = p.g1;
  if (threadIdx.x == 0) {
    // integration range of calcTwoPhotonLumi for this photon (point flux)
    const double k = exp(lnk);
    const double lb_lo = log(p.R);
    const double lb_hi = log(fmax(5. * g * kHc / k, 5. * p.R));
    const double lr1 = gf.lr0 + (gf.nr - 1) * gf.hr;
    const double hi = fmin(lb_hi, lr1);
    int j0 = (int)ceil((lb_lo - gf.lr0) / gf.hr);
    int j1 = (int)floor((hi - gf.lr0) / gf.hr);
    j0 = j0 < 0 ? 0 : j0;
    j1 = j1 > gf.nr - 1 ? gf.nr - 1 : j1;
    lim[0] = j0;
    lim[1] = j1;
    cut[0] = gf.lr0 + j0 * gf.hr - lb_lo;  // partial intervals at both ends
    cut[1] = hi - (gf.lr0 + j1 * gf.hr);
    // closed-form flux integral from the last radius to bmax
    double t = 0.;
    if (lb_hi > lr1) {
      const double c0 = g * kHc / k;  // b = c0 x
      const double xa = exp(lr1) / c0, xb = exp(lb_hi) / c0;
      t = p.factor * k / g / g * c0 * c0 * (lommel(xb, g) - lommel(xa, g));
    }
    tail[iw] = t;
  }
  __syncthreads();
  const int j0 = lim[0], j1 = lim[1];
  const float lnxk = (float)(lnk - log(g * kHc));  // ln x = ln b + ln(k / (g hc))
  const float lnc = (float)(log(p.factor / g / g) + lnk);
  const float hr = (float)gf.hr, lr0 = (float)gf.lr0;
  float part_f = 0.f;
  for (int j = threadIdx.x; j < gf.nr; j += kFluxThreads) {
    float v = 0.f;
    if (j >= j0 && j <= j1 && j1 >= j0) {
      const float lnb = fmaf((float)j, hr, lr0);
      float wgt = hr;  // trapezoid in ln b
      if (j == j0) wgt = 0.5f * hr + (float)cut[0];
      if (j == j1) wgt = (j0 == j1 ? (float)(cut[0] + cut[1]) : 0.5f * hr + (float)cut[1]);
      const float lnx = lnb + lnxk;
      const float x = expf(lnx);
      // N b^2 dln b = factor k/g^2 exp(S - 2x) b^2 w
      v = expf(lnc + s_table(gf, lnx) - 2.f * x + 2.f * lnb) * wgt;
    }
    const __nv_bfloat16 h = __float2bfloat16(v);
    nh[row + j] = h;
    nl[row + j] = __float2bfloat16(v - __bfloat162float(h));
    part_f += v;
  }
  double part = (double)part_f;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = part;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.;
    for (int w = 0; w < kFluxThreads / 32; ++w) s += red[w];
    rowsum[iw] = s;
  }
}

__device__ __forceinline__ int lag4d(double t, int n, double w[4]) {
  int p0 = (int)floor(t) - 1;
  p0 = p0 < 0 ? 0 : (p0 > n - 4 ? n - 4 : p0);
  const double s = t - p0;
  w[0] = -(s - 1.) * (s - 2.) * (s - 3.) * (1. / 6.);
  w[1] = s * (s - 2.) * (s - 3.) * 0.5;
  w[2] = -s * (s - 1.) * (s - 3.) * 0.5;
  w[3] = s * (s - 1.) * (s - 2.) * (1. / 6.);
  return p0;
}

__global__ void k_grid_cells(LumiParams p, GridForm gf, const float* __restrict__ lg,
                             const double* __restrict__ rowsum, const double* __restrict__ tail,
                             double* __restrict__ lumi) {
  const int cell = blockIdx.x * blockDim.x + threadIdx.x;
  if (cell >= p.nm * p.ny) return;
  const int im = cell / p.ny, iy = cell - im * p.ny;
  const double M = p.mmin + p.dm * im, Y = p.ymin + p.dy * iy;  // left edges (:540, :542)
  const double lnm2 = log(M / 2.);
  double w1[4], w2[4];
  const int a = lag4d((lnm2 + Y - gf.lw0) / gf.hw, gf.nw, w1);
  const int b = lag4d((lnm2 - Y - gf.lw0) / gf.hw, gf.nw, w2);
  double lnn = 0., s1 = 0., s2 = 0., f1 = 0., f2 = 0.;
  for (int u = 0; u < 4; ++u) {
    const float* r = lg + (size_t)(a + u) * gf.nw + b;
    lnn += w1[u] * (w2[0] * (double)__ldg(r) + w2[1] * (double)__ldg(r + 1) +
                    w2[2] * (double)__ldg(r + 2) + w2[3] * (double)__ldg(r + 3));
    s1 += w1[u] * rowsum[a + u];
    f1 += w1[u] * tail[a + u];
    s2 += w2[u] * rowsum[b + u];
    f2 += w2[u] * tail[b + u];
  }
  const double L = lnn + gf.c_far * (f1 * (s2 + f2) + s1 * f2);
  lumi[cell] = 2 * kPi * kPi * M * L * p.dm * p.dy;
}

}  // namespace

cudaError_t launch_grid_flux(const LumiParams& p, const GridForm& gf, void* nh, void* nl,
                             double* rowsum, double* tail, cudaStream_t st) {
  const int rows = (gf.nw + 127) / 128 * 128;
  note_launch();
  k_grid_flux<<<rows, kFluxThreads, 0, st>>>(p, gf, static_cast<__nv_bfloat16*>(nh),
                                             static_cast<__nv_bfloat16*>(nl), rowsum, tail);
  return cudaGetLastError();
}

cudaError_t launch_grid_cells(const LumiParams& p, const GridForm& gf, const float* lg,
                              const double* rowsum, const double* tail, double* lumi,
                              cudaStream_t st) {
  const int n = p.nm * p.ny;
  note_launch();
  k_grid_cells<<<(n + 255) / 256, 256, 0, st>>>(p, gf, lg, rowsum, tail, lumi);
  return cudaGetLastError();
}

}  // namespace upcg
