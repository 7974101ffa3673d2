// Elementary cross sections, nuclear cross-section fold and sampling CDFs.
//
// Reference:
//   UpcTwoPhotonDilep::calcCrossSectionM/ZM (+ polarized parts)
//       src/UpcTwoPhotonDilep.cpp:46-134
//   UpcTwoPhotonALP::calcCrossSectionM   src/UpcTwoPhotonALP.cpp:28-33
//   fillCrossSectionZM                   src/UpcCrossSection.cpp:337-362
//   calcNucCrossSectionYM                src/UpcCrossSection.cpp:594-698
//   gsl_histogram{,2d}_pdf_init used by UpcSampler1D/2D (include/UpcSampler.h:37-142):
//       cdf[0] = 0, cdf[i+1] = cdf[i] + (w_i / mean) / n.
#include "upcg_internal.h"

namespace upcg {

namespace {

__device__ double cs_m(const FoldParams& f, double m, int flag) {
  if (f.procID == 51) {
    if (flag) return 0.;
    double cs = 4. * kPi * kPi * f.alpWidth / (f.mPart * f.mPart);
    cs *= kHc * kHc * 1e7 * kAlpha * kAlpha;
    return cs;
  }
  const double mPart = f.mPart, aLep = f.aLep;
  if (flag == 0) {
    const double s = m * m;
    const double x = 4 * mPart * mPart / s;
    const double b = sqrt(1 - x);
    const double y = atanh(b);
    double cs = 0;
    cs += (2 + 2 * x - x * x) * y - b * (1 + x);
    cs += 4 * y * aLep;
    cs += (4 * b / x + y) * aLep * aLep;
    cs += (4 * b / x - 2 * y) * aLep * aLep * aLep;
    cs += ((7. / 12.) * b / x + (1. / 6.) * b / x / x - 0.5 * y) * aLep * aLep * aLep * aLep;
    cs *= 4 * kHc * kHc * 1e7 * kAlpha * kAlpha * kPi / s;
    return cs;
  }
  const double r = 2 * mPart / m;
  if (r > 1) return 0;
  if (flag == 1)
    return 4 * kPi * kAlpha * kAlpha * kHc * kHc / m / m *
           ((1 + r * r - 3. / 4. * r * r * r * r) * 2 * log(1 / r + sqrt(1 / r / r - 1)) -
            (1 + 3. / 2. * r * r) * sqrt(1 - r * r));
  return 4 * kPi * kAlpha * kAlpha * kHc * kHc / m / m *
         ((1 + r * r - 1. / 4. * r * r * r * r) * 2 * log(1 / r + sqrt(1 / r / r - 1)) -
          (1 + 1. / 2. * r * r) * sqrt(1 - r * r));
}

__device__ double cs_zm(const FoldParams& f, double z, double m, int flag) {
  if (f.procID == 51) return 0.;
  const double mPart = f.mPart, aLep = f.aLep;
  if (flag == 0) {
    const double s = m * m;
    const double k = sqrt(s) / 2.;
    const double p = sqrt(k * k - mPart * mPart);
    const double norm = 2 * kPi * kAlpha * kAlpha / s * p / k;
    const double kt = -2 * k * (k - z * p) / mPart / mPart;
    const double ku = -2 * k * (k + z * p) / mPart / mPart;
    const double ks = kt + ku, kp = kt * ku, kq = 1. / kt + 1. / ku, kr = ku / kt + kt / ku;
    double cs = 0;
    cs += -8. * (4. * kq * kq + 4. * kq - kr);
    cs += 16. * (2. + kr) * aLep;
    cs += 4. * (2. - 4. * ks + kr) * aLep * aLep;
    cs += -8. * (2. + 2. * ks + kr) * aLep * aLep * aLep;
    cs += -4. * (4. + 2. * ks + 2. * kr - kp) * aLep * aLep * aLep * aLep;
    return cs * norm;
  }
  const double mLep2 = mPart * mPart, m2 = m * m, z2 = z * z;
  double cs = 2 * kPi * kAlpha * kAlpha;
  if (flag == 1) {
    cs *= m2 - 4 * mLep2;
    cs *= sqrt(m2 - 4 * mLep2);
    cs *= (4 * mLep2 * (3 - 2 * z2 + z2 * z2)) + m2 * (1 - z2 * z2);
  } else {
    cs *= sqrt(m2 - 4 * mLep2);
    cs *= m2 * m2 * (1 - z2 * z2) + 8 * m2 * mLep2 * (1 - z2 + z2 * z2) -
          16 * mLep2 * mLep2 * (1 - z2) * (1 - z2);
  }
  cs /= m2 * m * (m2 * (1 - z2) + 4 * mLep2 * z2) * (m2 * (1 - z2) + 4 * mLep2 * z2);
  return cs;
}

__global__ void k_cs_zm(FoldParams f, int flag, double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= f.nm * f.nz) return;
  const int im = i / f.nz, iz = i - im * f.nz;
  constexpr double scalingFactor = 0.1973269718 * 0.1973269718 * 1e7;
  const double m = f.mmin + f.dm * im;
  const double z = f.zmin + f.dz * iz;
  out[i] = cs_zm(f, z, m, flag) * scalingFactor / f.dm;
}

__global__ void k_cs_m_pts(FoldParams f, const double* __restrict__ m, double* __restrict__ out,
                           int n, int flag) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = cs_m(f, m[i], flag);
}

constexpr int kFoldThreads = 256;

// cs[iy][im] and one partial sum of cs per block (fixed order).
__global__ void __launch_bounds__(kFoldThreads) k_fold(FoldParams f, const double* __restrict__ lumi,
                                                       const double* __restrict__ lumi2,
                                                       double* __restrict__ cs,
                                                       double* __restrict__ ratio,
                                                       double* __restrict__ partial) {
  __shared__ double red[kFoldThreads];
  const int n = f.nm * f.ny;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;  // i = im*ny + iy
  double v = 0.;
  if (i < n) {
    const int im = i / f.ny, iy = i - im * f.ny;
    const double m = f.mmin + f.dm * im;
    const size_t co = (size_t)iy * f.nm + im;
    if (!f.polarized) {
      v = cs_m(f, m, 0) * lumi[i];
    } else {
      const double s = lumi[i] * cs_m(f, m, 1);
      const double p = lumi2[i] * cs_m(f, m, 2);
      v = (s + p) * 1e7;
      ratio[co] = s / p;
    }
    cs[co] = v;
  }
  red[threadIdx.x] = v;
  __syncthreads();
  for (int s = kFoldThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

__global__ void k_reduce_total(const double* __restrict__ partial, int n, double scale,
                               double* __restrict__ out) {
  __shared__ double red[1024];
  double v = 0.;
  for (int i = threadIdx.x; i < n; i += blockDim.x) v += partial[i];
  red[threadIdx.x] = v;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0] * scale;
}

// One CTA builds the normalised cumulative sum of n weights (n up to a few 1e6).
constexpr int kCdfThreads = 1024;

__global__ void __launch_bounds__(kCdfThreads) k_cdf_2d(const double* __restrict__ w, int64_t n,
                                                        double* __restrict__ cdf) {
  __shared__ double red[kCdfThreads];
  const int t = threadIdx.x;
  const int64_t chunk = (n + kCdfThreads - 1) / kCdfThreads;
  const int64_t lo = t * chunk, hi = lo + chunk < n ? lo + chunk : n;
  double s = 0.;
  for (int64_t i = lo; i < hi; ++i) s += w[i];
  red[t] = s;
  __syncthreads();
  for (int st = kCdfThreads / 2; st > 0; st >>= 1) {
    if (t < st) red[t] += red[t + st];
    __syncthreads();
  }
  const double mean = red[0] / (double)n;
  __syncthreads();
  double loc = 0.;
  for (int64_t i = lo; i < hi; ++i) loc += (w[i] / mean) / n;
  red[t] = loc;
  __syncthreads();
  // inclusive Hillis-Steele scan of the per-thread sums
  for (int off = 1; off < kCdfThreads; off <<= 1) {
    const double add = t >= off ? red[t - off] : 0.;
    __syncthreads();
    red[t] += add;
    __syncthreads();
  }
  double run = t > 0 ? red[t - 1] : 0.;
  if (t == 0) cdf[0] = 0.;
  for (int64_t i = lo; i < hi; ++i) {
    run += (w[i] / mean) / n;
    cdf[i + 1] = run;
  }
}

// One thread per row, exactly the sequential GSL recurrence (running mean).
__global__ void k_cdf_rows(const double* __restrict__ w, int rows, int len,
                           double* __restrict__ cdf) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rows) return;
  const double* x = w + (size_t)r * len;
  double* c = cdf + (size_t)r * (len + 1);
  double mean = 0;
  for (int i = 0; i < len; i++) mean += (x[i] - mean) / ((double)(i + 1));
  double s = 0;
  c[0] = 0;
  for (int i = 0; i < len; i++) {
    s += (x[i] / mean) / len;
    c[i + 1] = s;
  }
}

}  // namespace

cudaError_t launch_cs_zm(const FoldParams& f, int flag, double* d_out, cudaStream_t st) {
  const int n = f.nm * f.nz;
  k_cs_zm<<<(n + 255) / 256, 256, 0, st>>>(f, flag, d_out);
  return cudaGetLastError();
}

cudaError_t launch_cs_m_points(const FoldParams& f, const double* d_m, double* d_out, int n,
                               int flag, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  k_cs_m_pts<<<(n + 255) / 256, 256, 0, st>>>(f, d_m, d_out, n, flag);
  return cudaGetLastError();
}

cudaError_t launch_fold(const FoldParams& f, const double* d_lumi, const double* d_lumi2,
                        double* d_cs, double* d_ratio, double* d_partial, double* d_tot,
                        cudaStream_t st) {
  const int n = f.nm * f.ny;
  const int blocks = (n + kFoldThreads - 1) / kFoldThreads;
  k_fold<<<blocks, kFoldThreads, 0, st>>>(f, d_lumi, d_lumi2, d_cs, d_ratio, d_partial);
  k_reduce_total<<<1, 1024, 0, st>>>(d_partial, blocks, 1e-6, d_tot);
  return cudaGetLastError();
}

cudaError_t launch_cdf_2d(const double* d_w, int64_t n, double* d_cdf, double* d_scratch,
                          cudaStream_t st) {
  (void)d_scratch;
  k_cdf_2d<<<1, kCdfThreads, 0, st>>>(d_w, n, d_cdf);
  return cudaGetLastError();
}

cudaError_t launch_cdf_rows(const double* d_w, int rows, int len, double* d_cdf,
                            cudaStream_t st) {
  k_cdf_rows<<<(rows + 127) / 128, 128, 0, st>>>(d_w, rows, len, d_cdf);
  return cudaGetLastError();
}

}  // namespace upcg
