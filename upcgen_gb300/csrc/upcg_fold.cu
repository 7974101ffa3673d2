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

// The unpolarized dilepton dsigma/dz of cs_zm (flag 0) with fewer FP64
// divisions (the 1/64-rate pipe): 1 / mPart^2 and the scale per launch, one
// reciprocal 1 / (kt ku) for kq = 1/kt + 1/ku and kr = ku/kt + kt/ku.  The
// same terms in the same order otherwise; they do not cancel, so the values
// move by rounding only (~1e-16 relative).
__device__ __forceinline__ double cs_zm_dilep(const FoldParams& f, double z, double m,
                                              double inv_mp2) {
  const double mPart = f.mPart, aLep = f.aLep;
  const double s = m * m;
  const double k = sqrt(s) / 2.;
  const double p = sqrt(k * k - mPart * mPart);
  const double norm = 2 * kPi * kAlpha * kAlpha / s * p / k;
  const double kt = -2 * k * (k - z * p) * inv_mp2;
  const double ku = -2 * k * (k + z * p) * inv_mp2;
  const double ks = kt + ku, kp = kt * ku, ir = 1. / kp;
  const double kq = ks * ir, kr = (ku * ku + kt * kt) * ir;
  double cs = 0;
  cs += -8. * (4. * kq * kq + 4. * kq - kr);
  cs += 16. * (2. + kr) * aLep;
  cs += 4. * (2. - 4. * ks + kr) * aLep * aLep;
  cs += -8. * (2. + 2. * ks + kr) * aLep * aLep * aLep;
  cs += -4. * (4. + 2. * ks + 2. * kr - kp) * aLep * aLep * aLep * aLep;
  return cs * norm;
}

__global__ void k_cs_zm(FoldParams f, int flag, double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= f.nm * f.nz) return;
  const int im = i / f.nz, iz = i - im * f.nz;
  constexpr double scalingFactor = 0.1973269718 * 0.1973269718 * 1e7;
  const double m = f.mmin + f.dm * im;
  const double z = f.zmin + f.dz * iz;
  if (flag == 0 && f.procID != 51)
    out[i] = cs_zm_dilep(f, z, m, 1. / (f.mPart * f.mPart)) * (scalingFactor / f.dm);
  else
    out[i] = cs_zm(f, z, m, flag) * scalingFactor / f.dm;
}

__global__ void k_cs_m_pts(FoldParams f, const double* __restrict__ m, double* __restrict__ out,
                           int n, int flag) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = cs_m(f, m[i], flag);
}


// sigma(m) of every mass row, once per row rather than once per cell: the FP64
// cross section runs on the 1/64-rate pipe, which a warp of cells of one row
// would occupy 32 times for one value.  Polarized: scalar in csm[0, nm),
// pseudoscalar in csm[nm, 2 nm).
__global__ void k_cs_m_rows(FoldParams f, double* __restrict__ csm) {
  const int im = blockIdx.x * blockDim.x + threadIdx.x;
  if (im >= f.nm) return;
  const double m = f.mmin + f.dm * im;
  if (!f.polarized) {
    csm[im] = cs_m(f, m, 0);
  } else {
    csm[im] = cs_m(f, m, 1);
    csm[f.nm + im] = cs_m(f, m, 2);
  }
}

// Normalised cumulative sum of n weights (gsl_histogram_pdf_init:
// cdf[0] = 0, cdf[i+1] = cdf[i] + (w_i / mean) / n) as a three-level scan over
// tiles of kCdfTile weights: tile sums of w -> mean; tile sums of the scaled
// terms -> exclusive tile offsets; per-tile scan with its offset.  Only the
// summation order differs from the sequential recurrence (relative 1e-16).
constexpr int kCdfThreads = 256;
constexpr int kCdfItems = 4;
constexpr int kCdfTile = kCdfThreads * kCdfItems;

__device__ __forceinline__ double block_sum(double v, double* red) {
  const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if (lane == 0) red[wid] = v;
  __syncthreads();
  double s = 0.;
  for (int w = 0; w < kCdfThreads / 32; ++w) s += red[w];
  __syncthreads();
  return s;
}

// mode 0: tile sums of w; mode 1: tile sums of (w / mean) / n
__global__ void __launch_bounds__(kCdfThreads) k_cdf_tiles(const double* __restrict__ w, int64_t n,
                                                          const double* __restrict__ mean, int mode,
                                                          double* __restrict__ part) {
  __shared__ double red[kCdfThreads / 32];
  const int64_t base = (int64_t)blockIdx.x * kCdfTile;
  const double m = mode ? *mean : 1.;
  double v = 0.;
#pragma unroll
  for (int k = 0; k < kCdfItems; ++k) {
    const int64_t i = base + (int64_t)threadIdx.x * kCdfItems + k;
    if (i < n) v += mode ? (w[i] / m) / (double)n : w[i];
  }
  const double s = block_sum(v, red);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// one CTA: mode 0 -> mean = sum(part) / n; mode 1 -> exclusive scan of part
__global__ void __launch_bounds__(1024) k_cdf_top(double* __restrict__ part, int ntiles, int64_t n,
                                                  int mode, double* __restrict__ mean) {
  __shared__ double sh[1024];
  const int t = threadIdx.x;
  const int per = (ntiles + 1023) / 1024;
  const int lo = t * per, hi = lo + per < ntiles ? lo + per : ntiles;
  double loc = 0.;
  for (int i = lo; i < hi; ++i) loc += part[i];
  sh[t] = loc;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {  // inclusive Hillis-Steele scan
    const double add = t >= off ? sh[t - off] : 0.;
    __syncthreads();
    sh[t] += add;
    __syncthreads();
  }
  if (mode == 0) {
    if (t == 0) *mean = sh[1023] / (double)n;
    return;
  }
  double run = t > 0 ? sh[t - 1] : 0.;
  for (int i = lo; i < hi; ++i) {
    const double v = part[i];
    part[i] = run;
    run += v;
  }
}

__global__ void __launch_bounds__(kCdfThreads) k_cdf_write(const double* __restrict__ w, int64_t n,
                                                          const double* __restrict__ mean,
                                                          const double* __restrict__ off,
                                                          double* __restrict__ cdf) {
  __shared__ double sh[kCdfThreads];
  const int t = threadIdx.x;
  const int64_t base = (int64_t)blockIdx.x * kCdfTile + (int64_t)t * kCdfItems;
  const double m = *mean;
  double v[kCdfItems];
  double loc = 0.;
#pragma unroll
  for (int k = 0; k < kCdfItems; ++k) {
    const int64_t i = base + k;
    v[k] = i < n ? (w[i] / m) / (double)n : 0.;
    loc += v[k];
  }
  sh[t] = loc;
  __syncthreads();
  for (int o = 1; o < kCdfThreads; o <<= 1) {
    const double add = t >= o ? sh[t - o] : 0.;
    __syncthreads();
    sh[t] += add;
    __syncthreads();
  }
  double run = off[blockIdx.x] + (t > 0 ? sh[t - 1] : 0.);
  if (blockIdx.x == 0 && t == 0) cdf[0] = 0.;
#pragma unroll
  for (int k = 0; k < kCdfItems; ++k) {
    const int64_t i = base + k;
    run += v[k];
    if (i < n) cdf[i + 1] = run;
  }
}

// Row-wise normalised cumulative sums (gsl_histogram_pdf_init per row:
// cdf[0] = 0, cdf[i+1] = cdf[i] + (w_i / mean) / len), one warp per row: the
// mean as the row's sum / len, the terms (w_i / mean) / len by all lanes, and
// their running sum by a warp scan.  Only the summation order (and the mean's
// rounding) differs from the sequential recurrence (relative 1e-16).
__global__ void k_cdf_rows(const double* __restrict__ w, int rows, int len,
                           double* __restrict__ cdf) {
  const int r = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (r >= rows) return;  // the whole warp: r is the same for its lanes
  const double* x = w + (size_t)r * len;
  double* c = cdf + (size_t)r * (len + 1);
  double sum = 0.;
  for (int i = lane; i < len; i += 32) sum += x[i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
  const double mean = sum / (double)len;
  if (lane == 0) c[0] = 0.;
  double run = 0.;
  for (int i0 = 0; i0 < len; i0 += 32) {
    const int i = i0 + lane;
    double t = i < len ? (x[i] / mean) / (double)len : 0.;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const double u = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += u;
    }
    t += run;
    if (i < len) c[i + 1] = t;
    run = __shfl_sync(0xffffffffu, t, 31);
  }
}

// The two-photon cross section's fold and its sampling CDF in three launches
// (the samplers' cell order co = iy * nm + im, tiles of kCdfTile cells):
//   k_fold_tiles     cs[co] = sigma(m) L (calcNucCrossSectionYM,
//                    src/UpcCrossSection.cpp:594-698; the polarized ratio),
//                    and each tile's sum of cs;
//   k_cdf_top_total  exclusive offsets of the tile sums, the total (sigma_tot
//                    = total * scale) and 1 / total;
//   k_cdf_write_fx   cdf[i + 1] = (w_0 + ... + w_i) / total per tile from its
//                    offset, with the fixed-point copy of every entry.
// The CDF is gsl_histogram2d_pdf_init's, (w_i / mean) / n summed, up to the
// rounding of the normalisation: the sum is taken first and scaled once.
__global__ void __launch_bounds__(kCdfThreads) k_fold_tiles(FoldParams f,
                                                           const double* __restrict__ lumi,
                                                           const double* __restrict__ lumi2,
                                                           const double* __restrict__ csm,
                                                           double* __restrict__ cs,
                                                           double* __restrict__ ratio,
                                                           double* __restrict__ part) {
  __shared__ double red[kCdfThreads / 32];
  const int64_t n = (int64_t)f.nm * f.ny;
  const int64_t base = (int64_t)blockIdx.x * kCdfTile;
  double loc = 0.;
#pragma unroll
  for (int k = 0; k < kCdfItems; ++k) {
    const int64_t co = base + (int64_t)k * kCdfThreads + threadIdx.x;
    if (co < n) {
      const int iy = (int)(co / f.nm), im = (int)(co - (int64_t)iy * f.nm);
      const size_t i = (size_t)im * f.ny + iy;
      double v;
      if (!f.polarized) {
        v = __ldg(csm + im) * lumi[i];
      } else {
        const double sc = lumi[i] * __ldg(csm + im);
        const double ps = lumi2[i] * __ldg(csm + f.nm + im);
        v = (sc + ps) * 1e7;
        ratio[co] = sc / ps;
      }
      cs[co] = v;
      loc += v;
    }
  }
  const double sum = block_sum(loc, red);
  if (threadIdx.x == 0) part[blockIdx.x] = sum;
}

__global__ void __launch_bounds__(1024) k_cdf_top_total(double* __restrict__ part, int ntiles,
                                                        double scale, double* __restrict__ tot,
                                                        double* __restrict__ inv) {
  __shared__ double sh[1024];
  const int t = threadIdx.x;
  const int per = (ntiles + 1023) / 1024;
  const int lo = t * per, hi = lo + per < ntiles ? lo + per : ntiles;
  double loc = 0.;
  for (int i = lo; i < hi; ++i) loc += part[i];
  sh[t] = loc;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {  // inclusive Hillis-Steele scan
    const double add = t >= off ? sh[t - off] : 0.;
    __syncthreads();
    sh[t] += add;
    __syncthreads();
  }
  if (t == 0) {
    *tot = sh[1023] * scale;
    *inv = 1. / sh[1023];
  }
  double run = t > 0 ? sh[t - 1] : 0.;
  for (int i = lo; i < hi; ++i) {
    const double v = part[i];
    part[i] = run;
    run += v;
  }
}

__global__ void __launch_bounds__(kCdfThreads) k_cdf_write_fx(const double* __restrict__ w,
                                                             int64_t n,
                                                             const double* __restrict__ inv_p,
                                                             const double* __restrict__ off,
                                                             double* __restrict__ cdf,
                                                             uint64_t* __restrict__ cdffx) {
  __shared__ double sh[kCdfThreads];
  const int t = threadIdx.x;
  const int64_t base = (int64_t)blockIdx.x * kCdfTile + (int64_t)t * kCdfItems;
  const double inv = *inv_p;
  double v[kCdfItems];
  double loc = 0.;
#pragma unroll
  for (int k = 0; k < kCdfItems; ++k) {
    const int64_t i = base + k;
    v[k] = i < n ? w[i] : 0.;
    loc += v[k];
  }
  sh[t] = loc;
  __syncthreads();
  for (int o = 1; o < kCdfThreads; o <<= 1) {
    const double add = t >= o ? sh[t - o] : 0.;
    __syncthreads();
    sh[t] += add;
    __syncthreads();
  }
  double run = off[blockIdx.x] + (t > 0 ? sh[t - 1] : 0.);
  if (blockIdx.x == 0 && t == 0) {
    cdf[0] = 0.;
    cdffx[0] = 0ull;
  }
#pragma unroll
  for (int k = 0; k < kCdfItems; ++k) {
    const int64_t i = base + k;
    run += v[k];
    if (i < n) {
      const double c = run * inv;
      cdf[i + 1] = c;
      cdffx[i + 1] = cdf_to_fx(c);
    }
  }
}

}  // namespace

cudaError_t launch_cs_zm(const FoldParams& f, int flag, double* d_out, cudaStream_t st) {
  const int n = f.nm * f.nz;
  note_launch();
  carveout_max_shared<k_cs_zm>();
  k_cs_zm<<<(n + 255) / 256, 256, 0, st>>>(f, flag, d_out);
  return cudaGetLastError();
}

cudaError_t launch_cs_m_points(const FoldParams& f, const double* d_m, double* d_out, int n,
                               int flag, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  note_launch();
  k_cs_m_pts<<<(n + 255) / 256, 256, 0, st>>>(f, d_m, d_out, n, flag);
  return cudaGetLastError();
}

cudaError_t launch_cs_m_rows(const FoldParams& f, double* d_csm, cudaStream_t st) {
  note_launch();
  carveout_max_shared<k_cs_m_rows>();
  k_cs_m_rows<<<(f.nm + 127) / 128, 128, 0, st>>>(f, d_csm);
  return cudaGetLastError();
}

cudaError_t launch_fold_cdf(const FoldParams& f, const double* d_lumi, const double* d_lumi2,
                            const double* d_csm, double* d_cs, double* d_ratio, double* d_scratch,
                            double* d_tot, double* d_cdf, uint64_t* d_cdffx, cudaStream_t st) {
  const int64_t n = (int64_t)f.nm * f.ny;
  const int ntiles = (int)((n + kCdfTile - 1) / kCdfTile);
  double* part = d_scratch;  // cdf_2d_scratch_doubles(n): tile sums | 1 / total
  double* inv = d_scratch + ntiles + 1;
  note_launch();
  k_fold_tiles<<<ntiles, kCdfThreads, 0, st>>>(f, d_lumi, d_lumi2, d_csm, d_cs, d_ratio, part);
  note_launch();
  k_cdf_top_total<<<1, 1024, 0, st>>>(part, ntiles, 1e-6, d_tot, inv);
  note_launch();
  k_cdf_write_fx<<<ntiles, kCdfThreads, 0, st>>>(d_cs, n, inv, part, d_cdf, d_cdffx);
  return cudaGetLastError();
}

int cdf_2d_scratch_doubles(int64_t n) { return (int)((n + kCdfTile - 1) / kCdfTile) + 2; }

cudaError_t launch_cdf_2d(const double* d_w, int64_t n, double* d_cdf, double* d_scratch,
                          cudaStream_t st) {
  // d_scratch: tile sums | mean (cdf_2d_scratch_doubles(n))
  const int ntiles = (int)((n + kCdfTile - 1) / kCdfTile);
  double* part = d_scratch;
  double* mean = d_scratch + ntiles + 1;
  note_launch();
  k_cdf_tiles<<<ntiles, kCdfThreads, 0, st>>>(d_w, n, mean, 0, part);
  note_launch();
  k_cdf_top<<<1, 1024, 0, st>>>(part, ntiles, n, 0, mean);
  note_launch();
  k_cdf_tiles<<<ntiles, kCdfThreads, 0, st>>>(d_w, n, mean, 1, part);
  note_launch();
  k_cdf_top<<<1, 1024, 0, st>>>(part, ntiles, n, 1, mean);
  note_launch();
  k_cdf_write<<<ntiles, kCdfThreads, 0, st>>>(d_w, n, mean, part, d_cdf);
  return cudaGetLastError();
}

cudaError_t launch_cdf_rows(const double* d_w, int rows, int len, double* d_cdf,
                            cudaStream_t st) {
  note_launch();
  // one warp per row, four rows per block
  carveout_max_shared<k_cdf_rows>();
  k_cdf_rows<<<(rows + 3) / 4, 128, 0, st>>>(d_w, rows, len, d_cdf);
  return cudaGetLastError();
}

}  // namespace upcg
