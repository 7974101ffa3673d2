// Two-photon luminosity, plain FP64 path.
//
// Reference: src/UpcCrossSection.cpp
//   fluxPoint :166-178, fluxFormIntegrand/fluxForm :181-218
//   calcTwoPhotonLumi :221-271, calcTwoPhotonLumiPol :274-335
//   prepareTwoPhotonLumi :463-592 (cells at left bin edges, lumi*dm*dy)
//
// Three launches per batch of (m,y) cells:
//   k_lumi_nodes  one CTA per cell: the 2x120 log-spaced impact-parameter nodes
//                 of the cell and the point-charge flux at every node that does
//                 not need the form-factor integral (K0/K1 in FP64);
//   k_lumi_qags   one warp per (cell, side): the Woods-Saxon flux at the nodes
//                 with b <= 2R by QUADPACK QAGS, the 21 Gauss-Kronrod points of
//                 a rule evaluated by 21 lanes and the adaptive bookkeeping
//                 replicated on every lane, the interval list in shared memory;
//   k_lumi_band   one CTA per cell: the 120x120x5 quadrature.  For b >= 20 fm
//                 the survival weight is the constant P(20) (G_AA = 1), so
//                 L = 2 pi^2 M [c S1 S2 + sum_{band} w1_i w2_j (g_ij - c)],
//                 with c = P(20) * sum_k w_k and S = sum_i w_i, where the band
//                 is the set of node pairs for which some azimuth gives b < 20.
//                 This is the reference's sum regrouped; pairs outside the band
//                 contribute exactly zero to the second term.
#include <mutex>

#include "upcg_internal.h"

namespace upcg {

namespace {

struct CellGeom {
  double M, Y, k[2], bmin, ld[2];
};

__device__ __forceinline__ void cell_geom(const LumiParams& p, int cell, CellGeom& g) {
  const int im = cell / p.ny, iy = cell - (cell / p.ny) * p.ny;
  g.M = p.mmin + p.dm * im;
  g.Y = p.ymin + p.dy * iy;
  g.k[0] = g.M / 2. * exp(g.Y);
  g.k[1] = g.M / 2. * exp(-g.Y);
  g.bmin = p.isPoint ? p.R : 0.05 * p.R;
  const double b1max = fmax(5. * p.g1 * kHc / g.k[0], 5. * p.R);
  const double b2max = fmax(5. * p.g2 * kHc / g.k[1], 5. * p.R);
  g.ld[0] = (log(b1max) - log(g.bmin)) / kNb;
  g.ld[1] = (log(b2max) - log(g.bmin)) / kNb;
}

__device__ __forceinline__ void node_b(double bmin, double ld, int i, double& b, double& w) {
  const double bl = bmin * exp(i * ld);
  const double bh = bmin * exp((i + 1) * ld);
  b = (bh + bl) / 2.;
  w = b * (bh - bl);
}

__device__ __forceinline__ double flux_point(const LumiParams& p, double b, double k) {
  const double g = p.g1;
  const double x = b * k / g / kHc;
  double K0 = 0, K1 = 0;
  if (x > 1e-10) bessel_k01(x, K0, K1);
  return p.factor * k / g / g * (K1 * K1 + K0 * K0 / g / g);
}

// ------------------------------------------------------------ nodes ----
__global__ void __launch_bounds__(256) k_lumi_nodes(LumiParams p, int cell0, double* __restrict__ flux,
                                                    int* __restrict__ nq) {
  __shared__ int cnt[2];
  const int cell = cell0 + blockIdx.x;
  const int side = threadIdx.x >> 7, i = threadIdx.x & 127;
  if (threadIdx.x < 2) cnt[threadIdx.x] = 0;
  __syncthreads();
  const int iy = cell - (cell / p.ny) * p.ny;
  const bool mirrored = side == 1 && p.mirror != nullptr && p.mirror[iy] >= 0;
  if (i < kNb && !mirrored) {
    CellGeom g;
    cell_geom(p, cell, g);
    double b, w;
    node_b(g.bmin, g.ld[side], i, b, w);
    double* out = flux + ((size_t)blockIdx.x * 2 + side) * kNb;
    if (p.isPoint || b > 2. * p.R) {
      out[i] = flux_point(p, b, g.k[side]);
    } else {
      atomicAdd(&cnt[side], 1);
    }
  }
  __syncthreads();
  if (threadIdx.x < 2) nq[(size_t)blockIdx.x * 2 + threadIdx.x] = cnt[threadIdx.x];
}

// ------------------------------------------------------------- QAGS ----
template <int CAP>
struct QWs {
  double lo[CAP], hi[CAP], r[CAP], e[CAP];
  int order[CAP], level[CAP];
  double tab[54];  // the epsilon table never holds more than 50 entries
  double hist[3];
};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ double ff_integrand(const LumiParams& p, double q, double b,
                                               double wg2) {
  const double t = q * q + wg2;
  const double ffv = spline_eval(p.ff, t < p.q2max ? t : p.q2clamp);
  return q * q * ffv / t * j1(b * q / kHc);
}

__device__ __forceinline__ double rescale_err(double err, double resabs, double resasc) {
  err = fabs(err);
  if (resasc != 0 && err != 0) {
    const double q = 200 * err / resasc;
    const double scale = q * sqrt(q);  // (200 err / resasc)^1.5
    err = scale < 1 ? resasc * scale : resasc;
  }
  if (resabs > 2.2250738585072014e-308 / (50 * 2.220446049250313e-16)) {
    const double fl = 50 * 2.220446049250313e-16 * resabs;
    if (fl > err) err = fl;
  }
  return err;
}

// 21-point Gauss-Kronrod rule on [a, bb]; lanes 0..20 hold one node each.
__device__ void warp_qk21(const LumiParams& p, double bq, double wg2, double a, double bb,
                          double& result, double& abserr, double& resabs, double& resasc) {
  const int lane = threadIdx.x & 31;
  const double center = 0.5 * (a + bb);
  const double half = 0.5 * (bb - a);
  double x = center, wk = 0.0, wgs = 0.0;
  if (lane == 0) {
    wk = kWgk[10];
  } else if (lane < 21) {
    const int j = (lane - 1) >> 1;
    const double dx = half * kXgk[j];
    x = (lane & 1) ? center - dx : center + dx;
    wk = kWgk[j];
    wgs = (j & 1) ? kWg[j >> 1] : 0.0;
  }
  const double f = lane < 21 ? ff_integrand(p, x, bq, wg2) : 0.0;
  const double sk = warp_sum(wk * f);
  const double sg = warp_sum(wgs * f);
  const double sa = warp_sum(wk * fabs(f));
  const double mean = 0.5 * sk;
  const double sc = warp_sum(lane < 21 ? wk * fabs(f - mean) : 0.0);
  const double err = (sk - sg) * half;
  result = sk * half;
  resabs = sa * fabs(half);
  resasc = sc * fabs(half);
  abserr = rescale_err(err, resabs, resasc);
}

constexpr double kEps = 2.220446049250313e-16;
constexpr double kDblMax = 1.7976931348623157e308;
constexpr double kDblMin = 2.2250738585072014e-308;

// Insertion of the newest intervals into the error-ordered list (QUADPACK qpsrt).
template <int CAP>
__device__ __forceinline__ void qs_sort(QWs<CAP>* w, int size, int& nrmax, int& cur) {
  const int last = size - 1;
  int nr = nrmax;
  const int imax = w->order[nr];
  if (last < 2) {
    w->order[0] = 0;
    w->order[1] = 1;
    cur = imax;
    return;
  }
  const double emax = w->e[imax];
  while (nr > 0 && emax > w->e[w->order[nr - 1]]) {
    w->order[nr] = w->order[nr - 1];
    --nr;
  }
  const int top = (last < kQagsLimit / 2 + 2) ? last : kQagsLimit - last + 1;
  int i = nr + 1;
  while (i < top && emax < w->e[w->order[i]]) {
    w->order[i - 1] = w->order[i];
    ++i;
  }
  w->order[i - 1] = imax;
  const double emin = w->e[last];
  int k = top - 1;
  while (k > i - 2 && emin >= w->e[w->order[k]]) {
    w->order[k + 1] = w->order[k];
    --k;
  }
  w->order[k + 1] = last;
  cur = w->order[nr];
  nrmax = nr;
}

// Wynn epsilon extrapolation (QUADPACK qelg, with GSL's result-history update).
template <int CAP>
__device__ void qs_eps(QWs<CAP>* w, int& n, int& nres, double* result, double* abserr) {
  double* tab = w->tab;
  const int n0 = n - 1;
  const double cur = tab[n0];
  *result = cur;
  *abserr = kDblMax;
  if (n0 < 2) return;
  tab[n0 + 2] = tab[n0];
  const int newelm = n0 / 2;
  tab[n0] = kDblMax;
  int nfin = n0;
  for (int i = 0; i < newelm; ++i) {
    double res = tab[n0 - 2 * i + 2];
    const double e0 = tab[n0 - 2 * i - 2];
    const double e1 = tab[n0 - 2 * i - 1];
    const double e2 = res;
    const double d2 = e2 - e1, a2 = fabs(d2);
    const double t2 = fmax(fabs(e2), fabs(e1)) * kEps;
    const double d3 = e1 - e0, a3 = fabs(d3);
    const double t3 = fmax(fabs(e1), fabs(e0)) * kEps;
    if (a2 < t2 && a3 < t3) {
      *result = res;
      *abserr = fmax(a2 + a3, 5 * kEps * fabs(res));
      return;
    }
    const double e3 = tab[n0 - 2 * i];
    tab[n0 - 2 * i] = e1;
    const double d1 = e1 - e3, a1 = fabs(d1);
    const double t1 = fmax(fabs(e1), fabs(e3)) * kEps;
    if (a1 < t1 || a2 < t2 || a3 < t3) {
      nfin = 2 * i;
      break;
    }
    const double ss = (1 / d1 + 1 / d2) - 1 / d3;
    if (fabs(ss * e1) <= 1e-4) {
      nfin = 2 * i;
      break;
    }
    res = e1 + 1 / ss;
    tab[n0 - 2 * i] = res;
    const double err = a2 + fabs(res - e2) + a3;
    if (err <= *abserr) {
      *abserr = err;
      *result = res;
    }
  }
  if (nfin == 49) nfin = 48;
  if (n0 % 2 == 1) {
    for (int i = 0; i <= newelm; ++i) tab[1 + 2 * i] = tab[2 * i + 3];
  } else {
    for (int i = 0; i <= newelm; ++i) tab[2 * i] = tab[2 * i + 2];
  }
  if (n0 != nfin)
    for (int i = 0; i <= nfin; ++i) tab[i] = tab[n0 - nfin + i];
  n = nfin + 1;
  if (nres < 3) {
    w->hist[nres] = *result;
    *abserr = kDblMax;
  } else {
    *abserr = fabs(*result - w->hist[2]) + fabs(*result - w->hist[1]) + fabs(*result - w->hist[0]);
    w->hist[0] = w->hist[1];
    w->hist[1] = w->hist[2];
    w->hist[2] = *result;
  }
  ++nres;
  *abserr = fmax(*abserr, 5 * kEps * fabs(*result));
}

// QAGS of the form-factor flux integrand on [0, 10] with epsabs = epsrel = 1e-4
// and limit 1000 (src/UpcCrossSection.cpp:209).  Returns the GSL status, or -1
// when more than CAP intervals would be needed (the caller re-runs the node
// with a larger workspace).
template <int CAP>
__device__ int warp_qags(const LumiParams& p, double bq, double wg2, QWs<CAP>* w,
                         double* out, int* nint, int* nevals) {
  const double a = 0., b = 10., epsabs = 1e-4, epsrel = 1e-4;
  const int limit = kQagsLimit;
  int nev = 21;
  double r0, e0, rabs0, rasc0;
  warp_qk21(p, bq, wg2, a, b, r0, e0, rabs0, rasc0);
  double tol = fmax(epsabs, epsrel * fabs(r0));
  *nint = 1;
  if (e0 <= 100 * kEps * rabs0 && e0 > tol) { *out = r0; *nevals = nev; return 18; }
  if ((e0 <= tol && e0 != rasc0) || e0 == 0.0) { *out = r0; *nevals = nev; return 0; }
  const int lane = threadIdx.x & 31;
  int size = 1, nrmax = 0, cur = 0, max_level = 0;
  int tn = 0, nres = 0;
  if (lane == 0) {
    w->lo[0] = a; w->hi[0] = b; w->r[0] = r0; w->e[0] = e0; w->order[0] = 0; w->level[0] = 0;
    w->tab[0] = r0;
  }
  tn = 1;
  __syncwarp();
  double area = r0, errsum = e0, res_ext = r0, err_ext = kDblMax;
  double ertest = 0, err_large = 0, correc = 0;
  int ktmin = 0, rt1 = 0, rt2 = 0, rt3 = 0, err_type = 0, err_type2 = 0;
  int iter = 1;
  const bool positive = fabs(r0) >= (1 - 50 * kEps) * rabs0;
  bool extrap = false, no_extrap = false, final_sum = false, to_return = false;
  do {
    const int im = cur;
    const double ai = w->lo[im], bi = w->hi[im], ri = w->r[im], ei = w->e[im];
    const int lvl = w->level[im] + 1;
    const double a1 = ai, b1 = 0.5 * (ai + bi), a2 = b1, b2 = bi;
    ++iter;
    double ar1, er1, rb1, rc1, ar2, er2, rb2, rc2;
    warp_qk21(p, bq, wg2, a1, b1, ar1, er1, rb1, rc1);
    warp_qk21(p, bq, wg2, a2, b2, ar2, er2, rb2, rc2);
    nev += 42;
    const double ar12 = ar1 + ar2, er12 = er1 + er2;
    errsum = errsum + er12 - ei;
    area = area + ar12 - ri;
    tol = fmax(epsabs, epsrel * fabs(area));
    if (rc1 != er1 && rc2 != er2) {
      const double delta = ri - ar12;
      if (fabs(delta) <= 1.0e-5 * fabs(ar12) && er12 >= 0.99 * ei) {
        if (!extrap) ++rt1; else ++rt2;
      }
      if (iter > 10 && er12 > ei) ++rt3;
    }
    if (rt1 + rt2 >= 10 || rt3 >= 20) err_type = 2;
    if (rt2 >= 5) err_type2 = 1;
    {
      const double tmp = (1 + 100 * kEps) * (fabs(a2) + 1000 * kDblMin);
      if (fabs(a1) <= tmp && fabs(b2) <= tmp) err_type = 4;
    }
    if (size >= CAP) { *nevals = nev; *nint = size; return -1; }
    {  // replace the bisected interval by its halves (lane 0 owns the list)
      const int in = size;
      ++size;
      if (lvl > max_level) max_level = lvl;
      if (lane == 0) {
        if (er2 > er1) {
          w->lo[im] = a2; w->r[im] = ar2; w->e[im] = er2; w->level[im] = lvl;
          w->lo[in] = a1; w->hi[in] = b1; w->r[in] = ar1; w->e[in] = er1; w->level[in] = lvl;
        } else {
          w->hi[im] = b1; w->r[im] = ar1; w->e[im] = er1; w->level[im] = lvl;
          w->lo[in] = a2; w->hi[in] = b2; w->r[in] = ar2; w->e[in] = er2; w->level[in] = lvl;
        }
        qs_sort(w, size, nrmax, cur);
      }
      __syncwarp();
      nrmax = __shfl_sync(0xffffffffu, nrmax, 0);
      cur = __shfl_sync(0xffffffffu, cur, 0);
    }
    if (errsum <= tol) { final_sum = true; break; }
    if (err_type) break;
    if (iter >= limit - 1) { err_type = 1; break; }
    if (iter == 2) {
      err_large = errsum;
      ertest = tol;
      if (tn < 52) {
        if (lane == 0) w->tab[tn] = area;
        ++tn;
      }
      __syncwarp();
      continue;
    }
    if (no_extrap) continue;
    err_large += -ei;
    if (lvl < max_level) err_large += er12;
    if (!extrap) {
      if (w->level[cur] < max_level) continue;
      extrap = true;
      nrmax = 1;
    }
    if (!err_type2 && err_large > ertest) {
      const int last = size - 1;
      const int bound = (last > 1 + limit / 2) ? limit + 1 - last : last;
      bool found = false;
      for (int k = nrmax; k <= bound; ++k) {
        cur = w->order[nrmax];
        if (w->level[cur] < max_level) { found = true; break; }
        ++nrmax;
      }
      if (found) continue;
    }
    double reseps = 0., abseps = 0.;
    if (lane == 0) {
      if (tn < 52) w->tab[tn++] = area;
      qs_eps(w, tn, nres, &reseps, &abseps);
    }
    __syncwarp();
    tn = __shfl_sync(0xffffffffu, tn, 0);
    nres = __shfl_sync(0xffffffffu, nres, 0);
    reseps = __shfl_sync(0xffffffffu, reseps, 0);
    abseps = __shfl_sync(0xffffffffu, abseps, 0);
    ++ktmin;
    if (ktmin > 5 && err_ext < 0.001 * errsum) err_type = 5;
    if (abseps < err_ext) {
      ktmin = 0;
      err_ext = abseps;
      res_ext = reseps;
      correc = err_large;
      ertest = fmax(epsabs, epsrel * fabs(reseps));
      if (err_ext <= ertest) break;
    }
    if (tn == 1) no_extrap = true;
    if (err_type == 5) break;
    nrmax = 0;
    cur = w->order[0];
    extrap = false;
    err_large = errsum;
  } while (iter < limit);

  double result = res_ext;
  if (!final_sum) {
    if (err_ext == kDblMax) {
      final_sum = true;
    } else {
      if (err_type || err_type2) {
        if (err_type2) err_ext += correc;
        if (err_type == 0) err_type = 3;
        if (res_ext != 0.0 && area != 0.0) {
          if (err_ext / fabs(res_ext) > errsum / fabs(area)) final_sum = true;
        } else if (err_ext > errsum) {
          final_sum = true;
        } else if (area == 0.0) {
          to_return = true;
        }
      }
      if (!final_sum && !to_return) {
        const double max_area = fmax(fabs(res_ext), fabs(area));
        if (!(!positive && max_area < 0.01 * rabs0)) {
          const double ratio = res_ext / area;
          if (ratio < 0.01 || ratio > 100.0 || errsum > fabs(area)) err_type = 6;
        }
      }
    }
  }
  if (final_sum) {
    double s = 0;
    for (int k = 0; k < size; ++k) s += w->r[k];
    result = s;
  }
  if (err_type > 2) --err_type;
  const int codes[6] = {0, 11, 18, 21, 18, 22};
  *out = result;
  *nint = size;
  *nevals = nev;
  return codes[err_type < 0 ? 0 : (err_type > 5 ? 5 : err_type)];
}

__device__ __forceinline__ void record_stats(QagsStats* st, int status, int nint, int nev) {
  if ((threadIdx.x & 31) != 0 || st == nullptr) return;
  if (status > 0) atomicAdd(&st->failures, 1u);
  atomicMax(&st->max_intervals, (unsigned)nint);
  atomicAdd(&st->evals, (unsigned long long)nev);
}

constexpr int kQagsWarps = 8;

// One warp per (cell, side) pair, pairs handed out by an atomic counter.
__global__ void __launch_bounds__(kQagsWarps * 32) k_lumi_qags(
    LumiParams p, int cell0, int ncells, double* __restrict__ flux, const int* __restrict__ nq,
    unsigned int* __restrict__ work, int* __restrict__ ovf_list, int ovf_cap, QagsStats* stats) {
  __shared__ QWs<kQagsCapSmem> ws[kQagsWarps];
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  QWs<kQagsCapSmem>* w = &ws[wid];
  const unsigned npairs = 2u * (unsigned)ncells;
  unsigned fails = 0, maxint = 0;
  unsigned long long nevals = 0;
  for (;;) {
    unsigned pr = 0;
    if (lane == 0) pr = atomicAdd(work, 1u);
    pr = __shfl_sync(0xffffffffu, pr, 0);
    if (pr >= npairs) break;
    const int lc = pr >> 1, side = pr & 1;
    const int n = nq[pr];
    if (n == 0) continue;
    CellGeom g;
    cell_geom(p, cell0 + lc, g);
    const double k = g.k[side];
    const double wg2 = k * k / p.g1 / p.g1;
    double* out = flux + (size_t)pr * kNb;
    for (int i = 0; i < n; ++i) {
      double b, wt;
      node_b(g.bmin, g.ld[side], i, b, wt);
      double res;
      int nint, nev;
      const int st = warp_qags<kQagsCapSmem>(p, b, wg2, w, &res, &nint, &nev);
      if (st < 0) {
        if (lane == 0) {
          const unsigned slot = atomicAdd(&stats->overflow, 1u);
          if ((int)slot < ovf_cap) ovf_list[slot] = (int)(pr * kNb + i);
          out[i] = __longlong_as_double(0x7ff8000000000000ULL);
        }
        continue;
      }
      fails += st > 0 ? 1u : 0u;
      maxint = max(maxint, (unsigned)nint);
      nevals += (unsigned long long)nev;
      if (lane == 0) {
        const double Q = res / p.A;
        out[i] = p.factor * Q * Q / k;
      }
    }
  }
  if (lane == 0 && stats != nullptr) {
    if (fails) atomicAdd(&stats->failures, fails);
    atomicMax(&stats->max_intervals, maxint);
    atomicAdd(&stats->evals, nevals);
  }
}

// Nodes that overflowed the shared-memory interval list: re-run with the full
// 1000-interval workspace in global memory.
__global__ void __launch_bounds__(128) k_lumi_qags_overflow(
    LumiParams p, int cell0, double* __restrict__ flux, const int* __restrict__ list, int n_list,
    unsigned int* __restrict__ work, QagsStats* stats, double* __restrict__ gws, int gws_warps) {
  const int lane = threadIdx.x & 31;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (gw >= gws_warps) return;
  QWs<kQagsLimit>* w = reinterpret_cast<QWs<kQagsLimit>*>(gws) + gw;
  for (;;) {
    unsigned t = 0;
    if (lane == 0) t = atomicAdd(work, 1u);
    t = __shfl_sync(0xffffffffu, t, 0);
    if ((int)t >= n_list) break;
    const int idx = list[t];
    const int pr = idx / kNb, i = idx - pr * kNb;
    const int lc = pr >> 1, side = pr & 1;
    CellGeom g;
    cell_geom(p, cell0 + lc, g);
    const double k = g.k[side];
    const double wg2 = k * k / p.g1 / p.g1;
    double b, wt;
    node_b(g.bmin, g.ld[side], i, b, wt);
    double res;
    int nint, nev;
    const int st = warp_qags<kQagsLimit>(p, b, wg2, w, &res, &nint, &nev);
    record_stats(stats, st, nint, nev);
    if (lane == 0) {
      const double Q = res / p.A;
      flux[(size_t)idx] = p.factor * Q * Q / k;
    }
  }
}

// ------------------------------------------------------------- band ----
constexpr int kBandThreads = 128;

__device__ __forceinline__ double survival(const LumiParams& p, const double4* sg, double bsq,
                                           double P20) {
  // breakup * gaa of src/UpcCrossSection.cpp:257-263 at b = sqrt(bsq)
  if (bsq < 400.) {
    const double b = sqrt(bsq);
    if (b < 20.) {
      const double brk = p.breakupMode != 1 ? spline_eval(p.brk, b) : 1.;
      return brk * spline_eval_smem(p.gaa, sg, b);
    }
  }
  return P20 * 1.;
}

__global__ void __launch_bounds__(kBandThreads) k_lumi_band(LumiParams p, int cell0,
                                                          const double* __restrict__ flux,
                                                          double* __restrict__ lumi,
                                                          double* __restrict__ lumi2) {
  __shared__ double4 sg[200];
  __shared__ double sb[2][kNb], sw[2][kNb];
  __shared__ float sbf[2][kNb];
  __shared__ double sred[3][kBandThreads / 32];
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int cell = cell0 + blockIdx.x;
  CellGeom g;
  cell_geom(p, cell, g);
  for (int i = tid; i < p.gaa.n - 1; i += kBandThreads) sg[i] = p.gaa.coef[i];
  if (tid < kNb) {
    const double* f = flux + (size_t)blockIdx.x * 2 * kNb;
    const int iy = cell - (cell / p.ny) * p.ny;
    const double* f2 = f + kNb;
    if (p.mirror != nullptr && p.mirror[iy] >= 0)  // side 0 of the mirror cell (same m-row)
      f2 = flux + ((size_t)blockIdx.x + (p.mirror[iy] - iy)) * 2 * kNb;
    for (int s = 0; s < 2; ++s) {
      double b, w;
      node_b(g.bmin, g.ld[s], tid, b, w);
      sb[s][tid] = b;
      sbf[s][tid] = (float)b;
      sw[s][tid] = (s ? f2 : f)[tid] * w;  // flux * b * (bh - bl)
    }
  }
  __syncthreads();
  const double P20 = p.breakupMode != 1 ? spline_eval(p.brk, 20.) : 1.;
  double c = 0., cs = 0., cp = 0.;
  for (int q = 0; q < 5; ++q) {
    c += P20 * 1. * p.wk[q];
    cs += P20 * 1. * p.wk[q] * p.cosk[q] * p.cosk[q];
    cp += P20 * 1. * p.wk[q] * p.sink[q] * p.sink[q];
  }
  // Band rows: warp `wid` takes rows i = wid, wid+4, ...
  // cosine that gives the smallest b over the five azimuths (b^2 = b1^2 + b2^2 + 2 b1 b2 cmin)
  const float cmin = (float)(p.polarized ? -p.cosk[0] : p.cosk[4]);
  const float sgn = p.polarized ? -1.f : 1.f;
  double acc = 0., acc2 = 0.;
  for (int i = wid; i < kNb; i += kBandThreads / 32) {
    const float b1f = sbf[0][i];
    unsigned first = 0xffffffffu, last = 0;
    for (int jb = 0; jb < 4; ++jb) {
      const int j = jb * 32 + lane;
      bool in = false;
      if (j < kNb) {
        const float b2f = sbf[1][j];
        const float bmin2 = b1f * b1f + b2f * b2f + 2.f * b1f * b2f * cmin;
        in = bmin2 < 400.f * 1.001f;
      }
      const unsigned m = __ballot_sync(0xffffffffu, in);
      if (m) {
        if (first == 0xffffffffu) first = jb * 32 + __ffs(m) - 1;
        last = jb * 32 + 31 - __clz(m);
      }
    }
    if (first == 0xffffffffu) continue;
    const double b1 = sb[0][i];
    const double b1sq = b1 * b1;
    double row = 0., row2 = 0.;
    for (int j = (int)first + lane; j <= (int)last; j += 32) {
      const double b2 = sb[1][j];
      const double base = b1sq + b2 * b2;
      const double tb = 2. * b1 * b2 * sgn;
      if (!p.polarized) {
        double sphi = 0.;
#pragma unroll
        for (int q = 0; q < 5; ++q) sphi += survival(p, sg, base + tb * p.cosk[q], P20) * p.wk[q];
        row += sw[1][j] * (sphi - c);
      } else {
        double ss = 0., sp = 0.;
#pragma unroll
        for (int q = 0; q < 5; ++q) {
          const double v = survival(p, sg, base + tb * p.cosk[q], P20);
          ss += v * p.wk[q] * p.cosk[q] * p.cosk[q];
          sp += v * p.wk[q] * p.sink[q] * p.sink[q];
        }
        row += sw[1][j] * (ss - cs);
        row2 += sw[1][j] * (sp - cp);
      }
    }
    row = warp_sum(row);
    acc += sw[0][i] * row;
    if (p.polarized) {
      row2 = warp_sum(row2);
      acc2 += sw[0][i] * row2;
    }
  }
  double s1 = 0., s2 = 0.;
  if (tid < kNb) { s1 = sw[0][tid]; s2 = sw[1][tid]; }
  s1 = warp_sum(s1);
  s2 = warp_sum(s2);
  if (lane == 0) {
    sred[0][wid] = s1;
    sred[1][wid] = s2;
    sred[2][wid] = acc;
  }
  __syncthreads();
  if (tid == 0) {
    double S1 = 0, S2 = 0, A = 0;
    for (int w = 0; w < kBandThreads / 32; ++w) { S1 += sred[0][w]; S2 += sred[1][w]; A += sred[2][w]; }
    const double cc = p.polarized ? cs : c;
    const double L = 2 * kPi * kPi * g.M * (cc * S1 * S2 + A);
    lumi[cell] = L * p.dm * p.dy;
  }
  if (p.polarized) {
    __syncthreads();
    if (lane == 0) sred[2][wid] = acc2;
    __syncthreads();
    if (tid == 0) {
      double S1 = 0, S2 = 0, A = 0;
      for (int w = 0; w < kBandThreads / 32; ++w) { S1 += sred[0][w]; S2 += sred[1][w]; A += sred[2][w]; }
      const double L = 2. * kPi * kPi * g.M * (cp * S1 * S2 + A);
      lumi2[cell] = L * p.dm * p.dy;
    }
  }
}

// ------------------------------------------------------ point entries ---
__global__ void k_flux_point_pts(LumiParams p, const double* __restrict__ b,
                                 const double* __restrict__ k, double* __restrict__ out, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = flux_point(p, b[i], k[i]);
}

__global__ void __launch_bounds__(128) k_flux_form_pts(LumiParams p, const double* __restrict__ b,
                                                       const double* __restrict__ k,
                                                       double* __restrict__ out, int n,
                                                       QagsStats* stats, double* __restrict__ gws,
                                                       int gws_warps) {
  const int lane = threadIdx.x & 31;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (gw >= gws_warps) return;
  QWs<kQagsLimit>* w = reinterpret_cast<QWs<kQagsLimit>*>(gws) + gw;
  for (int t = gw; t < n; t += gws_warps) {
    const double bb = b[t], kk = k[t];
    if (p.isPoint || bb > 2. * p.R) {
      if (lane == 0) out[t] = flux_point(p, bb, kk);
      continue;
    }
    const double wg2 = kk * kk / p.g1 / p.g1;
    double res;
    int nint, nev;
    const int st = warp_qags<kQagsLimit>(p, bb, wg2, w, &res, &nint, &nev);
    record_stats(stats, st, nint, nev);
    if (lane == 0) {
      const double Q = res / p.A;
      out[t] = p.factor * Q * Q / kk;
    }
  }
}

__global__ void k_spline_pts(SplineU s, const double* __restrict__ x, double* __restrict__ y,
                             int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = spline_eval(s, x[i]);
}

}  // namespace

size_t qags_global_ws_doubles_per_warp() {
  return (sizeof(QWs<kQagsLimit>) + sizeof(double) - 1) / sizeof(double);
}

cudaError_t launch_lumi_nodes(const LumiParams& p, int cell0, int ncells, double* d_flux,
                              int* d_nq, cudaStream_t st) {
  note_launch();
  k_lumi_nodes<<<ncells, 256, 0, st>>>(p, cell0, d_flux, d_nq);
  return cudaGetLastError();
}

cudaError_t launch_lumi_qags(const LumiParams& p, int cell0, int ncells, double* d_flux,
                             const int* d_nq, unsigned int* d_work, int* d_ovf_list, int ovf_cap,
                             QagsStats* d_stats, double* d_gws, int gws_warps, cudaStream_t st) {
  (void)d_gws;
  (void)gws_warps;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_lumi_qags, kQagsWarps * 32, 0);
  const int blocks = sms * (per_sm > 0 ? per_sm : 1);
  cudaMemsetAsync(d_work, 0, sizeof(unsigned int), st);
  note_launch();
  k_lumi_qags<<<blocks, kQagsWarps * 32, 0, st>>>(p, cell0, ncells, d_flux, d_nq, d_work,
                                                   d_ovf_list, ovf_cap, d_stats);
  return cudaGetLastError();
}

cudaError_t launch_lumi_qags_overflow(const LumiParams& p, int cell0, double* d_flux,
                                      const int* d_ovf_list, int n_ovf, unsigned int* d_work,
                                      QagsStats* d_stats, double* d_gws, int gws_warps,
                                      cudaStream_t st) {
  if (n_ovf <= 0) return cudaSuccess;
  cudaMemsetAsync(d_work, 0, sizeof(unsigned int), st);
  const int threads = 128;
  const int blocks = (gws_warps * 32 + threads - 1) / threads;
  note_launch();
  k_lumi_qags_overflow<<<blocks, threads, 0, st>>>(p, cell0, d_flux, d_ovf_list, n_ovf, d_work,
                                                   d_stats, d_gws, gws_warps);
  return cudaGetLastError();
}

cudaError_t launch_lumi_band(const LumiParams& p, int cell0, int ncells, const double* d_flux,
                             double* d_lumi, double* d_lumi2, cudaStream_t st) {
  note_launch();
  k_lumi_band<<<ncells, kBandThreads, 0, st>>>(p, cell0, d_flux, d_lumi, d_lumi2);
  return cudaGetLastError();
}

cudaError_t launch_flux_points(const LumiParams& p, const double* d_b, const double* d_k,
                               double* d_out, int n, int form, QagsStats* d_stats,
                               cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  if (!form || p.isPoint) {
    note_launch();
    k_flux_point_pts<<<(n + 255) / 256, 256, 0, st>>>(p, d_b, d_k, d_out, n);
    return cudaGetLastError();
  }
  const int warps = n < 256 ? n : 256;
  double* gws = nullptr;
  cudaError_t e = cudaMallocAsync((void**)&gws,
                                  qags_global_ws_doubles_per_warp() * sizeof(double) * warps, st);
  if (e != cudaSuccess) return e;
  note_launch();
  k_flux_form_pts<<<(warps * 32 + 127) / 128, 128, 0, st>>>(p, d_b, d_k, d_out, n, d_stats, gws,
                                                            warps);
  e = cudaGetLastError();
  cudaFreeAsync(gws, st);
  return e;
}

// ---- no-allocation flux entry ------------------------------------------------
// Scratch of upcg_flux_form_device_noalloc in static device memory: the QAGS
// workspaces of kNoAllocWarps warps (40.5 KB each, 2.6 MB in all) and one
// statistics word.  Every call uses all of it, so calls that overlap in time
// (two streams, two host threads) race on it.
namespace {
constexpr int kNoAllocWarps = 64;
__device__ __align__(256) unsigned char g_noalloc_ws[kNoAllocWarps * sizeof(QWs<kQagsLimit>)];
__device__ __align__(256) QagsStats g_noalloc_stats;
}  // namespace

// Device addresses of the static scratch, looked up once per device with that
// device current (cudaGetSymbolAddress; no allocation).
static cudaError_t noalloc_scratch(double** ws, QagsStats** stats) {
  constexpr int kMaxDev = 64;
  static std::mutex mu;
  static void* ws_ptr[kMaxDev];
  static void* st_ptr[kMaxDev];
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDev) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(mu);
  if (!ws_ptr[dev]) {
    void* w = nullptr;
    void* t = nullptr;
    if ((e = cudaGetSymbolAddress(&w, g_noalloc_ws)) != cudaSuccess) return e;
    if ((e = cudaGetSymbolAddress(&t, g_noalloc_stats)) != cudaSuccess) return e;
    ws_ptr[dev] = w;
    st_ptr[dev] = t;
  }
  *ws = static_cast<double*>(ws_ptr[dev]);
  *stats = static_cast<QagsStats*>(st_ptr[dev]);
  return cudaSuccess;
}

cudaError_t launch_flux_form_noalloc(const LumiParams& p, const double* d_b, const double* d_k,
                                     double* d_out, int n, unsigned* d_failures,
                                     cudaStream_t st) {
  double* ws = nullptr;
  QagsStats* stats = nullptr;
  cudaError_t e = noalloc_scratch(&ws, &stats);
  if (e != cudaSuccess) return e;
  // the statistics word must start at zero; the workspaces need no clearing
  // (each warp writes an interval before it reads it)
  if ((e = cudaMemsetAsync(stats, 0, sizeof(QagsStats), st)) != cudaSuccess) return e;
  if (p.isPoint) {
    note_launch();
    k_flux_point_pts<<<(n + 255) / 256, 256, 0, st>>>(p, d_b, d_k, d_out, n);
  } else {
    const int warps = n < kNoAllocWarps ? n : kNoAllocWarps;
    note_launch();
    k_flux_form_pts<<<(warps * 32 + 127) / 128, 128, 0, st>>>(p, d_b, d_k, d_out, n, stats, ws,
                                                              warps);
  }
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if (d_failures)
    e = cudaMemcpyAsync(d_failures, &stats->failures, sizeof(unsigned), cudaMemcpyDeviceToDevice,
                        st);
  return e;
}

cudaError_t launch_spline_eval(const SplineU& s, const double* d_x, double* d_y, int n,
                               cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  note_launch();
  k_spline_pts<<<(n + 255) / 256, 256, 0, st>>>(s, d_x, d_y, n);
  return cudaGetLastError();
}

}  // namespace upcg
