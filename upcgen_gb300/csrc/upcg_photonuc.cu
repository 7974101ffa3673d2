// Photonuclear path: coherent vector-meson photoproduction (PROC_ID 443,
// 100443, 553) in the impulse approximation.
//
//   calcPhotonFlux (src/UpcCrossSection.cpp:700-722)      -> k_pflux_nodes,
//       flux at the nodes (launch_flux_points), k_pflux_sum
//   UpcPhotoNuclearVM::calcCrossSectionY (src/UpcPhotoNuclearVM.cpp:340-381,
//       SHADOWING 0)                                      -> k_vm_cs_y
//   calcNucCrossSectionY (src/UpcCrossSection.cpp:724-748) -> k_vm_fold
//   getMomentumVM's pomeron transverse momentum (src/UpcCrossSection.cpp:
//       1087-1096)                                        -> k_pom_cells + a
//       cumulative table the event kernel inverts
//
// The photon flux is the reference's 120-bin log b-sum per (m, y) with the
// survival factors at each node; the flux at a node is fluxForm (QAGS for
// b <= 2R with the form-factor flux).  PhiA, the integral of calcFormFac^2
// over t in [tmin, tmin + 1] GeV^2 that the reference takes with
// TF1::Integral, is a 64-panel x 16-node Gauss-Legendre rule in q = sqrt(t)
// (dt = 2q dq): each panel spans a sixth of the form factor's oscillation
// period pi hc / R, so the rule is converged far below double rounding.
//
// The pomeron momentum: the reference draws ptPom uniformly on
// [0, 32 hc R] and accepts it with probability (F(tmin + ptPom^2)/A)^2 ptPom,
// so t = tmin + ptPom^2 has the density F(t)^2 on [tmin, tmin + (32 hc R)^2].
// One cumulative table of F^2 over q in [0, kPomQmax] serves every event (the
// integral beyond 2 GeV is below 1e-11 of the whole for Pb, Au, Xe and O): t
// is the inverse of the table between G(tmin) and 1, linear in t inside a
// cell.
#include "upcg_device.cuh"
#include "upcg_internal.h"

namespace upcg {

namespace {

__global__ void k_pflux_nodes(LumiParams p, const double* __restrict__ m,
                              const double* __restrict__ y, int npts, double* __restrict__ b_out,
                              double* __restrict__ k_out, double* __restrict__ w_out) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= npts * kNb) return;
  const int pt = idx / kNb, i = idx - pt * kNb;
  const double k = m[pt] / 2. * exp(y[pt]);
  const double bmin = p.isPoint ? 1 * p.R : 0.05 * p.R;
  const double bmax = fmax(5. * p.g1 * kHc / k, 5 * p.R);
  const double ldb = (log(bmax) - log(bmin)) / kNb;
  const double bl = bmin * exp(i * ldb);
  const double bh = bmin * exp((i + 1) * ldb);
  const double b = (bh + bl) / 2.;
  double bu = 1.;
  if (p.breakupMode != 1) bu = spline_eval(p.brk, b < 20. ? b : 20.);
  const double g = b < 20. ? spline_eval(p.gaa, b) : 1.;
  b_out[idx] = b;
  k_out[idx] = k;
  w_out[idx] = bu * g;  // times the flux, then b (bh - bl) in k_pflux_sum: the reference's order
}

__global__ void k_pflux_sum(LumiParams p, const double* __restrict__ m, const double* __restrict__ y,
                            const double* __restrict__ flux, const double* __restrict__ w, int npts,
                            double* __restrict__ out) {
  const int pt = blockIdx.x * blockDim.x + threadIdx.x;
  if (pt >= npts) return;
  const double k = m[pt] / 2. * exp(y[pt]);
  const double bmin = p.isPoint ? 1 * p.R : 0.05 * p.R;
  const double bmax = fmax(5. * p.g1 * kHc / k, 5 * p.R);
  const double ldb = (log(bmax) - log(bmin)) / kNb;
  double sum = 0;
  for (int i = 0; i < kNb; ++i) {
    const double bl = bmin * exp(i * ldb);
    const double bh = bmin * exp((i + 1) * ldb);
    const double b = (bh + bl) / 2.;
    const size_t o = (size_t)pt * kNb + i;
    sum += w[o] * flux[o] * b * (bh - bl);
  }
  out[pt] = 2. * kPi * k * sum;
}

constexpr int kPhiPanels = 64;

__global__ void k_vm_cs_y(VmParams v, const double* __restrict__ y, int n, double* __restrict__ out) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= n) return;
  const double w = v.mPart / 2. * exp(y[warp]);
  const double beamE = 0.5 * v.sqrts;
  const double Wgp2 = 4. * w * beamE;
  const double Wgp = sqrt(Wgp2);
  double csGammaP = 0.;
  if (Wgp > v.wmin) csGammaP = v.c0 * pow(1. - (v.wmin * v.wmin) / Wgp2, 1.5) * pow(Wgp2 * 1e-4, v.pw);
  const double x = v.mPart * v.mPart / Wgp2;
  const double tmin = x * x * v.mNucl * v.mNucl;
  const double q0 = sqrt(tmin), q1 = sqrt(tmin + 1.);
  const double hq = (q1 - q0) / kPhiPanels;
  double s = 0.;
  for (int pn = lane; pn < kPhiPanels; pn += 32) {
    const double a0 = q0 + pn * hq;
    double ps = 0.;
#pragma unroll 4
    for (int j = 0; j < 16; ++j) {
      const double q = a0 + 0.5 * hq * (v.glx[j] + 1.);
      const double f = calc_form_fac(q * q, v.rho0, v.R, v.a);
      ps += v.glw[j] * f * f * 2. * q;
    }
    s += ps * 0.5 * hq;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) out[warp] = csGammaP * s * 1e-6;
}

// dsigma/dy = N(y) s(y) + N(-y) s(-y) per y-bin; flux and s hold the +y
// values in [0, ny) and the -y values in [ny, 2 ny)
__global__ void k_vm_fold(const double* __restrict__ flux, const double* __restrict__ s, int ny,
                          double dy, double* __restrict__ cs, double* __restrict__ ratio,
                          double* __restrict__ tot) {
  for (int iy = threadIdx.x; iy < ny; iy += blockDim.x) {
    const double u1 = flux[iy] * s[iy], u2 = flux[ny + iy] * s[ny + iy];
    cs[iy] = u1 + u2;
    ratio[iy] = u1 / u2;
  }
  if (threadIdx.x == 0) {  // the reference's running sum, in y order
    double total = 0;
    for (int iy = 0; iy < ny; ++iy) total += flux[iy] * s[iy] + flux[ny + iy] * s[ny + iy];
    *tot = total * dy;
  }
}

// F(t)^2 integrated over cell j of the q grid (t = q^2): 4-point Gauss-Legendre in q
__global__ void k_pom_cells(double rho0, double R, double a, double dq, int n,
                            double* __restrict__ vals) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const double x4[4] = {-0.8611363115940526, -0.3399810435848563, 0.3399810435848563,
                        0.8611363115940526};
  const double w4[4] = {0.3478548451374538, 0.6521451548625461, 0.6521451548625461,
                        0.3478548451374538};
  double s = 0.;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const double q = dq * (j + 0.5 * (x4[k] + 1.));
    const double f = calc_form_fac(q * q, rho0, R, a);
    s += w4[k] * f * f * 2. * q;
  }
  vals[j] = s * 0.5 * dq;
}

}  // namespace

cudaError_t launch_photon_flux(const LumiParams& p, const double* d_m, const double* d_y, int npts,
                               double* d_b, double* d_k, double* d_w, double* d_flux, double* d_out,
                               QagsStats* d_stats, cudaStream_t st) {
  if (npts <= 0) return cudaSuccess;
  const int nn = npts * kNb;
  note_launch();
  k_pflux_nodes<<<(nn + 255) / 256, 256, 0, st>>>(p, d_m, d_y, npts, d_b, d_k, d_w);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  e = launch_flux_points(p, d_b, d_k, d_flux, nn, 1, d_stats, st);
  if (e != cudaSuccess) return e;
  note_launch();
  k_pflux_sum<<<(npts + 127) / 128, 128, 0, st>>>(p, d_m, d_y, d_flux, d_w, npts, d_out);
  return cudaGetLastError();
}

cudaError_t launch_vm_cs_y(const VmParams& v, const double* d_y, int n, double* d_out,
                           cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  note_launch();
  k_vm_cs_y<<<(n * 32 + 127) / 128, 128, 0, st>>>(v, d_y, n, d_out);
  return cudaGetLastError();
}

cudaError_t launch_vm_fold(const double* d_flux, const double* d_s, int ny, double dy, double* d_cs,
                           double* d_ratio, double* d_tot, cudaStream_t st) {
  note_launch();
  k_vm_fold<<<1, 256, 0, st>>>(d_flux, d_s, ny, dy, d_cs, d_ratio, d_tot);
  return cudaGetLastError();
}

cudaError_t launch_pom_table(const VmParams& v, double* d_vals, double* d_cdf, cudaStream_t st) {
  note_launch();
  k_pom_cells<<<(kPomN + 255) / 256, 256, 0, st>>>(v.rho0, v.R, v.a, kPomQmax / kPomN, kPomN, d_vals);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return launch_cdf_rows(d_vals, 1, kPomN, d_cdf, st);
}

}  // namespace upcg
