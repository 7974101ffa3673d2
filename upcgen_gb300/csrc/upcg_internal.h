// Internal interface between the host library (upcg_api.cpp) and the kernels.
#pragma once

#include <cuda_runtime.h>

#include <utility>
#include <vector>
#include <stdint.h>

#include <atomic>

#include "upcg_device.cuh"

struct upcg_generator;

namespace upcg {

// cudaFuncSetAttribute(MaxDynamicSharedMemorySize) once per device for one
// kernel; done holds a bit per device id (< 64), so handles on several
// devices, from several threads, each see the limit raised on theirs
template <typename Kernel>
inline cudaError_t smem_attr_once(std::atomic<uint64_t>& done, Kernel kernel, int bytes) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  const uint64_t bit = 1ull << dev;
  if (done.load(std::memory_order_acquire) & bit) return cudaSuccess;
  e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess) done.fetch_or(bit, std::memory_order_acq_rel);
  return e;
}

constexpr int kNb = 120;                // b-bins per side (include/UpcCrossSection.h:116-117)
constexpr int kBreakupTabMax = 1024;    // capacity of the photo-neutron energy table
constexpr int kQagsCapSmem = 64;        // QAGS intervals held in shared memory per warp
constexpr int kQagsLimit = 1000;        // QAGS limit of src/UpcCrossSection.cpp:209

struct GaaConsts {
  double cosk[5];  // cos(pi x_k) for the positive GL-10 abscissas
  double wk[5];    // their weights (include/UpcCrossSection.h:91-111)
};

// Everything a luminosity kernel needs about one configuration.
struct LumiParams {
  int nm, ny;
  double mmin, dm, ymin, dy;
  double R, g1, g2, factor;
  int A, isPoint, breakupMode, polarized;
  double cosk[5], sink[5], wk[5];
  SplineU gaa, brk, ff;
  double q2max, q2clamp;  // Q2max and Q2max - dQ2 (src/UpcCrossSection.cpp:188)
  // mirror[iy] = iy' with y_iy' = -y_iy to within 8 ulps (or -1): the second
  // photon of cell (m, y) then has the first photon's energy of cell (m, y'),
  // k2 = m/2 e^{-y} = m/2 e^{y'}, and reuses that side's fluxes (identical to
  // ~1e-15).  nullptr disables the reuse.
  const int* mirror;
};

// Per-launch statistics of the QAGS flux kernel.
struct QagsStats {
  unsigned int failures;     // nodes whose QAGS returned a non-zero GSL status
  unsigned int overflow;     // nodes needing more than kQagsCapSmem intervals
  unsigned int max_intervals;
  unsigned long long evals;  // integrand evaluations
};

// Every kernel launch of the library calls note_launch() first; the count
// (upcg_kernel_launches) lets a caller see how many kernels a call issued.
void note_launch();
// the library's error status: records the message for upcg_last_error, returns code
int fail(int code, const char* fmt, ...);
// host <-> device byte counters of upcg_copy_bytes
void count_copy(size_t n, cudaMemcpyKind k);
// the CUDA stream a handle launches on
cudaStream_t handle_stream(::upcg_generator* g);
// fidNuclX after n accepted events with `rejected` rejections
void set_fiducial(::upcg_generator* g, int64_t n, int64_t rejected);
unsigned long long launch_count();

// grid (precision) form of the luminosity, point flux: see upcg_grid.cu
struct GridForm {
  int nw, nr;                // photon-energy and radial grid points
  double lw0, hw, lr0, hr;   // ln w = lw0 + i hw, ln r = lr0 + j hr
  const float* s32;          // point-flux table S(ln x)
  double su0, sinv_h;        // its grid: index = (ln x - su0) * sinv_h
  int sn;
  double c_far;              // survival kernel beyond 20 fm
};
// flux matrix N[w][r] b^2 dln(b) weights (bf16 hi/lo, rows padded to 128) and
// per-row sums / analytic tails beyond the last radius (FP64)
cudaError_t launch_grid_flux(const LumiParams& p, const GridForm& gf, void* nh, void* nl,
                             double* rowsum, double* tail, cudaStream_t st);
// cells of the table from Lg[w1][w2] (FP32) and the row sums / tails
cudaError_t launch_grid_cells(const LumiParams& p, const GridForm& gf, const float* lg,
                              const double* rowsum, const double* tail, double* lumi,
                              cudaStream_t st);

// tables; d_coef32 (optional): an FP32 copy of the coefficients, (float) of each
cudaError_t build_spline_uniform(const double* d_y, int n, double x0, double h, double* d_c,
                                 double4* d_coef, cudaStream_t st, float4* d_coef32 = nullptr);
// fast: the fast form's knots, the closed form with fewer FP64 transcendentals
cudaError_t launch_formfac_values(double* d_out, int n, double x0, double h, double rho0,
                                  double R, double a, cudaStream_t st, int fast = 0);
// G_AA spline (199 intervals into d_coef); d_ta_coef: 199 intervals of the
// T_A spline; d_work: 800 doubles of scratch
// d_coef32: FP32 copy of the G_AA coefficients; d_ta32 (199 float4): the fast
// form's variant -- T_A and G_AA integrands in FP32 (sums in FP64), the T_A
// spline's FP32 copy written there
cudaError_t launch_gaa(double rho0, double R, double a, double csNN, const GaaConsts& k,
                       double4* d_coef, double4* d_ta_coef, double* d_work, cudaStream_t st,
                       float4* d_coef32 = nullptr, float4* d_ta32 = nullptr);
// calcBreakupProb's energy / cross-section table (host); returns its length
int breakup_energy_table(double gammatarg, double* ee, double* se);
// d_tab = [ee | se | ln ee | 1/ee], each kBreakupTabMax long, nt entries used
// fp32: the fast form's table, FP32 sums (~1e-6 of the FP64 ones)
cudaError_t launch_breakup_values(const double* d_tab, int nt, double gammatarg, double omaxx,
                                  double zcon, int mode, int n, double x0, double h,
                                  double* d_out, cudaStream_t st,
                                  int fp32 = 0);
cudaError_t launch_spline_eval(const SplineU& s, const double* d_x, double* d_y, int n,
                               cudaStream_t st);

// luminosity (plain FP64)
cudaError_t launch_lumi_nodes(const LumiParams& p, int cell0, int ncells, double* d_flux,
                              int* d_nq, cudaStream_t st);
cudaError_t launch_lumi_qags(const LumiParams& p, int cell0, int ncells, double* d_flux,
                             const int* d_nq, unsigned int* d_work, int* d_ovf_list,
                             int ovf_cap, QagsStats* d_stats, double* d_gws, int gws_warps,
                             cudaStream_t st);
cudaError_t launch_lumi_qags_overflow(const LumiParams& p, int cell0, double* d_flux,
                                      const int* d_ovf_list, int n_ovf, unsigned int* d_work,
                                      QagsStats* d_stats, double* d_gws, int gws_warps,
                                      cudaStream_t st);
size_t qags_global_ws_doubles_per_warp();
cudaError_t launch_lumi_band(const LumiParams& p, int cell0, int ncells, const double* d_flux,
                             double* d_lumi, double* d_lumi2, cudaStream_t st);
// point evaluations for the parity entry points
// fluxForm on device buffers with the QAGS scratch in static device memory
// (no allocation); d_failures (device, may be null) receives the count of
// points whose QAGS returned a non-zero status
cudaError_t launch_flux_form_noalloc(const LumiParams& p, const double* d_b, const double* d_k,
                                     double* d_out, int n, unsigned* d_failures,
                                     cudaStream_t st);
cudaError_t launch_flux_points(const LumiParams& p, const double* d_b, const double* d_k,
                               double* d_out, int n, int form, QagsStats* d_stats,
                               cudaStream_t st);
cudaError_t launch_breakup_points(double gammatarg, double omaxx, double zcon, int mode,
                                  const double* d_ee, const double* d_se, const int* d_ntab,
                                  const double* d_b, double* d_out, int n, cudaStream_t st);
cudaError_t launch_formfac_points(const double* d_q2, double* d_out, int n, double rho0,
                                  double R, double a, cudaStream_t st);

// fast form (tensor-core contraction), upcg_fast.cu
int fast_grid_points();
// d_gaa32 / d_brk32: FP32 copies of the G_AA and breakup splines' intervals
// convert = 0: the FP32 coefficient copies d_gaa32 / d_brk32 are already
// written (build_spline_uniform's coef32); far_out: P(20 fm) and the far
// constant computed by the kernel itself into far_out[0..1] (k_far_consts
// skipped), and *err0 reset to 0
cudaError_t launch_fast_G(const LumiParams& p, double u0, double h, int P, double P20,
                          float4* d_gaa32, float4* d_brk32, void* gh, void* gl, cudaStream_t st,
                          const double* P20d = nullptr, int convert = 1, double* far_out = nullptr,
                          unsigned* err0 = nullptr, int delta = 0);
// P(20 fm) and the survival kernel beyond 20 fm into d_out[0..1]
cudaError_t launch_far_consts(const LumiParams& p, int has_brk, double* d_out, cudaStream_t st);
// Flux tables of the fast form: scaled K0/K1 on ln x, and Q(w, b) of the
// form-factor flux on (ln w, ln b) (built by the Hankel product H.J).
struct FastFluxTables {
  double* st;    // point-flux table S(ln x) (FP64)
  float* st32;   // its FP32 copy
  double* qt;    // form-factor flux amplitude Q[nw][nb] (FP64)
  float* qt32;   // its FP32 copy
  int nw, nb;
  double lw0, hw, lb0, hb;
};
int flux_table_ktab_n();
// the point-flux table's grid: S at u0 + i (u1 - u0) / (n - 1), u = ln x
void flux_table_ktab_range(double* u0, double* u1);
// d_part: flux_table_part_doubles(nw, nb) doubles of split-K scratch
int flux_table_part_doubles(int nw, int nb);
// point-flux table, and the Q(w, b) rows [w_lo, nw) by the Hankel quadrature;
// js: a stream for the Bessel part J (with d_qn written in its order), whose
// completion ev_j is recorded there and joined into st before the rest
cudaError_t build_flux_tables(const LumiParams& p, FastFluxTables* t, double* d_qn, double* d_wn,
                              int nq, double* d_H, double* d_J, double* d_part, cudaStream_t st,
                              int w_lo = 0, int with_ktab = 1, cudaStream_t js = nullptr,
                              cudaEvent_t ev_j = nullptr);
// the point-flux table S(ln x) of the fast form alone; with d_lk (2 * N
// doubles, flux_table_ktab_n() points) from cached Bessel logs, computed
// there first unless lk_ready
cudaError_t launch_ktab(double g1, double* st, float* st32, cudaStream_t stream,
                        void* d_lk = nullptr, int lk_ready = 0);
// lnm2[im] = ln(m_im / 2); c_far = P(20 fm) sum_k w_k, the survival kernel
// wherever every azimuth has b >= 20 fm
// rep_y (optional, n_rep_y entries): rows map to cells (m0 + r / n_rep_y,
// rep_y[r % n_rep_y]) -- one of each pair of mirror rapidities, whose
// luminosities are equal; launch_fast_finish then also writes the mirror cell
// rep_mir[r % n_rep_y] (-1: none).  Without it row r is cell r.
// Per side the rows are written either dense on the radial grid -- side 0 as
// the A1 bf16 hi / lo pair when ah and al are given, side 1 as the FP32 A2 row
// when a2 is -- or as node lists (fast_node_floats_per_row() floats per row,
// both sides) in nodes.  side_part gets (ln scale, near sum, far sum) per row
// and side (2 float4 per row, for launch_fast_finish).  ncells_pad: a
// multiple of 128.  part: 0 both kernels, 1 the side constants only (they
// read no table values: they may run before the flux tables are ready), 2 the
// weights only (on side constants computed by a part-1 call).
cudaError_t launch_fast_project(const LumiParams& p, double u0, double h, int P, int cell0,
                                int ncells, int ncells_pad, const double* lnm2, double c_far,
                                const double* flux_nodes, const FastFluxTables* t, void* d_sides,
                                void* ah, void* al, float* a2, void* side_part, cudaStream_t st,
                                const int* rep_y = nullptr, int n_rep_y = 0, int m0 = 0,
                                float* nodes = nullptr, int part = 0);
int fast_node_floats_per_row();
// The persistent contraction with the projection folded in (k_contract_fused):
// the same work list and partial sums as launch_contract_pers, the A1 operand
// built in shared memory and the A2 row-dot gathered from the node lists.
cudaError_t launch_contract_fused(const void* gh, const void* gl, int nconf, int rows_total, int P,
                                  const void* items, int nitems, const float* nodes,
                                  float* partial, unsigned* d_err, int shape, int grid,
                                  cudaStream_t st, int kt0 = 0);
// the persistent contractions' work list for grid CTAs (CTA b: items b,
// b + grid, ...), each round's items rotated by its index so that every CTA
// meets every N tile (items of unequal K ranges); in place
void rotate_rounds(std::vector<int4>& items, int grid);
cudaError_t launch_fill_nodes_synthetic(float* nodes, int rows, cudaStream_t st);
// bytes of the per-(cell, photon) constants (d_sides holds 2 per cell)
size_t fast_side_bytes();
// General product on tcgen05, three-term bf16 split with FP32 accumulation:
// D[M][N] = A B^T for A [ceil128(M)][K], B [N][K] (K contiguous, bf16 hi/lo
// pairs; N % 256 == 0, K % 64 == 0).  D goes to out_f32 (FP32) or to
// out_hi / out_lo (a bf16 hi/lo pair for a following product), ld = N.
cudaError_t launch_gemm_bf16x3(const void* ah, const void* al, const void* bh, const void* bl,
                               int M, int N, int K, float* out_f32, void* out_hi, void* out_lo,
                               unsigned* d_err, cudaStream_t st);
// The same product on tcgen05 kind::tf32 (one product per k step, FP32
// operands A [ceil128(M)][K], B [N][K], K % 32 == 0, N % 256 == 0) into out.
cudaError_t launch_gemm_tf32(const float* a, const float* b, int M, int N, int K, float* out,
                             unsigned* d_err, cudaStream_t st);
// out[i] = hi[i] + lo[i] (FP32) of a bf16 hi / lo pair
cudaError_t launch_pair_to_f32(const void* hi, const void* lo, size_t n, float* out,
                               cudaStream_t st);
// Persistent contraction over a work list of {128-row tile of the stacked A,
// N tile, configuration (plane of the stacked G), valid rows} items (int4
// each, contract_item_bytes()); rows_total = rows of the stacked A (multiple
// of 128).  shape 0 = 256-wide N tiles x 2 stages, 1 = 128-wide x 3 stages;
// partial is [rows][P / tile width].  The row-dot of the epilogue takes the
// dense A2 rows, or with a2 == nullptr side 1's node lists in nodes.
cudaError_t launch_contract_pers(const void* ah, const void* al, const void* gh, const void* gl,
                                 int nconf, int rows_total, int P, const void* items, int nitems,
                                 const float* a2, float* partial, unsigned* d_err, int shape,
                                 int grid, cudaStream_t st, const float* nodes = nullptr,
                                 int kt0 = 0);
// kt0 for launch_contract_pers / launch_contract_fused: the first K tile that
// can be nonzero when every node lies at b >= b_min on the grid (u0, h)
int fast_first_ktile(double b_min, double u0, double h);
int contract_item_bytes();
cudaError_t launch_contract(const void* ah, const void* al, const void* gh, const void* gl,
                            const float* a2, int ncells_pad, int ncells, int P, float* partial,
                            unsigned* d_err, cudaStream_t st);
// delta: the contraction's survival kernel was G - c (launch_fast_G's delta)
cudaError_t launch_fast_finish(const LumiParams& p, int cell0, int ncells, int ntiles,
                               double c_far, const float* partial, const void* side_part,
                               double* lumi, cudaStream_t st, const double* c_far_d = nullptr,
                               const int* rep_y = nullptr, const int* rep_mir = nullptr,
                               int n_rep_y = 0, int m0 = 0, int delta = 0);
// The K-tile range [lo, hi) of each N tile (tbn columns) where the delta
// survival kernel G - c on the radial grid r_i = exp(u0 + i h), i < P, can be
// nonzero for the azimuths cosk (a superset: b^2 < 400 (1 + 1e-3) somewhere
// in the tile pair); out[nt] = (lo, hi), hi = lo when none.  Packed into the
// items' bits 8-23 by pack_item.
void delta_tile_ranges(int P, double u0, double h, const double* cosk, int ncos, int tbn, int bk,
                       std::vector<std::pair<int, int>>& out);
inline int pack_item(int rows, int klo, int khi) { return rows | (klo << 8) | (khi << 16); }
// The luminosity-independent samplers share the SMs with the persistent
// contraction, whose shared memory sets the SM's carveout to its maximum: the
// samplers' kernels ask for the same carveout, so that their blocks can be
// resident beside its CTA.  Once per kernel and process.
template <auto Kernel>
inline void carveout_max_shared() {
  static const bool done = [] {
    cudaFuncSetAttribute(Kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                         (int)cudaSharedmemCarveoutMaxShared);
    cudaGetLastError();  // a refusal only leaves the default carveout
    return true;
  }();
  (void)done;
}
constexpr int kContractBK = 64;  // K tile of the contraction kernels
cudaError_t contract_selftest(int ncells, int P, uint64_t seed, double* max_rel, double* ms);

// fold + samplers
struct FoldParams {
  int nm, ny, nz;
  double mmin, dm, zmin, dz;
  int procID, polarized;
  double mPart, aLep, alpWidth;
};
cudaError_t launch_cs_zm(const FoldParams& f, int flag, double* d_out, cudaStream_t st);
// sigma(m) per m-row (both polarized parts, [nm] each, when polarized)
cudaError_t launch_cs_m_rows(const FoldParams& f, double* d_csm, cudaStream_t st);
// the fold with sigma(m) from launch_cs_m_rows, sigma_tot into d_tot, and the
// (m, y) sampling CDF (FP64 and fixed point, n + 1 entries each) in three
// launches; d_scratch: cdf_2d_scratch_doubles(nm * ny)
cudaError_t launch_fold_cdf(const FoldParams& f, const double* d_lumi, const double* d_lumi2,
                            const double* d_csm, double* d_cs, double* d_ratio, double* d_scratch,
                            double* d_tot, double* d_cdf, uint64_t* d_cdffx, cudaStream_t st);
cudaError_t launch_cs_m_points(const FoldParams& f, const double* d_m, double* d_out, int n,
                               int flag, cudaStream_t st);
int cdf_2d_scratch_doubles(int64_t n);
cudaError_t launch_cdf_2d(const double* d_w, int64_t n, double* d_cdf, double* d_scratch,
                          cudaStream_t st);
cudaError_t launch_cdf_rows(const double* d_w, int rows, int len, double* d_cdf,
                            cudaStream_t st);

// events
struct EventParams {
  int nm, ny, nz;
  double mmin, mmax, dm, ymin, dy, zmin, dz;
  int ignoreCSZ, procID, useNonzeroGamPt, doPtCut, doEtaCut;
  double minPt, minEta, maxEta;
  // FP32 copies of the values the per-candidate FP32 code uses (a conversion
  // from FP64 runs on the 1/64-rate FP64 pipe), nm as a double
  float f_dy, f_ymin, f_dz, f_zmin, f_minPt, f_minEta, f_maxEta, f_ptw;
  double nm_d;
  const double2* medges;  // per mass bin: lower edge mmin + dm im, width (or null)
  float mPart;
  int partPDG;
  uint64_t seed;
  // photon-pT tables
  int pt_ne, pt_nbins;
  double pt_lne0, pt_dlne, pt_width, gtot;
  float pt_c0, pt_inv_dlne;  // table coordinate of ln k: (2 ln k - pt_c0) * pt_inv_dlne
  // guide tables of the CDF inversions: bucket j of K holds the largest bin k
  // with cdf[k] <= j / K, so a search starts at most a few bins below its answer
  const int* g2;        // (y, m) CDF, K = g2_n buckets
  int g2_n;
  const int* gz;        // z CDF of every mass row, gz_n buckets per row
  int gz_n;
  const uint16_t* gpt;  // photon-pT tables, gpt_n buckets per table
  int gpt_n;
  // polarized cross section: the z CDFs passed to the kernels are the scalar
  // ones, cdfz_ps the pseudoscalar ones, ratio[iy][im] the reference's
  // nuccs_s / nuccs_p threshold (src/UpcCrossSection.cpp:658, UpcGenerator.cpp:744-751)
  int polarized;
  const double* ratio;
  const double* cdfz_ps;
  // vector mesons (getMomentumVM, twoPartDecayVM): the emitter ratio per
  // y-bin, the pomeron table (kPomN + 1 cumulative values over q in
  // [0, kPomQmax]), the beam gamma, the daughters' mass and angular law
  // (0: 1 + cos^2, 1: 1 + 0.605 cos^2), a device counter of candidates whose
  // decay-angle draw ran out of tries
  // getBinY's int(n / (mmax_edge - mmin)) for n < mbin_lut_n, and that edge
  int mbin_lut_n;
  const int* mbin_lut;
  double medge_hi;
  // 64-bit fixed-point copies of the (y, m) CDF and the z CDFs, searched with
  // the guides g2 / gz (2^g2_bits, 2^gz_bits buckets per row)
  const uint64_t* cdf2fx;
  const uint64_t* cdfzfx;
  int g2_bits, gz_bits;
  int vm;
  const double* vm_ratio;
  const double* pom_cdf;
  double vm_g1;
  float mDght;
  int dght_law;
  unsigned* vm_err;
};
// the (m, y) guide table from the fixed-point CDF that launch_fold_cdf wrote
cudaError_t launch_guide2_fx(const EventParams& e, const uint64_t* d_cdf2fx, int* d_g2,
                             cudaStream_t st);
// guide tables (EventParams) of the built CDFs, with their fixed-point copies;
// d_g2 / d_gz sized g2_n, nm * gz_n (null: skipped)
cudaError_t launch_guides(const EventParams& e, const double* d_cdf2, const double* d_cdfz,
                          int* d_g2, int* d_gz, cudaStream_t st, uint64_t* d_cdf2fx = nullptr,
                          uint64_t* d_cdfzfx = nullptr);
struct EventRecord {  // 48 bytes
  float m, y, z, sign;
  float p0[4];
  float p1[4];
};
// d_ff32: scratch for the FP32 copy of the form-factor spline (ff.n - 1
// intervals); d_gpt (optional): the pT guide tables (e.gpt_n per photon
// energy), built by the same kernel
cudaError_t launch_photon_pt_tables(const EventParams& e, const SplineU& ff, float4* d_ff32,
                                    float* d_cdf, cudaStream_t st, uint16_t* d_gpt = nullptr);
cudaError_t launch_events_flags(const EventParams& e, const double* d_cdf2, const double* d_cdfz,
                                const float* d_ptcdf, uint64_t cand0, int64_t ncand,
                                uint32_t* d_mask, cudaStream_t st, EventRecord* d_stage = nullptr,
                                int32_t* d_stage_mbin = nullptr);
// pass 2 from pass 1's staging slots (launch_events_flags with d_stage)
cudaError_t launch_events_copy(const EventRecord* d_stage, const int32_t* d_stage_mbin,
                               const uint32_t* d_mask, const int64_t* d_tile_off, int64_t tiles,
                               int64_t out_base, int64_t nmax, EventRecord* d_out, int32_t* d_mbin,
                               cudaStream_t st);
cudaError_t launch_sampler_bins(const EventParams& e, const double* d_x, int n, int axis,
                                int* d_out, cudaStream_t st);
cudaError_t launch_events_write(const EventParams& e, const double* d_cdf2, const double* d_cdfz,
                                const float* d_ptcdf, uint64_t cand0, int64_t ncand,
                                const uint32_t* d_mask, const int64_t* d_tile_off,
                                int64_t out_base, int64_t nmax, EventRecord* d_out,
                                int32_t* d_mbin, cudaStream_t st);
cudaError_t launch_events_all(const EventParams& e, const double* d_cdf2, const double* d_cdfz,
                              const float* d_ptcdf, uint64_t cand0, int64_t n, EventRecord* d_out,
                              uint8_t* d_flag, cudaStream_t st);
cudaError_t launch_philox_dump(uint64_t seed, uint64_t c0, int64_t n, uint32_t* d_out,
                               cudaStream_t st);
cudaError_t launch_scan_tiles(const int* d_count, const uint32_t* d_mask, int64_t* d_off, int n,
                              int64_t* d_total, cudaStream_t st);

// fast form's Q(w, b) table: Gauss-Legendre nodes cover q in [0, kQNodeMax]
// GeV (beyond it q^2 > Q2max, where the reference's integrand holds the form
// factor at its clamp value and the integral has a closed form)
constexpr double kQNodeMax = 1.5;

// photonuclear path (upcg_photonuc.cu)
constexpr int kPomN = 65536;       // cells of the pomeron table
constexpr double kPomQmax = 2.0;   // its q range [0, kPomQmax] GeV
struct VmParams {
  double mPart, sqrts, c0, pw, wmin, mNucl;  // dsdt constants, wmin = m_p + m_V
  double rho0, R, a;
  double glx[16], glw[16];                   // 16-point Gauss-Legendre on [-1, 1]
};
// calcPhotonFlux at npts (m, y) points; d_b / d_k / d_w / d_flux: npts * kNb scratch
cudaError_t launch_photon_flux(const LumiParams& p, const double* d_m, const double* d_y, int npts,
                               double* d_b, double* d_k, double* d_w, double* d_flux, double* d_out,
                               QagsStats* d_stats, cudaStream_t st);
cudaError_t launch_vm_cs_y(const VmParams& v, const double* d_y, int n, double* d_out,
                           cudaStream_t st);
cudaError_t launch_vm_fold(const double* d_flux, const double* d_s, int ny, double dy, double* d_cs,
                           double* d_ratio, double* d_tot, cudaStream_t st);
// d_vals: kPomN scratch, d_cdf: kPomN + 1
cudaError_t launch_pom_table(const VmParams& v, double* d_vals, double* d_cdf, cudaStream_t st);

// learned flux surrogate (upcg_mlp.cu).  Box of the training points: ln w in
// [lw_lo, lw_hi], ln b from ln(bf_lo R) to lb_hi, R, a uniform, g uniform.
struct MlpBox {
  float lw_lo, lw_hi, bf_lo, lb_hi, R_lo, R_hi, a_lo, a_hi, g_lo, g_hi;
};
int mlp_param_count();
int mlp_step_samples();
cudaError_t launch_mlp_labels(const MlpBox& bx, uint64_t seed, uint64_t i0, int n,
                              const double* d_glx, const double* d_glw, float* xs, float* ys,
                              float* ws, cudaStream_t st);
cudaError_t launch_mlp_step(const void* pb, const float* pf, const float* xs, const float* ys,
                            const float* ws, const int* idx, int nbatch, float inv_wsum,
                            float* part, float* lossp, cudaStream_t st);
cudaError_t launch_mlp_adam(const float* part, int nparts, float* pf, void* pb, float* m, float* v,
                            float lr, int step, float* grad_out, cudaStream_t st);
cudaError_t launch_mlp_to_bf16(const float* pf, void* pb, cudaStream_t st);
cudaError_t launch_mlp_infer(const void* pb, const float* pf, const float* xs, int n, float* out,
                             cudaStream_t st);
// inputs of the surrogate on the fast form's Q(w, b) table rows [w0, w1)
// (normalised to the box) and the table entries A Q_pt e^y from its outputs
cudaError_t launch_mlp_table_inputs(const MlpBox& bx, const FastFluxTables& t, int w0, int w1,
                                    float R, float a, float g, float* xs, cudaStream_t st);
cudaError_t launch_mlp_table_fill(const FastFluxTables& t, int w0, int w1, double g, double A,
                                  const float* ys, cudaStream_t st);

}  // namespace upcg
