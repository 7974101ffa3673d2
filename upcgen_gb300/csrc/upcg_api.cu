// Host side of the C ABI (include/upcgen_gb300.h): configuration with the
// reference's parameters.in keys, table / luminosity / fold / sampler set-up
// on the GPU, and the accepted-event loop.
//
// Reference: src/UpcGenerator.cpp (UpcGenerator), src/UpcCrossSection.cpp
// (UpcCrossSection::init and its prepare* helpers).
#include <fcntl.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <map>
#include <tuple>
#include <mutex>
#include <new>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/upcgen_gb300.h"
#include "upcg_cache.h"
#include "upcg_internal.h"

using namespace upcg;

namespace upcg {
static std::atomic<unsigned long long> g_launches{0};
void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
unsigned long long launch_count() { return g_launches.load(std::memory_order_relaxed); }
}  // namespace upcg

namespace {
// host <-> device bytes the library has copied (upcg_copy_bytes)
std::atomic<unsigned long long> g_h2d{0}, g_d2h{0};
}  // namespace

namespace upcg {
void count_copy(size_t n, cudaMemcpyKind k) {
  if (k == cudaMemcpyHostToDevice) g_h2d.fetch_add(n, std::memory_order_relaxed);
  if (k == cudaMemcpyDeviceToHost) g_d2h.fetch_add(n, std::memory_order_relaxed);
}
}  // namespace upcg

namespace {

cudaError_t mcpy(void* dst, const void* src, size_t n, cudaMemcpyKind k, cudaStream_t s) {
  count_copy(n, k);
  return cudaMemcpyAsync(dst, src, n, k, s);
}

cudaError_t mcpy_sync(void* dst, const void* src, size_t n, cudaMemcpyKind k) {
  count_copy(n, k);
  return cudaMemcpy(dst, src, n, k);
}
}  // namespace

namespace {
thread_local std::string g_err;
}  // namespace

namespace upcg {
int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}
}  // namespace upcg

namespace {

#define CK(call)                                                                         \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess)                                                               \
      return fail(UPCG_ERR_CUDA, "%s:%d %s: %s", __FILE__, __LINE__, #call,             \
                  cudaGetErrorString(e_));                                               \
  } while (0)

// include/UpcCrossSection.h:91-111 (positive half of the reference's GL-10 table)
const double kW10pos[5] = {0.2955242247147529, 0.2692667193099963, 0.2190863625159820,
                           0.1494513491505806, 0.0666713443086881};
const double kX10pos[5] = {0.1488743389816312, 0.4333953941292472, 0.6794095682990244,
                           0.8650633666889845, 0.9739065285171717};
const double kQ2min = 1e-9, kQ2max = 2.;
const int kNQ2 = 1000000;
// the fast form's form-factor spline: 65,536 knots on the same range (a
// cubic spline error below 1e-9 of F; the Q(w, b) table and the photon-pT
// spectra are its only users there)
const int kNQ2Fast = 65536;
// largest (m, y) or (m, z) table a handle builds: 2^24 cells (138 times the
// 1001 x 121 grid), so that every per-cell index stays far inside int range
const int kMaxGridCells = 1 << 24;

template <class T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  ~DBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  cudaError_t ensure(size_t count) {
    if (count <= n && p) return cudaSuccess;
    release();
    cudaError_t e = cudaMalloc((void**)&p, std::max<size_t>(count, 1) * sizeof(T));
    if (e == cudaSuccess) n = count;
    return e;
  }
};

}  // namespace

// The learned flux surrogate (upcg_mlp.cu): parameters, Adam state,
// training points, and the scratch of a training step.
struct upcg_mlp {
  MlpBox box{};
  cudaStream_t own = nullptr;
  DBuf<float> pf, m, v, part, lossp, xs, ys, ws, tx, ty, tw, out;
  DBuf<uint16_t> pb;
  DBuf<int> idx;
  DBuf<double> glx, glw;
  int64_t ndata = 0;
  int step = 0;
  uint64_t seed = 0;
  double train_ms = 0, labels_ms = 0;
  ~upcg_mlp() {
    if (own) cudaStreamDestroy(own);
  }
  cudaStream_t st() {
    if (!own) cudaStreamCreateWithFlags(&own, cudaStreamNonBlocking);
    return own;
  }
};

namespace {
// Autotuner of the persistent contraction: for a work size it times both
// tile shapes (256-wide x 2 stages, 128-wide x 3 stages) on synthetic
// operands of that size, once per process and device, and keeps the faster.
struct TuneKey {
  int dev, rows, P, fused;
  bool operator<(const TuneKey& o) const {
    if (dev != o.dev) return dev < o.dev;
    if (rows != o.rows) return rows < o.rows;
    return P != o.P ? P < o.P : fused < o.fused;
  }
};
std::mutex g_tune_mu;
std::map<TuneKey, int> g_tune;
std::map<int, std::pair<double, double>> g_tune_ms;  // last timings per rows bucket

int tune_bucket(int rows) {  // power-of-two buckets of the row count
  int b = 128;
  while (b < rows) b <<= 1;
  return b;
}
}  // namespace

// shape and grid for `rows_pad` stacked rows (nvalid of them valid) at P, for
// the staged contraction (fused = 0, dense operands) or the fused one (node
// lists; timed on synthetic lists shaped like form-factor rows)
int contract_plan(int rows_pad, int nvalid, int P, int* shape, int* grid, int fused) {
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  *grid = sms;
  const TuneKey key{dev, tune_bucket(rows_pad), P, fused ? 1 : 0};
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    auto it = g_tune.find(key);
    if (it != g_tune.end()) {
      *shape = it->second;
      return UPCG_OK;
    }
  }
  // synthetic operands of the bucket's size, timed with events on a private stream
  const int rows = key.rows;
  DBuf<uint16_t> a, g;
  DBuf<float> a2, part, nodes;
  DBuf<int4> items;
  DBuf<unsigned> err;
  // the private stream and the timing events are released on every return
  struct Owned {
    cudaStream_t s = nullptr;
    cudaEvent_t e[2] = {nullptr, nullptr};
    ~Owned() {
      for (cudaEvent_t x : e)
        if (x) cudaEventDestroy(x);
      if (s) cudaStreamDestroy(s);
    }
  } own;
  CK(cudaStreamCreateWithFlags(&own.s, cudaStreamNonBlocking));
  CK(cudaEventCreate(&own.e[0]));
  CK(cudaEventCreate(&own.e[1]));
  cudaStream_t s = own.s;
  cudaEvent_t e0 = own.e[0], e1 = own.e[1];
  CK(g.ensure((size_t)P * P));
  CK(part.ensure((size_t)rows * (P / 128)));
  CK(err.ensure(1));
  CK(cudaMemsetAsync(g.p, 0, (size_t)P * P * 2, s));
  CK(cudaMemsetAsync(err.p, 0, 4, s));
  if (fused) {
    CK(nodes.ensure((size_t)rows * fast_node_floats_per_row()));
    CK(launch_fill_nodes_synthetic(nodes.p, rows, s));
  } else {
    CK(a.ensure((size_t)rows * P));
    CK(a2.ensure((size_t)rows * P));
    CK(cudaMemsetAsync(a.p, 0, (size_t)rows * P * 2, s));
    CK(cudaMemsetAsync(a2.p, 0, (size_t)rows * P * 4, s));
  }
  double best = 1e30;
  int pick = 0;
  double t[2] = {0, 0};
  for (int sh = 0; sh < 2; ++sh) {
    const int tbn = sh == 0 ? 256 : 128;
    std::vector<int4> it;
    for (int mt = 0; mt < rows / 128; ++mt)
      for (int nt = 0; nt < P / tbn; ++nt) it.push_back(make_int4(mt, nt, 0, 128));
    CK(items.ensure(it.size()));
    CK(cudaMemcpyAsync(items.p, it.data(), it.size() * sizeof(int4), cudaMemcpyHostToDevice, s));
    float ms = 0;
    for (int rep = 0; rep < 3; ++rep) {  // warm-up, then the best of two
      CK(cudaEventRecord(e0, s));
      if (fused)
        CK(launch_contract_fused(g.p, g.p, 1, rows, P, items.p, (int)it.size(), nodes.p, part.p,
                                 err.p, sh, *grid, s));
      else
        CK(launch_contract_pers(a.p, a.p, g.p, g.p, 1, rows, P, items.p, (int)it.size(), a2.p,
                                part.p, err.p, sh, *grid, s));
      CK(cudaEventRecord(e1, s));
      CK(cudaEventSynchronize(e1));
      float m = 0;
      CK(cudaEventElapsedTime(&m, e0, e1));
      if (rep == 1 || (rep == 2 && m < ms)) ms = m;
    }
    t[sh] = ms;
    if (ms < best) {
      best = ms;
      pick = sh;
    }
  }
  unsigned herr = 0;
  CK(cudaMemcpy(&herr, err.p, 4, cudaMemcpyDeviceToHost));
  if (herr) return fail(UPCG_ERR_CUDA, "contraction autotune timed out (code %u)", herr);
  (void)nvalid;
  std::lock_guard<std::mutex> lock(g_tune_mu);
  g_tune[key] = pick;
  g_tune_ms[key.rows] = {t[0], t[1]};
  *shape = pick;
  return UPCG_OK;
}

struct upcg_scan;

struct upcg_generator {
  // ---- configuration (defaults: include/UpcCrossSection.h:73-172,
  //      include/UpcGenerator.h:62-73, UpcGenerator() :30-40)
  double R = 6.68, a = 0.447;
  int Z = 82, A = 208;
  double sqrts = 5020., g1 = 0, g2 = 0, gtot = 0;
  int procID = 15;
  double aLep = 0, alpMass = 1., alpWidth = 0.010;
  // vector mesons (src/UpcPhotoNuclearVM.cpp:55-93): the SHADOWING and
  // DECAY_PDG keys and the meson's dsdt constants
  bool isVM = false;
  int shadowing = 0, dghtPDG = 0;
  double mDght = 0, vm_c0 = 0, vm_pw = 0.4;
  double zmin = -1, zmax = 1, mmin = 3.56, mmax = 50., ymin = -6., ymax = 6.;
  int nz = 100, nm = 1001, ny = 121;
  bool isPoint = true, useNonzeroGamPt = true, usePolarizedCS = false;
  int breakupMode = 1;
  bool doPtCut = false, doEtaCut = false;
  double minPt = 0, minEta = 0, maxEta = 0;
  long seed = 0, nEvents = 1000;
  // generateEvents' files: the reference writes the particles tree unless
  // USE_ROOT_OUTPUT says 0 (include/UpcGenerator.h:135-136, src/UpcGenerator.cpp:284-289)
  int useROOTOut = 1, useHepMCOut = 0;
  int numThreads = 1, debug = 0;
  std::string lumiDir = ".";
  bool lumiCache = false;
  int lumi_cache_hit = -1;  // last init: 1 table read from the cache, 0 computed, -1 cache unused
  int lumiMethod = 0;
  // the fast form's tables (65,536-knot form factor, FP32 breakup sums): methods 1, 4, 5, 6
  bool fast_tables() const { return lumiMethod == 1 || lumiMethod == 4 || lumiMethod == 5 || lumiMethod == 6; }
  int row_lo = 0, row_hi = -1;  // m-rows of the luminosity this handle computes (-1: all)
  upcg_mlp* surrogate = nullptr;  // luminosity method 4: Q(w, b) rows from the MLP
  int surrogate_rows = 0;         // rows of the last Q table that came from it
  bool cap = false;               // enqueue device work only (stream capture of a scan)
  // scan: earlier configurations whose form factor / G_AA / breakup tables
  // have the same inputs (their tables are copied, not rebuilt)
  upcg_generator* ff_donor = nullptr;
  int ff_n = kNQ2;  // knots of the form-factor spline (kNQ2Fast for methods 1 and 4)
  upcg_generator* gaa_donor = nullptr;
  upcg_generator* brk_donor = nullptr;
  FastFluxTables ftab_last{};     // the fast form's flux tables of the last build
  int nqn_last = 0;
  int enqueue_scan_front(upcg_scan& sc, int ci);
  int enqueue_scan_back(upcg_scan& sc, int ci);
  // ---- derived
  double mPart = 0;
  int partPDG = 0;
  bool isCharged = true, ignoreCSZ = false;
  double factor = 0, rho0 = 0, csNN = 0;
  double bu_gammatarg = 0, bu_omaxx = 0, bu_zcon = 0;
  // ---- device state
  cudaStream_t own = nullptr, stream = nullptr;
  DBuf<double> ff_y, ff_c, brk_y, brk_c, lumi, lumi2, cs, ratio, cszm, cszm2, cszm3;
  DBuf<double> cdf2, cdfz, cdfz2, cdfz3, flux, csm, tot, gws, pts_a, pts_b, pts_c;
  DBuf<double4> ff_coef, gaa_coef, ta_coef, brk_coef;
  DBuf<double> gaa_work, bu_tab, cdf_scratch;
  DBuf<double> vm_m, vm_y, vm_b, vm_k, vm_w, vm_f, vm_flux, vm_s, pom_vals, pom_cdf;
  DBuf<unsigned> vm_err;
  DBuf<int> mbinlut;  // getBinY of int(nm (m - mmin)), see EventParams
  DBuf<uint64_t> cdf2fx, cdfzfx;  // fixed-point CDF copies (EventParams)
  int mbinlut_n = 0;
  std::vector<int> mbinlut_host;  // its host copy and (lo, hi) edges
  DBuf<double2> medges;  // per mass bin (mmin + dm im, bin width), EventParams::medges
  std::vector<double2> medges_host;
  bool medges_ok = false;
  double mbinlut_key[2] = {0., 0.};
  int64_t contract_rows = 0;  // rows of the last fast-form contraction
  // multiply-adds per row of its A1 . (G - c) product over the nonzero tiles
  int64_t contract_macs_row = 0;
  int fast_nrep = 0;          // rapidity bins per m-row the fast form computes (frep), 0: all  // bu_tab: ee | se | ln ee | 1/ee (kBreakupTabMax each)
  std::vector<double> bu_host;
  int bu_nt = 0;
  // side streams of the table set-up (form factor, breakup, the
  // luminosity-independent samplers) and their fork / join events; ev_ff:
  // the form-factor spline is complete (side[0])
  cudaStream_t side[4] = {nullptr, nullptr, nullptr, nullptr};
  cudaEvent_t ev_fork = nullptr, ev_join[4] = {nullptr, nullptr, nullptr, nullptr}, ev_ff = nullptr;
  cudaEvent_t ev_ktab = nullptr;  // the point-flux table (side[2]) is complete
  cudaEvent_t ev_qj = nullptr;    // the Q table's Bessel part (side[2]) is complete
  // host event output: generation done / slot copied out (side[1] copies)
  cudaEvent_t ev_gen = nullptr, ev_out[3] = {nullptr, nullptr, nullptr};
  cudaError_t side_streams() {
    int least = 0, greatest = 0;
    cudaError_t pe = cudaDeviceGetStreamPriorityRange(&least, &greatest);
    if (pe != cudaSuccess) return pe;
    for (int i = 0; i < 4; ++i) {
      if (!side[i]) {
        // the form factor -> flux tables chain (side[0]) feeds the
        // projection, the breakup / G_AA chain and the survival kernel
        // (side[1]) the contraction: their blocks go first; the
        // luminosity-independent samplers (side[2]: z, side[3]: photon pT)
        // fill the SMs they leave
        const int prio = i < 2 ? greatest : least;
        cudaError_t e = cudaStreamCreateWithPriority(&side[i], cudaStreamNonBlocking, prio);
        if (e != cudaSuccess) return e;
      }
      if (!ev_join[i]) {
        cudaError_t e = cudaEventCreateWithFlags(&ev_join[i], cudaEventDisableTiming);
        if (e != cudaSuccess) return e;
      }
    }
    for (cudaEvent_t* ev : {&ev_ff, &ev_ktab, &ev_gaa, &ev_survival}) {
      if (!*ev) {
        cudaError_t e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
        if (e != cudaSuccess) return e;
      }
    }
    if (!ev_fork) return cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming);
    return cudaSuccess;
  }
  DBuf<int> ntab, nq, ovf, mirror, guide2, guidez, frep;
  DBuf<int4> fitems;
  DBuf<uint16_t> guidept;
  DBuf<unsigned int> work;
  DBuf<QagsStats> stats;
  DBuf<float> ptcdf;
  DBuf<uint32_t> mask;
  DBuf<int64_t> tile_off, total;
  DBuf<EventRecord> evbuf;
  DBuf<EventRecord> evstage;  // pass 1's accepted records, 256 slots per candidate tile
  DBuf<int32_t> evstage_mbin;
  DBuf<uint16_t> fgh, fgl, fah, fal;  // fast form: bf16 hi/lo of G and of the projections
  DBuf<float> fa2, fpart, fnodes;
  DBuf<double> ffar, fk1, fq, fqn, fwn, fH, fJ, flnm2, fpartq, fsides, ffc;
  DBuf<double> fk01;        // ln K0 + x, ln K1 + x on the K table's x grid (any gamma)
  DBuf<double> ffc2;        // polarized: the pseudoscalar far constants
  DBuf<uint16_t> fgh2, fgl2;  // polarized: the pseudoscalar survival kernel (bf16 hi/lo)
  DBuf<float> fpart2;
  bool fk01_ready = false;
  DBuf<float> fs32, fq32;
  DBuf<float4> fgaa32, fbrk32, ff32, fta32;
  // grid form: G, flux matrix, T = N G (bf16 hi/lo), Lg, row sums and tails
  DBuf<uint16_t> gg_h, gg_l, gn_h, gn_l, gt_h, gt_l;
  DBuf<float> g_lg;
  DBuf<float> g_n32, g_g32, g_t32;  // grid form, TF32 arm: FP32 N, G and T = N G
  DBuf<double> g_rowsum, g_tail;
  DBuf<unsigned> ferr;
  DBuf<int32_t> mbinbuf;
  int brk_n = 0;
  bool tables_ready = false, lumi_ready = false, xsec_ready = false;
  double totCS = 0, fidCS = 0;
  uint64_t next_cand = 0;
  double acc_rate = 1.0;
  QagsStats last_stats{};
  double timings[8] = {0};
  // single-event interface
  std::vector<EventRecord> ev_batch;
  std::vector<uint8_t> ev_flag;
  size_t ev_pos = 0;

  upcg_generator() {
    const double g0 = 5020. / (2. * kMProt);
    // UpcCrossSection() runs before any parameter is read: gtot keeps the
    // default sqrt(s) (src/UpcCrossSection.cpp:51-54, include/UpcCrossSection.h:83-85).
    gtot = std::cosh((std::acosh(g0) + std::acosh(g0)) / 2.);
    set_collision(5020.f, 82, 208);
  }
  ~upcg_generator() {
    for (int i = 0; i < 4; ++i) {
      if (side[i]) cudaStreamDestroy(side[i]);
      if (ev_join[i]) cudaEventDestroy(ev_join[i]);
    }
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_ff) cudaEventDestroy(ev_ff);
    if (ev_ktab) cudaEventDestroy(ev_ktab);
    if (ev_qj) cudaEventDestroy(ev_qj);
    if (ev_static_go) cudaEventDestroy(ev_static_go);
    if (ev_gaa) cudaEventDestroy(ev_gaa);
    if (ev_pt) cudaEventDestroy(ev_pt);
    if (ev_survival) cudaEventDestroy(ev_survival);
    if (ev_gen) cudaEventDestroy(ev_gen);
    for (auto e : ev_out)
      if (e) cudaEventDestroy(e);
    if (ev_static) cudaEventDestroy(ev_static);
    if (hstat) cudaFreeHost(hstat);
    for (auto e : ev_ft)
      if (e) cudaEventDestroy(e);
    if (own) cudaStreamDestroy(own);
    if (hp) cudaStreamDestroy(hp);
    for (auto e : ev_hp)
      if (e) cudaEventDestroy(e);
  }
  void set_collision(float s, int z, int aa) {
    sqrts = s;
    g1 = sqrts / (2. * kMProt);
    g2 = sqrts / (2. * kMProt);
    Z = z;
    A = aa;
  }
  cudaStream_t st() {
    if (hp_active) return hp;
    return user_st();
  }
  cudaStream_t user_st() {
    if (stream) return stream;
    if (!own) cudaStreamCreateWithFlags(&own, cudaStreamNonBlocking);
    return own;
  }
  // upcg_init runs its main-stream work on hp, a high-priority stream forked
  // from the caller's and joined back before the host synchronisation: the
  // projection and the contraction take the SMs ahead of the samplers beside
  // them, the table chains' kernels ahead of theirs
  cudaStream_t hp = nullptr;
  cudaEvent_t ev_hp[2] = {nullptr, nullptr};
  bool hp_active = false;
  cudaError_t hp_begin() {
    cudaStream_t u = user_st();
    if (!hp) {
      // one level below the table chains' streams (greatest): the chains'
      // short kernels are dispatched ahead of the projection's pending blocks
      int least = 0, greatest = 0;
      cudaError_t e = cudaDeviceGetStreamPriorityRange(&least, &greatest);
      const int prio = greatest < least ? greatest + 1 : greatest;
      if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&hp, cudaStreamNonBlocking, prio);
      if (e != cudaSuccess) return e;
    }
    for (auto& e : ev_hp)
      if (!e) {
        cudaError_t r = cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
        if (r != cudaSuccess) return r;
      }
    cudaError_t e = cudaEventRecord(ev_hp[0], u);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(hp, ev_hp[0], 0);
    if (e == cudaSuccess) hp_active = true;
    return e;
  }
  cudaError_t hp_end() {
    if (!hp_active) return cudaSuccess;
    hp_active = false;
    cudaError_t e = cudaEventRecord(ev_hp[1], hp);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(user_st(), ev_hp[1], 0);
    return e;
  }
  void invalidate() {
    tables_ready = lumi_ready = xsec_ready = false;
    up_cache.clear();
  }
  // Small host-computed tables uploaded at every init (grids, node sets, the
  // breakup energy table, work lists): skipped when the bytes for the same
  // device buffer are unchanged.  A buffer only moves when it must grow, and
  // then its new contents are larger, so a size match means the same buffer.
  std::map<const void*, std::vector<char>> up_cache;
  cudaError_t upload(void* dst, const void* src, size_t n, cudaStream_t ss) {
    std::vector<char>& c = up_cache[dst];
    if (!cap && c.size() == n && std::memcmp(c.data(), src, n) == 0) return cudaSuccess;
    c.assign(static_cast<const char*>(src), static_cast<const char*>(src) + n);
    return mcpy(dst, src, n, cudaMemcpyHostToDevice, ss);
  }

  int set_param(const std::string& k, const std::string& v);
  int setup_process();
  int check_config();
  // vector mesons: the decay-angle draws of the last events all ended
  int vm_check() {
    if (!isVM) return UPCG_OK;
    unsigned n = 0;
    const cudaError_t e = cudaMemcpyAsync(&n, vm_err.p, sizeof n, cudaMemcpyDeviceToHost, st());
    if (e != cudaSuccess || cudaStreamSynchronize(st()) != cudaSuccess)
      return fail(UPCG_ERR_CUDA, "reading the decay-angle error count failed");
    if (n) return fail(UPCG_ERR_NUMERIC, "%u candidates ran out of decay-angle draws", n);
    return UPCG_OK;
  }
  int build_tables();
  int build_lumi();
  int build_vm();
  // js: the stream of the table's Bessel part (and of the node uploads)
  int setup_flux_tables(cudaStream_t ss, int with_ktab = 1, cudaStream_t js = nullptr);
  bool ftab_early = false;  // build_tables enqueued the flux tables
  // build_tables wrote the FP32 copies of the G_AA and breakup splines
  // (fgaa32, fbrk32) beside their FP64 coefficients
  bool g32_ready = false;
  bool herr_copy_pending = false;  // the contraction's error word, copied in complete_deferred
  // per-N-tile K ranges of the delta survival kernel (delta_tile_ranges),
  // kept for the last (P, N tile, azimuth set)
  std::vector<std::pair<int, int>> dkr;
  int dkr_key[3] = {0, 0, -1};
  const std::vector<std::pair<int, int>>& delta_ranges(int P, double u0, double h, int tbn,
                                                       const LumiParams& p, bool negated) {
    if (dkr_key[0] != P || dkr_key[1] != tbn || dkr_key[2] != (negated ? 1 : 0)) {
      double ck[5];
      for (int q = 0; q < 5; ++q) ck[q] = negated ? -p.cosk[q] : p.cosk[q];
      delta_tile_ranges(P, u0, h, ck, 5, tbn, kContractBK, dkr);
      dkr_key[0] = P;
      dkr_key[1] = tbn;
      dkr_key[2] = negated ? 1 : 0;
    }
    return dkr;
  }
  bool lumi_stats = true;          // the deferred luminosity copied its QAGS statistics
  bool ftab_early_done = false;  // ... and build_lumi used them (deferred timing)
  // upcg_init enqueues tables, luminosity and cross section with one host
  // synchronisation at its end: the phases' timing events, the contraction's
  // error word, the QAGS statistics and sigma_tot are collected then
  // (complete_deferred); other callers of the phases synchronise per phase
  bool defer = false;
  struct HostStatus {
    unsigned herr, pad;
    QagsStats stats;
    double tot;
  };
  HostStatus* hstat = nullptr;  // pinned
  cudaEvent_t tab_ev[2] = {nullptr, nullptr}, xs_ev[2] = {nullptr, nullptr};
  std::vector<cudaEvent_t> lumi_ev;
  std::vector<std::pair<int, std::pair<int, int>>> lumi_spans;
  int lumi_w0 = 0, lumi_w1 = 0;
  bool tab_pending = false, lumi_pending = false, lumi_fast = false, xs_pending = false;
  int complete_deferred(int rc);
  cudaEvent_t ev_ft[2] = {nullptr, nullptr};
  // pts (optional): a stream for the photon-pT part, joined back into ss
  // parts: 1 the z samplers (and the mass-bin tables, sigma(m)), 2 the
  // photon-pT spectra and guides (on pts when given, ev_pt recorded there)
  int enqueue_static_samplers(cudaStream_t ss, cudaEvent_t ff_ready = nullptr,
                              cudaStream_t pts = nullptr, int parts = 3);
  cudaEvent_t ev_pt = nullptr;
  // the main stream waits for the form factor + flux-table chain (once)
  cudaError_t join_flux_tables() {
    if (!ff_join_pending) return cudaSuccess;
    ff_join_pending = false;
    const cudaError_t e = cudaStreamWaitEvent(st(), ev_ktab, 0);  // the point-flux table
    return e != cudaSuccess ? e : cudaStreamWaitEvent(st(), ev_join[0], 0);
  }
  // the breakup chain (side[1]), and the survival kernel the fast form
  // launches after it there (ev_survival), not yet joined into the main
  // stream: the projection needs neither, only the contraction does
  bool brk_join_pending = false, survival_on_side = false;
  cudaEvent_t ev_gaa = nullptr, ev_survival = nullptr;
  cudaError_t join_survival() {
    if (!brk_join_pending) return cudaSuccess;
    brk_join_pending = false;
    const bool side_g = survival_on_side;
    survival_on_side = false;
    // without the survival kernel (a cached luminosity), ev_gaa: the G_AA
    // chain runs after the breakup chain on side[1]
    return cudaStreamWaitEvent(st(), side_g ? ev_survival : ev_gaa, 0);
  }
  // parts as enqueue_static_samplers'; ev_static (side[2]) covers both once
  // the z part is forked
  int fork_static_samplers(int parts = 3);
  bool pt_forked = false;
  bool static_pending = false;   // static samplers enqueued on side[2], not yet joined
  // upcg_init's z samplers not enqueued yet: the fast form's luminosity step
  // enqueues them just before the contraction's launch (they wait for
  // ev_static_go, recorded there), so that the projection's kernels go ahead
  // of theirs and the samplers share the SMs with the contraction
  bool statics_deferred = false;
  cudaEvent_t ev_static_go = nullptr;  // where the deferred samplers start
  bool static_go = false;
  // the form factor + flux-table chain (side[0], ev_join[0]) not yet joined
  // into the main stream: the fast form joins it only where the projection
  // first reads the flux tables, so that the survival kernel and the side
  // constants run beside that chain
  bool ff_join_pending = false;
  cudaEvent_t ev_static = nullptr;
  VmParams vm_params() const;
  int build_lumi_cached();
  std::string lumi_cache_key() const;
  bool lumi_cache_usable() const {
    return lumiCache && lumiMethod != 4 && !cap && row_lo <= 0 && (row_hi < 0 || row_hi >= nm);
  }
  int build_lumi_grid();
  int breakup_at_20(double* P20);
  int build_xsec();
  LumiParams lumi_params() const;
  FoldParams fold_params() const;
  EventParams event_params() const;
  int gen_events_device(int64_t n, EventRecord* out, int32_t* mbin, int64_t* rejected);
};

int upcg_generator::set_param(const std::string& k, const std::string& v) {
  // src/UpcGenerator.cpp:183-305
  try {
    // keys of the event loop alone: no table depends on them
    if (k == "NEVENTS") { nEvents = std::stol(v); return UPCG_OK; }
    if (k == "USE_ROOT_OUTPUT") { useROOTOut = std::stoi(v); return UPCG_OK; }
    if (k == "USE_HEPMC_OUTPUT") { useHepMCOut = std::stoi(v); return UPCG_OK; }
    if (k == "SQRTS") { sqrts = std::stod(v); g1 = g2 = sqrts / (2. * kMProt); }
    else if (k == "PROC_ID") procID = std::stoi(v);
    else if (k == "LEP_A") aLep = std::stod(v);
    else if (k == "ALP_MASS") alpMass = std::stod(v);
    else if (k == "ALP_WIDTH") alpWidth = std::stod(v);
    else if (k == "DO_PT_CUT") doPtCut = std::stoi(v);
    else if (k == "PT_MIN") minPt = std::stod(v);
    else if (k == "DO_ETA_CUT") doEtaCut = std::stoi(v);
    else if (k == "ETA_MIN") minEta = std::stod(v);
    else if (k == "ETA_MAX") maxEta = std::stod(v);
    else if (k == "ZMIN") zmin = std::stod(v);
    else if (k == "ZMAX") zmax = std::stod(v);
    else if (k == "MMIN") mmin = std::stod(v);
    else if (k == "MMAX") mmax = std::stod(v);
    else if (k == "YMIN") ymin = std::stod(v);
    else if (k == "YMAX") ymax = std::stod(v);
    else if (k == "BINS_Z") nz = std::stoi(v);
    else if (k == "BINS_M") nm = std::stoi(v);
    else if (k == "BINS_Y") ny = std::stoi(v);
    else if (k == "WS_R") R = std::stod(v);
    else if (k == "WS_A") a = std::stod(v);
    else if (k == "NUCLEUS_Z") Z = std::stoi(v);
    else if (k == "NUCLEUS_A") A = std::stoi(v);
    else if (k == "FLUX_POINT") isPoint = std::stoi(v);
    else if (k == "BREAKUP_MODE") breakupMode = std::stoi(v);
    else if (k == "NON_ZERO_GAM_PT") useNonzeroGamPt = std::stoi(v);
    else if (k == "USE_POLARIZED_CS") usePolarizedCS = std::stoi(v);
    else if (k == "SHADOWING") shadowing = std::stoi(v);  // src/UpcGenerator.cpp:299-304
    else if (k == "DECAY_PDG") dghtPDG = std::stoi(v);
    else if (k == "SEED") seed = std::stol(v);
    else return UPCG_OK;  // keys of other paths: accepted and ignored
  } catch (...) {
    return fail(UPCG_ERR_ARG, "bad value '%s' for %s", v.c_str(), k.c_str());
  }
  invalidate();
  return UPCG_OK;
}

// Process-specific overrides of UpcGenerator::init (src/UpcGenerator.cpp:66-140)
// and the lepton masses of UpcTwoPhotonDilep (src/UpcTwoPhotonDilep.cpp:29-44).
namespace upcg {
cudaStream_t handle_stream(upcg_generator* g) { return g->st(); }
void set_fiducial(upcg_generator* g, int64_t n, int64_t rejected) {
  g->fidCS = g->totCS * (double)n / (double)(n + rejected);  // src/UpcGenerator.cpp:889
}
}  // namespace upcg

int upcg_generator::setup_process() {
  ignoreCSZ = false;
  isVM = false;
  if (procID == 443 || procID == 100443 || procID == 553) {
    // UpcPhotoNuclearVM::UpcPhotoNuclearVM (src/UpcPhotoNuclearVM.cpp:55-93)
    // and the generator's settings for it (src/UpcGenerator.cpp:131-140)
    isVM = true;
    ignoreCSZ = true;
    partPDG = procID;
    isCharged = false;
    vm_pw = 0.4;
    if (procID == 443) { mPart = 3.0969; vm_c0 = 342.; }
    if (procID == 100443) { mPart = 3.6861; vm_c0 = 56.8; }
    if (procID == 553) { mPart = 9.3987; vm_c0 = 0.902; vm_pw = 0.447; }
    if (dghtPDG == 11) mDght = kMEl;
    else if (dghtPDG == 13) mDght = kMMu;
    else if (dghtPDG == 2212) mDght = kMProt;
    else return fail(UPCG_ERR_ARG, "DECAY_PDG %d: the vector mesons decay to 11, 13 or 2212", dghtPDG);
    if (shadowing != 0)
      return fail(UPCG_ERR_PROCESS,
                  "SHADOWING %d needs the nuclear-shadowing tables (EPS09 / LTA); this path has the "
                  "impulse approximation (SHADOWING 0)", shadowing);
    if (usePolarizedCS) return fail(UPCG_ERR_PROCESS, "polarized cross section needs a dilepton process");
    mmin = mPart - 1e-6;
    mmax = mPart + 1e-6;
    nm = 1;
    return UPCG_OK;
  }
  if (procID == 51) {
    ignoreCSZ = true;
    mmin = alpMass - 4. * alpWidth;
    mmax = alpMass + 4. * alpWidth;
    mPart = alpMass;
    partPDG = 51;
    isCharged = false;
    if (usePolarizedCS) return fail(UPCG_ERR_PROCESS, "polarized cross section needs a dilepton process");
    return UPCG_OK;
  }
  if (procID == 11 || procID == 13 || procID == 15) {
    partPDG = procID;
    isCharged = true;
    mPart = procID == 11 ? kMEl : (procID == 13 ? kMMu : kMTau);
    if (mmin < mPart * 2.) mmin = mPart * 2.;
    return UPCG_OK;
  }
  return fail(UPCG_ERR_PROCESS, "PROC_ID %d is not on the two-photon luminosity path", procID);
}

// The process overrides, then the values no table can be built from.  The
// reference reads these keys unchecked (src/UpcGenerator.cpp:183-305); here a
// NaN or a reversed range would reach the kernels' index arithmetic, so it is
// refused on the host before any device work.
int upcg_generator::check_config() {
  const int rc = setup_process();
  if (rc) return rc;
  if (nm < 1 || ny < 1 || nz < 1) return fail(UPCG_ERR_ARG, "empty grid");
  if ((int64_t)nm * ny > kMaxGridCells || (int64_t)nm * nz > kMaxGridCells)
    return fail(UPCG_ERR_SIZE, "grid of %d x %d x %d bins: at most %d (m, y) or (m, z) cells", nm,
                ny, nz, kMaxGridCells);
  if (!(mmin > 0.) || !(mmax > mmin) || !std::isfinite(mmax))
    return fail(UPCG_ERR_ARG, "mass range [%g, %g] GeV: 0 < MMIN < MMAX needed", mmin, mmax);
  if (!(ymax > ymin) || !std::isfinite(ymin) || !std::isfinite(ymax))
    return fail(UPCG_ERR_ARG, "rapidity range [%g, %g]: YMIN < YMAX needed", ymin, ymax);
  if (!(zmax > zmin) || !std::isfinite(zmin) || !std::isfinite(zmax))
    return fail(UPCG_ERR_ARG, "z range [%g, %g]: ZMIN < ZMAX needed", zmin, zmax);
  if (!(g1 > 1.) || !(g2 > 1.) || !std::isfinite(g1) || !std::isfinite(g2))
    return fail(UPCG_ERR_ARG, "SQRTS %g GeV: the beams' Lorentz factor must exceed 1", sqrts);
  if (!(R > 0.) || !(a > 0.) || !std::isfinite(R) || !std::isfinite(a))
    return fail(UPCG_ERR_ARG, "WS_R %g, WS_A %g: both must be positive", R, a);
  if (Z < 1 || A < 1) return fail(UPCG_ERR_ARG, "NUCLEUS_Z %d, NUCLEUS_A %d: both must be >= 1", Z, A);
  if (breakupMode < 1 || breakupMode > 4) return fail(UPCG_ERR_ARG, "BREAKUP_MODE must be 1..4");
  return UPCG_OK;
}

LumiParams upcg_generator::lumi_params() const {
  LumiParams p{};
  p.nm = nm; p.ny = ny;
  p.mmin = mmin; p.dm = (mmax - mmin) / nm;
  p.ymin = ymin; p.dy = (ymax - ymin) / ny;
  p.R = R; p.g1 = g1; p.g2 = g2; p.factor = factor;
  p.A = A; p.isPoint = isPoint; p.breakupMode = breakupMode; p.polarized = usePolarizedCS;
  for (int q = 0; q < 5; ++q) {
    p.cosk[q] = std::cos(M_PI * kX10pos[q]);
    p.sink[q] = std::sin(M_PI * kX10pos[q]);
    p.wk[q] = kW10pos[q];
  }
  const double dbg = 20. / (200 - 1);
  p.gaa = SplineU{gaa_coef.p, 0.0, dbg, 1.0 / dbg, 200};
  const double dbb = (1000. - 1e-6) / 1000000;
  p.brk = SplineU{brk_coef.p, 1e-6, dbb, 1.0 / dbb, brk_n};
  const double dq = (kQ2max - kQ2min) / ff_n;
  p.ff = SplineU{ff_coef.p, kQ2min, dq, 1.0 / dq, ff_n};
  p.q2max = kQ2max;
  p.q2clamp = kQ2max - (kQ2max - kQ2min) / kNQ2;  // the reference's clamp, Q2max - dQ2
  p.mirror = nullptr;
  return p;
}

FoldParams upcg_generator::fold_params() const {
  FoldParams f{};
  f.nm = nm; f.ny = ny; f.nz = nz;
  f.mmin = mmin; f.dm = (mmax - mmin) / nm;
  f.zmin = zmin; f.dz = (zmax - zmin) / nz;
  f.procID = procID; f.polarized = usePolarizedCS;
  f.mPart = mPart; f.aLep = aLep; f.alpWidth = alpWidth;
  return f;
}

EventParams upcg_generator::event_params() const {
  EventParams e{};
  e.nm = nm; e.ny = ny; e.nz = nz;
  e.mmin = mmin; e.mmax = mmax; e.dm = (mmax - mmin) / nm;
  e.ymin = ymin; e.dy = (ymax - ymin) / ny;
  e.zmin = zmin; e.dz = (zmax - zmin) / nz;
  e.ignoreCSZ = ignoreCSZ; e.procID = procID; e.useNonzeroGamPt = useNonzeroGamPt;
  e.doPtCut = doPtCut; e.doEtaCut = doEtaCut;
  e.minPt = minPt; e.minEta = minEta; e.maxEta = maxEta;
  e.mPart = (float)mPart; e.partPDG = partPDG;
  e.seed = (uint64_t)seed;
  // photon-pT spectra on a log grid of e = k^2/gtot^2 covering the cell range
  const double kmin = mmin / 2. * std::exp(-std::max(std::fabs(ymin), std::fabs(ymax))) * 0.5;
  const double kmax = mmax / 2. * std::exp(std::max(std::fabs(ymin), std::fabs(ymax))) * 2.0;
  e.gtot = gtot;
  e.pt_ne = 1024;
  e.pt_nbins = 5000;
  e.pt_lne0 = std::log(kmin * kmin / (gtot * gtot));
  e.pt_dlne = (std::log(kmax * kmax / (gtot * gtot)) - e.pt_lne0) / (e.pt_ne - 1);
  e.pt_width = 6. * kHc / R / 5000;
  e.f_dy = (float)e.dy; e.f_ymin = (float)e.ymin; e.f_dz = (float)e.dz; e.f_zmin = (float)e.zmin;
  e.f_minPt = (float)e.minPt; e.f_minEta = (float)e.minEta; e.f_maxEta = (float)e.maxEta;
  e.f_ptw = (float)e.pt_width;
  e.nm_d = (double)nm;
  e.medges = medges.p && medges.n >= (size_t)nm && medges_ok ? medges.p : nullptr;
  e.pt_c0 = (float)(2. * std::log(gtot) + e.pt_lne0);
  e.pt_inv_dlne = (float)(1. / e.pt_dlne);
  int g2n = 1, g2b = 0;
  while (g2n < nm * ny) {
    g2n <<= 1;
    ++g2b;
  }
  e.g2 = guide2.p;
  e.g2_n = g2n;
  e.g2_bits = g2b;
  e.gz = guidez.p;
  e.gz_n = 128;
  e.gz_bits = 7;
  e.cdf2fx = cdf2fx.p;
  e.cdfzfx = cdfzfx.p;
  e.gpt = guidept.p;
  e.gpt_n = 4096;
  e.polarized = usePolarizedCS ? 1 : 0;
  e.ratio = usePolarizedCS ? ratio.p : nullptr;
  e.cdfz_ps = usePolarizedCS ? cdfz3.p : nullptr;
  e.medge_hi = mmin + (mmax - mmin) / nm * nm;  // binEdgesM.back() (src/UpcGenerator.cpp:677-678)
  e.mbin_lut = mbinlut.p;
  e.mbin_lut_n = mbinlut.p && mbinlut.n >= (size_t)mbinlut_n ? mbinlut_n : 0;
  e.vm = isVM ? 1 : 0;
  e.vm_ratio = isVM ? ratio.p : nullptr;
  e.pom_cdf = isVM ? pom_cdf.p : nullptr;
  e.vm_g1 = g1;
  e.mDght = (float)mDght;
  e.dght_law = dghtPDG == 2212 ? 1 : 0;
  e.vm_err = isVM ? vm_err.p : nullptr;
  return e;
}

namespace {
// Nodes and weights of the n-point Gauss-Legendre rule on [-1, 1] (Newton
// iteration on P_n from the Chebyshev-like initial guesses).
void gauss_legendre(int n, std::vector<double>& x, std::vector<double>& w) {
  x.resize(n);
  w.resize(n);
  for (int i = 0; i < n; ++i) {
    double z = std::cos(M_PI * (i + 0.75) / (n + 0.5)), dp = 0;
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = z;
      for (int k = 2; k <= n; ++k) {
        const double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      dp = n * (z * p1 - p0) / (z * z - 1.0);
      const double dz = p1 / dp;
      z -= dz;
      if (std::fabs(dz) < 1e-16) break;
    }
    x[i] = z;
    w[i] = 2.0 / ((1.0 - z * z) * dp * dp);
  }
}

// calcWSRho (src/UpcCrossSection.cpp:152-163): a 200-term Simpson sum in the
// reference's order, on the host (one serial FP64 chain).
double ws_rho_host(double R, double a, int A) {
  const int nb = 200;
  const double db = 20. / (nb - 1.);
  auto v = [&](int ib) {
    const double r = ib * db;
    return r * r / (1. + std::exp((r - R) / a));
  };
  double sum = v(0) + v(nb - 1);
  for (int i = 1; i < nb - 1; i += 2) sum += 4. * v(i);
  for (int i = 2; i < nb - 1; i += 2) sum += 2. * v(i);
  return A / (sum * db / 3.) / 4. / kPi;
}
}  // namespace

int upcg_generator::build_tables() {
  int rc = check_config();
  if (rc) return rc;
  cudaStream_t s = st();
  CK(side_streams());
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  if (!cap) {
    cudaEventCreate(&t0);
    cudaEventCreate(&t1);
    cudaEventRecord(t0, s);
  }
  factor = Z * Z * kAlpha / M_PI / M_PI / kHc / kHc;  // src/UpcCrossSection.cpp:120
  rho0 = ws_rho_host(R, a, A);
  // sigma_NN (PDG 2016 fit), src/UpcCrossSection.cpp:368-369
  const double ssm = std::pow(sqrts, 2) / std::pow(2 * kMProt + 2.1206, 2);
  csNN = 0.1 * (34.41 + 0.2720 * std::pow(std::log(ssm), 2) + 13.07 * std::pow(ssm, -0.4473) -
                7.394 * std::pow(ssm, -0.5486));
  GaaConsts gk;
  for (int q = 0; q < 5; ++q) {
    gk.cosk[q] = std::cos(M_PI * kX10pos[q]);
    gk.wk[q] = kW10pos[q];
  }
  // breakup: calcBreakupProb's static set-up, per configuration
  bu_gammatarg = 2. * g1 * g1 - 1.;
  bu_omaxx = g1 > 500. ? 1.E10 : 1.E7;
  {
    const double zp = 82, pi = 3.14159, hbarcmev = 197.3269718;
    bu_zcon = zp / (bu_gammatarg * (pi) * (hbarcmev)) * zp / (bu_gammatarg * (pi) * (hbarcmev)) / 137.04;
  }
  bu_host.assign(4 * kBreakupTabMax, 0.);
  bu_nt = breakup_energy_table(bu_gammatarg, bu_host.data(), bu_host.data() + kBreakupTabMax);
  for (int k = 1; k < bu_nt; ++k) {
    bu_host[2 * kBreakupTabMax + k] = std::log(bu_host[k]);
    bu_host[3 * kBreakupTabMax + k] = 1. / bu_host[k];
  }
  // the table chains on forked streams
  CK(cudaEventRecord(ev_fork, s));
  CK(cudaStreamWaitEvent(side[0], ev_fork, 0));
  CK(cudaStreamWaitEvent(side[1], ev_fork, 0));
  // side[2] and side[3] (the luminosity-independent samplers,
  // fork_static_samplers) start here too
  CK(cudaStreamWaitEvent(side[2], ev_fork, 0));
  CK(cudaStreamWaitEvent(side[3], ev_fork, 0));
  CK(gaa_coef.ensure(199));
  CK(ta_coef.ensure(199));
  CK(gaa_work.ensure(800));
  // the survival kernel of the fast forms reads FP32 copies of the G_AA and
  // breakup splines: written here by the spline kernels themselves
  const bool want32 = !cap && !isVM && (lumiMethod == 2 || fast_tables());
  g32_ready = false;
  if (want32) CK(fgaa32.ensure(200));
  // The fast form's projection (k_fast_sides, k_fast_weights) waits for the
  // form factor -> flux tables chain alone: it is enqueued first, on the
  // stream of greatest priority.  The breakup and G_AA chains feed only the
  // survival kernel, which the contraction needs: in the single-configuration
  // fast form they run one after the other on side[1] (least priority) and the
  // survival kernel after them there; otherwise G_AA runs on the handle's
  // stream and the breakup chain on side[1].
  const bool survival_side = defer && !cap && !isVM && fast_tables() && !usePolarizedCS;
  cudaStream_t gs = survival_side ? side[1] : s;
  // form factor on 1e6 knots (the reference's), 65,536 for the fast form
  ff_n = fast_tables() ? kNQ2Fast : kNQ2;
  const double dq = (kQ2max - kQ2min) / ff_n;
  CK(ff_y.ensure(ff_n));
  CK(ff_c.ensure(ff_n));
  CK(ff_coef.ensure(ff_n - 1));
  if (cap && ff_donor && ff_donor->ff_n == ff_n) {
    CK(cudaMemcpyAsync(ff_coef.p, ff_donor->ff_coef.p, (size_t)(ff_n - 1) * sizeof(double4),
                       cudaMemcpyDeviceToDevice, side[0]));
  } else {
    CK(launch_formfac_values(ff_y.p, ff_n, kQ2min, dq, rho0, R, a, side[0],
                             fast_tables() ? 1 : 0));
    CK(build_spline_uniform(ff_y.p, ff_n, kQ2min, dq, ff_c.p, ff_coef.p, side[0]));
  }
  CK(cudaEventRecord(ev_ff, side[0]));
  ftab_early = false;
  if (!cap && !isVM && (lumiMethod == 2 || fast_tables())) {
    // the fast form's flux tables need only the form factor: they run here,
    // ahead of the breakup and G_AA chains
    for (auto& e : ev_ft)
      if (!e) CK(cudaEventCreate(&e));
    CK(cudaEventRecord(ev_ft[0], side[0]));
    // the Q table's Bessel part on side[2] (setup_flux_tables), then the
    // point-flux table there, ahead of the samplers
    const int frc = setup_flux_tables(side[0], 0, side[2]);
    if (frc) return frc;
    CK(cudaEventRecord(ev_ft[1], side[0]));
    CK(fk1.ensure(flux_table_ktab_n()));
    CK(fs32.ensure(flux_table_ktab_n()));
    CK(fk01.ensure(2 * (size_t)flux_table_ktab_n()));
    CK(launch_ktab(g1, fk1.p, fs32.p, side[2], fk01.p, fk01_ready ? 1 : 0));
    CK(cudaEventRecord(ev_ktab, side[2]));
    fk01_ready = true;
    ftab_early = true;
  }
  CK(cudaEventRecord(ev_join[0], side[0]));  // the form factor -> flux tables chain
  // breakup probability: knots up to 20 fm + margin (the path evaluates the
  // spline at min(b, 20))
  CK(bu_tab.ensure(4 * kBreakupTabMax));
  CK(ntab.ensure(1));
  if (!cap) {  // a captured replay reuses the table uploaded by the set-up run
    CK(upload(bu_tab.p, bu_host.data(), 4 * kBreakupTabMax * sizeof(double), side[1]));
    CK(upload(ntab.p, &bu_nt, sizeof(int), side[1]));
  }
  const double dbb = (1000. - 1e-6) / 1000000;
  brk_n = (int)((20. - 1e-6) / dbb) + 257;
  CK(brk_y.ensure(brk_n));
  CK(brk_c.ensure(brk_n));
  CK(brk_coef.ensure(brk_n - 1));
  if (breakupMode > 1 && cap && brk_donor) {
    CK(cudaMemcpyAsync(brk_coef.p, brk_donor->brk_coef.p, (size_t)(brk_n - 1) * sizeof(double4),
                       cudaMemcpyDeviceToDevice, side[1]));
  } else if (breakupMode > 1) {
    if (want32) CK(fbrk32.ensure(brk_n));
    // the fast form (methods 1, 4; budget 1e-4) takes the FP32 sums (~1e-6);
    // the reference's sum steps where an energy crosses omax(b), so every
    // knot is summed (an interpolated table smears those steps to 1.5e-5)
    const int brk_fp32 = fast_tables() ? 1 : 0;
    CK(launch_breakup_values(bu_tab.p, bu_nt, bu_gammatarg, bu_omaxx, bu_zcon, breakupMode, brk_n,
                             1e-6, dbb, brk_y.p, side[1], brk_fp32));
    CK(build_spline_uniform(brk_y.p, brk_n, 1e-6, dbb, brk_c.p, brk_coef.p, side[1],
                            want32 ? fbrk32.p : nullptr));
  }
  g32_ready = want32;
  CK(cudaEventRecord(ev_join[1], side[1]));
  // in a captured scan, a configuration with the same inputs as an earlier one
  // copies that one's tables instead of rebuilding them
  if (cap && gaa_donor) {
    CK(cudaMemcpyAsync(gaa_coef.p, gaa_donor->gaa_coef.p, 199 * sizeof(double4),
                       cudaMemcpyDeviceToDevice, gs));
  } else {
    // the fast forms (budget 1e-4) evaluate the T_A / G_AA integrands in FP32
    const bool gaa_f = !isVM && fast_tables();
    if (gaa_f) CK(fta32.ensure(199));
    CK(launch_gaa(rho0, R, a, csNN, gk, gaa_coef.p, ta_coef.p, gaa_work.p, gs,
                  want32 ? fgaa32.p : nullptr, gaa_f ? fta32.p : nullptr));
  }
  CK(cudaEventRecord(ev_gaa, gs));  // the G_AA spline (and its FP32 copy) is complete
  // only inside upcg_init (defer), whose luminosity step joins the chain
  ff_join_pending = defer && ftab_early && fast_tables() && !usePolarizedCS;
  if (!ff_join_pending) CK(cudaStreamWaitEvent(s, ev_join[0], 0));
  // the fast form's survival kernel runs after the breakup chain on its
  // stream; the main stream joins it before the contraction (join_survival)
  brk_join_pending = ff_join_pending && g32_ready;
  survival_on_side = false;
  if (!brk_join_pending) CK(cudaStreamWaitEvent(s, ev_join[1], 0));
  // the point-flux table: joined with the flux tables where the projection
  // first reads them (join_flux_tables), else here
  if (ftab_early && !ff_join_pending) CK(cudaStreamWaitEvent(s, ev_ktab, 0));
  if (!cap) {
    cudaEventRecord(t1, s);
    if (defer) {
      tab_ev[0] = t0;
      tab_ev[1] = t1;
      tab_pending = true;
    } else {
      CK(cudaEventSynchronize(t1));
      float ms = 0;
      cudaEventElapsedTime(&ms, t0, t1);
      timings[0] = ms;
      cudaEventDestroy(t0);
      cudaEventDestroy(t1);
    }
  }
  tables_ready = true;
  return UPCG_OK;
}

// the breakup probability at 20 fm (the survival kernel beyond b = 20 fm)
int upcg_generator::breakup_at_20(double* P20) {
  *P20 = 1.;
  if (breakupMode == 1) return UPCG_OK;
  cudaStream_t s = st();
  const LumiParams p = lumi_params();
  const double x20 = 20.;
  CK(pts_a.ensure(1));
  CK(pts_c.ensure(1));
  CK(mcpy(pts_a.p, &x20, sizeof x20, cudaMemcpyHostToDevice, s));
  CK(launch_spline_eval(p.brk, pts_a.p, pts_c.p, 1, s));
  CK(mcpy(P20, pts_c.p, sizeof(double), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  return UPCG_OK;
}

// Luminosity method 3: the grid (precision) form of upcg_grid.cu -- a 4096 x
// 2048 flux matrix on the table's photon-energy range and radii 1 .. 500 fm,
// G on the radial grid, T = N G and Lg = T N^T on the tensor cores.
int upcg_generator::build_lumi_grid() {
  if (!isPoint) return fail(UPCG_ERR_PROCESS, "the grid form covers the point flux (FLUX_POINT 1)");
  if (usePolarizedCS) return fail(UPCG_ERR_PROCESS, "the grid form covers the unpolarized luminosity");
  cudaStream_t s = st();
  const int ncell = nm * ny;
  CK(lumi.ensure(ncell));
  const LumiParams p = lumi_params();
  const int nw = 4096, nr = 2048;
  GridForm gf{};
  gf.nw = nw;
  gf.nr = nr;
  const double ymx = std::max(std::fabs(ymin), std::fabs(ymax));
  const double kmin = mmin / 2. * std::exp(-ymx) * 0.99, kmax = mmax / 2. * std::exp(ymx) * 1.01;
  gf.lw0 = std::log(kmin);
  gf.hw = (std::log(kmax) - gf.lw0) / (nw - 1);
  gf.lr0 = std::log(1.0);
  gf.hr = (std::log(500.0) - gf.lr0) / (nr - 1);
  double P20 = 1.;
  int rc = breakup_at_20(&P20);
  if (rc) return rc;
  gf.c_far = 0.;
  for (int q = 0; q < 5; ++q) gf.c_far += P20 * 1. * p.wk[q];
  std::vector<cudaEvent_t> ev(4);
  for (auto& e : ev) {
    cudaEventCreate(&e);
  }
  cudaEventRecord(ev[0], s);
  // point-flux table S(ln x)
  const int nk = flux_table_ktab_n();
  CK(fk1.ensure(nk));
  CK(fs32.ensure(nk));
  FastFluxTables ftab{};
  ftab.st = fk1.p;
  ftab.st32 = fs32.p;
  CK(build_flux_tables(p, &ftab, nullptr, nullptr, 0, nullptr, nullptr, nullptr, s));
  double su0 = 0, su1 = 0;
  flux_table_ktab_range(&su0, &su1);
  gf.s32 = fs32.p;
  gf.su0 = su0;
  gf.sinv_h = (nk - 1) / (su1 - su0);
  gf.sn = nk;
  // G on the radial grid, the flux matrix
  CK(gg_h.ensure((size_t)nr * nr));
  CK(gg_l.ensure((size_t)nr * nr));
  CK(fgaa32.ensure(p.gaa.n));
  CK(fbrk32.ensure(breakupMode != 1 ? p.brk.n : 1));
  CK(launch_fast_G(p, gf.lr0, gf.hr, nr, P20, fgaa32.p, fbrk32.p, gg_h.p, gg_l.p, s));
  const size_t nwp = (size_t)(nw + 127) / 128 * 128;
  CK(gn_h.ensure(nwp * nr));
  CK(gn_l.ensure(nwp * nr));
  CK(gt_h.ensure(nwp * nr));
  CK(gt_l.ensure(nwp * nr));
  CK(g_rowsum.ensure(nw));
  CK(g_tail.ensure(nw));
  CK(g_lg.ensure((size_t)nw * nw));
  CK(launch_grid_flux(p, gf, gn_h.p, gn_l.p, g_rowsum.p, g_tail.p, s));
  cudaEventRecord(ev[1], s);
  CK(ferr.ensure(1));
  CK(cudaMemsetAsync(ferr.p, 0, sizeof(unsigned), s));
  if (lumiMethod == 7) {
    // TF32 arm: FP32 operands (the hi / lo pairs summed), one kind::tf32
    // product per k step instead of the three bf16 ones
    CK(g_n32.ensure(nwp * nr));
    CK(g_g32.ensure((size_t)nr * nr));
    CK(g_t32.ensure(nwp * nr));
    CK(launch_pair_to_f32(gn_h.p, gn_l.p, nwp * nr, g_n32.p, s));
    CK(launch_pair_to_f32(gg_h.p, gg_l.p, (size_t)nr * nr, g_g32.p, s));
    cudaEventRecord(ev[1], s);
    CK(launch_gemm_tf32(g_n32.p, g_g32.p, nw, nr, nr, g_t32.p, ferr.p, s));
    CK(launch_gemm_tf32(g_t32.p, g_n32.p, nw, nw, nr, g_lg.p, ferr.p, s));
  } else {
    CK(launch_gemm_bf16x3(gn_h.p, gn_l.p, gg_h.p, gg_l.p, nw, nr, nr, nullptr, gt_h.p, gt_l.p,
                          ferr.p, s));
    CK(launch_gemm_bf16x3(gt_h.p, gt_l.p, gn_h.p, gn_l.p, nw, nw, nr, g_lg.p, nullptr, nullptr,
                          ferr.p, s));
  }
  cudaEventRecord(ev[2], s);
  CK(launch_grid_cells(p, gf, g_lg.p, g_rowsum.p, g_tail.p, lumi.p, s));
  cudaEventRecord(ev[3], s);
  CK(cudaEventSynchronize(ev[3]));
  float t01 = 0, t12 = 0, t03 = 0;
  cudaEventElapsedTime(&t01, ev[0], ev[1]);
  cudaEventElapsedTime(&t12, ev[1], ev[2]);
  cudaEventElapsedTime(&t03, ev[0], ev[3]);
  for (auto e : ev) cudaEventDestroy(e);
  for (int k = 3; k < 8; ++k) timings[k] = 0;
  timings[1] = t03;
  timings[5] = t12;  // the two tensor-core products
  timings[6] = t01;  // tables, G, flux matrix
  unsigned herr = 0;
  CK(mcpy_sync(&herr, ferr.p, sizeof herr, cudaMemcpyDeviceToHost));
  if (herr) return fail(UPCG_ERR_CUDA, "tensor-core product timed out (code %u)", herr);
  lumi_ready = true;
  return UPCG_OK;
}

// Revision of the table-producing code; part of every cache key, raised
// whenever a change moves the values of any luminosity method.
constexpr int kLumiAlgorithmRevision = 3;
constexpr double kLumiLockTimeoutS = 600.;
// the wait for another process's lock: kLumiLockTimeoutS, or UPCG_LUMI_LOCK_TIMEOUT seconds
double lumi_lock_timeout() {
  if (const char* env = getenv("UPCG_LUMI_LOCK_TIMEOUT")) {
    const double t = atof(env);
    if (t >= 0) return t;
  }
  return kLumiLockTimeoutS;
}

std::string upcg_generator::lumi_cache_key() const {
  // every input of the table, doubles as exact hex floats
  char buf[768];
  snprintf(buf, sizeof buf,
           "upcgen_gb300 two-photon luminosity L dm dy [nm][ny]; revision %d; method %d; "
           "Z %d; A %d; R %a; a %a; sqrts %a; g1 %a; g2 %a; point flux %d; breakup mode %d; "
           "polarized %d; m [%a, %a] bins %d; y [%a, %a] bins %d",
           kLumiAlgorithmRevision, lumiMethod, Z, A, R, a, sqrts, g1, g2, isPoint ? 1 : 0,
           breakupMode, usePolarizedCS ? 1 : 0, mmin, mmax, nm, ymin, ymax, ny);
  return buf;
}

namespace {
struct LockGuard {
  std::string path;
  bool held = false;
  LockGuard(const std::string& p, double timeout) : path(p) {
    held = lumi_lock_acquire(path, timeout) == 1;
  }
  ~LockGuard() {
    if (held) lumi_lock_release(path);
  }
};
}  // namespace

int upcg_generator::build_lumi_cached() {
  // src/UpcCrossSection.cpp:463-592 with a keyed cache file (upcg_cache.cpp)
  const std::string key = lumi_cache_key();
  const std::string path = lumiDir + "/" + lumi_cache_file_name(key);
  const int ntab = usePolarizedCS ? 2 : 1;
  const size_t ncell = (size_t)nm * ny;
  const auto t0 = std::chrono::steady_clock::now();
  LockGuard lock(path + ".lock", lumi_lock_timeout());
  std::vector<double> host;
  if (lumi_cache_read(path, key, ntab, nm, ny, host)) {
    cudaStream_t s = st();
    CK(lumi.ensure(ncell));
    CK(mcpy(lumi.p, host.data(), ncell * sizeof(double), cudaMemcpyHostToDevice, s));
    if (usePolarizedCS) {
      CK(lumi2.ensure(ncell));
      CK(mcpy(lumi2.p, host.data() + ncell, ncell * sizeof(double), cudaMemcpyHostToDevice, s));
    }
    CK(cudaStreamSynchronize(s));
    for (int k = 1; k < 8; ++k) timings[k] = 0;
    timings[1] = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    lumi_cache_hit = 1;
    lumi_ready = true;
    return UPCG_OK;
  }
  const int rc = build_lumi();
  if (rc) return rc;
  lumi_cache_hit = 0;
  if (!lock.held) return UPCG_OK;  // another process holds the file: compute only
  host.resize((size_t)ntab * ncell);
  CK(cudaStreamSynchronize(st()));  // build_lumi may have left its work in flight
  CK(mcpy_sync(host.data(), lumi.p, ncell * sizeof(double), cudaMemcpyDeviceToHost));
  if (usePolarizedCS)
    CK(mcpy_sync(host.data() + ncell, lumi2.p, ncell * sizeof(double), cudaMemcpyDeviceToHost));
  if (lumi_cache_write(path, key, ntab, nm, ny, host.data()) != 0 && debug > 0)
    fprintf(stderr, "upcgen_gb300: could not write the luminosity cache %s\n", path.c_str());
  return UPCG_OK;
}

// The fast form's flux tables: K0/K1 on ln x and the Q(w, b) table (or its
// surrogate rows), on stream ss; the result is in ftab_last.
int upcg_generator::setup_flux_tables(cudaStream_t ss, int with_ktab, cudaStream_t js) {
  const LumiParams p = lumi_params();
  FastFluxTables ftab{};
  // flux tables: K0/K1 on ln x; Q(w, b) on 512 x 256 (ln w, ln b) points by
  // a Gauss-Legendre product on q in [0, kQNodeMax] (nodes below) and the
  // closed-form rest to q = 10.
  const int nk = flux_table_ktab_n();
  CK(fk1.ensure(nk));
  CK(fs32.ensure(nk));
  ftab.st = fk1.p;
  ftab.st32 = fs32.p;
  ftab.nw = 512;
  ftab.nb = 256;
  const double ymx = std::max(std::fabs(ymin), std::fabs(ymax));
  const double kmin = mmin / 2. * std::exp(-ymx) * 0.9, kmax = mmax / 2. * std::exp(ymx) * 1.1;
  ftab.lw0 = std::log(kmin);
  ftab.hw = (std::log(kmax) - ftab.lw0) / (ftab.nw - 1);
  ftab.lb0 = std::log(0.05 * R * 0.999);
  ftab.hb = (std::log(2. * R * 1.001) - ftab.lb0) / (ftab.nb - 1);
  // Q(w, b) nodes on q in [0, kQNodeMax]: the integrand q^2 F / (q^2 + e^2)
  // J1(b q / hc), e = w / gamma, turns on at q ~ e, anywhere from 1e-6 to 0.05
  // GeV over the table's rows, so [1e-7, q1] is taken in ln q (three panels:
  // smooth there for every e; below 1e-7 the integrand's share is < 1e-14),
  // [q1, kQNodeMax] in 13 uniform panels (J1 at b = 2R has ~1.3 periods per
  // panel).  16 Gauss-Legendre nodes per panel; against the integral
  // converged to 1e-10, 7e-7 at worst over the table's w < 0.05 gamma and b
  // (uniform panels from q = 0 were 1e-4 off at e ~ 5e-4 GeV, b ~ 2R).
  const int nlogp = 3, npan = 16, ngl = 16, nqn = npan * ngl;
  if (!isPoint) {
    std::vector<double> gx, gw, qn(nqn), wn(nqn);
    gauss_legendre(ngl, gx, gw);
    const double q0 = 1e-7, q1 = kQNodeMax / npan;
    const double u0 = std::log(q0), du = (std::log(q1) - u0) / nlogp;
    const double hq = (kQNodeMax - q1) / (npan - nlogp);
    for (int pa = 0; pa < npan; ++pa) {
      const bool lg = pa < nlogp;
      const double lo = lg ? u0 + du * pa : q1 + hq * (pa - nlogp);
      const double hi = lg ? u0 + du * (pa + 1) : q1 + hq * (pa - nlogp + 1);
      for (int j = 0; j < ngl; ++j) {
        const double x = 0.5 * (hi - lo) * gx[j] + 0.5 * (hi + lo);
        const double wx = 0.5 * (hi - lo) * gw[j];
        qn[pa * ngl + j] = lg ? std::exp(x) : x;
        wn[pa * ngl + j] = lg ? wx * std::exp(x) : wx;  // dq = q du
      }
    }
    CK(fqn.ensure(nqn));
    CK(fwn.ensure(nqn));
    CK(fq.ensure((size_t)ftab.nw * ftab.nb));
    CK(fq32.ensure((size_t)ftab.nw * ftab.nb));
    CK(fH.ensure((size_t)ftab.nw * nqn));
    CK(fJ.ensure((size_t)nqn * ftab.nb));
    CK(upload(fqn.p, qn.data(), nqn * sizeof(double), js ? js : ss));
    CK(upload(fwn.p, wn.data(), nqn * sizeof(double), js ? js : ss));
    ftab.qt = fq.p;
    ftab.qt32 = fq32.p;
  }
  // method 4: the rows inside the surrogate's box from the MLP (rows in
  // blocks of 64), the others from the quadrature
  int w_sur = 0;
  const double gam = g1;
  if (lumiMethod == 4 && !isPoint) {
    const MlpBox& bx = surrogate->box;
    const bool inside = R >= bx.R_lo && R <= bx.R_hi && a >= bx.a_lo && a <= bx.a_hi &&
                        gam >= bx.g_lo && gam <= bx.g_hi && ftab.lw0 >= bx.lw_lo &&
                        ftab.lb0 >= std::log(bx.bf_lo * R) &&
                        ftab.lb0 + (ftab.nb - 1) * ftab.hb <= bx.lb_hi;
    if (inside) {
      const int nin = (int)std::floor((bx.lw_hi - ftab.lw0) / ftab.hw) + 1;
      w_sur = std::max(0, std::min(ftab.nw, nin)) / 64 * 64;
    }
  }
  if (!isPoint) CK(fpartq.ensure(flux_table_part_doubles(ftab.nw, ftab.nb)));
  if (js && !ev_qj) CK(cudaEventCreateWithFlags(&ev_qj, cudaEventDisableTiming));
  CK(build_flux_tables(p, &ftab, fqn.p, fwn.p, nqn, fH.p, fJ.p, fpartq.p, ss, w_sur, with_ktab, js,
                       js ? ev_qj : nullptr));
  if (w_sur > 0) {
    const int n = w_sur * ftab.nb;
    CK(surrogate->tx.ensure((size_t)n * 5));
    CK(surrogate->out.ensure(n));
    CK(launch_mlp_table_inputs(surrogate->box, ftab, 0, w_sur, (float)R, (float)a, (float)gam,
                               surrogate->tx.p, ss));
    CK(launch_mlp_infer(surrogate->pb.p, surrogate->pf.p, surrogate->tx.p, n, surrogate->out.p, ss));
    CK(launch_mlp_table_fill(ftab, 0, w_sur, gam, (double)A, surrogate->out.p, ss));
  }
  surrogate_rows = w_sur;
  ftab_last = ftab;
  nqn_last = nqn;
  return UPCG_OK;
}

int upcg_generator::complete_deferred(int rc) {
  defer = false;
  join_flux_tables();  // no side-stream work left behind on any path
  join_survival();
  if (herr_copy_pending) {
    mcpy(&hstat->herr, ferr.p, sizeof(unsigned), cudaMemcpyDeviceToHost, st());
    herr_copy_pending = false;
  }
  const cudaError_t he = hp_end();  // the caller's stream waits for init's work
  const cudaError_t se = he != cudaSuccess ? he : cudaStreamSynchronize(st());
  auto elapsed = [](cudaEvent_t a, cudaEvent_t b) {
    float t = 0;
    cudaEventElapsedTime(&t, a, b);
    return t;
  };
  if (tab_pending) {
    timings[0] = elapsed(tab_ev[0], tab_ev[1]);
    cudaEventDestroy(tab_ev[0]);
    cudaEventDestroy(tab_ev[1]);
    tab_pending = false;
  }
  bool herr = false;
  if (lumi_pending) {
    timings[1] = elapsed(lumi_ev[lumi_w0], lumi_ev[lumi_w1]);
    for (int k = 3; k < 8; ++k) timings[k] = 0;
    for (auto& sp : lumi_spans)
      timings[2 + sp.first] += elapsed(lumi_ev[sp.second.first], lumi_ev[sp.second.second]);
    if (lumi_fast && ev_ft[0] && ftab_early_done) timings[7] = elapsed(ev_ft[0], ev_ft[1]);
    for (auto e : lumi_ev) cudaEventDestroy(e);
    lumi_ev.clear();
    lumi_spans.clear();
    last_stats = lumi_stats ? hstat->stats : QagsStats{};
    herr = lumi_fast && hstat->herr != 0;
    lumi_pending = false;
  }
  ftab_early_done = false;
  if (xs_pending) {
    timings[2] = elapsed(xs_ev[0], xs_ev[1]);
    cudaEventDestroy(xs_ev[0]);
    cudaEventDestroy(xs_ev[1]);
    totCS = hstat->tot;
    fidCS = totCS;
    xs_pending = false;
  }
  if (rc) return rc;
  if (se != cudaSuccess) return fail(UPCG_ERR_CUDA, "upcg_init: %s", cudaGetErrorString(se));
  if (herr) {
    xsec_ready = false;
    return fail(UPCG_ERR_CUDA, "tensor-core contraction timed out (code %u)", hstat->herr);
  }
  return UPCG_OK;
}

int upcg_generator::build_lumi() {
  if (lumiMethod == 3 || lumiMethod == 7) return build_lumi_grid();
  cudaStream_t s = st();
  const int ncell = nm * ny;
  CK(lumi.ensure(ncell));
  if (usePolarizedCS) CK(lumi2.ensure(ncell));
  // a shard computes the m-rows [row_lo, row_hi) and leaves the others zero
  const int r0 = std::min(std::max(row_lo, 0), nm);
  const int r1 = row_hi < 0 ? nm : std::min(std::max(row_hi, r0), nm);
  const int cell_lo = r0 * ny, cell_hi = r1 * ny;
  if (cell_lo > 0 || cell_hi < ncell) {
    CK(cudaMemsetAsync(lumi.p, 0, (size_t)ncell * sizeof(double), s));
    if (usePolarizedCS) CK(cudaMemsetAsync(lumi2.p, 0, (size_t)ncell * sizeof(double), s));
  }
  // mirror rapidities (see LumiParams::mirror); chunks hold whole m-rows
  std::vector<int> mir(ny, -1);
  const double dy = (ymax - ymin) / ny;
  for (int ia = 0; ia < ny; ++ia) {
    const double ya = ymin + dy * ia;
    for (int ib = 0; ib < ny; ++ib) {
      const double yb = ymin + dy * ib;
      if (ib != ia && std::fabs(ya + yb) <= 8 * 2.220446049250313e-16 * std::fabs(ya)) { mir[ia] = ib; break; }
    }
  }
  CK(mirror.ensure(ny));
  CK(upload(mirror.p, mir.data(), ny * sizeof(int), s));
  LumiParams p = lumi_params();
  p.mirror = mirror.p;
  // 1: fast form (flux tables + tensor-core contraction); 2: the same
  // contraction on the plain path's exact node fluxes (QAGS / K0,K1).  The
  // contraction's operands: methods 1, 2, 4 write both rows dense on the
  // radial grid (A1 bf16 hi / lo through TMA, A2 FP32 read by the epilogue:
  // the fastest on GB300); 5 writes the dense A1 rows and side 1's node lists
  // (the epilogue gathers the A2 row-dot at the node stencils); 6 writes node
  // lists only and builds A1 in shared memory (k_contract_fused)
  const bool fast = lumiMethod == 2 || fast_tables();
  const bool node_flux = lumiMethod == 2 || !fast;
  const bool fused = lumiMethod == 6, staged = lumiMethod != 5 && !fused;  // staged: dense A2
  // cells per chunk: the node-flux paths hold 1.9 KB of node fluxes per cell,
  // the fast form 8 KB of contraction operands; its chunks are larger, so
  // that a table needs fewer persistent contractions (2 GB at 2^18 cells)
  const int chunk = std::max(1, std::min(ncell, node_flux ? 65536 : 262144) / ny) * ny;
  if (node_flux) {
    CK(flux.ensure((size_t)chunk * 2 * kNb));
    CK(nq.ensure((size_t)chunk * 2));
  }
  CK(work.ensure(1));
  CK(stats.ensure(1));
  const int ovf_cap = 1 << 20;
  CK(ovf.ensure(ovf_cap));
  // the QAGS statistics: zero unless a path with node fluxes fills them
  if (node_flux) CK(cudaMemsetAsync(stats.p, 0, sizeof(QagsStats), s));
  if (lumiMethod == 4 && !surrogate)
    return fail(UPCG_ERR_STATE, "luminosity method 4 needs a surrogate (upcg_set_flux_surrogate)");
  const int P = fast_grid_points();
  const double fu0 = std::log(0.1), fh = (std::log(256.) - std::log(0.1)) / (P - 1);
  const int chunk_pad = (chunk + 127) / 128 * 128;
  if (fast) {
    CK(fgh.ensure((size_t)P * P));
    CK(fgl.ensure((size_t)P * P));
    if (!fused) {
      CK(fah.ensure((size_t)chunk_pad * P));
      CK(fal.ensure((size_t)chunk_pad * P));
    }
    if (staged) CK(fa2.ensure((size_t)chunk_pad * P));
    else CK(fnodes.ensure((size_t)chunk_pad * fast_node_floats_per_row()));
    CK(ffar.ensure(4 * (size_t)chunk_pad));  // per row and side: (ln scale, near, far) float4
    CK(fsides.ensure((2 * (size_t)chunk * fast_side_bytes() + 7) / 8));
    CK(fpart.ensure((size_t)chunk_pad * (P / 128)));
    CK(ferr.ensure(1));
    // the single-configuration survival kernel resets the error word itself
    if (!g32_ready || usePolarizedCS) CK(cudaMemsetAsync(ferr.p, 0, sizeof(unsigned), s));
  }
  // phase timers: 0 whole, 1 nodes, 2 qags, 3 band / contraction, 4 projection + G
  std::vector<cudaEvent_t> ev;
  auto mark = [&]() {
    cudaEvent_t e;
    cudaEventCreate(&e);
    cudaEventRecord(e, s);
    ev.push_back(e);
    return (int)ev.size() - 1;
  };
  std::vector<std::pair<int, std::pair<int, int>>> spans;  // (phase, (begin, end))
  const int w0 = mark();
  FastFluxTables ftab{};
  double c_far = 0.;
  if (fast) {
    const int b = mark();
    // the breakup probability at 20 fm (the survival kernel beyond b = 20 fm)
    // and c_far, on the device: no host round trip between the phases
    CK(ffc.ensure(2));
    CK(fgaa32.ensure(p.gaa.n));
    CK(fbrk32.ensure(breakupMode != 1 ? p.brk.n : 1));
    if (!usePolarizedCS && g32_ready) {
      // the FP32 spline copies come from build_tables; k_fast_G also writes
      // the far constants and resets the error word.  With the breakup chain
      // not joined it runs after that chain on side[1] (and after the G_AA
      // spline), beside the projection
      cudaStream_t gs = s;
      if (brk_join_pending) {
        gs = side[1];
        CK(cudaStreamWaitEvent(gs, ev_gaa, 0));
      }
      CK(launch_fast_G(p, fu0, fh, P, 1.0, fgaa32.p, fbrk32.p, fgh.p, fgl.p, gs, nullptr, 0,
                       ffc.p, ferr.p, 1));
      if (brk_join_pending) {
        CK(cudaEventRecord(ev_survival, gs));
        survival_on_side = true;
      }
    } else if (!usePolarizedCS) {
      CK(join_survival());
      CK(launch_far_consts(p, breakupMode != 1, ffc.p, s));
      CK(launch_fast_G(p, fu0, fh, P, 1.0, fgaa32.p, fbrk32.p, fgh.p, fgl.p, s, ffc.p, 1, nullptr,
                       nullptr, 1));
    } else {
      // calcTwoPhotonLumiPol (src/UpcCrossSection.cpp:274-335): b^2 = b1^2 + b2^2
      // - 2 b1 b2 cos(phi), weights w cos^2(phi) (scalar) and w sin^2(phi)
      // (pseudoscalar): two survival kernels and two far constants
      LumiParams ps = p, pp = p;
      for (int q = 0; q < 5; ++q) {
        ps.cosk[q] = pp.cosk[q] = -p.cosk[q];
        ps.wk[q] = p.wk[q] * p.cosk[q] * p.cosk[q];
        pp.wk[q] = p.wk[q] * p.sink[q] * p.sink[q];
      }
      CK(ffc2.ensure(2));
      CK(fgh2.ensure((size_t)P * P));
      CK(fgl2.ensure((size_t)P * P));
      CK(launch_far_consts(ps, breakupMode != 1, ffc.p, s));
      CK(launch_far_consts(pp, breakupMode != 1, ffc2.p, s));
      CK(launch_fast_G(ps, fu0, fh, P, 1.0, fgaa32.p, fbrk32.p, fgh.p, fgl.p, s, ffc.p, 1, nullptr,
                       nullptr, 1));
      CK(launch_fast_G(pp, fu0, fh, P, 1.0, fgaa32.p, fbrk32.p, fgh2.p, fgl2.p, s, ffc2.p, 1,
                       nullptr, nullptr, 1));
    }
    // the flux tables, unless build_tables already enqueued them beside the
    // breakup and G_AA chains
    if (!ftab_early) {
      const int ft0 = mark();
      const int rc = setup_flux_tables(s);
      if (rc) return rc;
      spans.push_back({5, {ft0, mark()}});
    }
    ftab = ftab_last;
    // ln(m/2) per mass row, and the survival kernel beyond b = 20 fm
    std::vector<double> lnm2(nm);
    for (int im = 0; im < nm; ++im) lnm2[im] = std::log((p.mmin + p.dm * im) / 2.);
    CK(flnm2.ensure(nm));
    CK(upload(flnm2.p, lnm2.data(), nm * sizeof(double), s));
    spans.push_back({4, {b, mark()}});
  }
  // the fast form on table fluxes computes one cell of each pair of mirror
  // rapidities: L(m, -y) = L(m, y) (the photons swap and the survival kernel
  // is symmetric), with equal beams
  const bool use_map = fast && !node_flux && g1 == g2;
  int row_lo = cell_lo, row_hi = cell_hi, n_rep = 0;
  if (use_map) {
    std::vector<int> rm;
    for (int iy = 0; iy < ny; ++iy)
      if (mir[iy] < 0 || iy < mir[iy]) rm.push_back(iy);
    n_rep = (int)rm.size();
    for (int j = 0; j < n_rep; ++j) rm.push_back(mir[rm[j]]);
    CK(frep.ensure(2 * (size_t)n_rep));
    CK(upload(frep.p, rm.data(), rm.size() * sizeof(int), s));
    row_lo = 0;
    row_hi = (r1 - r0) * n_rep;
  }
  contract_rows = fast ? (int64_t)(row_hi - row_lo) : 0;
  fast_nrep = use_map ? n_rep : 0;
  for (int c0 = row_lo; c0 < row_hi; c0 += chunk) {
    const int nc = std::min(chunk, row_hi - c0);
    int b = 0;
    if (node_flux) {
      b = mark();
      CK(launch_lumi_nodes(p, c0, nc, flux.p, nq.p, s));
      spans.push_back({1, {b, mark()}});
    }
    if (!isPoint && node_flux) {
      CK(cudaMemsetAsync(&stats.p->overflow, 0, sizeof(unsigned), s));
      b = mark();
      CK(launch_lumi_qags(p, c0, nc, flux.p, nq.p, work.p, ovf.p, ovf_cap, stats.p, nullptr, 0, s));
      spans.push_back({2, {b, mark()}});
      unsigned novf = 0;
      CK(mcpy(&novf, &stats.p->overflow, sizeof novf, cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
      if (novf > 0) {
        if ((int)novf > ovf_cap) return fail(UPCG_ERR_NUMERIC, "too many QAGS overflows (%u)", novf);
        const int warps = 512;
        CK(gws.ensure(qags_global_ws_doubles_per_warp() * warps));
        CK(launch_lumi_qags_overflow(p, c0, flux.p, ovf.p, (int)novf, work.p, stats.p, gws.p,
                                     warps, s));
      }
    }
    if (!fast) {
      b = mark();
      CK(launch_lumi_band(p, c0, nc, flux.p, lumi.p + 0, usePolarizedCS ? lumi2.p : nullptr, s));
      spans.push_back({3, {b, mark()}});
    } else {
      const int ncp = (nc + 127) / 128 * 128;
      b = mark();
      int part = 0;
      if (ff_join_pending) {  // the side constants beside the flux-table chain, then join it
        CK(launch_fast_project(p, fu0, fh, P, c0, nc, ncp, flnm2.p, c_far,
                               node_flux ? flux.p : nullptr, &ftab, fsides.p,
                               fused ? nullptr : fah.p, fused ? nullptr : fal.p,
                               staged ? fa2.p : nullptr, ffar.p, s, use_map ? frep.p : nullptr,
                               n_rep, r0, staged ? nullptr : fnodes.p, 1));
        CK(join_flux_tables());
        part = 2;
        b = mark();  // the projection span: the node weights and dense rows alone
      }
      CK(launch_fast_project(p, fu0, fh, P, c0, nc, ncp, flnm2.p, c_far,
                             node_flux ? flux.p : nullptr, &ftab, fsides.p,
                             fused ? nullptr : fah.p, fused ? nullptr : fal.p,
                             staged ? fa2.p : nullptr, ffar.p, s, use_map ? frep.p : nullptr, n_rep,
                             r0, staged ? nullptr : fnodes.p, part));
      spans.push_back({4, {b, mark()}});
      // persistent contraction over this chunk's (row tile, N tile) work list
      int shape = 0, grid = 0;
      {
        const int rc = contract_plan(ncp, nc, P, &shape, &grid, fused ? 1 : 0);
        if (rc) return rc;
      }
      const int tbn = shape == 0 ? 256 : 128;
      // each N tile multiplies only the K tiles where G - c can be nonzero
      // (the polarized kernels' azimuths are the negated ones)
      const std::vector<std::pair<int, int>>& kr = delta_ranges(P, fu0, fh, tbn, p,
                                                                usePolarizedCS);
      std::vector<int4> items;
      for (int mt = 0; mt < ncp / 128; ++mt)
        for (int nt = 0; nt < P / tbn; ++nt)
          items.push_back(make_int4(mt, nt, 0, pack_item(std::min(128, nc - mt * 128),
                                                         kr[nt].first, kr[nt].second)));
      // the radial columns below the first node stencil are zero in every row
      const int kt0 = fast_first_ktile(isPoint ? R : 0.05 * R, fu0, fh);
      contract_macs_row = 0;
      for (int nt = 0; nt < P / tbn; ++nt) {
        const int lo = std::max(kt0, kr[nt].first), hi = std::min(P / kContractBK, kr[nt].second);
        if (hi > lo) contract_macs_row += (int64_t)(hi - lo) * kContractBK * tbn;
      }
      // items of unequal work: every CTA meets every N tile
      grid = std::min(grid, (int)items.size());
      rotate_rounds(items, grid);
      CK(fitems.ensure(items.size()));
      CK(upload(fitems.p, items.data(), items.size() * sizeof(int4), s));
      CK(join_survival());  // G (side[1]) before its first reader
      if (statics_deferred) {
        // the samplers from here: ready together with the contraction, whose
        // CTAs (the stream of greatest priority) take the SMs first; theirs
        // share the SMs with it (the contraction is tensor-bound with 6 warps
        // per SM) instead of the FP64 pipes with the table chains
        statics_deferred = false;
        if (!ev_static_go) CK(cudaEventCreateWithFlags(&ev_static_go, cudaEventDisableTiming));
        CK(cudaEventRecord(ev_static_go, s));
        static_go = true;
        const int frc = fork_static_samplers(1);
        if (frc) return frc;
      }
      b = mark();
      if (fused)
        CK(launch_contract_fused(fgh.p, fgl.p, 1, ncp, P, fitems.p, (int)items.size(), fnodes.p,
                                 fpart.p, ferr.p, shape, grid, s, kt0));
      else
        CK(launch_contract_pers(fah.p, fal.p, fgh.p, fgl.p, 1, ncp, P, fitems.p,
                                (int)items.size(), staged ? fa2.p : nullptr, fpart.p, ferr.p,
                                shape, grid, s, staged ? nullptr : fnodes.p, kt0));
      if (usePolarizedCS) {  // the same operands against the pseudoscalar kernel
        CK(fpart2.ensure(fpart.n));
        if (fused)
          CK(launch_contract_fused(fgh2.p, fgl2.p, 1, ncp, P, fitems.p, (int)items.size(),
                                   fnodes.p, fpart2.p, ferr.p, shape, grid, s, kt0));
        else
          CK(launch_contract_pers(fah.p, fal.p, fgh2.p, fgl2.p, 1, ncp, P, fitems.p,
                                  (int)items.size(), staged ? fa2.p : nullptr, fpart2.p, ferr.p,
                                  shape, grid, s, staged ? nullptr : fnodes.p, kt0));
      }
      spans.push_back({3, {b, mark()}});
      CK(launch_fast_finish(p, c0, nc, P / tbn, c_far, fpart.p, ffar.p, lumi.p, s, ffc.p,
                            use_map ? frep.p : nullptr, use_map ? frep.p + n_rep : nullptr, n_rep,
                            r0, 1));
      if (usePolarizedCS)
        CK(launch_fast_finish(p, c0, nc, P / tbn, c_far, fpart2.p, ffar.p, lumi2.p, s, ffc2.p,
                              use_map ? frep.p : nullptr, use_map ? frep.p + n_rep : nullptr,
                              n_rep, r0, 1));
    }
  }
  const int w1 = mark();
  if (defer) {  // collected by complete_deferred
    lumi_ev = std::move(ev);
    lumi_spans = std::move(spans);
    lumi_w0 = w0;
    lumi_w1 = w1;
    lumi_fast = fast;
    ftab_early_done = ftab_early && fast;
    ftab_early = false;
    herr_copy_pending = fast;  // copied at the end (complete_deferred)
    lumi_stats = node_flux;
    if (node_flux) CK(mcpy(&hstat->stats, stats.p, sizeof(QagsStats), cudaMemcpyDeviceToHost, s));
    lumi_pending = true;
    lumi_ready = true;
    return UPCG_OK;
  }
  CK(cudaEventSynchronize(ev[w1]));
  float ms = 0;
  cudaEventElapsedTime(&ms, ev[w0], ev[w1]);
  timings[1] = ms;
  for (int k = 3; k < 8; ++k) timings[k] = 0;
  for (auto& sp : spans) {
    float t = 0;
    cudaEventElapsedTime(&t, ev[sp.second.first], ev[sp.second.second]);
    timings[2 + sp.first] += t;  // [3] nodes [4] qags [5] band/contract [6] projection+G
  }
  if (ftab_early && fast) {  // the flux tables ran beside the table chains
    float t = 0;
    cudaEventElapsedTime(&t, ev_ft[0], ev_ft[1]);
    timings[7] = t;
  }
  ftab_early = false;
  ftab_early_done = false;
  for (auto e : ev) cudaEventDestroy(e);
  if (fast) {
    unsigned herr = 0;
    CK(mcpy_sync(&herr, ferr.p, sizeof herr, cudaMemcpyDeviceToHost));
    if (herr) return fail(UPCG_ERR_CUDA, "tensor-core contraction timed out (code %u)", herr);
  }
  if (node_flux) CK(mcpy(&last_stats, stats.p, sizeof last_stats, cudaMemcpyDeviceToHost, s));
  else last_stats = QagsStats{};
  CK(cudaStreamSynchronize(s));
  lumi_ready = true;
  return UPCG_OK;
}

VmParams upcg_generator::vm_params() const {
  VmParams v{};
  v.mPart = mPart;
  v.sqrts = sqrts;
  v.c0 = vm_c0;
  v.pw = vm_pw;
  v.wmin = kMProt + mPart;  // dsdt's threshold (src/UpcPhotoNuclearVM.cpp:89)
  v.mNucl = (Z * kMProt + (A - Z) * kMNeut) / A;  // src/UpcCrossSection.cpp:121
  v.rho0 = rho0;
  v.R = R;
  v.a = a;
  std::vector<double> x, w;
  gauss_legendre(16, x, w);
  for (int j = 0; j < 16; ++j) {
    v.glx[j] = x[j];
    v.glw[j] = w[j];
  }
  return v;
}

// calcNucCrossSectionY (src/UpcCrossSection.cpp:724-748): per y-bin the photon
// flux of either nucleus (calcPhotonFlux at m_V, +-y) times the meson's
// dsigma/dy; the pomeron table of getMomentumVM.
int upcg_generator::build_vm() {
  cudaStream_t s = st();
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  cudaEventCreate(&t0);
  cudaEventCreate(&t1);
  cudaEventRecord(t0, s);
  const int n2 = 2 * ny;
  const double dy = (ymax - ymin) / ny;
  std::vector<double> hm((size_t)n2, mPart), hy((size_t)n2);
  for (int iy = 0; iy < ny; ++iy) {
    hy[iy] = ymin + dy * iy;
    hy[ny + iy] = -hy[iy];
  }
  CK(vm_m.ensure(n2));
  CK(vm_y.ensure(n2));
  CK(mcpy(vm_m.p, hm.data(), n2 * sizeof(double), cudaMemcpyHostToDevice, s));
  CK(mcpy(vm_y.p, hy.data(), n2 * sizeof(double), cudaMemcpyHostToDevice, s));
  const size_t nn = (size_t)n2 * kNb;
  CK(vm_b.ensure(nn));
  CK(vm_k.ensure(nn));
  CK(vm_w.ensure(nn));
  CK(vm_f.ensure(nn));
  CK(vm_flux.ensure(n2));
  CK(vm_s.ensure(n2));
  CK(stats.ensure(1));
  CK(cudaMemsetAsync(stats.p, 0, sizeof(QagsStats), s));
  CK(launch_photon_flux(lumi_params(), vm_m.p, vm_y.p, n2, vm_b.p, vm_k.p, vm_w.p, vm_f.p, vm_flux.p,
                        stats.p, s));
  const VmParams v = vm_params();
  CK(launch_vm_cs_y(v, vm_y.p, n2, vm_s.p, s));
  CK(cs.ensure(ny));
  CK(ratio.ensure(ny));
  CK(tot.ensure(1));
  CK(launch_vm_fold(vm_flux.p, vm_s.p, ny, dy, cs.p, ratio.p, tot.p, s));
  CK(pom_vals.ensure(kPomN));
  CK(pom_cdf.ensure(kPomN + 1));
  CK(launch_pom_table(v, pom_vals.p, pom_cdf.p, s));
  CK(vm_err.ensure(1));
  CK(cudaMemsetAsync(vm_err.p, 0, sizeof(unsigned), s));
  cudaEventRecord(t1, s);
  CK(cudaEventSynchronize(t1));
  float ms = 0;
  cudaEventElapsedTime(&ms, t0, t1);
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  for (int k = 1; k < 8; ++k) timings[k] = 0;
  timings[1] = ms;
  CK(mcpy_sync(&last_stats, stats.p, sizeof(QagsStats), cudaMemcpyDeviceToHost));
  lumi_ready = false;
  return UPCG_OK;
}

// The samplers that do not depend on the luminosity: the dsigma/dz tables
// and their CDFs, the photon-pT spectra, their guide tables.  upcg_init
// enqueues them on a side stream as soon as the nuclear tables exist, so that
// they run beside the luminosity; build_xsec joins them.
int upcg_generator::enqueue_static_samplers(cudaStream_t ss, cudaEvent_t ff_ready,
                                            cudaStream_t pts, int parts) {
  const FoldParams f = fold_params();
  if (parts & 1) {  // getBinY (include/UpcSampler.h:130-133) of every numerator int(nm (m - mmin))
    const double lo = mmin, hi = mmin + (mmax - mmin) / nm * nm;
    const double nmax = std::floor(nm * (hi - lo)) + 2;
    mbinlut_n = nmax < (double)(1 << 22) ? (int)nmax : 0;
    if (mbinlut_n > 0 && !cap) {  // a captured replay reuses the set-up run's table
      if ((int)mbinlut_host.size() != mbinlut_n || mbinlut_key[0] != lo || mbinlut_key[1] != hi) {
        mbinlut_host.resize((size_t)mbinlut_n);
        for (int n = 0; n < mbinlut_n; ++n) mbinlut_host[n] = (int)((double)n / (hi - lo));
        mbinlut_key[0] = lo;
        mbinlut_key[1] = hi;
      }
      CK(mbinlut.ensure(mbinlut_n));
      CK(upload(mbinlut.p, mbinlut_host.data(), (size_t)mbinlut_n * sizeof(int), ss));
    }
    if (!cap) {  // the gsl histogram's mass edges mmin + dm i (src/UpcGenerator.cpp:677-678)
      const double dmv = (mmax - mmin) / nm;
      medges_host.resize((size_t)nm);
      for (int i = 0; i < nm; ++i) {
        const double a = mmin + dmv * i, b = mmin + dmv * (i + 1);
        medges_host[i] = make_double2(a, b - a);
      }
      CK(medges.ensure((size_t)nm));
      CK(upload(medges.p, medges_host.data(), (size_t)nm * sizeof(double2), ss));
      medges_ok = true;
    }
  }
  if ((parts & 1) && !isVM) {  // sigma(m) per m-row for the fold (build_xsec)
    CK(csm.ensure(usePolarizedCS ? 2 * (size_t)nm : (size_t)nm));
    CK(launch_cs_m_rows(f, csm.p, ss));
  }
  if (!(parts & 1)) {
    // the photon-pT part only
  } else if (isVM) {
    CK(cdfz.ensure(1));  // no z distribution (ignoreCSZ)
  } else if (!usePolarizedCS) {
    CK(cszm.ensure((size_t)nm * nz));
    CK(launch_cs_zm(f, 0, cszm.p, ss));
    CK(cdfz.ensure((size_t)nm * (nz + 1)));
    if (!ignoreCSZ) CK(launch_cdf_rows(cszm.p, nm, nz, cdfz.p, ss));
  } else {
    CK(cszm2.ensure((size_t)nm * nz));
    CK(cszm3.ensure((size_t)nm * nz));
    CK(launch_cs_zm(f, 1, cszm2.p, ss));
    CK(launch_cs_zm(f, 2, cszm3.p, ss));
    CK(cdfz2.ensure((size_t)nm * (nz + 1)));
    CK(cdfz3.ensure((size_t)nm * (nz + 1)));
    CK(launch_cdf_rows(cszm2.p, nm, nz, cdfz2.p, ss));
    CK(launch_cdf_rows(cszm3.p, nm, nz, cdfz3.p, ss));
  }
  const EventParams e = event_params();
  CK(ptcdf.ensure((size_t)e.pt_ne * (e.pt_nbins + 1)));
  CK(ff32.ensure(ff_n));
  CK(guidez.ensure((size_t)nm * e.gz_n));
  CK(guidept.ensure((size_t)e.pt_ne * e.gpt_n));
  CK(cdfzfx.ensure((size_t)nm * (nz + 1)));
  const EventParams eg = event_params();  // with the guide buffers allocated
  if (parts & 1) CK(launch_guides(eg, nullptr, cdfz.p, nullptr, guidez.p, ss, nullptr, cdfzfx.p));
  if (parts & 2) {
    // the photon-pT spectra (they read the form factor) and their guide tables
    // (photon pT drawn: NON_ZERO_GAM_PT, vector mesons), on pts when given
    cudaStream_t ps = pts ? pts : ss;
    if (ff_ready) CK(cudaStreamWaitEvent(ps, ff_ready, 0));
    const bool pt_guides = eg.useNonzeroGamPt || eg.vm;
    CK(launch_photon_pt_tables(eg, lumi_params().ff, ff32.p, ptcdf.p, ps,
                               pt_guides ? guidept.p : nullptr));
    if (pts) {
      if (!ev_pt) CK(cudaEventCreateWithFlags(&ev_pt, cudaEventDisableTiming));
      CK(cudaEventRecord(ev_pt, pts));
    }
  }
  return UPCG_OK;
}

// On side[2], which build_tables forked at its start: the samplers need
// nothing of the luminosity and, of the tables, only the form factor
// (ev_ff), so they run beside the table chains, whose small grids leave most
// SMs idle, and are done before the weights and the contraction fill the GPU.
int upcg_generator::fork_static_samplers(int parts) {
  CK(side_streams());
  if (!ev_static) CK(cudaEventCreateWithFlags(&ev_static, cudaEventDisableTiming));
  if (parts & 2) {
    // the photon-pT part on side[3], after the form factor (beside the flux
    // tables: after them it would meet the projection's pending blocks and
    // hold SMs when the contraction starts)
    const int rc = enqueue_static_samplers(side[2], ev_ff, side[3], 2);
    if (rc) return rc;
    pt_forked = true;
  }
  if (parts & 1) {  // the z part on side[2] (from the go event when one is set)
    if (static_go) {
      static_go = false;
      CK(cudaStreamWaitEvent(side[2], ev_static_go, 0));
    }
    const int rc = enqueue_static_samplers(side[2], ev_ff, nullptr, 1);
    if (rc) return rc;
    if (pt_forked) {
      CK(cudaStreamWaitEvent(side[2], ev_pt, 0));
      pt_forked = false;
    }
    CK(cudaEventRecord(ev_static, side[2]));
    static_pending = true;
  }
  return UPCG_OK;
}

int upcg_generator::build_xsec() {
  cudaStream_t s = st();
  const FoldParams f = fold_params();
  const int ncell = nm * ny;
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  if (!cap) {
    cudaEventCreate(&t0);
    cudaEventCreate(&t1);
    cudaEventRecord(t0, s);
  }
  CK(cdf2.ensure((size_t)ncell + 1));
  CK(cdf2fx.ensure((size_t)ncell + 1));
  CK(cdf_scratch.ensure(cdf_2d_scratch_doubles(ncell)));
  if (isVM) {  // vector mesons: cs, ratio and tot come from build_vm
    CK(launch_cdf_2d(cs.p, ncell, cdf2.p, cdf_scratch.p, s));
  }
  // the luminosity-independent samplers (sigma(m) among them) before the fold
  if (static_pending) {  // enqueued on a side stream before the luminosity
    CK(cudaStreamWaitEvent(s, ev_static, 0));
    static_pending = false;
  } else {
    const int rc = enqueue_static_samplers(s);
    if (rc) return rc;
  }
  if (!isVM) {
    CK(cs.ensure(ncell));
    CK(ratio.ensure(usePolarizedCS ? ncell : 1));
    CK(tot.ensure(1));
    CK(launch_fold_cdf(f, lumi.p, usePolarizedCS ? lumi2.p : nullptr, csm.p, cs.p, ratio.p,
                       cdf_scratch.p, tot.p, cdf2.p, cdf2fx.p, s));
  }
  {
    const EventParams e = event_params();
    CK(guide2.ensure(e.g2_n));
    const EventParams eg = event_params();  // with the guide buffer allocated
    if (isVM)
      CK(launch_guides(eg, cdf2.p, nullptr, guide2.p, nullptr, s, cdf2fx.p, nullptr));
    else
      CK(launch_guide2_fx(eg, cdf2fx.p, guide2.p, s));
  }
  if (cap) {  // a captured replay leaves sigma_tot on the device (read after the replay)
    xsec_ready = true;
    return UPCG_OK;
  }
  if (defer) {  // collected by complete_deferred
    CK(mcpy(&hstat->tot, tot.p, sizeof(double), cudaMemcpyDeviceToHost, s));
    cudaEventRecord(t1, s);
    xs_ev[0] = t0;
    xs_ev[1] = t1;
    xs_pending = true;
    next_cand = 0;
    ev_batch.clear();
    ev_flag.clear();
    ev_pos = 0;
    xsec_ready = true;
    return UPCG_OK;
  }
  CK(mcpy(&totCS, tot.p, sizeof(double), cudaMemcpyDeviceToHost, s));
  cudaEventRecord(t1, s);
  CK(cudaEventSynchronize(t1));
  float ms = 0;
  cudaEventElapsedTime(&ms, t0, t1);
  timings[2] = ms;
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  fidCS = totCS;
  next_cand = 0;
  ev_batch.clear();
  ev_flag.clear();
  ev_pos = 0;
  xsec_ready = true;
  return UPCG_OK;
}

namespace {
// Candidate index of the need-th accepted candidate (need >= 1) of a chunk.
// The candidate index of the need-th accepted candidate of a chunk, from the
// tiles' output offsets and accept words (-1 if the chunk holds fewer).
__global__ void k_find_cut(const int64_t* off, const uint32_t* mask, int ntiles, int64_t need,
                           int64_t* out) {
  if (threadIdx.x != 0) return;
  int lo = 0, hi = ntiles;  // last tile with off <= need-1
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (off[mid] <= need - 1) lo = mid; else hi = mid;
  }
  int rem = (int)(need - 1 - off[lo]);
  for (int w = 0; w < 8; ++w) {
    uint32_t b = mask[(size_t)lo * 8 + w];
    const int pc = __popc(b);
    if (rem < pc) {
      for (;;) {
        const int bit = __ffs(b) - 1;
        if (rem == 0) { *out = (int64_t)lo * 256 + w * 32 + bit; return; }
        b &= b - 1;
        --rem;
      }
    }
    rem -= pc;
  }
  *out = -1;
}
}  // namespace

int upcg_generator::gen_events_device(int64_t n, EventRecord* out, int32_t* mbin,
                                      int64_t* rejected) {
  if (!xsec_ready) return fail(UPCG_ERR_STATE, "upcg_init has not run");
  cudaStream_t s = st();
  const EventParams e = event_params();
  const double* zc = ignoreCSZ ? cdf2.p : (usePolarizedCS ? cdfz2.p : cdfz.p);
  int64_t rej = 0;
  if (!doPtCut && !doEtaCut) {
    CK(launch_events_write(e, cdf2.p, zc, ptcdf.p, next_cand, n, nullptr, nullptr, 0, n, out, mbin, s));
    next_cand += (uint64_t)n;
    *rejected = 0;
    return vm_check();
  }
  int64_t done = 0;
  // pass 1 stages the accepted records (48 bytes per candidate slot), so a
  // chunk holds at most 2^26 candidates: 3.2 GB of staging
  const int64_t kMaxChunk = (int64_t)1 << 26;
  // the reference's loop never ends when the cuts reject everything
  // (src/UpcGenerator.cpp:840-889); this one gives up after 2^34 candidates
  // in a row without an accepted event
  int64_t dry = 0;
  while (done < n) {
    const int64_t need = n - done;
    int64_t nc = (int64_t)std::ceil(need / std::max(acc_rate, 1e-4) * 1.05) + 4096;
    nc = std::min(std::max<int64_t>(nc, 1 << 16), kMaxChunk);
    nc = (nc + 255) / 256 * 256;
    const int tiles = (int)(nc / 256);
    CK(mask.ensure((size_t)tiles * 8));
    CK(tile_off.ensure(tiles + 1));
    CK(total.ensure(2));
    CK(evstage.ensure((size_t)nc));
    if (mbin) CK(evstage_mbin.ensure((size_t)nc));
    CK(launch_events_flags(e, cdf2.p, zc, ptcdf.p, next_cand, nc, mask.p, s, evstage.p,
                           mbin ? evstage_mbin.p : nullptr));
    CK(launch_scan_tiles(nullptr, mask.p, tile_off.p, tiles, total.p, s));
    CK(launch_events_copy(evstage.p, mbin ? evstage_mbin.p : nullptr, mask.p, tile_off.p, tiles,
                          done, n, out, mbin, s));
    int64_t acc = 0;
    CK(mcpy(&acc, total.p, sizeof acc, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    acc_rate = std::max(1e-6, (double)acc / (double)nc);
    dry = acc == 0 ? dry + nc : 0;
    if (dry >= ((int64_t)1 << 34))
      return fail(UPCG_ERR_NUMERIC, "no candidate passed the cuts in %lld draws", (long long)dry);
    if (acc >= need) {
      CK(cudaMemsetAsync(total.p + 1, 0xff, sizeof(int64_t), s));
      note_launch();
      k_find_cut<<<1, 32, 0, s>>>(tile_off.p, mask.p, tiles, need, total.p + 1);
      CK(cudaGetLastError());
      int64_t cut = -1;
      CK(mcpy(&cut, total.p + 1, sizeof cut, cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
      if (cut < 0) return fail(UPCG_ERR_CUDA, "event cut search failed");
      rej += (cut + 1) - need;
      next_cand += (uint64_t)(cut + 1);
      done = n;
    } else {
      rej += nc - acc;
      next_cand += (uint64_t)nc;
      done += acc;
    }
  }
  *rejected = rej;
  return vm_check();
}

// ---------------------------------------------------------------- scans ----
// Many configurations in one captured graph: per configuration the table
// chains, the survival kernel (one plane of a stacked G) and the projection
// (rows of a stacked A), then ONE persistent contraction over the work list
// of every configuration's tiles, then per configuration the finish, the
// fold and the samplers.
struct upcg_scan {
  std::vector<upcg_generator*> gens;
  DBuf<uint16_t> ah, al, gh, gl;  // stacked A1 rows (bf16 hi / lo), survival kernels
  DBuf<float> a2, part;           // stacked A2 rows (FP32), partial row-dots
  DBuf<double> far, fc;
  DBuf<int4> items;
  DBuf<unsigned> err;
  std::vector<int> row0, rows;
  int rows_total = 0, nitems = 0, shape = 0, grid = 0, P = 0;
  cudaStream_t s = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  double setup_ms = 0, run_ms = 0;
  ~upcg_scan() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (s) cudaStreamDestroy(s);
  }
};

int upcg_generator::enqueue_scan_front(upcg_scan& sc, int ci) {
  cudaStream_t s = st();
  cap = true;
  int rc = build_tables();
  if (rc) {
    cap = false;
    return rc;
  }
  const LumiParams p = lumi_params();
  const int P = sc.P;
  const double fu0 = std::log(0.1), fh = (std::log(256.) - std::log(0.1)) / (P - 1);
  const size_t plane = (size_t)P * P;
  double* fc = sc.fc.p + 2 * ci;
  CK(launch_far_consts(p, breakupMode != 1, fc, s));
  CK(launch_fast_G(p, fu0, fh, P, 1.0, fgaa32.p, fbrk32.p, sc.gh.p + ci * plane,
                   sc.gl.p + ci * plane, s, fc, 1, nullptr, nullptr, 1));
  FastFluxTables ft = ftab_last;
  CK(build_flux_tables(p, &ft, fqn.p, fwn.p, nqn_last, fH.p, fJ.p, fpartq.p, s, 0));
  const size_t r0 = (size_t)sc.row0[ci];
  const int nrows = nm * (fast_nrep > 0 ? fast_nrep : ny);
  CK(launch_fast_project(p, fu0, fh, P, 0, nrows, sc.rows[ci], flnm2.p, 0.0, nullptr, &ft,
                         fsides.p, sc.ah.p + r0 * P, sc.al.p + r0 * P, sc.a2.p + r0 * P,
                         sc.far.p + 4 * r0, s, fast_nrep > 0 ? frep.p : nullptr, fast_nrep, 0));
  cap = false;
  return UPCG_OK;
}

int upcg_generator::enqueue_scan_back(upcg_scan& sc, int ci) {
  cudaStream_t s = st();
  const LumiParams p = lumi_params();
  const int ntiles = sc.P / (sc.shape == 0 ? 256 : 128);
  const size_t r0 = (size_t)sc.row0[ci];
  const int nrows = nm * (fast_nrep > 0 ? fast_nrep : ny);
  CK(launch_fast_finish(p, 0, nrows, ntiles, 0.0, sc.part.p + r0 * ntiles, sc.far.p + 4 * r0,
                        lumi.p, s, sc.fc.p + 2 * ci, fast_nrep > 0 ? frep.p : nullptr,
                        fast_nrep > 0 ? frep.p + fast_nrep : nullptr, fast_nrep, 0, 1));
  lumi_ready = true;
  cap = true;
  const int rc = build_xsec();
  cap = false;
  return rc;
}

// ------------------------------------------------------------------ ABI ----
extern "C" {

int upcg_create(upcg_generator** out) {
  // No device work here: configuration calls run without a GPU and the first
  // computing call reports a missing device.
  if (!out) return fail(UPCG_ERR_ARG, "null handle pointer");
  *out = new upcg_generator();
  return UPCG_OK;
}

int upcg_destroy(upcg_generator* g) {
  delete g;
  return UPCG_OK;
}

int upcg_set_parameter(upcg_generator* g, const char* key, const char* value) {
  if (!g || !key || !value) return fail(UPCG_ERR_ARG, "null argument");
  return g->set_param(key, value);
}

int upcg_config_from_file(upcg_generator* g, const char* path) {
  // src/UpcGenerator.cpp:318-346, read as the reference reads it: a line that
  // starts with '#' is skipped; every other line is split into "KEY value"
  // by a stream made before the comment is trimmed, and the key and value
  // persist from line to line, so a token the line lacks keeps the previous
  // line's (a key without a value takes the value of the line before; an
  // empty line repeats the previous pair).  Unknown keys are ignored; a
  // missing file keeps the defaults.
  if (!g || !path) return fail(UPCG_ERR_ARG, "null argument");
  std::ifstream in(path);
  if (!in) return UPCG_OK;
  std::string line, key, val;
  while (std::getline(in, line)) {
    std::istringstream iss(line);
    if (line[0] == '#') continue;  // an empty line's [0] is '\0'
    iss >> key >> val;
    int rc = g->set_param(key, val);
    if (rc < 0) return rc;
  }
  return UPCG_OK;
}

int upcg_set_collision_system(upcg_generator* g, float sqrts, int z, int a) {
  if (!g) return fail(UPCG_ERR_ARG, "null handle");
  g->set_collision(sqrts, z, a);
  g->invalidate();
  return UPCG_OK;
}

int upcg_set_seed(upcg_generator* g, long seed) {
  if (!g) return fail(UPCG_ERR_ARG, "null handle");
  g->seed = seed;
  g->next_cand = 0;
  g->ev_batch.clear();
  g->ev_pos = 0;
  return UPCG_OK;
}

int upcg_set_num_threads(upcg_generator* g, int n) {
  if (!g || n < 1) return fail(UPCG_ERR_ARG, "bad thread count");
  g->numThreads = n;
  return UPCG_OK;
}

int upcg_set_debug_level(upcg_generator* g, int level) {
  if (!g) return fail(UPCG_ERR_ARG, "null handle");
  g->debug = level;
  return UPCG_OK;
}

int upcg_set_lumi_file_directory(upcg_generator* g, const char* dir) {
  if (!g || !dir) return fail(UPCG_ERR_ARG, "null argument");
  g->lumiDir = dir;
  return UPCG_OK;
}

int upcg_set_lumi_cache(upcg_generator* g, int enable) {
  if (!g) return fail(UPCG_ERR_ARG, "null handle");
  g->lumiCache = enable != 0;
  return UPCG_OK;
}

int upcg_set_stream(upcg_generator* g, void* stream) {
  if (!g) return fail(UPCG_ERR_ARG, "null handle");
  g->stream = (cudaStream_t)stream;
  return UPCG_OK;
}

int upcg_set_lumi_method(upcg_generator* g, int method) {
  if (!g || method < 0 || method > 7) return fail(UPCG_ERR_ARG, "bad luminosity method");
  if (method != g->lumiMethod) g->invalidate();
  g->lumiMethod = method;
  return UPCG_OK;
}

int upcg_init(upcg_generator* g) {
  if (!g) return fail(UPCG_ERR_ARG, "null handle");
  if (const int rc = g->check_config()) return rc;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
    return fail(UPCG_ERR_CUDA, "no CUDA device visible");
  if (!g->hstat && cudaMallocHost(&g->hstat, sizeof(upcg_generator::HostStatus)) != cudaSuccess)
    return fail(UPCG_ERR_CUDA, "pinned status block");
  g->defer = true;  // one host synchronisation, at the end (complete_deferred)
  if (const cudaError_t he = g->hp_begin(); he != cudaSuccess)
    return g->complete_deferred(fail(UPCG_ERR_CUDA, "upcg_init: %s", cudaGetErrorString(he)));
  int rc = g->build_tables();
  if (rc) return g->complete_deferred(rc);
  g->lumi_cache_hit = -1;
  if (g->isVM) {  // photonuclear: calcNucCrossSectionY instead of the two-photon luminosity
    rc = g->build_vm();
    if (rc) return g->complete_deferred(rc);
    return g->complete_deferred(g->build_xsec());
  }
  // the photon-pT spectra now (beside the table chains); the z samplers from
  // the luminosity step's contraction launch (beside the contraction)
  g->pt_forked = false;
  rc = g->fork_static_samplers(2);
  if (rc) return g->complete_deferred(rc);
  g->statics_deferred = true;
  rc = g->lumi_cache_usable() ? g->build_lumi_cached() : g->build_lumi();
  if (!rc && g->statics_deferred) {  // a path that did not enqueue them
    g->statics_deferred = false;
    rc = g->fork_static_samplers(1);
  }
  g->statics_deferred = false;
  if (const cudaError_t je = g->join_flux_tables(); je != cudaSuccess && !rc)
    rc = fail(UPCG_ERR_CUDA, "upcg_init: %s", cudaGetErrorString(je));
  if (const cudaError_t je = g->join_survival(); je != cudaSuccess && !rc)
    rc = fail(UPCG_ERR_CUDA, "upcg_init: %s", cudaGetErrorString(je));
  if (rc) {
    if (g->static_pending) {  // leave no side-stream work behind a failed init
      cudaStreamWaitEvent(g->st(), g->ev_static, 0);
      g->static_pending = false;
    }
    if (g->pt_forked) {
      cudaStreamWaitEvent(g->st(), g->ev_pt, 0);
      g->pt_forked = false;
    }
    return g->complete_deferred(rc);
  }
  return g->complete_deferred(g->build_xsec());
}

int upcg_lumi_cache_file(upcg_generator* g, char* path, size_t len, int* last_hit) {
  if (!g || !path || len == 0) return fail(UPCG_ERR_ARG, "null argument");
  const int rc = g->setup_process();  // the key holds the derived mass range
  if (rc) return rc;
  const std::string p = g->lumiDir + "/" + lumi_cache_file_name(g->lumi_cache_key());
  if (p.size() + 1 > len) return fail(UPCG_ERR_SIZE, "path needs %zu bytes", p.size() + 1);
  std::memcpy(path, p.c_str(), p.size() + 1);
  if (last_hit) *last_hit = g->lumi_cache_hit;
  return UPCG_OK;
}

int upcg_compute_nucl_xsection(upcg_generator* g) {
  if (!g) return fail(UPCG_ERR_ARG, "null handle");
  if (!g->lumi_ready) return fail(UPCG_ERR_STATE, "luminosity not computed");
  return g->build_xsec();
}

int upcg_tot_nucl_x(const upcg_generator* g, double* mb) {
  if (!g || !mb) return fail(UPCG_ERR_ARG, "null argument");
  *mb = g->totCS;
  return UPCG_OK;
}

int upcg_fid_nucl_x(const upcg_generator* g, double* mb) {
  if (!g || !mb) return fail(UPCG_ERR_ARG, "null argument");
  *mb = g->fidCS;
  return UPCG_OK;
}

int upcg_get_grid(const upcg_generator* g, double* mmin, double* mmax, int* nm, double* ymin,
                  double* ymax, int* ny, double* zmin, double* zmax, int* nz) {
  if (!g) return fail(UPCG_ERR_ARG, "null handle");
  if (mmin) *mmin = g->mmin;
  if (mmax) *mmax = g->mmax;
  if (nm) *nm = g->nm;
  if (ymin) *ymin = g->ymin;
  if (ymax) *ymax = g->ymax;
  if (ny) *ny = g->ny;
  if (zmin) *zmin = g->zmin;
  if (zmax) *zmax = g->zmax;
  if (nz) *nz = g->nz;
  return UPCG_OK;
}

int upcg_lumi_table(upcg_generator* g, double* out, size_t n, double* out2) {
  if (!g || !out) return fail(UPCG_ERR_ARG, "null argument");
  if (g->isVM) return fail(UPCG_ERR_PROCESS, "PROC_ID %d has no two-photon luminosity", g->procID);
  if (!g->lumi_ready) return fail(UPCG_ERR_STATE, "luminosity not computed");
  const size_t need = (size_t)g->nm * g->ny;
  if (n < need) return fail(UPCG_ERR_SIZE, "need %zu doubles", need);
  CK(mcpy(out, g->lumi.p, need * sizeof(double), cudaMemcpyDeviceToHost, g->st()));
  if (out2 && g->usePolarizedCS)
    CK(mcpy(out2, g->lumi2.p, need * sizeof(double), cudaMemcpyDeviceToHost, g->st()));
  CK(cudaStreamSynchronize(g->st()));
  return UPCG_OK;
}

int upcg_lumi_table_device(upcg_generator* g, const double** out, const double** out2) {
  if (!g || !out) return fail(UPCG_ERR_ARG, "null argument");
  if (!g->lumi_ready) return fail(UPCG_ERR_STATE, "luminosity not computed");
  *out = g->lumi.p;
  if (out2) *out2 = g->usePolarizedCS ? g->lumi2.p : nullptr;
  return UPCG_OK;
}

int upcg_nuc_cs_ym(upcg_generator* g, double* out, size_t n, double* tot_mb) {
  if (!g || !out) return fail(UPCG_ERR_ARG, "null argument");
  if (!g->xsec_ready) return fail(UPCG_ERR_STATE, "cross section not computed");
  const size_t need = (size_t)g->nm * g->ny;
  if (n < need) return fail(UPCG_ERR_SIZE, "need %zu doubles", need);
  CK(mcpy(out, g->cs.p, need * sizeof(double), cudaMemcpyDeviceToHost, g->st()));
  CK(cudaStreamSynchronize(g->st()));
  if (tot_mb) *tot_mb = g->totCS;
  return UPCG_OK;
}

int upcg_cs_zm_table(upcg_generator* g, int flag, double* out, size_t n) {
  if (!g || !out || flag < 0 || flag > 2) return fail(UPCG_ERR_ARG, "bad argument");
  if (!g->tables_ready) {
    int rc = g->setup_process();
    if (rc) return rc;
  }
  const size_t need = (size_t)g->nm * g->nz;
  if (n < need) return fail(UPCG_ERR_SIZE, "need %zu doubles", need);
  DBuf<double> tmp;
  CK(tmp.ensure(need));
  CK(launch_cs_zm(g->fold_params(), flag, tmp.p, g->st()));
  CK(mcpy(out, tmp.p, need * sizeof(double), cudaMemcpyDeviceToHost, g->st()));
  CK(cudaStreamSynchronize(g->st()));
  return UPCG_OK;
}

namespace {
int points_in(upcg_generator* g, const double* a, const double* b, size_t n) {
  CK(g->pts_a.ensure(n));
  CK(g->pts_c.ensure(n));
  CK(mcpy(g->pts_a.p, a, n * sizeof(double), cudaMemcpyHostToDevice, g->st()));
  if (b) {
    CK(g->pts_b.ensure(n));
    CK(mcpy(g->pts_b.p, b, n * sizeof(double), cudaMemcpyHostToDevice, g->st()));
  }
  return UPCG_OK;
}
int points_out(upcg_generator* g, double* out, size_t n) {
  CK(mcpy(out, g->pts_c.p, n * sizeof(double), cudaMemcpyDeviceToHost, g->st()));
  CK(cudaStreamSynchronize(g->st()));
  return UPCG_OK;
}
int need_tables(upcg_generator* g) {
  if (g->tables_ready) return UPCG_OK;
  return g->build_tables();
}
}  // namespace

int upcg_flux_point(upcg_generator* g, const double* b, const double* k, double* out, size_t n) {
  if (!g || !b || !k || !out) return fail(UPCG_ERR_ARG, "null argument");
  if (n == 0) return UPCG_OK;
  int rc = need_tables(g);
  if (rc) return rc;
  rc = points_in(g, b, k, n);
  if (rc) return rc;
  CK(launch_flux_points(g->lumi_params(), g->pts_a.p, g->pts_b.p, g->pts_c.p, (int)n, 0, nullptr, g->st()));
  return points_out(g, out, n);
}

int upcg_flux_form(upcg_generator* g, const double* b, const double* k, double* out, size_t n) {
  if (!g || !b || !k || !out) return fail(UPCG_ERR_ARG, "null argument");
  if (n == 0) return UPCG_OK;
  int rc = need_tables(g);
  if (rc) return rc;
  rc = points_in(g, b, k, n);
  if (rc) return rc;
  CK(g->stats.ensure(1));
  CK(cudaMemsetAsync(g->stats.p, 0, sizeof(QagsStats), g->st()));
  CK(launch_flux_points(g->lumi_params(), g->pts_a.p, g->pts_b.p, g->pts_c.p, (int)n, 1, g->stats.p,
                        g->st()));
  rc = points_out(g, out, n);
  if (rc) return rc;
  CK(mcpy_sync(&g->last_stats, g->stats.p, sizeof(QagsStats), cudaMemcpyDeviceToHost));
  return UPCG_OK;
}

int upcg_flux_form_device_noalloc(upcg_generator* g, const double* b_device,
                                  const double* k_device, double* out_device, size_t n,
                                  uint32_t* failures_device) {
  if (!g || !b_device || !k_device || !out_device) return fail(UPCG_ERR_ARG, "null argument");
  if (n > UPCG_NOALLOC_MAX_POINTS)
    return fail(UPCG_ERR_SIZE, "upcg_flux_form_device_noalloc: %zu points, at most %d per call", n,
                UPCG_NOALLOC_MAX_POINTS);
  if (!g->tables_ready)
    return fail(UPCG_ERR_STATE, "upcg_flux_form_device_noalloc needs the tables of upcg_init");
  if (n == 0) return UPCG_OK;
  CK(launch_flux_form_noalloc(g->lumi_params(), b_device, k_device, out_device, (int)n,
                              failures_device, g->st()));
  return UPCG_OK;
}

int upcg_form_factor(upcg_generator* g, const double* q2, double* out, size_t n) {
  if (!g || !q2 || !out) return fail(UPCG_ERR_ARG, "null argument");
  if (n == 0) return UPCG_OK;
  int rc = need_tables(g);
  if (rc) return rc;
  rc = points_in(g, q2, nullptr, n);
  if (rc) return rc;
  CK(launch_formfac_points(g->pts_a.p, g->pts_c.p, (int)n, g->rho0, g->R, g->a, g->st()));
  return points_out(g, out, n);
}

int upcg_breakup_prob(upcg_generator* g, const double* b, int mode, double* out, size_t n) {
  if (!g || !b || !out || mode < 1 || mode > 4) return fail(UPCG_ERR_ARG, "bad argument");
  if (n == 0) return UPCG_OK;
  int rc = need_tables(g);
  if (rc) return rc;
  rc = points_in(g, b, nullptr, n);
  if (rc) return rc;
  CK(launch_breakup_points(g->bu_gammatarg, g->bu_omaxx, g->bu_zcon, mode, g->bu_tab.p, g->bu_tab.p + kBreakupTabMax,
                           g->ntab.p, g->pts_a.p, g->pts_c.p, (int)n, g->st()));
  return points_out(g, out, n);
}

int upcg_eval_spline(upcg_generator* g, int which, const double* x, double* out, size_t n) {
  if (!g || !x || !out || which < 0 || which > 2) return fail(UPCG_ERR_ARG, "bad argument");
  if (n == 0) return UPCG_OK;
  int rc = need_tables(g);
  if (rc) return rc;
  if (which == 1 && g->breakupMode == 1) return fail(UPCG_ERR_STATE, "no breakup spline for BREAKUP_MODE 1");
  rc = points_in(g, x, nullptr, n);
  if (rc) return rc;
  const LumiParams p = g->lumi_params();
  const SplineU& s = which == 0 ? p.gaa : (which == 1 ? p.brk : p.ff);
  CK(launch_spline_eval(s, g->pts_a.p, g->pts_c.p, (int)n, g->st()));
  return points_out(g, out, n);
}

int upcg_two_photon_lumi(upcg_generator* g, const double* m, const double* y, double* out,
                         double* out2, size_t n) {
  // Cells at arbitrary (m, y): a one-row grid per point through the same kernels.
  if (!g || !m || !y || !out) return fail(UPCG_ERR_ARG, "null argument");
  if (n == 0) return UPCG_OK;
  int rc = need_tables(g);
  if (rc) return rc;
  const bool pol = out2 != nullptr;
  for (size_t i = 0; i < n; ++i) {
    LumiParams p = g->lumi_params();
    p.nm = 1; p.ny = 1; p.mmin = m[i]; p.ymin = y[i]; p.dm = 1.0; p.dy = 1.0;
    p.polarized = pol;
    CK(g->flux.ensure(2 * kNb));
    CK(g->nq.ensure(2));
    CK(g->work.ensure(1));
    CK(g->stats.ensure(1));
    CK(g->ovf.ensure(1 << 10));
    CK(g->pts_c.ensure(2));
    CK(launch_lumi_nodes(p, 0, 1, g->flux.p, g->nq.p, g->st()));
    if (!g->isPoint) {
      CK(cudaMemsetAsync(g->stats.p, 0, sizeof(QagsStats), g->st()));
      CK(launch_lumi_qags(p, 0, 1, g->flux.p, g->nq.p, g->work.p, g->ovf.p, 1 << 10, g->stats.p,
                          nullptr, 0, g->st()));
      unsigned novf = 0;
      CK(mcpy(&novf, &g->stats.p->overflow, sizeof novf, cudaMemcpyDeviceToHost, g->st()));
      CK(cudaStreamSynchronize(g->st()));
      if (novf > 0) {
        const int warps = 64;
        CK(g->gws.ensure(qags_global_ws_doubles_per_warp() * warps));
        CK(launch_lumi_qags_overflow(p, 0, g->flux.p, g->ovf.p, (int)novf, g->work.p, g->stats.p,
                                     g->gws.p, warps, g->st()));
      }
    }
    CK(launch_lumi_band(p, 0, 1, g->flux.p, g->pts_c.p, pol ? g->pts_c.p + 1 : nullptr, g->st()));
    double v[2] = {0, 0};
    CK(mcpy(v, g->pts_c.p, sizeof v, cudaMemcpyDeviceToHost, g->st()));
    CK(cudaStreamSynchronize(g->st()));
    out[i] = v[0];
    if (pol) out2[i] = v[1];
  }
  return UPCG_OK;
}

int upcg_cs_m(upcg_generator* g, const double* m, int flag, double* out, size_t n) {
  if (!g || !m || !out || flag < 0 || flag > 2) return fail(UPCG_ERR_ARG, "bad argument");
  if (n == 0) return UPCG_OK;
  int rc = g->setup_process();
  if (rc) return rc;
  rc = points_in(g, m, nullptr, n);
  if (rc) return rc;
  CK(launch_cs_m_points(g->fold_params(), g->pts_a.p, g->pts_c.p, (int)n, flag, g->st()));
  return points_out(g, out, n);
}

int upcg_generate_events_device(upcg_generator* g, int64_t n, upcg_event* out_device,
                                int32_t* mbin_device, int64_t* rejected) {
  if (!g || !out_device || !rejected || n < 0) return fail(UPCG_ERR_ARG, "bad argument");
  if (n == 0) { *rejected = 0; return UPCG_OK; }
  int rc = g->gen_events_device(n, reinterpret_cast<EventRecord*>(out_device), mbin_device, rejected);
  if (rc) return rc;
  g->fidCS = g->totCS * (double)n / (double)(n + *rejected);  // src/UpcGenerator.cpp:889
  return UPCG_OK;
}

// Host output in slices of 2^21 events through a ring of 3 device slots: the
// copy of slice k to the host (on side[1]) overlaps the generation of slice
// k+1; a slot is reused once its copy has finished.  The slices take the
// candidate sequence in order, so the events are those of one device call.
int upcg_generate_events(upcg_generator* g, int64_t n, upcg_event* out, int32_t* mbin,
                         int64_t* rejected) {
  if (!g || !out || !rejected || n < 0) return fail(UPCG_ERR_ARG, "bad argument");
  if (n == 0) { *rejected = 0; return UPCG_OK; }
  if (!g->xsec_ready) return fail(UPCG_ERR_STATE, "upcg_init has not run");
  const int64_t chunk = std::min<int64_t>(n, (int64_t)1 << 21);
  const int nslot = n > chunk ? 3 : 1;
  CK(g->evbuf.ensure((size_t)chunk * nslot));
  if (mbin) CK(g->mbinbuf.ensure((size_t)chunk * nslot));
  CK(g->side_streams());
  if (!g->ev_gen) CK(cudaEventCreateWithFlags(&g->ev_gen, cudaEventDisableTiming));
  for (auto& e : g->ev_out)
    if (!e) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  cudaStream_t s = g->st(), cs = g->side[1];
  auto* rec = reinterpret_cast<EventRecord*>(out);
  int64_t rej = 0;
  int rc = UPCG_OK;
  // on an error the loop stops, and both streams are drained before returning:
  // no copy into the caller's buffers outlives the call
  cudaError_t ce = cudaSuccess;
  for (int64_t off = 0, k = 0; off < n; off += chunk, ++k) {
    const int slot = (int)(k % nslot);
    const int64_t c = std::min(chunk, n - off);
    if (k >= nslot) ce = cudaStreamWaitEvent(s, g->ev_out[slot], 0);
    if (ce != cudaSuccess) break;
    EventRecord* dv = g->evbuf.p + (size_t)slot * chunk;
    int32_t* dm = mbin ? g->mbinbuf.p + (size_t)slot * chunk : nullptr;
    int64_t r = 0;
    rc = g->gen_events_device(c, dv, dm, &r);
    if (rc) break;
    rej += r;
    ce = cudaEventRecord(g->ev_gen, s);
    if (ce == cudaSuccess) ce = cudaStreamWaitEvent(cs, g->ev_gen, 0);
    if (ce == cudaSuccess)
      ce = mcpy(rec + off, dv, (size_t)c * sizeof(EventRecord), cudaMemcpyDeviceToHost, cs);
    if (ce == cudaSuccess && mbin)
      ce = mcpy(mbin + off, dm, (size_t)c * sizeof(int32_t), cudaMemcpyDeviceToHost, cs);
    if (ce == cudaSuccess) ce = cudaEventRecord(g->ev_out[slot], cs);
    if (ce != cudaSuccess) break;
  }
  const cudaError_t e_cs = cudaStreamSynchronize(cs), e_s = cudaStreamSynchronize(s);
  if (rc) return rc;
  if (ce == cudaSuccess) ce = e_cs != cudaSuccess ? e_cs : e_s;
  if (ce != cudaSuccess)
    return fail(UPCG_ERR_CUDA, "event output to the host: %s", cudaGetErrorString(ce));
  *rejected = rej;
  g->fidCS = g->totCS * (double)n / (double)(n + rej);  // src/UpcGenerator.cpp:889
  return UPCG_OK;
}

int upcg_sampler_bins(upcg_generator* g, const double* x, size_t n, int axis, int32_t* out) {
  if (!g || !x || !out || axis < 0 || axis > 1) return fail(UPCG_ERR_ARG, "bad argument");
  if (n == 0) return UPCG_OK;
  if (n > (size_t)INT32_MAX) return fail(UPCG_ERR_SIZE, "too many values");
  if (!g->xsec_ready) return fail(UPCG_ERR_STATE, "upcg_init has not run");
  CK(g->pts_a.ensure(n));
  CK(g->pts_c.ensure((n + 1) / 2));  // n ints
  cudaStream_t s = g->st();
  CK(mcpy(g->pts_a.p, x, n * sizeof(double), cudaMemcpyHostToDevice, s));
  int* d_out = reinterpret_cast<int*>(g->pts_c.p);
  CK(launch_sampler_bins(g->event_params(), g->pts_a.p, (int)n, axis, d_out, s));
  CK(mcpy(out, d_out, n * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  return UPCG_OK;
}

int upcg_run_events(upcg_generator* g, int64_t n, int64_t* rejected) {
  if (!g || !rejected || n < 0) return fail(UPCG_ERR_ARG, "bad argument");
  if (n == 0) { *rejected = 0; return UPCG_OK; }
  if (!g->xsec_ready) return fail(UPCG_ERR_STATE, "upcg_init has not run");
  // slices of 2^21 events through one device slot, in candidate order
  const int64_t chunk = std::min<int64_t>(n, (int64_t)1 << 21);
  CK(g->evbuf.ensure((size_t)chunk));
  int64_t rej = 0;
  for (int64_t off = 0; off < n; off += chunk) {
    int64_t r = 0;
    const int rc = g->gen_events_device(std::min(chunk, n - off), g->evbuf.p, nullptr, &r);
    if (rc) return rc;
    rej += r;
  }
  CK(cudaStreamSynchronize(g->st()));
  *rejected = rej;
  g->fidCS = g->totCS * (double)n / (double)(n + rej);  // src/UpcGenerator.cpp:889
  return UPCG_OK;
}

int upcg_host_alloc(size_t bytes, void** out) {
  if (!out) return fail(UPCG_ERR_ARG, "null argument");
  *out = nullptr;
  if (bytes == 0) return UPCG_OK;
  CK(cudaMallocHost(out, bytes));
  return UPCG_OK;
}

int upcg_host_free(void* p) {
  if (p) CK(cudaFreeHost(p));
  return UPCG_OK;
}

int upcg_generate_event(upcg_generator* g, upcg_event* ev, int* accepted) {
  // The next candidate of the sequence upcg_generate_events draws from, with
  // its accept flag (1 = passes the cuts, 0 = rejected), as generateEvent.
  if (!g || !ev || !accepted) return fail(UPCG_ERR_ARG, "null argument");
  if (!g->xsec_ready) return fail(UPCG_ERR_STATE, "upcg_init has not run");
  if (g->ev_pos >= g->ev_flag.size()) {
    const int64_t nb = 4096;
    DBuf<EventRecord> rec;
    DBuf<uint8_t> flg;
    CK(rec.ensure(nb));
    CK(flg.ensure(nb));
    const EventParams e = g->event_params();
    const double* zc = g->ignoreCSZ ? g->cdf2.p : (g->usePolarizedCS ? g->cdfz2.p : g->cdfz.p);
    CK(launch_events_all(e, g->cdf2.p, zc, g->ptcdf.p, g->next_cand, nb, rec.p, flg.p, g->st()));
    g->ev_batch.resize(nb);
    g->ev_flag.resize(nb);
    CK(mcpy(g->ev_batch.data(), rec.p, nb * sizeof(EventRecord), cudaMemcpyDeviceToHost, g->st()));
    CK(mcpy(g->ev_flag.data(), flg.p, nb, cudaMemcpyDeviceToHost, g->st()));
    CK(cudaStreamSynchronize(g->st()));
    g->next_cand += (uint64_t)nb;
    g->ev_pos = 0;
  }
  const size_t i = g->ev_pos++;
  const bool cuts = g->doPtCut || g->doEtaCut;
  *accepted = cuts ? g->ev_flag[i] : 1;
  *reinterpret_cast<EventRecord*>(ev) = g->ev_batch[i];
  return UPCG_OK;
}

int upcg_philox(uint64_t seed, uint64_t counter0, size_t n, uint32_t* out4) {
  if (!out4) return fail(UPCG_ERR_ARG, "null argument");
  if (n == 0) return UPCG_OK;
  DBuf<uint32_t> d;
  CK(d.ensure(4 * n));
  CK(launch_philox_dump(seed, counter0, (int64_t)n, d.p, 0));
  CK(mcpy_sync(out4, d.p, 4 * n * sizeof(uint32_t), cudaMemcpyDeviceToHost));
  return UPCG_OK;
}

int upcg_last_timings(const upcg_generator* g, double* ms, size_t n) {
  if (!g || !ms) return fail(UPCG_ERR_ARG, "null argument");
  for (size_t i = 0; i < n && i < 8; ++i) ms[i] = g->timings[i];
  return UPCG_OK;
}

int upcg_qags_stats(const upcg_generator* g, uint64_t* failures, uint64_t* max_intervals,
                    uint64_t* evals) {
  if (!g) return fail(UPCG_ERR_ARG, "null handle");
  if (failures) *failures = g->last_stats.failures;
  if (max_intervals) *max_intervals = g->last_stats.max_intervals;
  if (evals) *evals = g->last_stats.evals;
  return UPCG_OK;
}

int upcg_fast_flux_table(upcg_generator* g, double* out, size_t n, double* grid) {
  if (!g || !out || !grid) return fail(UPCG_ERR_ARG, "null argument");
  if (!g->lumi_ready || !g->fast_tables() || g->isPoint || !g->fq.p)
    return fail(UPCG_ERR_STATE, "no fast-form flux table (fast method, FLUX_POINT 0, after init)");
  const size_t need = (size_t)512 * 256;
  if (n < need) return fail(UPCG_ERR_SIZE, "need %zu doubles", need);
  CK(mcpy_sync(out, g->fq.p, need * sizeof(double), cudaMemcpyDeviceToHost));
  const double ymx = std::max(std::fabs(g->ymin), std::fabs(g->ymax));
  const double kmin = g->mmin / 2. * std::exp(-ymx) * 0.9, kmax = g->mmax / 2. * std::exp(ymx) * 1.1;
  grid[0] = std::log(kmin);
  grid[1] = (std::log(kmax) - grid[0]) / 511;
  grid[2] = std::log(0.05 * g->R * 0.999);
  grid[3] = (std::log(2. * g->R * 1.001) - grid[2]) / 255;
  return UPCG_OK;
}

int upcg_selftest_contract(int ncells, int P, uint64_t seed, double* max_rel, double* ms) {
  if (!max_rel || !ms || ncells < 1 || P < 256 || P % 256) return fail(UPCG_ERR_ARG, "bad argument");
  CK(contract_selftest(ncells, P, seed, max_rel, ms));
  return UPCG_OK;
}

const char* upcg_last_error(void) { return g_err.c_str(); }
int upcg_set_row_range(upcg_generator* g, int im0, int im1) {
  if (!g || im0 < 0 || (im1 >= 0 && im1 < im0)) return fail(UPCG_ERR_ARG, "bad row range");
  g->row_lo = im0;
  g->row_hi = im1;
  g->invalidate();
  return UPCG_OK;
}

namespace {
int set_lumi_table(upcg_generator* g, const double* table, size_t n, const double* table2,
                   cudaMemcpyKind kind) {
  if (!g || !table) return fail(UPCG_ERR_ARG, "null argument");
  const size_t ncell = (size_t)g->nm * g->ny;
  if (n != ncell) return fail(UPCG_ERR_SIZE, "table has %zu cells, the grid %zu", n, ncell);
  if (g->usePolarizedCS && !table2) return fail(UPCG_ERR_ARG, "polarized: two tables needed");
  if (!g->tables_ready) {
    const int rc = g->build_tables();
    if (rc) return rc;
  }
  cudaStream_t s = g->st();
  CK(g->lumi.ensure(ncell));
  CK(mcpy(g->lumi.p, table, ncell * sizeof(double), kind, s));
  if (g->usePolarizedCS) {
    CK(g->lumi2.ensure(ncell));
    CK(mcpy(g->lumi2.p, table2, ncell * sizeof(double), kind, s));
  }
  CK(cudaStreamSynchronize(s));
  g->lumi_ready = true;
  return g->build_xsec();
}
}  // namespace

int upcg_set_lumi_table(upcg_generator* g, const double* table, size_t n, const double* table2) {
  return set_lumi_table(g, table, n, table2, cudaMemcpyHostToDevice);
}

int upcg_set_lumi_table_device(upcg_generator* g, const double* table_device, size_t n,
                               const double* table2_device) {
  return set_lumi_table(g, table_device, n, table2_device, cudaMemcpyDeviceToDevice);
}

int upcg_set_candidate_offset(upcg_generator* g, uint64_t counter) {
  if (!g) return fail(UPCG_ERR_ARG, "null handle");
  if (!g->xsec_ready) return fail(UPCG_ERR_STATE, "upcg_init has not run");
  g->next_cand = counter;
  g->ev_batch.clear();
  g->ev_flag.clear();
  g->ev_pos = 0;
  return UPCG_OK;
}

int upcg_event_output_config(const upcg_generator* g, int64_t* nevents, int* use_root,
                             int* use_hepmc) {
  if (!g || !nevents || !use_root || !use_hepmc) return fail(UPCG_ERR_ARG, "null argument");
  *nevents = g->nEvents;
  *use_root = g->useROOTOut;
  *use_hepmc = g->useHepMCOut;
  return UPCG_OK;
}

int upcg_get_candidate_offset(const upcg_generator* g, uint64_t* counter) {
  if (!g || !counter) return fail(UPCG_ERR_ARG, "null argument");
  *counter = g->next_cand;
  return UPCG_OK;
}

int upcg_decay_pdg(upcg_generator* g, int* pdg) {
  if (!g || !pdg) return fail(UPCG_ERR_ARG, "null argument");
  const int rc = g->setup_process();
  if (rc) return rc;
  *pdg = g->isVM ? g->dghtPDG : (g->procID == 51 ? 22 : 0);
  return UPCG_OK;
}

int upcg_photon_flux(upcg_generator* g, const double* m, const double* y, double* out, size_t n) {
  if (!g || !m || !y || !out) return fail(UPCG_ERR_ARG, "null argument");
  if (n == 0) return UPCG_OK;
  if (n > (size_t)(1 << 24)) return fail(UPCG_ERR_SIZE, "at most 2^24 points per call");
  int rc = need_tables(g);
  if (rc) return rc;
  rc = points_in(g, m, y, n);
  if (rc) return rc;
  cudaStream_t s = g->st();
  const size_t nn = n * kNb;
  DBuf<double> b, k, w, f;
  CK(b.ensure(nn));
  CK(k.ensure(nn));
  CK(w.ensure(nn));
  CK(f.ensure(nn));
  CK(g->stats.ensure(1));
  CK(cudaMemsetAsync(g->stats.p, 0, sizeof(QagsStats), s));
  CK(launch_photon_flux(g->lumi_params(), g->pts_a.p, g->pts_b.p, (int)n, b.p, k.p, w.p, f.p,
                        g->pts_c.p, g->stats.p, s));
  rc = points_out(g, out, n);
  if (rc) return rc;
  CK(mcpy_sync(&g->last_stats, g->stats.p, sizeof(QagsStats), cudaMemcpyDeviceToHost));
  return UPCG_OK;
}

int upcg_vm_cross_section_y(upcg_generator* g, const double* y, double* out, size_t n) {
  if (!g || !y || !out) return fail(UPCG_ERR_ARG, "null argument");
  int rc = g->setup_process();
  if (rc) return rc;
  if (!g->isVM) return fail(UPCG_ERR_PROCESS, "PROC_ID %d is not a vector meson", g->procID);
  if (n == 0) return UPCG_OK;
  rc = need_tables(g);  // rho0 of the form factor
  if (rc) return rc;
  rc = points_in(g, y, nullptr, n);
  if (rc) return rc;
  CK(launch_vm_cs_y(g->vm_params(), g->pts_a.p, (int)n, g->pts_c.p, g->st()));
  return points_out(g, out, n);
}

int upcg_nuc_cs_y(upcg_generator* g, double* cs, double* ratio, size_t ny, double* tot_mb) {
  if (!g || !cs) return fail(UPCG_ERR_ARG, "null argument");
  if (!g->isVM) return fail(UPCG_ERR_PROCESS, "PROC_ID %d is not a vector meson", g->procID);
  if (!g->xsec_ready) return fail(UPCG_ERR_STATE, "cross section not computed");
  if (ny < (size_t)g->ny) return fail(UPCG_ERR_SIZE, "need %d doubles", g->ny);
  CK(mcpy(cs, g->cs.p, g->ny * sizeof(double), cudaMemcpyDeviceToHost, g->st()));
  if (ratio) CK(mcpy(ratio, g->ratio.p, g->ny * sizeof(double), cudaMemcpyDeviceToHost, g->st()));
  CK(cudaStreamSynchronize(g->st()));
  if (tot_mb) *tot_mb = g->totCS;
  return UPCG_OK;
}

int upcg_particle_pdg(upcg_generator* g, int* pdg, int* charged) {
  if (!g || !pdg) return fail(UPCG_ERR_ARG, "null argument");
  const int rc = g->setup_process();
  if (rc) return rc;
  *pdg = g->partPDG;
  if (charged) *charged = g->isCharged ? 1 : 0;
  return UPCG_OK;
}

int upcg_contract_rows(const upcg_generator* g, int64_t* rows) {
  if (!g || !rows) return fail(UPCG_ERR_ARG, "null argument");
  *rows = g->contract_rows;
  return UPCG_OK;
}

int upcg_contract_work(const upcg_generator* g, int64_t* rows, int64_t* macs_per_row) {
  if (!g || !rows || !macs_per_row) return fail(UPCG_ERR_ARG, "null argument");
  *rows = g->contract_rows;
  *macs_per_row = g->contract_rows ? g->contract_macs_row : 0;
  return UPCG_OK;
}

int upcg_copy_bytes(uint64_t* h2d, uint64_t* d2h) {
  if (!h2d || !d2h) return fail(UPCG_ERR_ARG, "null pointer");
  *h2d = g_h2d.load(std::memory_order_relaxed);
  *d2h = g_d2h.load(std::memory_order_relaxed);
  return UPCG_OK;
}

int upcg_kernel_launches(uint64_t* n) {
  if (!n) return fail(UPCG_ERR_ARG, "null pointer");
  *n = launch_count();
  return UPCG_OK;
}

// ---- learned flux surrogate ------------------------------------------------
int upcg_mlp_create(upcg_mlp** out, uint64_t seed) {
  if (!out) return fail(UPCG_ERR_ARG, "null argument");
  upcg_mlp* h = new (std::nothrow) upcg_mlp();
  if (!h) return fail(UPCG_ERR_NOMEM, "out of host memory");
  // training box: w in [1e-3, 1e2] GeV, b in [0.049 R, 500] fm, R in [5, 7.5] fm,
  // a in [0.40, 0.60] fm, g in [100, 3000]
  h->box = MlpBox{(float)std::log(1e-3), (float)std::log(1e2), 0.049f, (float)std::log(500.),
                  5.f, 7.5f, 0.40f, 0.60f, 100.f, 3000.f};
  h->seed = seed;
  const int np = mlp_param_count();
  std::vector<float> p(np, 0.f);
  // uniform +-sqrt(6 / fan_in) for the SiLU layers (He, uniform), +-sqrt(3 / fan_in)
  // for the output layer; biases 0 (a counter-based splitmix64 stream)
  uint64_t st = seed * 0x9E3779B97F4A7C15ull + 1;
  auto uni = [&]() {
    st += 0x9E3779B97F4A7C15ull;
    uint64_t x = st;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    x ^= x >> 31;
    return (double)(x >> 11) * (1.0 / 9007199254740992.0);
  };
  const int kH = 128, kIn = 5;
  int o = 0;
  auto fill = [&](int n, int fan_in, double gain) {
    const double lim = std::sqrt(gain / fan_in);
    for (int i = 0; i < n; ++i) p[o++] = (float)((2. * uni() - 1.) * lim);
  };
  fill(kH * kIn, kIn, 6.);
  o += kH;
  for (int l = 0; l < 3; ++l) {
    fill(kH * kH, kH, 6.);
    o += kH;
  }
  fill(kH, kH, 3.);
  o += 1;
  cudaStream_t s = h->st();
  auto bad = [&](cudaError_t e) {
    if (e == cudaSuccess) return false;
    fail(UPCG_ERR_CUDA, "upcg_mlp_create: %s", cudaGetErrorString(e));
    return true;
  };
  if (bad(h->pf.ensure(np)) || bad(h->m.ensure(np)) || bad(h->v.ensure(np)) ||
      bad(h->pb.ensure(np)) ||
      bad(mcpy(h->pf.p, p.data(), np * sizeof(float), cudaMemcpyHostToDevice, s)) ||
      bad(cudaMemsetAsync(h->m.p, 0, np * sizeof(float), s)) ||
      bad(cudaMemsetAsync(h->v.p, 0, np * sizeof(float), s)) ||
      bad(launch_mlp_to_bf16(h->pf.p, h->pb.p, s)) || bad(cudaStreamSynchronize(s))) {
    delete h;
    return UPCG_ERR_CUDA;
  }
  std::vector<double> gx, gw;
  gauss_legendre(12, gx, gw);
  if (bad(h->glx.ensure(12)) || bad(h->glw.ensure(12)) ||
      bad(mcpy(h->glx.p, gx.data(), 12 * sizeof(double), cudaMemcpyHostToDevice, s)) ||
      bad(mcpy(h->glw.p, gw.data(), 12 * sizeof(double), cudaMemcpyHostToDevice, s)) ||
      bad(cudaStreamSynchronize(s))) {
    delete h;
    return UPCG_ERR_CUDA;
  }
  *out = h;
  return UPCG_OK;
}

int upcg_mlp_destroy(upcg_mlp* h) {
  delete h;
  return UPCG_OK;
}

int upcg_mlp_box(const upcg_mlp* h, float* out, size_t n) {
  if (!h || !out || n < 10) return fail(UPCG_ERR_ARG, "bad argument");
  const MlpBox& b = h->box;
  const float v[10] = {b.lw_lo, b.lw_hi, b.bf_lo, b.lb_hi, b.R_lo, b.R_hi, b.a_lo, b.a_hi, b.g_lo, b.g_hi};
  std::memcpy(out, v, sizeof v);
  return UPCG_OK;
}

int upcg_mlp_make_data(upcg_mlp* h, int64_t n, uint64_t seed) {
  if (!h || n <= 0 || n > (int64_t)1 << 26) return fail(UPCG_ERR_ARG, "bad argument");
  cudaStream_t s = h->st();
  CK(h->xs.ensure((size_t)n * 5));
  CK(h->ys.ensure(n));
  CK(h->ws.ensure(n));
  cudaEvent_t t0, t1;
  cudaEventCreate(&t0);
  cudaEventCreate(&t1);
  cudaEventRecord(t0, s);
  CK(launch_mlp_labels(h->box, seed, 0, (int)n, h->glx.p, h->glw.p, h->xs.p, h->ys.p, h->ws.p, s));
  cudaEventRecord(t1, s);
  CK(cudaEventSynchronize(t1));
  float ms = 0;
  cudaEventElapsedTime(&ms, t0, t1);
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  h->labels_ms = ms;
  h->ndata = n;
  return UPCG_OK;
}

int upcg_mlp_get_data(upcg_mlp* h, int64_t i0, int64_t n, float* x, float* y, float* w) {
  if (!h || i0 < 0 || n < 0 || i0 + n > h->ndata) return fail(UPCG_ERR_ARG, "bad range");
  cudaStream_t s = h->st();
  if (x) CK(mcpy(x, h->xs.p + i0 * 5, (size_t)n * 5 * sizeof(float), cudaMemcpyDeviceToHost, s));
  if (y) CK(mcpy(y, h->ys.p + i0, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost, s));
  if (w) CK(mcpy(w, h->ws.p + i0, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  return UPCG_OK;
}

int upcg_mlp_train(upcg_mlp* h, int epochs, int batch, float lr, double* last_loss) {
  if (!h || epochs < 0 || batch < 16 || h->ndata < batch) return fail(UPCG_ERR_ARG, "bad argument");
  cudaStream_t s = h->st();
  const int np = mlp_param_count();
  const int ctas = (batch + mlp_step_samples() - 1) / mlp_step_samples();
  CK(h->part.ensure((size_t)ctas * np));
  CK(h->lossp.ensure(ctas));
  CK(h->idx.ensure(h->ndata));
  std::vector<int> perm((size_t)h->ndata);
  for (int64_t i = 0; i < h->ndata; ++i) perm[i] = (int)i;
  uint64_t rs = h->seed ^ 0xD1B54A32D192ED03ull;
  auto next = [&]() {
    rs ^= rs << 13;
    rs ^= rs >> 7;
    rs ^= rs << 17;
    return rs;
  };
  const int steps_per_epoch = (int)(h->ndata / batch);
  const int total = epochs * steps_per_epoch;
  cudaEvent_t t0, t1;
  cudaEventCreate(&t0);
  cudaEventCreate(&t1);
  cudaEventRecord(t0, s);
  for (int ep = 0; ep < epochs; ++ep) {
    for (int64_t i = h->ndata - 1; i > 0; --i) std::swap(perm[i], perm[next() % (uint64_t)(i + 1)]);
    CK(mcpy(h->idx.p, perm.data(), h->ndata * sizeof(int), cudaMemcpyHostToDevice, s));
    for (int b = 0; b < steps_per_epoch; ++b) {
      // cosine decay of the step size over the run
      const int k = ep * steps_per_epoch + b;
      const float lrk = lr * 0.5f * (1.f + std::cos(3.14159265f * (float)k / (float)total));
      CK(launch_mlp_step(h->pb.p, h->pf.p, h->xs.p, h->ys.p, h->ws.p, h->idx.p + (size_t)b * batch,
                         batch, 1.f / batch, h->part.p, h->lossp.p, s));
      ++h->step;
      CK(launch_mlp_adam(h->part.p, ctas, h->pf.p, h->pb.p, h->m.p, h->v.p, lrk, h->step, nullptr, s));
    }
  }
  cudaEventRecord(t1, s);
  std::vector<float> lp(ctas);
  CK(mcpy(lp.data(), h->lossp.p, ctas * sizeof(float), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  float ms = 0;
  cudaEventElapsedTime(&ms, t0, t1);
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  h->train_ms = ms;
  if (last_loss) {
    double l = 0;
    for (float v : lp) l += v;
    *last_loss = l;
  }
  return UPCG_OK;
}

int upcg_mlp_gradients(upcg_mlp* h, const float* x, const float* y, const float* w, int n,
                       float* grads, size_t ng, double* loss) {
  const int np = mlp_param_count();
  if (!h || !x || !y || !w || !grads || n <= 0 || ng < (size_t)np)
    return fail(UPCG_ERR_ARG, "bad argument");
  cudaStream_t s = h->st();
  const int ctas = (n + mlp_step_samples() - 1) / mlp_step_samples();
  CK(h->tx.ensure((size_t)n * 5));
  CK(h->ty.ensure(n));
  CK(h->tw.ensure(n));
  CK(h->idx.ensure(std::max<int64_t>(h->ndata, n)));
  CK(h->part.ensure((size_t)ctas * np));
  CK(h->lossp.ensure(ctas));
  CK(h->out.ensure(np));
  std::vector<int> iota(n);
  for (int i = 0; i < n; ++i) iota[i] = i;
  CK(mcpy(h->tx.p, x, (size_t)n * 5 * sizeof(float), cudaMemcpyHostToDevice, s));
  CK(mcpy(h->ty.p, y, (size_t)n * sizeof(float), cudaMemcpyHostToDevice, s));
  CK(mcpy(h->tw.p, w, (size_t)n * sizeof(float), cudaMemcpyHostToDevice, s));
  CK(mcpy(h->idx.p, iota.data(), (size_t)n * sizeof(int), cudaMemcpyHostToDevice, s));
  CK(launch_mlp_step(h->pb.p, h->pf.p, h->tx.p, h->ty.p, h->tw.p, h->idx.p, n, 1.f / n, h->part.p,
                     h->lossp.p, s));
  CK(launch_mlp_adam(h->part.p, ctas, h->pf.p, h->pb.p, h->m.p, h->v.p, 0.f, 1, h->out.p, s));
  CK(mcpy(grads, h->out.p, np * sizeof(float), cudaMemcpyDeviceToHost, s));
  std::vector<float> lp(ctas);
  CK(mcpy(lp.data(), h->lossp.p, ctas * sizeof(float), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (loss) {
    double l = 0;
    for (float v : lp) l += v;
    *loss = l;
  }
  return UPCG_OK;
}

int upcg_mlp_params(upcg_mlp* h, float* out, size_t n) {
  const int np = mlp_param_count();
  if (!h || !out || n < (size_t)np) return fail(UPCG_ERR_ARG, "bad argument");
  CK(mcpy(out, h->pf.p, np * sizeof(float), cudaMemcpyDeviceToHost, h->st()));
  CK(cudaStreamSynchronize(h->st()));
  return UPCG_OK;
}

int upcg_mlp_set_params(upcg_mlp* h, const float* in, size_t n) {
  const int np = mlp_param_count();
  if (!h || !in || n != (size_t)np) return fail(UPCG_ERR_ARG, "bad argument");
  cudaStream_t s = h->st();
  CK(mcpy(h->pf.p, in, np * sizeof(float), cudaMemcpyHostToDevice, s));
  CK(launch_mlp_to_bf16(h->pf.p, h->pb.p, s));
  CK(cudaStreamSynchronize(s));
  return UPCG_OK;
}

int upcg_mlp_predict(upcg_mlp* h, const float* x, int n, float* y) {
  if (!h || !x || !y || n <= 0) return fail(UPCG_ERR_ARG, "bad argument");
  cudaStream_t s = h->st();
  CK(h->tx.ensure((size_t)n * 5));
  CK(h->out.ensure(std::max(n, mlp_param_count())));
  CK(mcpy(h->tx.p, x, (size_t)n * 5 * sizeof(float), cudaMemcpyHostToDevice, s));
  CK(launch_mlp_infer(h->pb.p, h->pf.p, h->tx.p, n, h->out.p, s));
  CK(mcpy(y, h->out.p, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  return UPCG_OK;
}

int upcg_mlp_timings(const upcg_mlp* h, double* labels_ms, double* train_ms) {
  if (!h) return fail(UPCG_ERR_ARG, "null handle");
  if (labels_ms) *labels_ms = h->labels_ms;
  if (train_ms) *train_ms = h->train_ms;
  return UPCG_OK;
}

int upcg_scan_create(upcg_scan** out, upcg_generator* const* gens, int n) {
  if (!out || !gens || n <= 0) return fail(UPCG_ERR_ARG, "bad argument");
  for (int i = 0; i < n; ++i)
    if (!gens[i]) return fail(UPCG_ERR_ARG, "null generator %d", i);
  upcg_scan* sc = new (std::nothrow) upcg_scan();
  if (!sc) return fail(UPCG_ERR_NOMEM, "out of host memory");
  sc->gens.assign(gens, gens + n);
  *out = sc;
  return UPCG_OK;
}

int upcg_scan_destroy(upcg_scan* sc) {
  delete sc;
  return UPCG_OK;
}

namespace {
int scan_setup(upcg_scan* sc) {
  const int n = (int)sc->gens.size();
  const auto t0 = std::chrono::steady_clock::now();
  CK(cudaStreamCreateWithFlags(&sc->s, cudaStreamNonBlocking));
  sc->P = fast_grid_points();
  const int P = sc->P;
  // one ordinary initialisation per configuration: allocations, static
  // uploads, checks; the generators then run on the scan's stream
  sc->row0.assign(n, 0);
  sc->rows.assign(n, 0);
  int64_t rows_total = 0;
  for (int i = 0; i < n; ++i) {
    upcg_generator* g = sc->gens[i];
    g->lumiMethod = 1;
    g->row_lo = 0;
    g->row_hi = -1;
    g->stream = sc->s;
    g->invalidate();
    int rc = upcg_init(g);
    if (rc) return rc;
    if (g->usePolarizedCS) return fail(UPCG_ERR_PROCESS, "scan: polarized configuration %d", i);
    // its rows: one cell of each mirror-rapidity pair (the map upcg_init made)
    const int ncell = g->nm * (g->fast_nrep > 0 ? g->fast_nrep : g->ny);
    CK(g->fsides.ensure((2 * (size_t)ncell * fast_side_bytes() + 7) / 8));
    sc->row0[i] = (int)rows_total;
    sc->rows[i] = (ncell + 127) / 128 * 128;
    rows_total += sc->rows[i];
  }
  if (rows_total > (int64_t)1 << 30) return fail(UPCG_ERR_SIZE, "scan too large");
  // table sharing: the form factor depends on (A, R, a), G_AA also on sqrt(s)
  // (sigma_NN), the breakup spline on (sqrt(s), mode)
  {
    std::map<std::tuple<int, double, double>, upcg_generator*> ffk;
    std::map<std::tuple<int, double, double, double>, upcg_generator*> gaak;
    std::map<std::pair<double, int>, upcg_generator*> brkk;
    for (upcg_generator* g : sc->gens) {
      const auto kf = std::make_tuple(g->A, g->R, g->a);
      const auto kg = std::make_tuple(g->A, g->R, g->a, g->sqrts);
      const auto kb = std::make_pair(g->sqrts, g->breakupMode);
      auto f = ffk.find(kf);
      g->ff_donor = f == ffk.end() ? nullptr : f->second;
      if (f == ffk.end()) ffk[kf] = g;
      auto q = gaak.find(kg);
      g->gaa_donor = q == gaak.end() ? nullptr : q->second;
      if (q == gaak.end()) gaak[kg] = g;
      auto b = brkk.find(kb);
      g->brk_donor = b == brkk.end() ? nullptr : b->second;
      if (b == brkk.end()) brkk[kb] = g;
    }
  }
  sc->rows_total = (int)rows_total;
  const size_t plane = (size_t)P * P;
  CK(sc->ah.ensure((size_t)rows_total * P));
  CK(sc->al.ensure((size_t)rows_total * P));
  CK(sc->a2.ensure((size_t)rows_total * P));
  CK(sc->part.ensure((size_t)rows_total * (P / 128)));
  CK(sc->far.ensure(4 * (size_t)rows_total));
  CK(sc->gh.ensure(n * plane));
  CK(sc->gl.ensure(n * plane));
  CK(sc->fc.ensure(2 * (size_t)n));
  CK(sc->err.ensure(1));
  // tile shape from the autotuner, then the work list: per configuration its
  // row tiles, the N tiles of a row tile adjacent (L2 reuse of A)
  int rc = contract_plan(std::min(sc->rows_total, 131072), sc->rows_total, P, &sc->shape,
                         &sc->grid, 0);
  if (rc) return rc;
  const int tbn = sc->shape == 0 ? 256 : 128;
  // the K tiles where the delta survival kernels can be nonzero (the same
  // radial grid and azimuths for every configuration)
  std::vector<std::pair<int, int>> kr;
  {
    const double fu0 = std::log(0.1), fh = (std::log(256.) - std::log(0.1)) / (P - 1);
    kr = sc->gens[0]->delta_ranges(P, fu0, fh, tbn, sc->gens[0]->lumi_params(), false);
  }
  std::vector<int4> items;
  for (int i = 0; i < n; ++i) {
    const upcg_generator* g = sc->gens[i];
    const int ncell = g->nm * (g->fast_nrep > 0 ? g->fast_nrep : g->ny);
    for (int mt = 0; mt < sc->rows[i] / 128; ++mt)
      for (int nt = 0; nt < P / tbn; ++nt)
        items.push_back(make_int4(sc->row0[i] / 128 + mt, nt, i,
                                  pack_item(std::min(128, ncell - mt * 128), kr[nt].first,
                                            kr[nt].second)));
  }
  sc->nitems = (int)items.size();
  // the first nonzero K tile of any configuration (the smallest b_min)
  int kt0 = P / kContractBK;
  {
    const double fu0 = std::log(0.1), fh = (std::log(256.) - std::log(0.1)) / (P - 1);
    for (const upcg_generator* g : sc->gens)
      kt0 = std::min(kt0, fast_first_ktile(g->isPoint ? g->R : 0.05 * g->R, fu0, fh));
  }
  // items of unequal work: every CTA meets every N tile
  sc->grid = std::min(sc->grid, (int)items.size());
  rotate_rounds(items, sc->grid);
  CK(sc->items.ensure(items.size()));
  CK(mcpy(sc->items.p, items.data(), items.size() * sizeof(int4), cudaMemcpyHostToDevice, sc->s));
  CK(cudaStreamSynchronize(sc->s));
  // capture the whole scan
  CK(cudaStreamBeginCapture(sc->s, cudaStreamCaptureModeThreadLocal));
  auto abort_capture = [&](int code) {
    cudaGraph_t gph = nullptr;
    cudaStreamEndCapture(sc->s, &gph);
    if (gph) cudaGraphDestroy(gph);
    return code;
  };
  if (cudaMemsetAsync(sc->err.p, 0, sizeof(unsigned), sc->s) != cudaSuccess)
    return abort_capture(fail(UPCG_ERR_CUDA, "scan: capture of the error word failed"));
  for (int i = 0; i < n; ++i) {
    rc = sc->gens[i]->enqueue_scan_front(*sc, i);
    if (rc) return abort_capture(rc);
  }
  if (launch_contract_pers(sc->ah.p, sc->al.p, sc->gh.p, sc->gl.p, n, sc->rows_total, P,
                           sc->items.p, sc->nitems, sc->a2.p, sc->part.p, sc->err.p, sc->shape,
                           sc->grid, sc->s, nullptr, kt0) != cudaSuccess)
    return abort_capture(fail(UPCG_ERR_CUDA, "scan: contraction capture failed"));
  for (int i = 0; i < n; ++i) {
    rc = sc->gens[i]->enqueue_scan_back(*sc, i);
    if (rc) return abort_capture(rc);
  }
  CK(cudaStreamEndCapture(sc->s, &sc->graph));
  CK(cudaGraphInstantiate(&sc->exec, sc->graph, 0));
  sc->setup_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return UPCG_OK;
}
}  // namespace

int upcg_scan_run(upcg_scan* sc, double* ms) {
  if (!sc) return fail(UPCG_ERR_ARG, "null handle");
  if (!sc->exec) {
    const int rc = scan_setup(sc);
    if (rc) return rc;
  }
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, sc->s);
  CK(cudaGraphLaunch(sc->exec, sc->s));
  cudaEventRecord(e1, sc->s);
  CK(cudaEventSynchronize(e1));
  float t = 0;
  cudaEventElapsedTime(&t, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  sc->run_ms = t;
  if (ms) *ms = t;
  unsigned herr = 0;
  CK(mcpy_sync(&herr, sc->err.p, sizeof herr, cudaMemcpyDeviceToHost));
  if (herr) return fail(UPCG_ERR_CUDA, "scan contraction timed out (code %u)", herr);
  for (upcg_generator* g : sc->gens) {
    CK(mcpy_sync(&g->totCS, g->tot.p, sizeof(double), cudaMemcpyDeviceToHost));
    g->fidCS = g->totCS;
    g->next_cand = 0;
    g->ev_batch.clear();
    g->ev_flag.clear();
    g->ev_pos = 0;
    g->tables_ready = g->lumi_ready = g->xsec_ready = true;
  }
  return UPCG_OK;
}

int upcg_scan_info(const upcg_scan* sc, int* nitems, int* shape, int* rows_total, double* setup_ms) {
  if (!sc) return fail(UPCG_ERR_ARG, "null handle");
  if (nitems) *nitems = sc->nitems;
  if (shape) *shape = sc->shape;
  if (rows_total) *rows_total = sc->rows_total;
  if (setup_ms) *setup_ms = sc->setup_ms;
  return UPCG_OK;
}

int upcg_set_flux_surrogate(upcg_generator* g, upcg_mlp* h) {
  if (!g) return fail(UPCG_ERR_ARG, "null handle");
  g->surrogate = h;
  if (g->lumiMethod == 4) g->invalidate();
  return UPCG_OK;
}

int upcg_surrogate_rows(const upcg_generator* g, int* rows) {
  if (!g || !rows) return fail(UPCG_ERR_ARG, "null argument");
  *rows = g->surrogate_rows;
  return UPCG_OK;
}

const char* upcg_version(void) { return "upcgen-gb300 0.1 (sm_103a)"; }

}  // extern "C"
