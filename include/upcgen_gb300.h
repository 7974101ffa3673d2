/* upcgen-gb300 -- C ABI of the GB300 two-photon luminosity / nuclear cross
 * section / event-sampling library.
 *
 * Drop-in boundary for upcgen's UpcGenerator / UpcCrossSection path.  The
 * reference exposes a C++ class API (include/UpcGenerator.h:55-128,
 * include/UpcCrossSection.h:65-240, built as the Upcgenlib library by
 * CMakeLists.txt:83-91); every entry point below names the method it
 * replaces.  A header-only C++ facade with the reference's class and method
 * names sits on top of this ABI in include/upcgen_gb300.hpp.
 *
 * Conventions
 *   - every function returns an int status (UPCG_OK = 0, negative on error)
 *     and never exits or aborts; upcg_last_error() gives a message;
 *   - the caller owns every buffer passed in; the handle owns device memory;
 *   - pointers are host pointers unless the name ends in _device;
 *   - a handle is bound to one CUDA stream (upcg_set_stream); distinct handles
 *     may be used from distinct threads.
 */
#ifndef UPCGEN_GB300_H_
#define UPCGEN_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define UPCG_OK 0
#define UPCG_ERR_ARG (-1)       /* bad argument / unknown value */
#define UPCG_ERR_CUDA (-2)      /* CUDA error (message in upcg_last_error) */
#define UPCG_ERR_STATE (-3)     /* call out of order (e.g. before upcg_init) */
#define UPCG_ERR_PROCESS (-4)   /* PROC_ID outside this path */
#define UPCG_ERR_NUMERIC (-5)   /* QAGS failure the reference would abort on */
#define UPCG_ERR_NOMEM (-6)
#define UPCG_ERR_SIZE (-7)      /* output buffer too small */
#define UPCG_ERR_IO (-8)        /* file could not be opened or written */

typedef struct upcg_generator upcg_generator;

/* One accepted event, 48 bytes: pair mass / rapidity / cos(theta), charge
 * sign of particle 0 (+1/-1; +1 for neutral products), then px,py,pz,E of the
 * two final-state particles (leptons; the two photons for an ALP). */
typedef struct upcg_event {
  float m, y, z, sign;
  float p0[4];
  float p1[4];
} upcg_event;

/* ---- life cycle / configuration (UpcGenerator) ------------------------ */
/* UpcGenerator::UpcGenerator, src/UpcGenerator.cpp:30-40 (Pb-Pb at 5020 GeV) */
int upcg_create(upcg_generator** out);
/* UpcGenerator::~UpcGenerator, src/UpcGenerator.cpp:42-55 */
int upcg_destroy(upcg_generator* g);
/* UpcGenerator::setParameterValue, src/UpcGenerator.cpp:183-305; parameters.in
 * keys; keys of other paths (PYTHIA_*, USE_*_OUTPUT, SHADOWING, ...) are
 * accepted and ignored as the reference ignores unknown keys */
int upcg_set_parameter(upcg_generator* g, const char* key, const char* value);
/* UpcGenerator::setParFile + configGeneratorFromFile, src/UpcGenerator.cpp:318-346 */
int upcg_config_from_file(upcg_generator* g, const char* path);
/* UpcGenerator::setCollisionSystem, src/UpcGenerator.cpp:307-316 */
int upcg_set_collision_system(upcg_generator* g, float sqrts, int nucl_z, int nucl_a);
/* UpcGenerator::setSeed, include/UpcGenerator.h:104-113 */
int upcg_set_seed(upcg_generator* g, long seed);
/* UpcGenerator::setNumThreads, include/UpcGenerator.h:95 (accepted; the GPU
 * path does not use host threads) */
int upcg_set_num_threads(upcg_generator* g, int n);
/* UpcGenerator::setDebugLevel, include/UpcGenerator.h:92 */
int upcg_set_debug_level(upcg_generator* g, int level);
/* UpcGenerator::setLumiFileDirectory, include/UpcGenerator.h:87: directory
 * of the luminosity cache (see upcg_set_lumi_cache) */
int upcg_set_lumi_file_directory(upcg_generator* g, const char* dir);
/* 1: reuse / write a luminosity cache keyed by a hash of every input of the
 * table (the reference's twoPhotonLumi.root is keyed by nothing,
 * src/UpcCrossSection.cpp:481-491); 0 (default): always compute */
int upcg_set_lumi_cache(upcg_generator* g, int enable);
/* The cache file of the current configuration (no counterpart in the
 * reference, whose file is always twoPhotonLumi[Pol].root,
 * src/UpcCrossSection.cpp:481-482): "<dir>/upcg_lumi_<16 hex>.bin", the hex
 * digits a 64-bit FNV-1a hash of a key text naming every input of the table.
 * last_hit (optional): 1 if the last upcg_init read the table from it, 0 if it
 * computed the table, -1 if the cache was not used.  Host only. */
int upcg_lumi_cache_file(upcg_generator* g, char* path, size_t len, int* last_hit);
/* CUDA stream (cudaStream_t) for every launch of this handle; NULL = the
 * handle's own stream.  upcg_init forks its work from this stream onto the
 * handle's internal streams (one of high priority for its main chain, side
 * streams for the table chains and samplers) and joins them back into it
 * before it returns: work queued on the stream before upcg_init precedes
 * init's, and init's completes before anything queued after it. */
int upcg_set_stream(upcg_generator* g, void* stream);
/* Luminosity method: 0 = plain FP64 (default; the reference's quadrature),
 * 1 = fast form (flux tables + tensor-core contraction, <= 1e-4 relative to
 * the converged quadrature), 2 = the fast form's contraction on the plain
 * path's node fluxes (diagnostic), 3 = grid form (point flux): fixed
 * 4096-energy x 2048-radius grids, L = N G N^T as two tensor-core products
 * (its own quadrature: the difference to the reference is stated by the tests)
 * in the three-term bf16 split, 7 = the same grid form with TF32 products
 * (tcgen05 kind::tf32, one product per k step),
 * 4 = the fast form with the form-factor flux rows inside the learned
 * surrogate's box from the surrogate (upcg_set_flux_surrogate).  Methods 5
 * and 6 are the fast form with other operand paths, for comparison: 1, 2 and
 * 4 write both contraction operands dense on the radial grid (A1 read by
 * TMA, A2 by the epilogue); 5 writes the dense A1 rows and side 1's node
 * lists (the epilogue gathers the A2 row-dot at the node stencils); 6 writes
 * node lists only and builds A1 in the contraction's shared memory.  All
 * three give the same table up to FP32 summation order.  With USE_POLARIZED_CS the fast form (1,
 * 4, 5, 6) builds the scalar and pseudoscalar tables of calcTwoPhotonLumiPol
 * from the same operands. */
int upcg_set_lumi_method(upcg_generator* g, int method);

/* ---- initialisation (UpcGenerator::init) ------------------------------ */
/* UpcGenerator::init, src/UpcGenerator.cpp:57-181: process overrides, nuclear
 * tables (UpcCrossSection::init :116-137), two-photon luminosity
 * (prepareTwoPhotonLumi :463-592), nuclear cross section and samplers
 * (computeNuclXsection :630-713) */
int upcg_init(upcg_generator* g);
/* UpcGenerator::computeNuclXsection, src/UpcGenerator.cpp:630-713 (re-run the
 * fold and sampler set-up on the current luminosity) */
int upcg_compute_nucl_xsection(upcg_generator* g);
/* UpcGenerator::totNuclX / fidNuclX, include/UpcGenerator.h:120-121 (mb) */
int upcg_tot_nucl_x(const upcg_generator* g, double* mb);
int upcg_fid_nucl_x(const upcg_generator* g, double* mb);
/* effective grid after the process overrides of UpcGenerator::init */
int upcg_get_grid(const upcg_generator* g, double* mmin, double* mmax, int* nm,
                  double* ymin, double* ymax, int* ny, double* zmin, double* zmax,
                  int* nz);

/* ---- sharding (no counterpart in the reference; the reference's OpenMP
 * m-slices of prepareTwoPhotonLumi, src/UpcCrossSection.cpp:537-538, across
 * processes) ------------------------------------------------------------- */
/* compute only the luminosity m-rows [im0, im1) in upcg_init (im1 = -1: to the
 * end); the other rows stay zero */
int upcg_set_row_range(upcg_generator* g, int im0, int im1);
/* install a full luminosity table (as upcg_lumi_table returns it; the
 * pseudoscalar one in table2 when polarized) and build the cross section and
 * samplers from it (upcg_compute_nucl_xsection) */
int upcg_set_lumi_table(upcg_generator* g, const double* table, size_t n, const double* table2);
/* the same from device memory of the handle's GPU (a table all-gathered
 * on the device); the copies run on the handle's stream, which is
 * synchronised before the call returns */
int upcg_set_lumi_table_device(upcg_generator* g, const double* table_device, size_t n,
                               const double* table2_device);
/* start the candidate sequence of the event entries at this Philox counter
 * (after upcg_init, which resets it to 0): disjoint ranges per shard */
int upcg_set_candidate_offset(upcg_generator* g, uint64_t counter);
/* the Philox counter the next event entry starts at */
int upcg_get_candidate_offset(const upcg_generator* g, uint64_t* counter);

/* ---- tables ------------------------------------------------------------ */
/* hD2LDMDY of prepareTwoPhotonLumi (src/UpcCrossSection.cpp:506-571):
 * out[im*ny + iy] = L(m_im, y_iy) dm dy (bin (im+1, iy+1)); polarized:
 * hD2LDMDY_s into out, hD2LDMDY_p into out2 (may be NULL otherwise) */
int upcg_lumi_table(upcg_generator* g, double* out, size_t n, double* out2);
int upcg_lumi_table_device(upcg_generator* g, const double** out, const double** out2);
/* nucCSYM of calcNucCrossSectionYM (src/UpcCrossSection.cpp:594-698):
 * out[iy*nm + im] (nb) and its total (mb) */
int upcg_nuc_cs_ym(upcg_generator* g, double* out, size_t n, double* tot_mb);
/* fillCrossSectionZM (src/UpcCrossSection.cpp:337-362), flag 0/1/2:
 * out[im*nz + iz] */
int upcg_cs_zm_table(upcg_generator* g, int flag, double* out, size_t n);

/* ---- point evaluations (UpcCrossSection methods, batched, on the GPU) ---- */
/* fluxPoint, src/UpcCrossSection.cpp:166-178 */
int upcg_flux_point(upcg_generator* g, const double* b, const double* k, double* out, size_t n);
/* fluxForm, src/UpcCrossSection.cpp:194-218 (QAGS on the device) */
int upcg_flux_form(upcg_generator* g, const double* b, const double* k, double* out, size_t n);
/* No counterpart in the reference.  upcg_flux_form on DEVICE buffers without
 * any device-memory allocation: for callers that may not allocate once they
 * run -- applications whose memory pool takes all of HBM at start-up, where a
 * driver allocation later fails or forces the pool to give memory back, and
 * hosts that grant a library a fixed device budget at start and forbid
 * cudaMalloc afterwards.
 * The QAGS scratch lives in 2.6 MB of static device memory of the library
 * (64 warp workspaces and one statistics word); nothing is allocated here.
 *   - n <= UPCG_NOALLOC_MAX_POINTS, else UPCG_ERR_SIZE;
 *   - needs the tables of a completed upcg_init (else UPCG_ERR_STATE);
 *   - the call clears the statistics word itself (cudaMemsetAsync on the
 *     handle's stream); the workspaces need no clearing;
 *   - asynchronous on the handle's stream; failures_device (device, may be
 *     NULL) receives the number of points whose QAGS returned a non-zero
 *     status (the reference aborts there);
 *   - the first call on a device looks up the scratch address
 *     (cudaGetSymbolAddress) and should come before any stream capture;
 *   - the scratch is shared by all handles: calls that overlap in time (two
 *     streams or two host threads) race on it and must be serialised. */
#define UPCG_NOALLOC_MAX_POINTS 16777216
int upcg_flux_form_device_noalloc(upcg_generator* g, const double* b_device,
                                  const double* k_device, double* out_device, size_t n,
                                  uint32_t* failures_device);
/* calcFormFac, src/UpcCrossSection.cpp:436-445 */
int upcg_form_factor(upcg_generator* g, const double* q2, double* out, size_t n);
/* calcBreakupProb, src/UpcCrossSection.cpp:752-1019 */
int upcg_breakup_prob(upcg_generator* g, const double* b, int mode, double* out, size_t n);
/* the splines gslSplineGAA / gslSplineBreakP / gslSplineFormFac
 * (src/UpcCrossSection.cpp:411-413, 431-433, 458-460): which = 0/1/2 */
int upcg_eval_spline(upcg_generator* g, int which, const double* x, double* out, size_t n);
/* calcTwoPhotonLumi, src/UpcCrossSection.cpp:221-271 (out2 == NULL), or
 * calcTwoPhotonLumiPol :274-335 (scalar into out, pseudoscalar into out2) */
int upcg_two_photon_lumi(upcg_generator* g, const double* m, const double* y, double* out,
                         double* out2, size_t n);
/* UpcElemProcess::calcCrossSectionM / MPolS / MPolPS of the configured
 * process (flag 0/1/2), src/UpcTwoPhotonDilep.cpp:46-122, src/UpcTwoPhotonALP.cpp:28-33 */
int upcg_cs_m(upcg_generator* g, const double* m, int flag, double* out, size_t n);

/* PDG code of the final-state particles of the configured process and
 * whether they are charged (UpcGenerator::init, src/UpcGenerator.cpp:66-140):
 * the lepton for PROC_ID 11/13/15, 51 for the ALP (its decay photons are 22) */
int upcg_particle_pdg(upcg_generator* g, int* pdg, int* charged);

/* ---- events (UpcGenerator::generateEvents) ------------------------------ */
/* The event loop of src/UpcGenerator.cpp:834-889: the first n accepted events
 * of the candidate sequence; *rejected = candidates rejected by the cuts
 * before the n-th accepted one; updates fidNuclX.  mbin (may be NULL) gets
 * UpcSampler2D::getBinY of each event's mass (include/UpcSampler.h:130-133). */
int upcg_generate_events(upcg_generator* g, int64_t n, upcg_event* out, int32_t* mbin,
                         int64_t* rejected);
int upcg_generate_events_device(upcg_generator* g, int64_t n, upcg_event* out_device,
                                int32_t* mbin_device, int64_t* rejected);
/* Page-locked host memory for event buffers (the caller owns it; free with
 * upcg_host_free): upcg_generate_events into such a buffer copies at the
 * link's rate instead of through the driver's pageable staging. */
int upcg_host_alloc(size_t bytes, void** out);
int upcg_host_free(void* p);
/* ---- photonuclear path: coherent vector mesons (PROC_ID 443 J/psi, 100443
 * psi(2S), 553 Upsilon(1S); DECAY_PDG 11, 13 or 2212; SHADOWING 0, the
 * impulse approximation -- the other options need the reference's
 * nuclear-shadowing tables and return UPCG_ERR_PROCESS).  upcg_init builds
 * calcNucCrossSectionY's dsigma/dy on the y-bins (one mass bin at m_V) and
 * the samplers of generateEvent's vector-meson branch. ---------------------
 * calcPhotonFlux, src/UpcCrossSection.cpp:700-722: the photon flux of one
 * nucleus integrated over b with the survival factors, at n (m, y) points */
int upcg_photon_flux(upcg_generator* g, const double* m, const double* y, double* out, size_t n);
/* UpcPhotoNuclearVM::calcCrossSectionY, src/UpcPhotoNuclearVM.cpp:340-381
 * (impulse approximation), at n rapidities */
int upcg_vm_cross_section_y(upcg_generator* g, const double* y, double* out, size_t n);
/* calcNucCrossSectionY, src/UpcCrossSection.cpp:724-748: dsigma/dy [ny] at
 * the left y-edges, the emitter ratio [ny] (optional) and sigma_tot (mb) */
int upcg_nuc_cs_y(upcg_generator* g, double* cs, double* ratio, size_t ny, double* tot_mb);
/* PDG code of the decay products of the configured process: DECAY_PDG for a
 * vector meson, 22 for the ALP, 0 for a lepton pair */
int upcg_decay_pdg(upcg_generator* g, int* pdg);

/* ---- event output (UpcGenerator::writeEvent / generateEvents' files,
 * src/UpcGenerator.cpp:589-628, 834-926) ----------------------------------
 * Particles per event as generateEvent lists them (:767-812): a lepton pair
 * is 2 (pdg +-PDG, status 23, mother 0), an ALP 3 (the ALP: pdg 51, status
 * 23, mother 0, momentum = the photons' sum; two photons: pdg 22, status 33,
 * mother 1). */
int upcg_particles_per_event(upcg_generator* g, int* n);
/* NEVENTS, USE_ROOT_OUTPUT and USE_HEPMC_OUTPUT as configured: the event
 * count and the files of the reference's generateEvents() (src/UpcGenerator.cpp:
 * 185-187, 284-289, 834-926) */
int upcg_event_output_config(const upcg_generator* g, int64_t* nevents, int* use_root,
                             int* use_hepmc);
/* Columns of the reference's ROOT tree "particles" (:842-853), one row per
 * particle, row = event * particles_per_event + (particleID - 1). */
typedef struct upcg_particle_columns {
  int32_t* eventNumber;
  int32_t* pdgCode;
  int32_t* particleID;
  int32_t* statusID;
  int32_t* motherID;
  double* px;
  double* py;
  double* pz;
  double* e;
} upcg_particle_columns;
/* Device records -> device columns (every pointer device memory), eventNumber
 * = first_event + index; one kernel on the handle's stream. */
int upcg_event_particles_device(upcg_generator* g, const upcg_event* ev_device, int64_t n,
                                int64_t first_event, const upcg_particle_columns* cols);
/* HepMC3 ASCII of n host records as WriterHepMC writes them
 * (include/UpcGenerator.h:192-242): "E", "U GEV MM" and "P" lines, numbers
 * as setprecision(9); without the version / listing lines.  *len = the text's
 * size; UPCG_ERR_SIZE when out is NULL or cap is smaller.  Host only. */
int upcg_format_hepmc3(upcg_generator* g, const upcg_event* ev, int64_t n, int64_t first_event,
                       char* out, size_t cap, size_t* len);
/* generateEvents with file output: the next n accepted events to path.
 * format 0: HepMC3 ASCII (the reference's events.hepmc, complete with the
 * version and listing lines); 1: the particle columns (the reference's
 * events.root tree) in a column file, converted to ROOT by
 * upcgen_gb300/particles_to_root.C.  threads: host formatting threads
 * (0 = every core).  Device generation of the next batch overlaps the file
 * work of the current one.  Sets fidNuclX over the n events. */
int upcg_write_events(upcg_generator* g, const char* path, int64_t n, int format, int threads,
                      int64_t* rejected);
/* The loop of the reference's generateEvents() with no file configured
 * (USE_ROOT_OUTPUT 0 and USE_HEPMC_OUTPUT 0, src/UpcGenerator.cpp:866-889):
 * the next n accepted events are drawn on the device and dropped, so that the
 * candidate sequence advances, *rejected counts the rejected candidates and
 * fidNuclX = totNuclX n / (n + rejected), as after the reference's loop. */
int upcg_run_events(upcg_generator* g, int64_t n, int64_t* rejected);

/* UpcGenerator::generateEvent, src/UpcGenerator.cpp:715-832: one candidate.
 * Returns 1 (accepted) or 0 (rejected by the cuts) in *accepted and the
 * event in *ev; candidates are drawn from the same sequence as
 * upcg_generate_events. */
int upcg_generate_event(upcg_generator* g, upcg_event* ev, int* accepted);
/* The event kernels' bin functions on given values, as the sampler of
 * include/UpcSampler.h:124-134 computes them: axis 0 = getBinY of the
 * (y, m) sampler for masses x (the z sampler and the polarized ratio are
 * picked with it), axis 1 = getBinX for rapidities x (the polarized pick);
 * out[i] = the bin, clamped to the grid.  Needs upcg_init. */
int upcg_sampler_bins(upcg_generator* g, const double* x, size_t n, int axis, int32_t* out);

/* ---- batched scans (no counterpart in the reference: one configuration per
 * process there) ----------------------------------------------------------
 * A scan builds the tables of n configurations (each a handle with its
 * parameters set) with the fast form: per configuration the nuclear tables,
 * its survival kernel and projection; ONE persistent tensor-core contraction
 * over every configuration's tiles (uneven grid sizes in one work list; the
 * tile shape picked by the library's autotuner); then per configuration the
 * cross section and samplers.  The first upcg_scan_run initialises every
 * handle, captures the whole sequence into a CUDA graph and replays it;
 * later runs replay the graph.  After a run each handle is ready for events.
 * The handles must outlive the scan and run on its stream from then on. */
typedef struct upcg_scan upcg_scan;
int upcg_scan_create(upcg_scan** out, upcg_generator* const* gens, int n);
int upcg_scan_run(upcg_scan* sc, double* ms);
int upcg_scan_info(const upcg_scan* sc, int* nitems, int* shape, int* rows_total, double* setup_ms);
int upcg_scan_destroy(upcg_scan* sc);

/* ---- learned flux surrogate (no counterpart in the reference) -------------
 * An MLP (inputs ln w, ln b, R, a, ln g; four hidden layers of 128 SiLU; BF16
 * weights, FP32 accumulation) for y = ln(Q_ff / Q_pt), the log-ratio of
 * fluxForm's form-factor amplitude (src/UpcCrossSection.cpp:181-218) to the
 * point-charge one, trained on the GPU by the library's own forward, backward
 * and Adam kernels on points labelled by the form-factor quadrature.
 * Training box: w in [1e-3, 1e2] GeV, b in [0.049 R, 500] fm, R in [5, 7.5]
 * fm, a in [0.40, 0.60] fm, g in [100, 3000].  Inputs x are normalised to
 * [-1, 1] over the box (upcg_mlp_box gives its bounds). */
typedef struct upcg_mlp upcg_mlp;
int upcg_mlp_create(upcg_mlp** out, uint64_t seed);
int upcg_mlp_destroy(upcg_mlp* h);
/* {ln w lo, ln w hi, b lo / R, ln b hi, R lo, R hi, a lo, a hi, g lo, g hi} */
int upcg_mlp_box(const upcg_mlp* h, float* out, size_t n);
/* n training points and labels on the device (weights 0 where k b / hc > 30) */
int upcg_mlp_make_data(upcg_mlp* h, int64_t n, uint64_t seed);
int upcg_mlp_get_data(upcg_mlp* h, int64_t i0, int64_t n, float* x, float* y, float* w);
/* Adam over the points: epochs x (n / batch) steps, cosine-decayed step size;
 * last_loss = weighted mean squared error of the last batch */
int upcg_mlp_train(upcg_mlp* h, int epochs, int batch, float lr, double* last_loss);
/* gradient of sum_i w_i (y(x_i) - y_i)^2 / n at the current parameters (no
 * update): grads[upcg_mlp parameter count] */
int upcg_mlp_gradients(upcg_mlp* h, const float* x, const float* y, const float* w, int n,
                       float* grads, size_t ng, double* loss);
/* FP32 master parameters: W1[128][5] b1 W2[128][128] b2 W3 b3 W4 b4 W5[128] b5 */
int upcg_mlp_params(upcg_mlp* h, float* out, size_t n);
int upcg_mlp_set_params(upcg_mlp* h, const float* in, size_t n);
int upcg_mlp_predict(upcg_mlp* h, const float* x, int n, float* y);
int upcg_mlp_timings(const upcg_mlp* h, double* labels_ms, double* train_ms);
/* luminosity method 4: the fast form with the Q(w, b) table rows inside the
 * surrogate's box from the MLP, the rest from the quadrature; the handle keeps
 * the pointer (the surrogate must outlive its use) */
int upcg_set_flux_surrogate(upcg_generator* g, upcg_mlp* h);
int upcg_surrogate_rows(const upcg_generator* g, int* rows);

/* ---- diagnostics --------------------------------------------------------- */
/* Philox4x32-10 uniforms of the event stream (seed, counter) -- for tests */
int upcg_philox(uint64_t seed, uint64_t counter0, size_t n, uint32_t* out4);
/* The tensor-core contraction of the fast form on random data (ncells x P
 * operands, P a multiple of 256) against an FP64 contraction of the same
 * bf16 hi/lo values: max relative error per cell (negative: the kernel's
 * error word) and the contraction time in ms -- for tests */
int upcg_selftest_contract(int ncells, int P, uint64_t seed, double* max_rel, double* ms);
/* The fast form's form-factor flux amplitude table Q[512][256] on
 * (ln w, ln b) and its grid {ln w0, h_w, ln b0, h_b} -- for tests */
int upcg_fast_flux_table(upcg_generator* g, double* out, size_t n, double* grid);
/* timings of the last upcg_init phases (ms): [0] tables [1] luminosity
 * [2] cross section + samplers [3] nodes [4] QAGS [5] band quadrature or
 * tensor-core contraction [6] fast-form projection + kernel build [7] of
 * which the flux tables (quadrature and surrogate rows) */
int upcg_last_timings(const upcg_generator* g, double* ms, size_t n);
int upcg_qags_stats(const upcg_generator* g, uint64_t* failures, uint64_t* max_intervals,
                    uint64_t* evals);
/* kernels launched by the library in this process so far (all handles) */
int upcg_kernel_launches(uint64_t* n);
/* host-to-device and device-to-host bytes the library has copied in this
 * process so far (all handles) */
int upcg_copy_bytes(uint64_t* h2d, uint64_t* d2h);
/* Rows of the last fast-form luminosity's contraction: the cells computed,
 * one of each pair of mirror rapidities (L(m, -y) = L(m, y), copied to the
 * other); 0 when the last luminosity was not the fast form */
int upcg_contract_rows(const upcg_generator* g, int64_t* rows);
/* The same rows and the multiply-adds per row that the last fast-form
 * contraction needed: A1 (rows x P) times the survival kernel minus its
 * constant, over the tiles where that can be nonzero (the constant's share
 * is added per cell in FP64); 0 when the last luminosity was not the fast
 * form.  The tensor cores issue each multiply-add three times (hi.hi +
 * hi.lo + lo.hi). */
int upcg_contract_work(const upcg_generator* g, int64_t* rows, int64_t* macs_per_row);
const char* upcg_last_error(void);
const char* upcg_version(void);

#ifdef __cplusplus
}
#endif
#endif /* UPCGEN_GB300_H_ */
