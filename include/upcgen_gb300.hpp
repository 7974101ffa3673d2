// upcgen-gb300 -- header-only C++ facade over the C ABI (upcgen_gb300.h) with
// the reference's class and method names, so that a host written against
// upcgen's UpcGenerator (include/UpcGenerator.h:55-128) and UpcCrossSection
// (include/UpcCrossSection.h:65-240) switches by changing its include and
// namespace.  ROOT-free: TLorentzVector / TParticle become the plain
// LorentzVector / Particle below.
//
// Differences from the reference's classes:
//   * errors throw upcgen_gb300::Error (the reference exits the process);
//   * generateEvents() writes NEVENTS events as the reference does, with the
//     particles tree as a column file (events.cols) in place of events.root;
//     generateEvents(n) returns the accepted events and eventRecords(n) the
//     raw 48-byte records; writeEvents(path, n, format) writes one file;
//   * setSeed() seeds the Philox event stream (the reference reseeds gRandom).
#ifndef UPCGEN_GB300_HPP_
#define UPCGEN_GB300_HPP_

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "upcgen_gb300.h"

namespace upcgen_gb300 {

class Error : public std::runtime_error {
 public:
  Error(int code, const char* what) : std::runtime_error(what ? what : "upcgen-gb300 error"), code_(code) {}
  int code() const { return code_; }

 private:
  int code_;
};

inline void check(int rc) {
  if (rc != UPCG_OK) throw Error(rc, upcg_last_error());
}

struct LorentzVector {  // px, py, pz, E (GeV)
  double px = 0, py = 0, pz = 0, e = 0;
};

struct Particle {  // the fields of TParticle the generator fills
  int pdg = 0, status = 0, mother = 0;
  LorentzVector p;
};

class UpcCrossSection;

class UpcGenerator {
 public:
  UpcGenerator() { check(upcg_create(&h_)); }
  ~UpcGenerator() { upcg_destroy(h_); }
  UpcGenerator(const UpcGenerator&) = delete;
  UpcGenerator& operator=(const UpcGenerator&) = delete;

  // ---- configuration (src/UpcGenerator.cpp:183-346)
  void setParameterValue(const std::string& parameter, const std::string& parValue) {
    check(upcg_set_parameter(h_, parameter.c_str(), parValue.c_str()));
  }
  void setParFile(const std::string& parfilename) { parFile_ = parfilename; }
  void configGeneratorFromFile() { check(upcg_config_from_file(h_, parFile_.c_str())); }
  void setLumiFileDirectory(const std::string& directory) {
    check(upcg_set_lumi_file_directory(h_, directory.c_str()));
  }
  void setDebugLevel(int level) { check(upcg_set_debug_level(h_, level)); }
  void setNumThreads(int n) { check(upcg_set_num_threads(h_, n)); }
  void setCollisionSystem(float sqrts, int nucl_z, int nucl_a) {
    check(upcg_set_collision_system(h_, sqrts, nucl_z, nucl_a));
  }
  void setSeed(int seedIn) { check(upcg_set_seed(h_, seedIn)); }
  // 0 plain FP64 (the reference's quadrature), 1 fast form
  void setLumiMethod(int method) { check(upcg_set_lumi_method(h_, method)); }
  void setStream(void* cuda_stream) { check(upcg_set_stream(h_, cuda_stream)); }

  // ---- initial calculations (src/UpcGenerator.cpp:57-181, 630-713)
  void init() { check(upcg_init(h_)); }
  void computeNuclXsection() { check(upcg_compute_nucl_xsection(h_)); }
  double totNuclX() const {
    double v = 0;
    check(upcg_tot_nucl_x(h_, &v));
    return v;
  }
  double fidNuclX() const {
    double v = 0;
    check(upcg_fid_nucl_x(h_, &v));
    return v;
  }

  // ---- events (src/UpcGenerator.cpp:715-926)
  // One candidate: 1 (accepted) or 0 (rejected by the cuts); the outputs are
  // cleared and filled like the reference's vectors.
  long generateEvent(std::vector<int>& pdgs, std::vector<int>& statuses, std::vector<int>& mothers,
                     std::vector<LorentzVector>& particles) {
    upcg_event ev;
    int accepted = 0;
    check(upcg_generate_event(h_, &ev, &accepted));
    pdgs.clear();
    statuses.clear();
    mothers.clear();
    particles.clear();
    fill(ev, pdgs, statuses, mothers, particles);
    genParticles_.clear();
    for (size_t i = 0; i < pdgs.size(); ++i)
      genParticles_.push_back(Particle{pdgs[i], statuses[i], mothers[i], particles[i]});
    return accepted;
  }
  const std::vector<Particle>& getParticles() const { return genParticles_; }

  // The reference's generateEvents with its file output (src/UpcGenerator.cpp:
  // 834-926): n events to path, format 0 = HepMC3 text (events.hepmc), 1 = the
  // particles tree as a column file (events.root via particles_to_root.C);
  // threads formatting on the host (0 = every core).  Returns the rejected count.
  int64_t writeEvents(const std::string& path, int64_t n, int format = 0, int threads = 0) {
    int64_t rej = 0;
    check(upcg_write_events(h_, path.c_str(), n, format, threads, &rej));
    return rej;
  }

  // The reference's generateEvents() itself: NEVENTS events to events.hepmc
  // (USE_HEPMC_OUTPUT) and to the particles tree's column file events.cols
  // (USE_ROOT_OUTPUT, on unless set to 0), in the working directory, the same
  // events in both.  With neither file the loop still runs: the events are
  // drawn and dropped, and fidNuclX() is set as after the reference's loop.
  void generateEvents() {
    int64_t n = 0;
    int use_root = 0, use_hepmc = 0;
    check(upcg_event_output_config(h_, &n, &use_root, &use_hepmc));
    if (!use_root && !use_hepmc) {
      int64_t rej = 0;
      check(upcg_run_events(h_, n, &rej));
      return;
    }
    uint64_t c0 = 0;
    check(upcg_get_candidate_offset(h_, &c0));
    if (use_hepmc) writeEvents("events.hepmc", n, 0);
    if (use_root) {
      if (use_hepmc) check(upcg_set_candidate_offset(h_, c0));
      writeEvents("events.cols", n, 1);
    }
  }

  // The first n accepted events of the candidate sequence (the reference's
  // loop without the file output); *rejected gets the rejected count.
  std::vector<upcg_event> eventRecords(int64_t n, int64_t* rejected = nullptr) {
    std::vector<upcg_event> out((size_t)n);
    int64_t rej = 0;
    check(upcg_generate_events(h_, n, out.data(), nullptr, &rej));
    if (rejected) *rejected = rej;
    return out;
  }
  std::vector<std::vector<Particle>> generateEvents(int64_t n) {
    std::vector<std::vector<Particle>> evs;
    std::vector<int> pdgs, st, mo;
    std::vector<LorentzVector> ps;
    for (const upcg_event& e : eventRecords(n)) {
      pdgs.clear();
      st.clear();
      mo.clear();
      ps.clear();
      fill(e, pdgs, st, mo, ps);
      std::vector<Particle> v;
      for (size_t i = 0; i < pdgs.size(); ++i) v.push_back(Particle{pdgs[i], st[i], mo[i], ps[i]});
      evs.push_back(std::move(v));
    }
    return evs;
  }

  upcg_generator* handle() const { return h_; }

 private:
  // pairProduction (src/UpcGenerator.cpp:388-423): two leptons, status 23,
  // mother 0, charges sign1 = +-1, sign2 = -sign1; the ALP (status 23) and its
  // two decay photons (pdg 22, status 33, mother 1) as twoPartDecayUniform
  // (:526-561); a vector meson and its two daughters likewise.
  void fill(const upcg_event& e, std::vector<int>& pdgs, std::vector<int>& statuses,
            std::vector<int>& mothers, std::vector<LorentzVector>& particles) {
    int pdg = 0, charged = 0, dpdg = 0;
    check(upcg_particle_pdg(h_, &pdg, &charged));
    check(upcg_decay_pdg(h_, &dpdg));
    const LorentzVector a{e.p0[0], e.p0[1], e.p0[2], e.p0[3]};
    const LorentzVector b{e.p1[0], e.p1[1], e.p1[2], e.p1[3]};
    if (dpdg != 0) {  // ALP -> 2 photons; vector meson -> +-DECAY_PDG (twoPartDecayVM, :425-472)
      particles.push_back(LorentzVector{a.px + b.px, a.py + b.py, a.pz + b.pz, a.e + b.e});
      pdgs.push_back(pdg);
      statuses.push_back(23);
      mothers.push_back(0);
      const int s1 = dpdg == 22 ? 1 : (e.sign > 0 ? 1 : -1);
      const int s2 = dpdg == 22 ? 1 : -s1;
      particles.push_back(a);
      particles.push_back(b);
      pdgs.push_back(s1 * dpdg);
      pdgs.push_back(s2 * dpdg);
      for (int k = 0; k < 2; ++k) {
        statuses.push_back(33);
        mothers.push_back(1);
      }
      return;
    }
    const int s1 = charged ? (e.sign > 0 ? 1 : -1) : 1;
    const int s2 = charged ? -s1 : 1;
    particles.push_back(a);
    particles.push_back(b);
    pdgs.push_back(s1 * pdg);
    pdgs.push_back(s2 * pdg);
    statuses.push_back(23);
    statuses.push_back(23);
    mothers.push_back(0);
    mothers.push_back(0);
  }

  upcg_generator* h_ = nullptr;
  std::string parFile_ = "parameters.in";
  std::vector<Particle> genParticles_;
};

// Batched views of UpcCrossSection's methods on a generator's tables
// (src/UpcCrossSection.cpp): each takes n points and returns n values.
class UpcCrossSection {
 public:
  explicit UpcCrossSection(UpcGenerator& g) : h_(g.handle()) {}
  std::vector<double> fluxPoint(const std::vector<double>& b, const std::vector<double>& k) {
    return pts2(b, k, &upcg_flux_point);
  }
  std::vector<double> fluxForm(const std::vector<double>& b, const std::vector<double>& k) {
    return pts2(b, k, &upcg_flux_form);
  }
  std::vector<double> calcFormFac(const std::vector<double>& q2) {
    std::vector<double> out(q2.size());
    check(upcg_form_factor(h_, q2.data(), out.data(), q2.size()));
    return out;
  }
  std::vector<double> calcBreakupProb(const std::vector<double>& b, int mode) {
    std::vector<double> out(b.size());
    check(upcg_breakup_prob(h_, b.data(), mode, out.data(), b.size()));
    return out;
  }
  std::vector<double> calcTwoPhotonLumi(const std::vector<double>& m, const std::vector<double>& y) {
    if (m.size() != y.size()) throw Error(UPCG_ERR_ARG, "m and y differ in length");
    std::vector<double> out(m.size());
    check(upcg_two_photon_lumi(h_, m.data(), y.data(), out.data(), nullptr, m.size()));
    return out;
  }
  // calcTwoPhotonLumiPol (src/UpcCrossSection.cpp:274-335): the scalar
  // luminosity into the result, the pseudoscalar one into *ps
  std::vector<double> calcTwoPhotonLumiPol(const std::vector<double>& m,
                                           const std::vector<double>& y, std::vector<double>* ps) {
    if (m.size() != y.size()) throw Error(UPCG_ERR_ARG, "m and y differ in length");
    if (!ps) throw Error(UPCG_ERR_ARG, "no pseudoscalar output");
    std::vector<double> out(m.size());
    ps->assign(m.size(), 0.);
    check(upcg_two_photon_lumi(h_, m.data(), y.data(), out.data(), ps->data(), m.size()));
    return out;
  }
  // the elementary process's sigma(m) (flag 0 unpolarized, 1 scalar, 2
  // pseudoscalar; src/UpcTwoPhotonDilep.cpp:46-122, src/UpcTwoPhotonALP.cpp:28-33)
  std::vector<double> calcCrossSectionM(const std::vector<double>& m, int flag = 0) {
    std::vector<double> out(m.size());
    check(upcg_cs_m(h_, m.data(), flag, out.data(), m.size()));
    return out;
  }
  // fillCrossSectionZM (src/UpcCrossSection.cpp:337-362): [nm][nz]
  std::vector<double> fillCrossSectionZM(size_t n, int flag = 0) {
    std::vector<double> out(n);
    check(upcg_cs_zm_table(h_, flag, out.data(), n));
    return out;
  }
  // calcPhotonFlux (src/UpcCrossSection.cpp:700-722) at points (m, y)
  std::vector<double> calcPhotonFlux(const std::vector<double>& m, const std::vector<double>& y) {
    return pts2(m, y, &upcg_photon_flux);
  }
  // calcNucCrossSectionY (src/UpcCrossSection.cpp:724-748): dsigma/dy [ny],
  // the emitter ratio into *ratio (may be null), the total (mb) into *tot_mb
  std::vector<double> calcNucCrossSectionY(size_t ny, std::vector<double>* ratio, double* tot_mb) {
    std::vector<double> out(ny);
    if (ratio) ratio->assign(ny, 0.);
    check(upcg_nuc_cs_y(h_, out.data(), ratio ? ratio->data() : nullptr, ny, tot_mb));
    return out;
  }
  // hD2LDMDY of prepareTwoPhotonLumi: [nm][ny], L dm dy
  std::vector<double> lumiTable(size_t n) {
    std::vector<double> out(n);
    check(upcg_lumi_table(h_, out.data(), n, nullptr));
    return out;
  }
  // nucCSYM of calcNucCrossSectionYM: [ny][nm] (nb) and the total (mb)
  std::vector<double> calcNucCrossSectionYM(size_t n, double* tot_mb) {
    std::vector<double> out(n);
    check(upcg_nuc_cs_ym(h_, out.data(), n, tot_mb));
    return out;
  }

 private:
  using Pts2 = int (*)(upcg_generator*, const double*, const double*, double*, size_t);
  std::vector<double> pts2(const std::vector<double>& b, const std::vector<double>& k, Pts2 f) {
    if (b.size() != k.size()) throw Error(UPCG_ERR_ARG, "b and k differ in length");
    std::vector<double> out(b.size());
    check(f(h_, b.data(), k.data(), out.data(), b.size()));
    return out;
  }
  upcg_generator* h_;
};

}  // namespace upcgen_gb300

#endif  // UPCGEN_GB300_HPP_
