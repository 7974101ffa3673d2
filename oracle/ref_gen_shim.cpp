// C entry point around the reference's own event generator
// (src/UpcGenerator.cpp with src/UpcCrossSection.cpp and the process classes),
// compiled from the reference sources where they lie by oracle/build.py into
// oracle/_ref/, with the GSL / ROOT stand-ins of oracle/refshim/ (TEST
// INFRASTRUCTURE ONLY).
//
// uref_gen_run does what the reference's main does for one configuration
// (main.cpp: setParameterValue per parameters.in key, init, then the event
// loop of generateEvents, src/UpcGenerator.cpp:834-889) and returns the
// accepted events' particles (generateEvent's pdg codes and 4-momenta, in
// its order) and the rejected count.  UpcGenerator::init runs as written:
// UpcCrossSection::init computes the luminosity with the reference's own
// prepareTwoPhotonLumi into the stand-in ROOT file (its lock file in
// `lumi_dir`, which must be a fresh directory), computeNuclXsection folds it
// and builds the GSL samplers, and gRandom is the TRandomMT64 stand-in.  Like
// the reference, one configuration per process (its nucleus, splines and
// breakup tables are process globals).
#include <pthread.h>

#include <cstdint>
#include <functional>
#include <string>
#include <vector>

#include "UpcGenerator.h"

namespace {
// prepareBreakupProb keeps two arrays of 10^6 doubles on the stack
// (src/UpcCrossSection.cpp:422-423, 16 MB): the run goes on a thread with a
// 256 MB stack.
int on_big_stack(std::function<void()> fn) {
  pthread_attr_t attr;
  pthread_attr_init(&attr);
  pthread_attr_setstacksize(&attr, (size_t)256 << 20);
  pthread_t th;
  auto body = [](void* p) -> void* {
    (*static_cast<std::function<void()>*>(p))();
    return nullptr;
  };
  const int rc = pthread_create(&th, &attr, body, &fn);
  pthread_attr_destroy(&attr);
  if (rc != 0) return -1;
  pthread_join(th, nullptr);
  return 0;
}
}  // namespace

extern "C" {

// keys / vals: nkv parameters.in pairs.  pdg, status, mother [n][max_particles]
// (generateEvent's lists; 0 where an event has fewer particles), p4
// [n][max_particles][4] (px, py, pz, E).  Returns 0, -1 (thread), -2 (an
// event with more than max_particles).
int uref_gen_run(const char* const* keys, const char* const* vals, int nkv, const char* lumi_dir,
                 int threads, int64_t n, int max_particles, int* pdg, int* status, int* mother,
                 double* p4, int64_t* rejected, double* tot_mb) {
  int result = 0;
  const int rc = on_big_stack([&] {
    auto* gen = new UpcGenerator();
    for (int i = 0; i < nkv; ++i) gen->setParameterValue(keys[i], vals[i]);
    gen->setLumiFileDirectory(lumi_dir);
    gen->setNumThreads(threads);
    gen->init();
    std::vector<int> pdgs, statuses, mothers;
    std::vector<TLorentzVector> particles;
    int64_t acc = 0, rej = 0;
    while (acc < n) {
      if (gen->generateEvent(pdgs, statuses, mothers, particles) == 1) {
        if ((int)particles.size() > max_particles) {
          result = -2;
          return;
        }
        for (int k = 0; k < max_particles; ++k) {
          const size_t r = (size_t)acc * max_particles + k;
          const bool has = k < (int)particles.size();
          pdg[r] = has ? pdgs[k] : 0;
          status[r] = has ? statuses[k] : 0;
          mother[r] = has ? mothers[k] : 0;
          p4[4 * r + 0] = has ? particles[k].Px() : 0.;
          p4[4 * r + 1] = has ? particles[k].Py() : 0.;
          p4[4 * r + 2] = has ? particles[k].Pz() : 0.;
          p4[4 * r + 3] = has ? particles[k].E() : 0.;
        }
        ++acc;
      } else {
        ++rej;
      }
    }
    *rejected = rej;
    *tot_mb = gen->totNuclX();
  });
  return rc != 0 ? -1 : result;
}
}

extern "C" {
// The reference's UpcSampler2D::getBinX / getBinY (include/UpcSampler.h:124-134)
// on n values: the sampler built as computeNuclXsection builds it
// (src/UpcGenerator.cpp:677-700: x = the nx + 1 rapidity edges, y = the ny + 1
// mass edges; the contents do not enter the bin functions); axis 0 -> getBinX,
// 1 -> getBinY.
int uref_sampler_bins(int nx, const double* edges_x, int ny, const double* edges_y,
                      const double* v, int64_t n, int axis, int* out) {
  std::vector<std::vector<double>> dist(nx, std::vector<double>(ny, 1.0));
  std::vector<double> ex(edges_x, edges_x + nx + 1), ey(edges_y, edges_y + ny + 1);
  UpcSampler2D s(dist, ex, ey, 1);
  for (int64_t i = 0; i < n; ++i) out[i] = axis == 0 ? s.getBinX(v[i]) : s.getBinY(v[i]);
  return 0;
}
}
