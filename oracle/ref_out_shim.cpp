// C entry point around the reference's own HepMC3 output: UpcGenerator's
// writeEvent (src/UpcGenerator.cpp:589-628) and its WriterHepMC
// (include/UpcGenerator.h:192-242), compiled from the reference sources with
// the stand-ins of oracle/refshim/ into oracle/_ref/libupcref_gen.so (TEST
// INFRASTRUCTURE ONLY).
//
// Both are private members of UpcGenerator: this translation unit alone opens
// them (every standard header is included first, then the class is read with
// its private members public; the layout does not change).  uref_write_hepmc
// writes given particle lists through the reference's code, so the library's
// HepMC3 text can be compared with the reference's byte for byte.
// uref_config_file reads a parameters.in with the reference's own
// configGeneratorFromFile (src/UpcGenerator.cpp:318-346) and runs its init
// (the process overrides, :57-181), and returns the resulting grid and flags.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <fstream>
#include <functional>
#include <iomanip>
#include <iostream>
#include <limits>
#include <map>
#include <memory>
#include <mutex>
#include <random>
#include <sstream>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>

#include <pthread.h>

#include "refshim.h"

#define private public
#include "UpcGenerator.h"
#undef private

extern "C" {

// n events of ppe particles: pdg, status, mother [n][ppe], p4 [n][ppe][4]
// (px, py, pz, E); the events are numbered first, first + 1, ...  Writes the
// reference's preamble, the events and its end-of-listing line to `path`.
int uref_write_hepmc(const char* path, int64_t n, int ppe, const int* pdg, const int* status,
                     const int* mother, const double* p4, int64_t first) {
  UpcGenerator gen;
  gen.useROOTOut = false;
  gen.useHepMCOut = true;
  gen.writerHepMC = new UpcGenerator::WriterHepMC(path);
  if (!gen.writerHepMC->outfile.is_open()) return -1;
  std::vector<int> pdgs(ppe), statuses(ppe), mothers(ppe);
  std::vector<TLorentzVector> particles(ppe);
  for (int64_t i = 0; i < n; ++i) {
    for (int k = 0; k < ppe; ++k) {
      const size_t r = (size_t)i * ppe + k;
      pdgs[k] = pdg[r];
      statuses[k] = status[r];
      mothers[k] = mother[r];
      particles[k].SetPxPyPzE(p4[4 * r], p4[4 * r + 1], p4[4 * r + 2], p4[4 * r + 3]);
    }
    gen.writeEvent(first + i, pdgs, statuses, mothers, particles);
  }
  delete gen.writerHepMC;  // the end-of-listing line, file closed
  gen.writerHepMC = nullptr;
  return 0;  // ~UpcGenerator deletes gRandom, which this run never set
}
}

namespace {
// prepareBreakupProb keeps two arrays of 10^6 doubles on the stack
// (src/UpcCrossSection.cpp:422-423, 16 MB): init runs on a thread with a
// 256 MB stack.
int on_big_stack_cfg(std::function<void()> fn) {
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

// grid: mmin, mmax, ymin, ymax, zmin, zmax; ints: nm, ny, nz, procID,
// breakupMode, isPoint, usePolarizedCS, useNonzeroGamPt, doPtCut, doEtaCut,
// useROOTOut, useHepMCOut; nevents.  lumi_dir: a fresh directory for the
// reference's lock file (init computes the luminosity: keep the grid small).
int uref_config_file(const char* path, const char* lumi_dir, double* grid, int* ints,
                     int64_t* nevents) {
  const int rc = on_big_stack_cfg([&] {
    UpcGenerator gen;
    gen.setParFile(path);
    gen.configGeneratorFromFile();
    gen.setLumiFileDirectory(lumi_dir);
    gen.setNumThreads(1);
    gen.init();
    const UpcCrossSection& c = *gen.nucProcessCS;
    const double g[6] = {c.mmin, c.mmax, c.ymin, c.ymax, c.zmin, c.zmax};
    for (int i = 0; i < 6; ++i) grid[i] = g[i];
    const int v[12] = {c.nm, c.ny, c.nz, gen.procID, c.breakupMode, c.isPoint ? 1 : 0,
                       gen.usePolarizedCS ? 1 : 0, c.useNonzeroGamPt ? 1 : 0,
                       gen.doPtCut ? 1 : 0, gen.doEtaCut ? 1 : 0, gen.useROOTOut ? 1 : 0,
                       gen.useHepMCOut ? 1 : 0};
    for (int i = 0; i < 12; ++i) ints[i] = v[i];
    *nevents = gen.nEvents;
  });
  gRandom = nullptr;  // deleted by ~UpcGenerator
  return rc;
}
}
