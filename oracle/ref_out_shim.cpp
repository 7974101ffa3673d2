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
  return 0;
}
}
