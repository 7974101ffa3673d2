// ROOT macro: a particle column file of upcgen_gb300 (upcg_write_events
// format 1) -> the reference's events.root tree "particles"
// (src/UpcGenerator.cpp:842-853): branches eventNumber/I, pdgCode/I,
// particleID/I, statusID/I, motherID/I, px/D, py/D, pz/D, e/D, one entry per
// particle.
//
//   root -b -q 'particles_to_root.C("events.cols", "events.root")'
//
// The file layout is documented in upcgen_gb300/event_output.py.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <vector>

#include "TFile.h"
#include "TTree.h"

int particles_to_root(const char* cols, const char* out = "events.root") {
  std::ifstream in(cols, std::ios::binary);
  char magic[8];
  uint32_t ver = 0, ncol = 0;
  uint64_t nrows = 0;
  if (!in.read(magic, 8) || std::memcmp(magic, "UPCGPRT1", 8) != 0 ||
      !in.read(reinterpret_cast<char*>(&ver), 4) || !in.read(reinterpret_cast<char*>(&ncol), 4) ||
      !in.read(reinterpret_cast<char*>(&nrows), 8) || ver != 1 || ncol != 9) {
    std::printf("%s: not a particle column file\n", cols);
    return 1;
  }
  in.seekg(24 + 24 * 9);
  std::vector<int32_t> iv[5];
  std::vector<double> dv[4];
  for (int c = 0; c < 9; ++c) {
    const size_t sz = c < 5 ? 4 : 8;
    char* dst;
    if (c < 5) {
      iv[c].resize(nrows);
      dst = reinterpret_cast<char*>(iv[c].data());
    } else {
      dv[c - 5].resize(nrows);
      dst = reinterpret_cast<char*>(dv[c - 5].data());
    }
    const size_t bytes = nrows * sz;
    if (!in.read(dst, (std::streamsize)bytes)) {
      std::printf("%s: truncated\n", cols);
      return 1;
    }
    in.seekg((std::streamoff)((bytes + 7) / 8 * 8 - bytes), std::ios::cur);
  }
  TFile f(out, "recreate");
  TTree tree("particles", "Generated particles");
  int32_t eventNumber, pdgCode, particleID, statusID, motherID;
  double px, py, pz, e;
  tree.Branch("eventNumber", &eventNumber, "eventNumber/I");
  tree.Branch("pdgCode", &pdgCode, "pdgCode/I");
  tree.Branch("particleID", &particleID, "particleID/I");
  tree.Branch("statusID", &statusID, "statusID/I");
  tree.Branch("motherID", &motherID, "motherID/I");
  tree.Branch("px", &px, "px/D");
  tree.Branch("py", &py, "py/D");
  tree.Branch("pz", &pz, "pz/D");
  tree.Branch("e", &e, "e/D");
  for (uint64_t r = 0; r < nrows; ++r) {
    eventNumber = iv[0][r];
    pdgCode = iv[1][r];
    particleID = iv[2][r];
    statusID = iv[3][r];
    motherID = iv[4][r];
    px = dv[0][r];
    py = dv[1][r];
    pz = dv[2][r];
    e = dv[3][r];
    tree.Fill();
  }
  tree.Write();
  f.Close();
  return 0;
}
