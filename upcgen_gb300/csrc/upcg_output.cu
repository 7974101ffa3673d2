// Event output: the reference's two writers of generateEvents
// (src/UpcGenerator.cpp:589-628, 834-926).
//
// * The ROOT tree "particles" (one row per particle: eventNumber/I, pdgCode/I,
//   particleID/I, statusID/I, motherID/I, px/D, py/D, pz/D, e/D) becomes
//   columns built on the device by k_event_columns; upcg_write_events format 1
//   writes them to a column file (ROOT is not a dependency; the macro
//   upcgen_gb300/particles_to_root.C turns one into the reference's tree).
// * The HepMC3 ASCII file of WriterHepMC (include/UpcGenerator.h:192-242):
//   "E <event> <vertices> <particles>", "U GEV MM", then per particle
//   "P <id> <mother> <pdg> <px> <py> <pz> <e> <m> <status>" with
//   setprecision(9) (printf "%.9g"), between the version / listing lines.
//
// Particles per event follow generateEvent (src/UpcGenerator.cpp:767-812):
// a lepton pair is two leptons (pdg +-PDG by the event's charge sign, status
// 23, mother 0); an ALP is the ALP (pdg 51, status 23, mother 0, momentum =
// the photons' sum) and its two photons (pdg 22, status 33, mother 1); a
// vector meson is the meson (status 23, mother 0, momentum = the daughters'
// sum) and its two daughters (pdg +-DECAY_PDG by the event's sign, status 33,
// mother 1; twoPartDecayVM, :425-472).
//
// upcg_write_events generates batches on the device while host threads format
// and write the previous batch: the device work of batch k+1 overlaps the file
// work of batch k, and formatting runs on every host core.
#include <fcntl.h>
#include <unistd.h>

#include <algorithm>
#include <charconv>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/upcgen_gb300.h"
#include "upcg_internal.h"

namespace upcg {
namespace {

struct ProcOut {
  int pdg, charged, ppe;  // particles per event
  int dpdg, dsigned;      // decay products (3-particle events), signed by the event's sign
};

int proc_out(upcg_generator* g, ProcOut* p) {
  int pdg = 0, ch = 0, d = 0;
  int rc = upcg_particle_pdg(g, &pdg, &ch);
  if (rc) return rc;
  rc = upcg_decay_pdg(g, &d);
  if (rc) return rc;
  p->pdg = pdg;
  p->charged = ch;
  p->ppe = d != 0 ? 3 : 2;
  p->dpdg = d;
  p->dsigned = d != 22;
  return UPCG_OK;
}

__global__ void k_event_columns(const float4* __restrict__ ev, int64_t n, int64_t first, ProcOut po,
                                upcg_particle_columns c) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  // EventRecord: {m, y, z, sign}, p0[4], p1[4]
  const float4 h = __ldg(ev + 3 * i), a = __ldg(ev + 3 * i + 1), b = __ldg(ev + 3 * i + 2);
  const int evn = (int)(first + i);
  const int64_t r = i * po.ppe;
  if (po.ppe == 3) {
    const double q[4] = {(double)a.x + (double)b.x, (double)a.y + (double)b.y,
                         (double)a.z + (double)b.z, (double)a.w + (double)b.w};
    c.eventNumber[r] = evn;
    c.pdgCode[r] = po.pdg;
    c.particleID[r] = 1;
    c.statusID[r] = 23;
    c.motherID[r] = 0;
    c.px[r] = q[0];
    c.py[r] = q[1];
    c.pz[r] = q[2];
    c.e[r] = q[3];
    const float4 ph[2] = {a, b};
    const int s1 = po.dsigned ? (h.w > 0.f ? 1 : -1) : 1;
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      const int64_t rk = r + 1 + k;
      c.eventNumber[rk] = evn;
      c.pdgCode[rk] = (k == 0 ? s1 : (po.dsigned ? -s1 : 1)) * po.dpdg;
      c.particleID[rk] = 2 + k;
      c.statusID[rk] = 33;
      c.motherID[rk] = 1;
      c.px[rk] = ph[k].x;
      c.py[rk] = ph[k].y;
      c.pz[rk] = ph[k].z;
      c.e[rk] = ph[k].w;
    }
    return;
  }
  const int s1 = po.charged ? (h.w > 0.f ? 1 : -1) : 1;
  const int s2 = po.charged ? -s1 : 1;
  const float4 lp[2] = {a, b};
  const int sg[2] = {s1, s2};
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const int64_t rk = r + k;
    c.eventNumber[rk] = evn;
    c.pdgCode[rk] = sg[k] * po.pdg;
    c.particleID[rk] = 1 + k;
    c.statusID[rk] = 23;
    c.motherID[rk] = 0;
    c.px[rk] = lp[k].x;
    c.py[rk] = lp[k].y;
    c.pz[rk] = lp[k].z;
    c.e[rk] = lp[k].w;
  }
}

// TLorentzVector::M(): sqrt(E^2 - p^2), negative for space-like vectors
double lv_mass(double px, double py, double pz, double e) {
  const double mm = e * e - (px * px + py * py + pz * pz);
  return mm < 0. ? -std::sqrt(-mm) : std::sqrt(mm);
}

// The reference's stream prints doubles with setprecision(9), i.e. as printf's
// "%.9g".  std::to_chars with chars_format::general and a precision is
// specified to give exactly that text (the shortest correctly rounded
// digits, the same exponent form), about three times faster than snprintf.
char* put_g9(char* p, char* end, double v) {
  return std::to_chars(p, end, v, std::chars_format::general, 9).ptr;
}
template <class I>
char* put_int(char* p, char* end, I v) {
  return std::to_chars(p, end, v).ptr;
}

// "P id mother pdg px py pz e m status" (WriterHepMC::writeParticleInfo)
void append_particle(std::string& s, int id, int mother, int pdg, double px, double py, double pz,
                     double e, int status) {
  char buf[192];  // 3 ints, 5 doubles of at most 16 characters, 1 int, separators
  char* const end = buf + sizeof buf;
  char* p = buf;
  *p++ = 'P';
  *p++ = ' ';
  p = put_int(p, end, id);
  *p++ = ' ';
  p = put_int(p, end, mother);
  *p++ = ' ';
  p = put_int(p, end, pdg);
  const double v[5] = {px, py, pz, e, lv_mass(px, py, pz, e)};
  for (double x : v) {
    *p++ = ' ';
    p = put_g9(p, end, x);
  }
  *p++ = ' ';
  p = put_int(p, end, status);
  *p++ = '\n';
  s.append(buf, (size_t)(p - buf));
}

// one event of WriterHepMC::writeEventInfo + writeParticleInfo (the vertex
// count of writeEvent: mother-id changes along the list, starting from -1)
void append_event(std::string& s, int64_t evt, const EventRecord& r, const ProcOut& po) {
  char buf[96];
  char* const end = buf + sizeof buf;
  const int nvert = po.ppe == 3 ? 1 : 0;
  char* p = buf;
  *p++ = 'E';
  *p++ = ' ';
  p = put_int(p, end, (long long)evt);
  *p++ = ' ';
  p = put_int(p, end, nvert);
  *p++ = ' ';
  p = put_int(p, end, po.ppe);
  static const char kUnits[] = "\nU GEV MM\n";
  std::memcpy(p, kUnits, sizeof kUnits - 1);
  p += sizeof kUnits - 1;
  s.append(buf, (size_t)(p - buf));
  const double a[4] = {r.p0[0], r.p0[1], r.p0[2], r.p0[3]};
  const double b[4] = {r.p1[0], r.p1[1], r.p1[2], r.p1[3]};
  if (po.ppe == 3) {
    const int s1 = po.dsigned ? (r.sign > 0.f ? 1 : -1) : 1;
    const int s2 = po.dsigned ? -s1 : 1;
    append_particle(s, 1, 0, po.pdg, a[0] + b[0], a[1] + b[1], a[2] + b[2], a[3] + b[3], 23);
    append_particle(s, 2, 1, s1 * po.dpdg, a[0], a[1], a[2], a[3], 33);
    append_particle(s, 3, 1, s2 * po.dpdg, b[0], b[1], b[2], b[3], 33);
    return;
  }
  const int s1 = po.charged ? (r.sign > 0.f ? 1 : -1) : 1;
  const int s2 = po.charged ? -s1 : 1;
  append_particle(s, 1, 0, s1 * po.pdg, a[0], a[1], a[2], a[3], 23);
  append_particle(s, 2, 0, s2 * po.pdg, b[0], b[1], b[2], b[3], 23);
}

// events [0, n) formatted by up to `threads` threads; the pieces in order
void format_parallel(const EventRecord* ev, int64_t n, int64_t first, const ProcOut& po, int threads,
                     std::vector<std::string>& parts) {
  const int64_t per_min = 4096;
  int t = (int)std::min<int64_t>(threads, (n + per_min - 1) / per_min);
  t = std::max(t, 1);
  parts.assign((size_t)t, std::string());
  auto work = [&](int w) {
    const int64_t lo = n * w / t, hi = n * (w + 1) / t;
    std::string& s = parts[(size_t)w];
    s.reserve((size_t)(hi - lo) * (po.ppe * 96 + 32));
    for (int64_t i = lo; i < hi; ++i) append_event(s, first + i, ev[i], po);
  };
  std::vector<std::thread> pool;
  for (int w = 1; w < t; ++w) pool.emplace_back(work, w);
  work(0);
  for (auto& th : pool) th.join();
}

const char kHepmcHead[] = "HepMC::Version 3.02.04\nHepMC::Asciiv3-START_EVENT_LISTING\n";
const char kHepmcTail[] = "HepMC::Asciiv3-END_EVENT_LISTING\n";

// particle column file: magic, version, column count, rows, then per column
// {name[16], type 'I' (int32) or 'D' (double), 7 pad bytes}, then the columns
// in that order, each padded to 8 bytes
constexpr char kColMagic[8] = {'U', 'P', 'C', 'G', 'P', 'R', 'T', '1'};
const char* const kColNames[9] = {"eventNumber", "pdgCode", "particleID", "statusID", "motherID",
                                  "px", "py", "pz", "e"};
constexpr size_t kColHeader = 8 + 4 + 4 + 8 + 9 * 24;

size_t col_size(int c) { return c < 5 ? 4 : 8; }
size_t pad8(size_t b) { return (b + 7) / 8 * 8; }

struct PinnedBuf {
  void* p = nullptr;
  ~PinnedBuf() {
    if (p) cudaFreeHost(p);
  }
};
struct DevBuf {
  void* p = nullptr;
  ~DevBuf() {
    if (p) cudaFree(p);
  }
};

bool pwrite_all(int fd, const void* data, size_t n, off_t off) {
  const char* c = static_cast<const char*>(data);
  while (n > 0) {
    const ssize_t w = pwrite(fd, c, n, off);
    if (w <= 0) return false;
    c += w;
    n -= (size_t)w;
    off += w;
  }
  return true;
}

}  // namespace
}  // namespace upcg

using namespace upcg;

int upcg_particles_per_event(upcg_generator* g, int* n) {
  if (!g || !n) return fail(UPCG_ERR_ARG, "null argument");
  ProcOut po{};
  const int rc = proc_out(g, &po);
  if (rc) return rc;
  *n = po.ppe;
  return UPCG_OK;
}

int upcg_event_particles_device(upcg_generator* g, const upcg_event* ev_device, int64_t n,
                                int64_t first_event, const upcg_particle_columns* cols) {
  if (!g || !cols || n < 0 || (n > 0 && !ev_device)) return fail(UPCG_ERR_ARG, "bad argument");
  if (first_event < 0 || first_event + n > 2147483647LL)
    return fail(UPCG_ERR_SIZE, "eventNumber is a 32-bit column (UpcGenerator.cpp:847)");
  const upcg_particle_columns& c = *cols;
  if (!c.eventNumber || !c.pdgCode || !c.particleID || !c.statusID || !c.motherID || !c.px || !c.py ||
      !c.pz || !c.e)
    return fail(UPCG_ERR_ARG, "null column");
  // the kernel loads records as float4 and stores naturally aligned columns
  const auto mis = [](const void* p, uintptr_t a) { return (reinterpret_cast<uintptr_t>(p) & (a - 1)) != 0; };
  if (mis(ev_device, 16) || mis(c.eventNumber, 4) || mis(c.pdgCode, 4) || mis(c.particleID, 4) ||
      mis(c.statusID, 4) || mis(c.motherID, 4) || mis(c.px, 8) || mis(c.py, 8) || mis(c.pz, 8) ||
      mis(c.e, 8))
    return fail(UPCG_ERR_ARG, "records need 16-byte, int32 columns 4-byte, double columns 8-byte alignment");
  ProcOut po{};
  int rc = proc_out(g, &po);
  if (rc) return rc;
  if (n == 0) return UPCG_OK;
  note_launch();
  k_event_columns<<<(unsigned)((n + 255) / 256), 256, 0, handle_stream(g)>>>(
      reinterpret_cast<const float4*>(ev_device), n, first_event, po, c);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(UPCG_ERR_CUDA, "k_event_columns: %s", cudaGetErrorString(e));
  return UPCG_OK;
}

int upcg_format_hepmc3(upcg_generator* g, const upcg_event* ev, int64_t n, int64_t first_event,
                       char* out, size_t cap, size_t* len) {
  if (!g || !len || n < 0 || (n > 0 && !ev)) return fail(UPCG_ERR_ARG, "bad argument");
  ProcOut po{};
  const int rc = proc_out(g, &po);
  if (rc) return rc;
  std::vector<std::string> parts;
  const unsigned hw = std::thread::hardware_concurrency();
  format_parallel(reinterpret_cast<const EventRecord*>(ev), n, first_event, po, hw ? (int)hw : 1,
                  parts);
  size_t total = 0;
  for (const auto& s : parts) total += s.size();
  *len = total;
  if (!out || cap < total) return fail(UPCG_ERR_SIZE, "the text needs %zu bytes", total);
  size_t o = 0;
  for (const auto& s : parts) {
    std::memcpy(out + o, s.data(), s.size());
    o += s.size();
  }
  return UPCG_OK;
}

int upcg_write_events(upcg_generator* g, const char* path, int64_t n, int format, int threads,
                      int64_t* rejected) {
  if (!g || !path || !rejected || n < 0 || (format != 0 && format != 1))
    return fail(UPCG_ERR_ARG, "bad argument");
  if (n > 2147483647LL) return fail(UPCG_ERR_SIZE, "eventNumber is a 32-bit column");
  ProcOut po{};
  int rc = proc_out(g, &po);
  if (rc) return rc;
  if (threads <= 0) {
    const unsigned hw = std::thread::hardware_concurrency();
    threads = hw ? (int)hw : 1;
  }
  // events per batch: 2^21 (100 MB of records), or UPCG_OUTPUT_BATCH
  int64_t bmax = (int64_t)1 << 21;
  if (const char* env = getenv("UPCG_OUTPUT_BATCH")) bmax = std::min<int64_t>(std::max(atoll(env), 1LL), 1LL << 24);
  const int64_t B = std::max<int64_t>(1, std::min<int64_t>(n, bmax));
  const int64_t rows_b = B * po.ppe;
  const size_t rec_bytes = (size_t)B * sizeof(EventRecord);
  const size_t col_bytes = pad8((size_t)rows_b * 20) + (size_t)rows_b * 32;
  DevBuf dev_rec, dev_col;
  PinnedBuf host[2];
  cudaError_t ce = cudaMalloc(&dev_rec.p, rec_bytes);
  if (ce == cudaSuccess && format == 1) ce = cudaMalloc(&dev_col.p, col_bytes);
  for (int k = 0; k < 2 && ce == cudaSuccess; ++k)
    ce = cudaMallocHost(&host[k].p, format == 0 ? rec_bytes : col_bytes);
  if (ce != cudaSuccess) return fail(UPCG_ERR_CUDA, "output buffers: %s", cudaGetErrorString(ce));
  const int fd = open(path, O_WRONLY | O_CREAT | O_TRUNC, 0644);
  if (fd < 0) return fail(UPCG_ERR_IO, "cannot open %s for writing", path);
  const int64_t nrows = n * po.ppe;
  // column offsets of format 1
  size_t col_off[9];
  {
    size_t o = kColHeader;
    for (int c = 0; c < 9; ++c) {
      col_off[c] = o;
      o += pad8((size_t)nrows * col_size(c));
    }
  }
  bool io_ok = true;
  off_t text_off = 0;
  if (format == 0) {
    io_ok = pwrite_all(fd, kHepmcHead, sizeof kHepmcHead - 1, 0);
    text_off = sizeof kHepmcHead - 1;
  } else {
    std::vector<char> h(kColHeader, 0);
    std::memcpy(h.data(), kColMagic, 8);
    const uint32_t ver = 1, ncol = 9;
    const uint64_t nr = (uint64_t)nrows;
    std::memcpy(h.data() + 8, &ver, 4);
    std::memcpy(h.data() + 12, &ncol, 4);
    std::memcpy(h.data() + 16, &nr, 8);
    for (int c = 0; c < 9; ++c) {
      char* d = h.data() + 24 + 24 * c;
      std::strncpy(d, kColNames[c], 16);
      d[16] = c < 5 ? 'I' : 'D';
    }
    io_ok = pwrite_all(fd, h.data(), h.size(), 0);
    // size the file so every column's padding exists
    io_ok = io_ok && ftruncate(fd, (off_t)(col_off[8] + pad8((size_t)nrows * 8))) == 0;
  }
  cudaStream_t s = handle_stream(g);
  std::thread writer;
  bool writer_ok = true;
  int64_t rej_total = 0, done = 0;
  int slot = 0;
  while (done < n && io_ok) {
    const int64_t nb = std::min(B, n - done);
    int64_t rej = 0;
    rc = upcg_generate_events_device(g, nb, reinterpret_cast<upcg_event*>(dev_rec.p), nullptr, &rej);
    if (rc) break;
    rej_total += rej;
    void* hb = host[slot].p;
    if (format == 0) {
      count_copy((size_t)nb * sizeof(EventRecord), cudaMemcpyDeviceToHost);
      ce = cudaMemcpyAsync(hb, dev_rec.p, (size_t)nb * sizeof(EventRecord), cudaMemcpyDeviceToHost, s);
    } else {
      // five int32 columns, then (from an 8-byte boundary) four double columns
      const int64_t rb = nb * po.ppe;
      const size_t ioff = pad8((size_t)rb * 20);
      char* d = static_cast<char*>(dev_col.p);
      upcg_particle_columns c{};
      c.eventNumber = reinterpret_cast<int32_t*>(d);
      c.pdgCode = c.eventNumber + rb;
      c.particleID = c.pdgCode + rb;
      c.statusID = c.particleID + rb;
      c.motherID = c.statusID + rb;
      c.px = reinterpret_cast<double*>(d + ioff);
      c.py = c.px + rb;
      c.pz = c.py + rb;
      c.e = c.pz + rb;
      rc = upcg_event_particles_device(g, reinterpret_cast<const upcg_event*>(dev_rec.p), nb, done, &c);
      if (rc) break;
      count_copy(ioff + (size_t)rb * 32, cudaMemcpyDeviceToHost);
      ce = cudaMemcpyAsync(hb, dev_col.p, ioff + (size_t)rb * 32, cudaMemcpyDeviceToHost, s);
    }
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
    if (ce != cudaSuccess) {
      rc = fail(UPCG_ERR_CUDA, "event output copy: %s", cudaGetErrorString(ce));
      break;
    }
    if (writer.joinable()) writer.join();  // the previous batch is on disk; its slot is free
    if (!writer_ok) {
      io_ok = false;
      break;
    }
    const int64_t first = done;
    if (format == 0) {
      writer = std::thread([&, hb, nb, first, text_off_in = text_off]() mutable {
        std::vector<std::string> parts;
        format_parallel(static_cast<const EventRecord*>(hb), nb, first, po, threads, parts);
        for (const auto& p : parts) {
          writer_ok = writer_ok && pwrite_all(fd, p.data(), p.size(), text_off_in);
          text_off_in += (off_t)p.size();
        }
        text_off = text_off_in;
      });
      // text offsets depend on the formatted sizes: the next batch's writer
      // starts after this one has finished (joined above)
    } else {
      writer = std::thread([&, hb, nb, first]() {
        const int64_t rb = nb * po.ppe, r0 = first * po.ppe;
        const char* base = static_cast<const char*>(hb);
        const size_t ioff = pad8((size_t)rb * 20);
        for (int c = 0; c < 9; ++c) {
          const size_t sz = col_size(c);
          const char* src = c < 5 ? base + (size_t)c * rb * 4 : base + ioff + (size_t)(c - 5) * rb * 8;
          writer_ok = writer_ok && pwrite_all(fd, src, (size_t)rb * sz, (off_t)(col_off[c] + (size_t)r0 * sz));
        }
      });
    }
    done += nb;
    slot ^= 1;
  }
  if (writer.joinable()) writer.join();
  io_ok = io_ok && writer_ok;
  if (!rc && io_ok && format == 0) io_ok = pwrite_all(fd, kHepmcTail, sizeof kHepmcTail - 1, text_off);
  if (close(fd) != 0) io_ok = false;
  if (rc) return rc;
  if (!io_ok) return fail(UPCG_ERR_IO, "writing %s failed", path);
  *rejected = rej_total;
  if (n > 0) set_fiducial(g, n, rej_total);
  return UPCG_OK;
}
