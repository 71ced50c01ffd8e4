// io.cpp -- host-side data paths around the search (include/hella_io.h).
#include "hella_io.h"

#include <arpa/inet.h>
#include <cuda_runtime.h>
#include <errno.h>
#include <fcntl.h>
#include <netinet/in.h>
#include <poll.h>
#include <sys/socket.h>
#include <unistd.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <mutex>
#include <new>
#include <numeric>
#include <string>
#include <vector>

// ------------------------------------------------------------- SIGPROC

struct hella_fil {
  FILE *f = nullptr;
  hella_fil_header h{};
};

namespace {

// A header string: int32 length (1..80) then the characters.
bool get_string(FILE *f, std::string *s) {
  int32_t n = 0;
  if (std::fread(&n, sizeof(n), 1, f) != 1) return false;
  if (n < 1 || n > 80) {
    *s = "";  // not a header string (the reference reads it as "ERROR")
    return true;
  }
  char buf[81];
  if (std::fread(buf, 1, (size_t)n, f) != (size_t)n) return false;
  buf[n] = '\0';
  *s = buf;
  return true;
}

template <typename T>
bool get_value(FILE *f, T *v) {
  return std::fread(v, sizeof(T), 1, f) == 1;
}

}  // namespace

extern "C" {

hella_status hella_fil_open(hella_fil **out, const char *path, int expect_nchan, hella_fil_header *hdr) {
  if (!out || !path) return HELLA_ERR_INVALID_ARG;
  *out = nullptr;
  hella_fil *fl = new (std::nothrow) hella_fil;
  if (!fl) return HELLA_ERR_ALLOC;
  fl->f = std::fopen(path, "rb");
  if (!fl->f) {
    delete fl;
    return HELLA_ERR_INVALID_ARG;
  }
  auto fail = [&](hella_status s) {
    hella_fil_close(fl);
    return s;
  };
  hella_fil_header &h = fl->h;
  std::string key;
  if (!get_string(fl->f, &key)) return fail(HELLA_ERR_STATE);
  if (key != "HEADER_START") return fail(HELLA_ERR_INVALID_ARG);
  bool want_raw = false, want_src = false;
  for (;;) {
    if (!get_string(fl->f, &key)) return fail(HELLA_ERR_STATE);
    bool ok = true;
    if (key == "HEADER_END") break;
    if (key == "rawdatafile") {
      want_raw = true;
    } else if (key == "source_name") {
      want_src = true;
    } else if (key == "FREQUENCY_START") {
      h.nfreq = 0;
    } else if (key == "FREQUENCY_END") {
    } else if (key == "az_start") { ok = get_value(fl->f, &h.az_start);
    } else if (key == "za_start") { ok = get_value(fl->f, &h.za_start);
    } else if (key == "src_raj") { ok = get_value(fl->f, &h.src_raj);
    } else if (key == "src_dej") { ok = get_value(fl->f, &h.src_dej);
    } else if (key == "tstart") { ok = get_value(fl->f, &h.tstart);
    } else if (key == "tsamp") { ok = get_value(fl->f, &h.tsamp);
    } else if (key == "period") { ok = get_value(fl->f, &h.period);
    } else if (key == "fch1") { ok = get_value(fl->f, &h.fch1);
    } else if (key == "fchannel") {
      if (h.nfreq >= HELLA_FIL_MAX_FREQ) return fail(HELLA_ERR_INVALID_ARG);
      ok = get_value(fl->f, &h.frequency_table[h.nfreq]);
      h.nfreq++;
      h.fch1 = h.foff = 0.0;  // a frequency table is in use
    } else if (key == "foff") { ok = get_value(fl->f, &h.foff);
    } else if (key == "nchans") { ok = get_value(fl->f, &h.nchans);
    } else if (key == "telescope_id") { ok = get_value(fl->f, &h.telescope_id);
    } else if (key == "machine_id") { ok = get_value(fl->f, &h.machine_id);
    } else if (key == "data_type") { ok = get_value(fl->f, &h.data_type);
    } else if (key == "ibeam") { ok = get_value(fl->f, &h.ibeam);
    } else if (key == "nbeams") { ok = get_value(fl->f, &h.nbeams);
    } else if (key == "nbits") { ok = get_value(fl->f, &h.nbits);
    } else if (key == "barycentric") { ok = get_value(fl->f, &h.barycentric);
    } else if (key == "pulsarcentric") { ok = get_value(fl->f, &h.pulsarcentric);
    } else if (key == "nbins" || key == "nsamples") {
      int32_t skip;
      ok = get_value(fl->f, &skip);
    } else if (key == "nifs") { ok = get_value(fl->f, &h.nifs);
    } else if (key == "npuls") { ok = get_value(fl->f, &h.npuls);
    } else if (key == "refdm") { ok = get_value(fl->f, &h.refdm);
    } else if (key == "signed") { ok = get_value(fl->f, &h.isign);
    } else if (want_raw) {
      std::snprintf(h.rawdatafile, sizeof(h.rawdatafile), "%s", key.c_str());
      want_raw = false;
    } else if (want_src) {
      std::snprintf(h.source_name, sizeof(h.source_name), "%s", key.c_str());
      want_src = false;
    } else {
      return fail(HELLA_ERR_INVALID_ARG);  // unknown parameter (sigproc.cpp:168-172)
    }
    if (!ok) return fail(HELLA_ERR_STATE);
  }
  if (expect_nchan > 0 && h.nchans != expect_nchan) return fail(HELLA_ERR_INVALID_ARG);
  if (h.nbits != 8 || h.nchans < 1) return fail(HELLA_ERR_INVALID_ARG);
  h.header_bytes = std::ftell(fl->f);
  if (hdr) *hdr = h;
  *out = fl;
  return HELLA_OK;
}

hella_status hella_fil_read(hella_fil *f, uint8_t *out, int nsamp, int *got) {
  if (!f || !out || nsamp < 0 || !got) return HELLA_ERR_INVALID_ARG;
  *got = (int)std::fread(out, (size_t)f->h.nchans, (size_t)nsamp, f->f);
  return HELLA_OK;
}

void hella_fil_close(hella_fil *f) {
  if (!f) return;
  if (f->f) std::fclose(f->f);
  delete f;
}

// --------------------------------------------------------- candidates

namespace {

// One output_peaks line of candidate c.
int cand_line(const hella_cand &c, long samp0, const float *dms, int ndms, double tres, char *buf,
              size_t cap) {
  const long samp = c.samp + samp0;
  const double dm = (c.dm_idx >= 0 && c.dm_idx < ndms) ? (double)dms[c.dm_idx] : 0.0;
  return std::snprintf(buf, cap, "%g %d %g %d %d %g %d\n", (double)c.snr, (int)samp,
                       tres * (double)samp / 86400.0, c.width, c.dm_idx, dm, c.beam);
}

hella_status format_lines(const hella_cand *c, int n, long samp0, const float *dms, int ndms, double tres,
                          char *buf, size_t cap, size_t *len) {
  size_t at = *len;
  for (int i = 0; i < n; ++i) {
    const int k = cand_line(c[i], samp0, dms, ndms, tres, buf + at, cap > at ? cap - at : 0);
    if (k < 0 || at + (size_t)k >= cap) return HELLA_ERR_BUDGET;
    at += (size_t)k;
  }
  *len = at;
  return HELLA_OK;
}

}  // namespace

hella_status hella_cands_format(const hella_cand *c, int n, long samp0, const float *dms, int ndms,
                                double time_resolution, char *buf, size_t cap, size_t *len) {
  if ((n > 0 && (!c || !dms)) || n < 0 || !buf || !len) return HELLA_ERR_INVALID_ARG;
  *len = 0;
  if (cap) buf[0] = '\0';
  return format_lines(c, n, samp0, dms, ndms, time_resolution, buf, cap, len);
}

hella_status hella_cands_append(const char *path, const hella_cand *c, int n, long samp0, const float *dms,
                                int ndms, double time_resolution) {
  if (!path || n < 0 || (n > 0 && (!c || !dms))) return HELLA_ERR_INVALID_ARG;
  FILE *f = std::fopen(path, "a");
  if (!f) return HELLA_ERR_INVALID_ARG;
  bool ok = std::fseek(f, 0, SEEK_END) == 0;
  const long sz = ok ? std::ftell(f) : -1;
  ok = ok && sz >= 0;
  if (ok && sz == 0) ok = std::fprintf(f, "%s\n", HELLA_CAND_FILE_HEADER) > 0;
  char line[256];
  for (int i = 0; ok && i < n; ++i) {
    const int k = cand_line(c[i], samp0, dms, ndms, time_resolution, line, sizeof(line));
    ok = k > 0 && std::fwrite(line, 1, (size_t)k, f) == (size_t)k;
  }
  ok = (std::fclose(f) == 0) && ok;
  return ok ? HELLA_OK : HELLA_ERR_STATE;
}

hella_status hella_cands_coincidencer(int gulp_number, const char *utc_start, const char *picoseconds,
                                      const char *tsamp, const hella_cand *c, int n, long samp0,
                                      const float *dms, int ndms, double time_resolution, char *buf,
                                      size_t cap, size_t *len) {
  if (!buf || !len || n < 0 || (n > 0 && (!c || !dms))) return HELLA_ERR_INVALID_ARG;
  int k;
  if (utc_start)
    k = std::snprintf(buf, cap, "%d %s %s %s\n", gulp_number, utc_start, picoseconds ? picoseconds : "",
                      tsamp ? tsamp : "");
  else
    k = std::snprintf(buf, cap, "%d\n", gulp_number);
  if (k < 0 || (size_t)k >= cap) return HELLA_ERR_BUDGET;
  *len = (size_t)k;
  return format_lines(c, n, samp0, dms, ndms, time_resolution, buf, cap, len);
}

namespace {

// Waits until fd is ready for `events` (POLLOUT); false on timeout or error.
bool wait_fd(int fd, short events, int timeout_ms) {
  pollfd pf{fd, events, 0};
  for (;;) {
    const int r = poll(&pf, 1, timeout_ms);
    if (r > 0) return (pf.revents & (POLLERR | POLLHUP | POLLNVAL)) == 0 || (pf.revents & events);
    if (r == 0) return false;
    if (errno != EINTR) return false;
  }
}

hella_status send_on(int fd, const sockaddr_in &addr, const char *msg, size_t len, int timeout_ms) {
  if (timeout_ms > 0) {
    const int fl = fcntl(fd, F_GETFL, 0);
    if (fl < 0 || fcntl(fd, F_SETFL, fl | O_NONBLOCK) != 0) return HELLA_ERR_IO;
  }
  if (connect(fd, reinterpret_cast<const sockaddr *>(&addr), sizeof addr) != 0) {
    if (timeout_ms <= 0 || errno != EINPROGRESS || !wait_fd(fd, POLLOUT, timeout_ms)) return HELLA_ERR_IO;
    int err = 0;
    socklen_t el = sizeof err;
    if (getsockopt(fd, SOL_SOCKET, SO_ERROR, &err, &el) != 0 || err != 0) return HELLA_ERR_IO;
  }
  size_t at = 0;
  while (at < len) {
    const ssize_t k = send(fd, msg + at, len - at, MSG_NOSIGNAL);
    if (k > 0) {
      at += (size_t)k;
    } else if (k < 0 && errno == EINTR) {
      continue;
    } else if (k < 0 && (errno == EAGAIN || errno == EWOULDBLOCK) && timeout_ms > 0) {
      if (!wait_fd(fd, POLLOUT, timeout_ms)) return HELLA_ERR_IO;
    } else {
      return HELLA_ERR_IO;
    }
  }
  return HELLA_OK;
}

}  // namespace

hella_status hella_cands_send(const char *host, int port, const char *msg, size_t len, int timeout_ms) {
  if (!host || (!msg && len) || port < 1 || port > 65535) return HELLA_ERR_INVALID_ARG;
  sockaddr_in addr;
  std::memset(&addr, 0, sizeof addr);
  addr.sin_family = AF_INET;
  addr.sin_port = htons((uint16_t)port);
  if (inet_pton(AF_INET, host, &addr.sin_addr) != 1) return HELLA_ERR_INVALID_ARG;
  const int fd = socket(AF_INET, SOCK_STREAM, 0);
  if (fd < 0) return HELLA_ERR_IO;
  const hella_status st = send_on(fd, addr, msg, len, timeout_ms);
  const int cr = close(fd);
  return st != HELLA_OK ? st : (cr == 0 ? HELLA_OK : HELLA_ERR_IO);
}

// ---------------------------------------------------------- clustering

hella_status hella_cluster(const hella_cand *in, int n, int dsamp, int ddm, int dwidth, hella_cand *out,
                           int *nout, int *labels) {
  if (n < 0 || (n > 0 && (!in || !out)) || !nout || dsamp < 0 || ddm < 0 || dwidth < 0)
    return HELLA_ERR_INVALID_ARG;
  std::vector<int> parent(n), order(n);
  std::iota(parent.begin(), parent.end(), 0);
  std::iota(order.begin(), order.end(), 0);
  std::function<int(int)> root = [&](int i) {
    while (parent[i] != i) {
      parent[i] = parent[parent[i]];
      i = parent[i];
    }
    return i;
  };
  std::sort(order.begin(), order.end(), [&](int a, int b) {
    if (in[a].beam != in[b].beam) return in[a].beam < in[b].beam;
    if (in[a].samp != in[b].samp) return in[a].samp < in[b].samp;
    return a < b;
  });
  for (int x = 0; x < n; ++x) {
    const hella_cand &a = in[order[x]];
    for (int y = x + 1; y < n; ++y) {
      const hella_cand &b = in[order[y]];
      if (b.beam != a.beam || (long)b.samp - a.samp > dsamp) break;
      if (std::abs(b.dm_idx - a.dm_idx) <= ddm && std::abs(b.width - a.width) <= dwidth) {
        const int ra = root(order[x]), rb = root(order[y]);
        if (ra != rb) parent[std::max(ra, rb)] = std::min(ra, rb);
      }
    }
  }
  // representatives: highest snr, earliest index on ties; clusters in order of first member
  std::vector<int> best(n, -1), index(n, -1);
  int k = 0;
  for (int i = 0; i < n; ++i) {
    const int r = root(i);
    if (best[r] < 0 || in[i].snr > in[best[r]].snr) best[r] = i;
  }
  for (int i = 0; i < n; ++i) {
    const int r = root(i);
    if (index[r] < 0) {
      index[r] = k;
      out[k++] = in[best[r]];
    }
    if (labels) labels[i] = index[r];
  }
  *nout = k;
  return HELLA_OK;
}

}  // extern "C"

// ------------------------------------------------------ flag statistics

struct hella_flagstats {
  int nchan = 0, ntime = 0;
  std::vector<float> prev;
  std::vector<long> counts;
};

extern "C" {

hella_status hella_flagstats_create(hella_flagstats **s, int nchan, int ntime) {
  if (!s || nchan < 1 || ntime < 1) return HELLA_ERR_INVALID_ARG;
  hella_flagstats *f = new (std::nothrow) hella_flagstats;
  if (!f) return HELLA_ERR_ALLOC;
  f->nchan = nchan;
  f->ntime = ntime;
  f->prev.assign(nchan, 0.f);
  f->counts.assign(nchan, 0);
  *s = f;
  return HELLA_OK;
}

void hella_flagstats_destroy(hella_flagstats *s) { delete s; }

hella_status hella_flagstats_update(hella_flagstats *s, const float *cum) {
  if (!s || !cum) return HELLA_ERR_INVALID_ARG;
  for (int c = 0; c < s->nchan; ++c) {
    s->counts[c] += (int)(1. * s->ntime * (cum[c] - s->prev[c]));
    s->prev[c] = cum[c];
  }
  return HELLA_OK;
}

hella_status hella_flagstats_counts(const hella_flagstats *s, long *counts) {
  if (!s || !counts) return HELLA_ERR_INVALID_ARG;
  std::copy(s->counts.begin(), s->counts.end(), counts);
  return HELLA_OK;
}

hella_status hella_flagstats_append(const hella_flagstats *s, const char *path) {
  if (!s || !path) return HELLA_ERR_INVALID_ARG;
  FILE *f = std::fopen(path, "a");
  if (!f) return HELLA_ERR_INVALID_ARG;
  bool ok = true;
  for (int c = 0; ok && c < s->nchan; ++c) ok = std::fprintf(f, "%ld\n", s->counts[c]) > 0;
  ok = (std::fclose(f) == 0) && ok;
  return ok ? HELLA_OK : HELLA_ERR_STATE;
}

}  // extern "C"

// ------------------------------------------------------ in-process ring

struct hella_ring {
  size_t block_bytes = 0;
  int nblocks = 0;
  bool pinned = false;
  uint8_t *mem = nullptr;
  std::vector<size_t> fill;   // bytes in each filled block
  int w = 0, r = 0, filled = 0;
  bool writing = false, reading = false, eod = false;
  std::string header;
  bool have_header = false;
  std::mutex mu;
  std::condition_variable cv;
};

namespace {

template <typename Pred>
bool wait_for(hella_ring *r, std::unique_lock<std::mutex> &lk, int timeout_ms, Pred pred) {
  if (timeout_ms < 0) {
    r->cv.wait(lk, pred);
    return true;
  }
  return r->cv.wait_for(lk, std::chrono::milliseconds(timeout_ms), pred);
}

}  // namespace

extern "C" {

hella_status hella_ring_create(hella_ring **out, size_t block_bytes, int nblocks, int pinned) {
  if (!out || block_bytes == 0 || nblocks < 2) return HELLA_ERR_INVALID_ARG;
  *out = nullptr;
  hella_ring *r = new (std::nothrow) hella_ring;
  if (!r) return HELLA_ERR_ALLOC;
  r->block_bytes = block_bytes;
  r->nblocks = nblocks;
  r->pinned = pinned != 0;
  const size_t total = block_bytes * (size_t)nblocks;
  if (r->pinned) {
    if (cudaHostAlloc((void **)&r->mem, total, cudaHostAllocDefault) != cudaSuccess) {
      cudaGetLastError();
      delete r;
      return HELLA_ERR_ALLOC;
    }
  } else {
    r->mem = static_cast<uint8_t *>(std::malloc(total));
    if (!r->mem) {
      delete r;
      return HELLA_ERR_ALLOC;
    }
  }
  r->fill.assign(nblocks, 0);
  *out = r;
  return HELLA_OK;
}

void hella_ring_destroy(hella_ring *r) {
  if (!r) return;
  if (r->pinned)
    cudaFreeHost(r->mem);
  else
    std::free(r->mem);
  delete r;
}

size_t hella_ring_block_bytes(const hella_ring *r) { return r ? r->block_bytes : 0; }

hella_status hella_ring_write_header(hella_ring *r, const char *header, size_t len) {
  if (!r || !header) return HELLA_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(r->mu);
  if (r->have_header) return HELLA_ERR_STATE;
  r->header.assign(header, len);
  r->have_header = true;
  r->cv.notify_all();
  return HELLA_OK;
}

hella_status hella_ring_read_header(hella_ring *r, char *out, size_t cap, size_t *len, int timeout_ms) {
  if (!r || !len) return HELLA_ERR_INVALID_ARG;
  std::unique_lock<std::mutex> lk(r->mu);
  if (!wait_for(r, lk, timeout_ms, [&] { return r->have_header; })) return HELLA_ERR_TIMEOUT;
  *len = r->header.size();
  if (out && cap) {
    const size_t k = std::min(cap - 1, r->header.size());
    std::memcpy(out, r->header.data(), k);
    out[k] = '\0';
  }
  return HELLA_OK;
}

hella_status hella_ring_open_write(hella_ring *r, uint8_t **block, int timeout_ms) {
  if (!r || !block) return HELLA_ERR_INVALID_ARG;
  std::unique_lock<std::mutex> lk(r->mu);
  if (r->writing || r->eod) return HELLA_ERR_STATE;
  if (!wait_for(r, lk, timeout_ms, [&] { return r->filled < r->nblocks; })) return HELLA_ERR_TIMEOUT;
  r->writing = true;
  *block = r->mem + (size_t)r->w * r->block_bytes;
  return HELLA_OK;
}

hella_status hella_ring_mark_filled(hella_ring *r, size_t nbytes) {
  if (!r || nbytes > r->block_bytes) return HELLA_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(r->mu);
  if (!r->writing) return HELLA_ERR_STATE;
  r->fill[r->w] = nbytes;
  r->w = (r->w + 1) % r->nblocks;
  r->filled++;
  r->writing = false;
  r->cv.notify_all();
  return HELLA_OK;
}

hella_status hella_ring_end(hella_ring *r) {
  if (!r) return HELLA_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(r->mu);
  r->eod = true;
  r->cv.notify_all();
  return HELLA_OK;
}

hella_status hella_ring_open_read(hella_ring *r, const uint8_t **block, size_t *nbytes, int timeout_ms) {
  if (!r || !block || !nbytes) return HELLA_ERR_INVALID_ARG;
  std::unique_lock<std::mutex> lk(r->mu);
  if (r->reading) return HELLA_ERR_STATE;
  if (!wait_for(r, lk, timeout_ms, [&] { return r->filled > 0 || r->eod; })) return HELLA_ERR_TIMEOUT;
  if (r->filled == 0) {  // end of data
    *block = nullptr;
    *nbytes = 0;
    return HELLA_OK;
  }
  r->reading = true;
  *block = r->mem + (size_t)r->r * r->block_bytes;
  *nbytes = r->fill[r->r];
  return HELLA_OK;
}

hella_status hella_ring_mark_cleared(hella_ring *r) {
  if (!r) return HELLA_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(r->mu);
  if (!r->reading) return HELLA_ERR_STATE;
  r->r = (r->r + 1) % r->nblocks;
  r->filled--;
  r->reading = false;
  r->cv.notify_all();
  return HELLA_OK;
}

hella_status hella_header_get(const char *header, size_t len, const char *key, char *val, size_t cap) {
  if (!header || !key || !val || cap == 0) return HELLA_ERR_INVALID_ARG;
  const size_t end = std::find(header, header + len, '\0') - header;
  const std::string text(header, end), want(key);
  size_t pos = 0;
  bool found = false;
  std::string value;
  while (pos < text.size()) {
    size_t nl = text.find('\n', pos);
    if (nl == std::string::npos) nl = text.size();
    const std::string line = text.substr(pos, nl - pos);
    pos = nl + 1;
    if (line.empty()) continue;
    const size_t sp = line.find(' ');
    if (sp == std::string::npos) break;  // an invalid line ends the parse (dada.cpp:66-71)
    if (line.compare(0, sp, want) == 0 && sp == want.size()) {  // a later line wins, as in a map
      const size_t vp = line.find_first_not_of(' ', sp);
      value = vp == std::string::npos ? std::string() : line.substr(vp);
      found = true;
    }
  }
  if (!found) return HELLA_ERR_INVALID_ARG;
  std::snprintf(val, cap, "%s", value.c_str());
  return HELLA_OK;
}

}  // extern "C"
