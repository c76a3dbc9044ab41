// g4s_formats.cu — binary files of the library: the spike raster (streamed chunk by chunk
// by a writer thread while the GPU computes the next chunk) and the connectivity tables
// (a checkpoint that skips table generation).  Host code only.
//
// The reference writes its raster as text, one "t i" row per spike, from a host scan of a
// per-step flag array (gpu4snn.cu:1256-1261), and regenerates its tables on the host for
// every run (gpu4snn.cu:862-911).  The text files are still written by
// g4s_net_write_results; these are the compact alternatives for long or large runs.
//
// Raster file (little-endian):
//   char[8] "G4SRAS01"; int64 n; int64 first step; int64 steps; int64 spikes;
//   then chunks until the end of the file: int32 cs; int32 counts[cs]; int32 ids[sum counts]
//   (ids ascending within each step).  steps and spikes are written when the file is
//   closed; a reader of a file that was not closed takes the chunks as they are.
// Tables file:
//   char[8] "G4STAB01"; int64 n; int32 nsyn; int32 stride; uint64 seed; int32 conn_law;
//   int32 self_loops; int32 exc_permille; int32 flags (1 = rows sorted by target);
//   int32 reserved[2]; int32 idx[n][stride]; float w[n][stride].
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/gpu4snn.h"
#include "g4s_internal.h"

namespace g4s {

static_assert(sizeof(TableHeader) == 48, "tables header layout");

struct RasterFile {
  struct Chunk {
    std::vector<int32_t> counts, ids;
  };
  FILE *f = nullptr;
  std::string path;
  int64_t n = 0, t0 = 0, steps = 0, spikes = 0;
  std::mutex mu;
  std::condition_variable cv;
  std::deque<Chunk> q;
  bool stop = false, failed = false;
  std::thread th;

  void loop() {
    for (;;) {
      Chunk c;
      {
        std::unique_lock<std::mutex> lk(mu);
        cv.wait(lk, [&] { return stop || !q.empty(); });
        if (q.empty()) return;
        c = std::move(q.front());
        q.pop_front();
      }
      const int32_t cs = (int32_t)c.counts.size();
      bool ok = fwrite(&cs, 4, 1, f) == 1 && fwrite(c.counts.data(), 4, c.counts.size(), f) == c.counts.size() &&
                (c.ids.empty() || fwrite(c.ids.data(), 4, c.ids.size(), f) == c.ids.size());
      if (!ok) {
        std::lock_guard<std::mutex> lk(mu);
        failed = true;
      }
    }
  }
};

static bool write_raster_header(FILE *f, int64_t n, int64_t t0, int64_t steps, int64_t spikes) {
  const int64_t h[4] = {n, t0, steps, spikes};
  return fseek(f, 0, SEEK_SET) == 0 && fwrite("G4SRAS01", 1, 8, f) == 8 && fwrite(h, 8, 4, f) == 4;
}

int raster_open(const char *path, int64_t n, int64_t t0, RasterFile **out) {
  *out = nullptr;
  FILE *f = fopen(path, "wb");
  if (!f) return set_error(G4S_ERR_IO, std::string("cannot open ") + path);
  if (!write_raster_header(f, n, t0, 0, 0)) {
    fclose(f);
    return set_error(G4S_ERR_IO, std::string("cannot write ") + path);
  }
  RasterFile *r = new RasterFile;
  r->f = f;
  r->path = path;
  r->n = n;
  r->t0 = t0;
  r->th = std::thread([r] { r->loop(); });
  *out = r;
  return G4S_OK;
}

void raster_push(RasterFile *r, const int32_t *counts, int cs, const int32_t *ids, int64_t nids) {
  RasterFile::Chunk c;
  c.counts.assign(counts, counts + cs);
  c.ids.assign(ids, ids + nids);
  {
    std::lock_guard<std::mutex> lk(r->mu);
    r->steps += cs;
    r->spikes += nids;
    r->q.push_back(std::move(c));
  }
  r->cv.notify_one();
}

int raster_close(RasterFile *r) {
  if (!r) return G4S_OK;
  {
    std::lock_guard<std::mutex> lk(r->mu);
    r->stop = true;
  }
  r->cv.notify_one();
  r->th.join();
  bool ok = !r->failed && fflush(r->f) == 0 && write_raster_header(r->f, r->n, r->t0, r->steps, r->spikes);
  ok = fclose(r->f) == 0 && ok;
  const std::string path = r->path;
  delete r;
  return ok ? G4S_OK : set_error(G4S_ERR_IO, "writing " + path + " failed");
}

int raster_write_all(const char *path, int64_t n, int64_t t0, const std::vector<int32_t> &counts,
                     const std::vector<int32_t> &ids) {
  FILE *f = fopen(path, "wb");
  if (!f) return set_error(G4S_ERR_IO, std::string("cannot open ") + path);
  const int32_t cs = (int32_t)counts.size();
  bool ok = write_raster_header(f, n, t0, (int64_t)counts.size(), (int64_t)ids.size()) &&
            (cs == 0 || (fwrite(&cs, 4, 1, f) == 1 && fwrite(counts.data(), 4, counts.size(), f) == counts.size() &&
                         (ids.empty() || fwrite(ids.data(), 4, ids.size(), f) == ids.size())));
  ok = fclose(f) == 0 && ok;
  return ok ? G4S_OK : set_error(G4S_ERR_IO, std::string("writing ") + path + " failed");
}

int tables_write(const char *path, const TableHeader &h, const int32_t *idx, const float *w) {
  FILE *f = fopen(path, "wb");
  if (!f) return set_error(G4S_ERR_IO, std::string("cannot open ") + path);
  const size_t cnt = (size_t)h.n * (size_t)h.stride;
  bool ok = fwrite("G4STAB01", 1, 8, f) == 8 && fwrite(&h, sizeof h, 1, f) == 1 &&
            fwrite(idx, 4, cnt, f) == cnt && fwrite(w, 4, cnt, f) == cnt;
  ok = fclose(f) == 0 && ok;
  return ok ? G4S_OK : set_error(G4S_ERR_IO, std::string("writing ") + path + " failed");
}

int tables_read_header(const char *path, TableHeader *h) {
  FILE *f = fopen(path, "rb");
  if (!f) return set_error(G4S_ERR_IO, std::string("cannot open ") + path);
  char magic[8];
  const bool ok = fread(magic, 1, 8, f) == 8 && fread(h, sizeof *h, 1, f) == 1;
  fclose(f);
  if (!ok || memcmp(magic, "G4STAB01", 8) != 0) return set_error(G4S_ERR_IO, std::string(path) + ": not a tables file");
  if (h->n < 1 || h->nsyn < 1 || h->stride < h->nsyn || h->stride % 4 != 0)
    return set_error(G4S_ERR_IO, std::string(path) + ": bad tables header");
  return G4S_OK;
}

int tables_read(const char *path, const TableHeader &h, int32_t *idx, float *w) {
  FILE *f = fopen(path, "rb");
  if (!f) return set_error(G4S_ERR_IO, std::string("cannot open ") + path);
  const size_t cnt = (size_t)h.n * (size_t)h.stride;
  bool ok = fseek(f, 8 + (long)sizeof(TableHeader), SEEK_SET) == 0 && fread(idx, 4, cnt, f) == cnt &&
            fread(w, 4, cnt, f) == cnt;
  fclose(f);
  return ok ? G4S_OK : set_error(G4S_ERR_IO, std::string(path) + ": truncated tables file");
}

}  // namespace g4s
