// autotune.cpp -- the tuning cache of the march kernels' launch shapes.
//
// The library times candidate shapes of the one-element-per-thread kernel
// on the device the first time it meets a class of problems (see
// sem2d_gpu.cu, tune_march) and keeps the fastest here, so that later
// handles of the same class -- in this process or another -- start with it.
// The reference has no counterpart: it is serial (solver.f90:307-315).
//
// The cache is a text file of JSON objects, one per line:
//   {"key": "march ndof=2 mat=2 nodes=2^28 members=2^8 sm=152", "chunk_rows": 32,
//    "warps_per_cta": 1, "ms_per_step": 4.52}
// A later line with the same key replaces an earlier one.  Writes go to a
// temporary file renamed over the cache, so readers never see half a file.
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <sys/stat.h>
#include <unistd.h>

#include "../../include/sem2d_host.h"

namespace {

// value of "name": <number> in a line, or false
bool field(const std::string &line, const char *name, double *v) {
  const std::string pat = std::string("\"") + name + "\":";
  const size_t p = line.find(pat);
  if (p == std::string::npos) return false;
  const char *s = line.c_str() + p + pat.size();
  char *end = nullptr;
  *v = std::strtod(s, &end);
  return end != s;
}

bool key_of(const std::string &line, std::string *key) {
  const std::string pat = "\"key\": \"";
  const size_t p = line.find(pat);
  if (p == std::string::npos) return false;
  const size_t q = line.find('"', p + pat.size());
  if (q == std::string::npos) return false;
  *key = line.substr(p + pat.size(), q - p - pat.size());
  return true;
}

bool parse_entry(const std::string &line, std::string *key, sem2d_tune_entry *e) {
  double cz, w, ms;
  if (!key_of(line, key) || !field(line, "chunk_rows", &cz) || !field(line, "warps_per_cta", &w) ||
      !field(line, "ms_per_step", &ms))
    return false;
  e->chunk_rows = int(cz);
  e->warps_per_cta = int(w);
  e->ms_per_step = ms;
  return e->chunk_rows > 0 && (e->warps_per_cta == 1 || e->warps_per_cta == 2 || e->warps_per_cta == 4);
}

std::map<std::string, sem2d_tune_entry> read_all(const char *path) {
  std::map<std::string, sem2d_tune_entry> out;
  FILE *f = std::fopen(path, "r");
  if (!f) return out;
  char buf[1024];
  while (std::fgets(buf, sizeof(buf), f)) {
    std::string key;
    sem2d_tune_entry e;
    if (parse_entry(buf, &key, &e)) out[key] = e;
  }
  std::fclose(f);
  return out;
}

// mkdir -p of the directory part of path
void make_parent(const std::string &path) {
  for (size_t p = path.find('/', 1); p != std::string::npos; p = path.find('/', p + 1))
    mkdir(path.substr(0, p).c_str(), 0755);
}

int ilog2(long long v) {
  int k = 0;
  while (v > 1) {
    v >>= 1;
    ++k;
  }
  return k;
}

}  // namespace

extern "C" {

int sem2d_tune_cache_path(char *buf, int n) {
  std::string path;
  if (const char *e = std::getenv("SEM2D_TUNE_CACHE")) {
    path = e;
  } else if (const char *x = std::getenv("XDG_CACHE_HOME")) {
    path = std::string(x) + "/sem2dpack_gb300/tune.json";
  } else if (const char *h = std::getenv("HOME")) {
    path = std::string(h) + "/.cache/sem2dpack_gb300/tune.json";
  } else {
    return SEM2D_E_STATE;
  }
  if (!buf || n <= int(path.size())) return int(path.size()) + 1;
  std::memcpy(buf, path.c_str(), path.size() + 1);
  return SEM2D_OK;
}

int sem2d_tune_key(int ndof, int mat_layout, long long nodes, int members, int nsm, char *buf, int n) {
  if (!buf || n <= 0 || ndof < 1 || ndof > 2 || nodes <= 0 || members < 0 || nsm <= 0) return SEM2D_E_ARG;
  const int w = std::snprintf(buf, size_t(n), "march ndof=%d mat=%d nodes=2^%d members=2^%d sm=%d", ndof, mat_layout,
                              ilog2(nodes), ilog2(members > 0 ? members : 1), nsm);
  return w < n ? SEM2D_OK : SEM2D_E_ARG;
}

int sem2d_tune_lookup(const char *path, const char *key, sem2d_tune_entry *out) {
  if (!path || !key || !out) return SEM2D_E_ARG;
  const auto all = read_all(path);
  const auto it = all.find(key);
  if (it == all.end()) return 0;
  *out = it->second;
  return 1;
}

int sem2d_tune_record(const char *path, const char *key, const sem2d_tune_entry *e) {
  if (!path || !key || !e || std::strchr(key, '"') || std::strchr(key, '\n')) return SEM2D_E_ARG;
  auto all = read_all(path);
  all[key] = *e;
  const std::string p(path);
  make_parent(p);
  const std::string tmp = p + ".tmp" + std::to_string(getpid());
  FILE *f = std::fopen(tmp.c_str(), "w");
  if (!f) return SEM2D_E_STATE;
  for (const auto &kv : all)
    std::fprintf(f,
                 "{\"key\": \"%s\", \"chunk_rows\": %d, \"warps_per_cta\": %d, \"ms_per_step\": %.6g}\n",
                 kv.first.c_str(), kv.second.chunk_rows, kv.second.warps_per_cta, kv.second.ms_per_step);
  const bool ok = std::fclose(f) == 0;
  if (!ok || std::rename(tmp.c_str(), p.c_str()) != 0) {
    std::remove(tmp.c_str());
    return SEM2D_E_STATE;
  }
  return SEM2D_OK;
}

int sem2d_tune_select(const sem2d_tune_entry *cands, int n, double keep_margin) {
  if (!cands || n <= 0) return SEM2D_E_ARG;
  // the fastest; candidate 0 (the analytic default) is kept unless another
  // is faster by more than keep_margin (a fraction), so that timing noise
  // does not flip the shape
  int best = 0;
  for (int k = 1; k < n; ++k)
    if (cands[k].ms_per_step > 0 && cands[k].ms_per_step < cands[best].ms_per_step) best = k;
  if (best != 0 && !(cands[best].ms_per_step < cands[0].ms_per_step * (1.0 - keep_margin))) best = 0;
  return best;
}

}  // extern "C"
