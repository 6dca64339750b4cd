// Tile autotuner of the mixed path: for every Nk bucket of a context and every
// tunable GEMM kind (exchange products, commutators, sources) it times the
// engine's two N tiles (256: one accumulator set per SM, 128: two in flight) on the
// context's own workspace and keeps the faster; the choices are cached in a JSON
// file keyed by the device and the context's buckets, so that later contexts of the
// same shape load them instead of timing.
//
// File format (one entry per line, so that entries can be replaced line by line):
//   {"sbe_autotune": 1, "entries": [
//   {"key": "<device>|sm<cc>|<SMs>|f<flags>|<nk>x<nw>;...", "buckets": [{"nk": N,
//    "nw": W, "exchange_bn": B, "commutator_bn": B, "sources_bn": B, "hh_split": S,
//    "ms": {...}}, ...]},
//   ...
//   ]}
#include <cstdio>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "sbe_mixed.cuh"

namespace {

using namespace sbe;

constexpr int kKinds[3] = {JK_EXCH, JK_FULL, JK_SRC};
constexpr const char* kNames[3] = {"exchange", "commutator", "sources"};
constexpr int kTiles[2] = {256, 128};

int key_of(SbeCtx* c, std::string* key) {
  int dev = 0;
  cudaDeviceProp p{};
  int rc = cuda_check(cudaGetDevice(&dev), "sbe_autotune: device");
  if (!rc) rc = cuda_check(cudaGetDeviceProperties(&p, dev), "sbe_autotune: device properties");
  if (rc) return rc;
  std::ostringstream k;
  k << p.name << "|sm" << p.major << p.minor << "|" << p.multiProcessorCount << "|f" << std::hex
    << c->wires[0].flags << std::dec << "|";
  for (Mixed* m : all_of(c)->b) k << m->nk << "x" << m->nw << ";";
  std::string s = k.str();
  for (char& ch : s)
    if (ch == '"' || ch == '\\' || ch == '\n') ch = '_';
  *key = s;
  return SBE_OK;
}

std::string key_in(const std::string& line) {
  const std::string tag = "{\"key\": \"";
  const size_t a = line.find(tag);
  if (a == std::string::npos) return "";
  const size_t b = line.find('"', a + tag.size());
  return b == std::string::npos ? "" : line.substr(a + tag.size(), b - a - tag.size());
}

std::vector<std::string> entry_lines(const char* path) {
  std::vector<std::string> out;
  std::ifstream f(path);
  std::string line;
  while (std::getline(f, line))
    if (!key_in(line).empty()) {
      while (!line.empty() && (line.back() == ',' || line.back() == ' ')) line.pop_back();
      out.push_back(line);
    }
  return out;
}

// the choices of the entry with this key; false if absent or not matching the buckets
bool load(const char* path, const std::string& key, MixedAll* A) {
  for (const std::string& line : entry_lines(path)) {
    if (key_in(line) != key) continue;
    std::vector<int> v;
    size_t pos = 0;
    const std::string tag = "{\"nk\": ", htag = "\"hh_split\": ";
    while ((pos = line.find(tag, pos)) != std::string::npos) {
      int nk, nw, e, f, s;
      if (std::sscanf(line.c_str() + pos,
                      "{\"nk\": %d, \"nw\": %d, \"exchange_bn\": %d, \"commutator_bn\": %d, "
                      "\"sources_bn\": %d",
                      &nk, &nw, &e, &f, &s) != 5)
        return false;
      // optional hi*hi split of this bucket (before the next bucket's entry)
      const size_t next = line.find(tag, pos + tag.size());
      const size_t hp = line.find(htag, pos);
      int hs = nk >= 1024 ? 8 : (nk >= 256 ? 4 : 2);   // the default of mixed_ensure
      if (hp != std::string::npos && (next == std::string::npos || hp < next) &&
          std::sscanf(line.c_str() + hp + htag.size(), "%d", &hs) != 1)
        return false;
      v.insert(v.end(), {nk, nw, e, f, s, hs});
      pos += tag.size();
    }
    if (v.size() != 6 * A->b.size()) return false;
    for (size_t i = 0; i < A->b.size(); ++i) {
      Mixed* m = A->b[i];
      const int* r = &v[6 * i];
      if (r[0] != m->nk || r[1] != m->nw || r[5] < 1 || r[5] > 8) return false;
      for (int j = 2; j < 5; ++j)
        if (r[j] != 128 && r[j] != 256) return false;
    }
    for (size_t i = 0; i < A->b.size(); ++i) {
      Mixed* m = A->b[i];
      m->bn[JK_EXCH] = v[6 * i + 2];
      m->bn[JK_FULL] = v[6 * i + 3];
      m->bn[JK_SRC] = v[6 * i + 4];
      m->hs = v[6 * i + 5];
    }
    return true;
  }
  return false;
}

int save(const char* path, const std::string& key, const std::string& entry) {
  std::vector<std::string> lines;
  for (const std::string& l : entry_lines(path))
    if (key_in(l) != key) lines.push_back(l);
  lines.push_back(entry);
  const std::string tmp = std::string(path) + ".tmp";
  {
    std::ofstream f(tmp, std::ios::trunc);
    if (!f) return fail(SBE_ERR_ARG, std::string("sbe_autotune: cannot write ") + path);
    f << "{\"sbe_autotune\": 1, \"entries\": [\n";
    for (size_t i = 0; i < lines.size(); ++i) f << lines[i] << (i + 1 < lines.size() ? ",\n" : "\n");
    f << "]}\n";
    if (!f) return fail(SBE_ERR_ARG, std::string("sbe_autotune: cannot write ") + path);
  }
  if (std::rename(tmp.c_str(), path) != 0)
    return fail(SBE_ERR_ARG, std::string("sbe_autotune: cannot replace ") + path);
  return SBE_OK;
}

// mean time (ms) of reps launches of the job list, after one untimed launch
int time_jobs(const std::vector<tc::GemmJob>& jobs, cudaStream_t s, int reps, double* ms) {
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  int rc = launch_jobs(jobs, s);
  cudaEventRecord(a, s);
  for (int i = 0; !rc && i < reps; ++i) rc = launch_jobs(jobs, s);
  cudaEventRecord(b, s);
  if (!rc) rc = cuda_check(cudaEventSynchronize(b), "sbe_autotune: timing");
  float t = 0.f;
  if (!rc) rc = cuda_check(cudaEventElapsedTime(&t, a, b), "sbe_autotune: timing");
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  *ms = t / reps;
  return rc;
}

}  // namespace

// No counterpart in the reference (its wires run one after another): see
// include/sbe_gb300.h.
extern "C" int sbe_autotune(SbeCtx* c, const char* cache_json) {
  if (!c) return fail(SBE_ERR_ARG, "sbe_autotune: null context");
  cudaStream_t s = nullptr;
  int rc = cuda_check(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "sbe_autotune: stream");
  if (rc) return rc;
  rc = mixed_prepare(c, s);
  if (!rc) rc = cuda_check(cudaStreamSynchronize(s), "sbe_autotune: workspace");
  std::string key;
  if (!rc) rc = key_of(c, &key);
  MixedAll* A = rc ? nullptr : all_of(c);
  if (A && cache_json && load(cache_json, key, A)) {
    cudaStreamDestroy(s);
    return SBE_OK;
  }
  const bool have_x = (c->wires[0].flags & SBE_F_EXCITONS) != 0;
  std::ostringstream entry;
  if (A) entry << "{\"key\": \"" << key << "\", \"buckets\": [";
  for (size_t i = 0; A && !rc && i < A->b.size(); ++i) {
    Mixed* m = A->b[i];
    double ms[3][2] = {{0, 0}, {0, 0}, {0, 0}};
    for (int k = 0; !rc && k < 3; ++k) {
      const int kind = kKinds[k];
      if (kind == JK_EXCH && !have_x) {
        m->bn[kind] = 256;
        continue;
      }
      for (int t = 0; !rc && t < 2; ++t) {
        m->bn[kind] = kTiles[t];
        std::vector<tc::GemmJob> jobs;
        bucket_jobs(c, m, kind, jobs);
        rc = time_jobs(jobs, s, 5, &ms[k][t]);
      }
      m->bn[kind] = ms[k][1] < ms[k][0] ? 128 : 256;
    }
    char buf[512];
    std::snprintf(buf, sizeof(buf),
                  "%s{\"nk\": %d, \"nw\": %d, \"exchange_bn\": %d, \"commutator_bn\": %d, "
                  "\"sources_bn\": %d, \"hh_split\": %d, \"ms\": {\"%s\": [%.5f, %.5f], "
                  "\"%s\": [%.5f, %.5f], \"%s\": [%.5f, %.5f]}}",
                  i ? ", " : "", m->nk, m->nw, m->bn[JK_EXCH], m->bn[JK_FULL], m->bn[JK_SRC], m->hs,
                  kNames[0], ms[0][0], ms[0][1], kNames[1], ms[1][0], ms[1][1], kNames[2],
                  ms[2][0], ms[2][1]);
    entry << buf;
  }
  cudaStreamDestroy(s);
  if (rc) return rc;
  // the timing runs touched the engine's error flag only if a wait gave up
  rc = sbe_ctx_check(c, nullptr);
  if (rc) return rc;
  entry << "]}";
  return cache_json ? save(cache_json, key, entry.str()) : SBE_OK;
}

extern "C" int sbe_ctx_tiles(const SbeCtx* cc, int* out, int cap, int* nbuckets) {
  SbeCtx* c = const_cast<SbeCtx*>(cc);
  if (!c || !nbuckets || (cap > 0 && !out)) return fail(SBE_ERR_ARG, "sbe_ctx_tiles: bad arguments");
  MixedAll* A = all_of(c);
  *nbuckets = A ? (int)A->b.size() : 0;
  for (int i = 0; A && i < (int)A->b.size() && 6 * i + 5 < cap; ++i) {
    Mixed* m = A->b[i];
    const int v[6] = {m->nk, m->nw, m->bn[JK_EXCH] ? m->bn[JK_EXCH] : 256,
                      m->bn[JK_FULL] ? m->bn[JK_FULL] : 256, m->bn[JK_SRC] ? m->bn[JK_SRC] : 256,
                      m->hs};
    for (int j = 0; j < 6; ++j) out[6 * i + j] = v[j];
  }
  return SBE_OK;
}
