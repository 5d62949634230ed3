// Autotuned launch shapes (see autotune.h).
//
// Cache file: S2LET_GPU_AUTOTUNE_CACHE, else $XDG_CACHE_HOME/s2let_gb300/
// autotune.txt, else $HOME/.cache/s2let_gb300/autotune.txt.  Each line:
//   <GPU name, blanks as '_'> <family> <a> <b> <c> <choice> <best ms> <default ms>
// Lines of other GPU models are ignored; a later line for a key replaces an
// earlier one.  The file is read when tuning is first needed and appended to
// after each new measurement; an unwritable location only loses persistence.
#include <sys/stat.h>

#include <array>
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "autotune.h"
#include "common.h"
#include "runtime.h"

namespace s2g {

namespace {

constexpr int kTuneReps = 3;

struct Entry {
  int choice = 0;
  double best_ms = 0, def_ms = 0;
};

using Key = std::array<int, 4>;

std::mutex g_mu;
std::map<Key, Entry> g_table;
bool g_loaded = false;
int g_mode = -1;  // -1: not yet read from the environment
std::string g_gpu;

int mode_locked() {
  if (g_mode < 0) {
    const char *e = getenv("S2LET_GPU_AUTOTUNE");
    g_mode = (e && e[0] == '1') ? 1 : 0;
  }
  return g_mode;
}

std::string cache_path() {
  const char *e = getenv("S2LET_GPU_AUTOTUNE_CACHE");
  if (e && e[0]) return e;
  const char *x = getenv("XDG_CACHE_HOME");
  if (x && x[0]) return std::string(x) + "/s2let_gb300/autotune.txt";
  const char *h = getenv("HOME");
  return std::string(h && h[0] ? h : ".") + "/.cache/s2let_gb300/autotune.txt";
}

// directories of `path` created as needed (mkdir -p of the parent)
void make_parent(const std::string &path) {
  for (size_t i = 1; i < path.size(); ++i)
    if (path[i] == '/') {
      const std::string d = path.substr(0, i);
      if (mkdir(d.c_str(), 0755) != 0 && errno != EEXIST) return;
    }
}

std::string gpu_name() {
  int dev = 0;
  cudaDeviceProp pr;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&pr, dev) != cudaSuccess) return "unknown";
  std::string s = pr.name;
  for (char &ch : s)
    if (ch == ' ' || ch == '\t') ch = '_';
  return s;
}

void load_locked() {
  if (g_loaded) return;
  g_loaded = true;
  g_gpu = gpu_name();
  FILE *f = fopen(cache_path().c_str(), "r");
  if (!f) return;
  char name[256];
  Key k;
  Entry en;
  while (fscanf(f, "%255s %d %d %d %d %d %lf %lf", name, &k[0], &k[1], &k[2], &k[3], &en.choice, &en.best_ms,
                &en.def_ms) == 8)
    if (g_gpu == name && en.choice >= 0) g_table[k] = en;
  fclose(f);
}

void save_locked(const Key &k, const Entry &en) {
  const std::string path = cache_path();
  make_parent(path);
  FILE *f = fopen(path.c_str(), "a");
  if (!f) return;
  fprintf(f, "%s %d %d %d %d %d %.6f %.6f\n", g_gpu.c_str(), k[0], k[1], k[2], k[3], en.choice, en.best_ms,
          en.def_ms);
  fclose(f);
}

}  // namespace

int autotune_mode() {
  std::lock_guard<std::mutex> lk(g_mu);
  return mode_locked();
}

int tuned(int family, int a, int b, int c, int ncand, int def, cudaStream_t st,
          const std::function<void(int)> &trial) {
  if (ncand <= 1) return 0;
  const Key key{family, a, b, c};
  std::lock_guard<std::mutex> lk(g_mu);
  if (mode_locked() == 0) return def;
  load_locked();
  auto it = g_table.find(key);
  if (it != g_table.end() && it->second.choice < ncand) return it->second.choice;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  S2G_CUDA(cudaStreamIsCapturing(st, &cap));
  if (cap != cudaStreamCaptureStatusNone) return def;
  cudaEvent_t e0, e1;
  S2G_CUDA(cudaEventCreate(&e0));
  S2G_CUDA(cudaEventCreate(&e1));
  Entry en;
  en.best_ms = 1e300;
  try {
    for (int i = 0; i < ncand; ++i) {
      trial(i);  // warm-up (first launch of the instantiation, caches)
      S2G_CUDA(cudaEventRecord(e0, st));
      for (int r = 0; r < kTuneReps; ++r) trial(i);
      S2G_CUDA(cudaEventRecord(e1, st));
      S2G_CUDA(cudaEventSynchronize(e1));
      float ms = 0.f;
      S2G_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      const double t = ms / kTuneReps;
      if (i == def) en.def_ms = t;
      if (t < en.best_ms) {
        en.best_ms = t;
        en.choice = i;
      }
    }
  } catch (...) {
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    throw;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  g_table[key] = en;
  save_locked(key, en);
  return en.choice;
}

}  // namespace s2g

extern "C" {

// 1: tune unseen launch shapes and use the recorded choices; 0: the built-in
// choices.  Returns the previous mode.
int s2let_gpu_autotune(int mode) {
  std::lock_guard<std::mutex> lk(s2g::g_mu);
  const int old = s2g::mode_locked();
  s2g::g_mode = mode ? 1 : 0;
  return old;
}

// The choices recorded in this process or read from the cache file:
// keys[5 i + 0..4] = {family, a, b, c, choice}, ms[2 i + 0..1] = {best
// milliseconds, milliseconds of the built-in choice} for i < returned count
// (at most max entries written).
int s2let_gpu_autotune_entries(int *keys, double *ms, int max) {
  std::lock_guard<std::mutex> lk(s2g::g_mu);
  s2g::load_locked();
  int n = 0;
  for (const auto &kv : s2g::g_table) {
    if (n < max) {
      for (int j = 0; j < 4; ++j) keys[5 * n + j] = kv.first[j];
      keys[5 * n + 4] = kv.second.choice;
      ms[2 * n] = kv.second.best_ms;
      ms[2 * n + 1] = kv.second.def_ms;
    }
    ++n;
  }
  return n;
}

}  // extern "C"
