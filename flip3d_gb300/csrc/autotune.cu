/*
 * autotune.cu — the registry behind autotune.h and its C ABI
 * (flipgpu_set_autotune, flipgpu_autotune_report).
 */
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "autotune.h"
#include "devcommon.cuh"

namespace {

struct Decision {
  int choice = 0;
  std::vector<std::string> names;
  std::vector<float> ms; /* median per candidate, <0 when it failed */
};

std::mutex g_mu;
std::map<std::string, Decision> g_table;
int g_enabled = -1; /* -1: from the environment */

bool enabled() {
  if (g_enabled < 0) {
    const char *e = getenv("FLIPGPU_AUTOTUNE");
    g_enabled = (e && e[0] == '0') ? 0 : 1;
  }
  return g_enabled != 0;
}

} // namespace

namespace autotune {

int choose(const std::string &key, const std::vector<std::string> &names, cudaStream_t st,
           const std::function<cudaError_t(int)> &run) {
  const int n = (int)names.size();
  if (n <= 1) return 0;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_table.find(key);
    if (it != g_table.end()) return it->second.choice;
    if (!enabled()) return 0;
  }
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone)
    return 0;
  Decision d;
  d.names = names;
  d.ms.assign(n, -1.0f);
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess) return 0;
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return 0;
  }
  for (int i = 0; i < n; i++) {
    if (run(i) != cudaSuccess) continue; /* warm-up (and the check that it runs) */
    float t[3];
    bool ok = true;
    for (int r = 0; r < 3 && ok; r++) {
      ok = cudaEventRecord(e0, st) == cudaSuccess && run(i) == cudaSuccess &&
           cudaEventRecord(e1, st) == cudaSuccess && cudaEventSynchronize(e1) == cudaSuccess &&
           cudaEventElapsedTime(&t[r], e0, e1) == cudaSuccess;
    }
    if (!ok) continue;
    std::sort(t, t + 3);
    d.ms[i] = t[1];
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaGetLastError();
  int best = 0;
  for (int i = 0; i < n; i++)
    if (d.ms[i] >= 0.0f && (d.ms[best] < 0.0f || d.ms[i] < d.ms[best])) best = i;
  d.choice = best;
  std::lock_guard<std::mutex> lk(g_mu);
  g_table[key] = d;
  return best;
}

int cached(const std::string &key) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_table.find(key);
  return it == g_table.end() ? 0 : it->second.choice;
}

void record(const std::string &key, const std::vector<std::string> &names,
            const std::vector<float> &ms, int choice) {
  Decision d;
  d.names = names;
  d.ms = ms;
  d.choice = choice;
  std::lock_guard<std::mutex> lk(g_mu);
  g_table[key] = d;
}

} // namespace autotune

extern "C" {

int flipgpu_set_autotune(int on) {
  std::lock_guard<std::mutex> lk(g_mu);
  g_enabled = on ? 1 : 0;
  if (on < 0) g_table.clear();
  return FLIPGPU_OK;
}

int flipgpu_autotune_report(char *buf, int len) {
  std::lock_guard<std::mutex> lk(g_mu);
  std::string s;
  char line[512];
  for (const auto &kv : g_table) {
    snprintf(line, sizeof line, "%s -> %s", kv.first.c_str(),
             kv.second.names[(size_t)kv.second.choice].c_str());
    s += line;
    for (size_t i = 0; i < kv.second.names.size(); i++) {
      snprintf(line, sizeof line, " [%s %.4f ms]", kv.second.names[i].c_str(), kv.second.ms[i]);
      s += line;
    }
    s += "\n";
  }
  if (buf && len > 0) {
    strncpy(buf, s.c_str(), (size_t)len - 1);
    buf[len - 1] = 0;
  }
  return (int)s.size();
}

} // extern "C"
