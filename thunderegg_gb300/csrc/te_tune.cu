// te_tune.cu -- the autotuner's choice table, timing and cache file (te_tune.cuh).

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <limits>
#include <map>
#include <mutex>
#include <sstream>

#include "te_internal.cuh"
#include "te_tune.cuh"

namespace te {
namespace {

struct Choice {
  int index = 0;
  std::string label;
  std::vector<std::pair<std::string, double>> ms;  // candidate label, median milliseconds
  bool cached = false;
};

std::mutex g_mu;
std::map<std::string, Choice> g_choices;        // "device|family|key" -> choice
std::map<std::string, std::string> g_file;      // the same keys -> label, from TE_TUNE_CACHE
bool g_file_loaded = false;

bool tuning_on() {
  static const bool on = [] {
    const char* e = std::getenv("TE_TUNE");
    return !(e && e[0] == '0');
  }();
  return on;
}

std::string device_name() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return "?";
  cudaDeviceProp p;
  if (cudaGetDeviceProperties(&p, dev) != cudaSuccess) return "?";
  return std::string(p.name) + " sm_" + std::to_string(p.major) + std::to_string(p.minor);
}

const char* cache_path() { return std::getenv("TE_TUNE_CACHE"); }

void load_file() {
  if (g_file_loaded) return;
  g_file_loaded = true;
  const char* path = cache_path();
  if (!path) return;
  std::ifstream in(path);
  std::string line;
  while (std::getline(in, line)) {
    const size_t t = line.rfind('\t');
    if (t == std::string::npos) continue;
    g_file[line.substr(0, t)] = line.substr(t + 1);
  }
}

void append_file(const std::string& k, const std::string& label) {
  const char* path = cache_path();
  if (!path) return;
  std::ofstream out(path, std::ios::app);
  out << k << '\t' << label << '\n';
}

std::string json_escape(const std::string& s) {
  std::string o;
  for (char c : s) {
    if (c == '"' || c == '\\') o += '\\';
    o += c;
  }
  return o;
}

}  // namespace

bool tune_settled(const std::string& family, const std::string& key) {
  if (!tuning_on()) return true;
  std::lock_guard<std::mutex> lock(g_mu);
  const std::string k = device_name() + "|" + family + "|" + key;
  if (g_choices.count(k)) return true;
  load_file();
  return g_file.count(k) != 0;
}

int tune_select(const std::string& family, const std::string& key, const std::vector<TuneCandidate>& cands,
                cudaStream_t s, int reps) {
  if (cands.size() <= 1 || !tuning_on()) return 0;
  std::lock_guard<std::mutex> lock(g_mu);
  const std::string k = device_name() + "|" + family + "|" + key;
  auto label_index = [&](const std::string& label) {
    for (size_t i = 0; i < cands.size(); i++)
      if (cands[i].label == label) return (int)i;
    return 0;
  };
  auto it = g_choices.find(k);
  if (it != g_choices.end()) return label_index(it->second.label);
  load_file();
  auto f = g_file.find(k);
  if (f != g_file.end()) {
    Choice c;
    c.label = f->second;
    c.index = label_index(c.label);
    c.cached = true;
    g_choices[k] = c;
    return c.index;
  }
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  TE_CUDA(cudaStreamIsCapturing(s, &cap));
  if (cap != cudaStreamCaptureStatusNone) return 0;  // cannot time inside a capture; default for now
  cudaEvent_t e0, e1;
  TE_CUDA(cudaEventCreate(&e0));
  TE_CUDA(cudaEventCreate(&e1));
  Choice c;
  double best = std::numeric_limits<double>::infinity();
  for (size_t i = 0; i < cands.size(); i++) {
    double med = std::numeric_limits<double>::infinity();
    try {
      cands[i].run();  // warm-up (module load, caches)
      std::vector<float> t;
      for (int r = 0; r < reps; r++) {
        TE_CUDA(cudaEventRecord(e0, s));
        cands[i].run();
        TE_CUDA(cudaEventRecord(e1, s));
        TE_CUDA(cudaEventSynchronize(e1));
        float ms = 0;
        TE_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        t.push_back(ms);
      }
      std::sort(t.begin(), t.end());
      med = t[t.size() / 2];
    } catch (const Error&) {
      cudaGetLastError();  // a candidate that cannot launch here is skipped
    }
    c.ms.push_back({cands[i].label, med});
    if (med < best) {
      best = med;
      c.index = (int)i;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  c.label = cands[c.index].label;
  g_choices[k] = c;
  append_file(k, c.label);
  return c.index;
}

}  // namespace te

using namespace te;

extern "C" int te_tune_report(char* buf, int len, int* needed) {
  return guard([&] {
    std::lock_guard<std::mutex> lock(g_mu);
    std::ostringstream o;
    o << "[";
    bool first = true;
    for (const auto& kv : g_choices) {
      o << (first ? "" : ",") << "{\"key\":\"" << json_escape(kv.first) << "\",\"choice\":\""
        << json_escape(kv.second.label) << "\",\"cached\":" << (kv.second.cached ? "true" : "false") << ",\"ms\":{";
      for (size_t i = 0; i < kv.second.ms.size(); i++) {
        char v[32];
        std::snprintf(v, sizeof v, "%.5f", kv.second.ms[i].second);
        o << (i ? "," : "") << "\"" << json_escape(kv.second.ms[i].first) << "\":"
          << (std::isfinite(kv.second.ms[i].second) ? v : "null");
      }
      o << "}}";
      first = false;
    }
    o << "]";
    const std::string s = o.str();
    if (needed) *needed = (int)s.size() + 1;
    if (buf && len > 0) {
      std::strncpy(buf, s.c_str(), (size_t)len - 1);
      buf[len - 1] = 0;
    }
  });
}

extern "C" int te_tune_reset(void) {
  return guard([&] {
    std::lock_guard<std::mutex> lock(g_mu);
    g_choices.clear();
  });
}
