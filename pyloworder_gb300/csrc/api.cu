// Library-wide C-ABI entries: version and per-thread error string.
#include <map>
#include <string>
#include <vector>

#include "plom_common.cuh"

namespace plom {

static thread_local char g_err[1024] = "";

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

const char* last_error() { return g_err; }

Tuning& tuning() {
  static Tuning t;
  return t;
}

static thread_local std::vector<ProfEntry>* g_prof = nullptr;
bool prof_on() { return g_prof != nullptr; }
void prof_push(const ProfEntry& e) {
  if (g_prof) g_prof->push_back(e);
}

}  // namespace plom

extern "C" const char* plom_last_error_string(void) { return plom::last_error(); }
extern "C" int plom_version(void) { return 100; }

extern "C" int plom_profile_begin(void) {
  if (!plom::g_prof) plom::g_prof = new std::vector<plom::ProfEntry>();
  plom::g_prof->clear();
  return PLOM_OK;
}

extern "C" int plom_profile_end(char* buf, size_t cap) {
  using namespace plom;
  if (!g_prof) {
    if (buf && cap) buf[0] = 0;
    return PLOM_OK;
  }
  struct Agg {
    int count = 0, launches = 0;
    double ms = 0, flops = 0, bytes = 0;
  };
  std::map<std::string, Agg> agg;
  int status = PLOM_OK;
  for (auto& e : *g_prof) {
    float ms = 0.f;
    if (cudaEventSynchronize(e.b) != cudaSuccess || cudaEventElapsedTime(&ms, e.a, e.b) != cudaSuccess)
      status = PLOM_ERR_CUDA;
    Agg& a = agg[e.name];
    a.count += 1;
    a.launches += e.launches;
    a.ms += ms;
    a.flops += e.flops;
    a.bytes += e.bytes;
    cudaEventDestroy(e.a);
    cudaEventDestroy(e.b);
  }
  delete g_prof;
  g_prof = nullptr;
  std::string out;
  char line[256];
  for (auto& kv : agg) {
    snprintf(line, sizeof(line), "%s %d %.6f %.6e %.6e %d\n", kv.first.c_str(), kv.second.count,
             kv.second.ms, kv.second.flops, kv.second.bytes, kv.second.launches);
    out += line;
  }
  if (buf && cap) {
    size_t n = out.size() < cap - 1 ? out.size() : cap - 1;
    memcpy(buf, out.data(), n);
    buf[n] = 0;
  }
  if (status != PLOM_OK) set_error("plom_profile_end: event timing failed");
  return status;
}

// tuning parameters by name (see plom::Tuning); values outside the allowed
// set are rejected with PLOM_ERR_ARG
extern "C" int plom_set_tuning(const char* key, double value) {
  using namespace plom;
  if (!key) {
    set_error("plom_set_tuning: null key");
    return PLOM_ERR_ARG;
  }
  const std::string k(key);
  const int v = (int)value;
  if ((double)v != value) {
    set_error("plom_set_tuning: %s takes an integer", key);
    return PLOM_ERR_ARG;
  }
  Tuning& t = tuning();
  if (k == "gram_wave_mult" && v >= 1 && v <= 32) {
    t.gram_wave_mult = v;
  } else if (k == "gram_wide_wave_mult" && v >= 1 && v <= 256) {
    t.gram_wide_wave_mult = v;
  } else if (k == "reduce_blocks_per_sm" && v >= 1 && v <= 16) {
    t.reduce_blocks_per_sm = v;
  } else if (k == "apply_dense_tn" && (v == 128 || v == 256)) {
    t.apply_dense_tn = v;
  } else if (k == "apply_dense_by_rows" && (v == 0 || v == 1)) {
    t.apply_dense_by_rows = v;
  } else if (k == "apply_tri_by_rows" && (v == 0 || v == 1)) {
    t.apply_tri_by_rows = v;
  } else if (k == "pass1_chunks" && (v == 1 || v == 2 || v == 4 || v == 8)) {
    t.pass1_chunks = v;
  } else if (k == "apply_pair" && v >= 0 && v <= 2) {
    t.apply_pair = v;
  } else {
    set_error("plom_set_tuning: unknown key or value out of range: %s = %g", key, value);
    return PLOM_ERR_ARG;
  }
  return PLOM_OK;
}

extern "C" double plom_get_tuning(const char* key) {
  using namespace plom;
  if (!key) return -1.0;
  const std::string k(key);
  const Tuning& t = tuning();
  if (k == "gram_wave_mult") return t.gram_wave_mult;
  if (k == "gram_wide_wave_mult") return t.gram_wide_wave_mult;
  if (k == "reduce_blocks_per_sm") return t.reduce_blocks_per_sm;
  if (k == "apply_dense_tn") return t.apply_dense_tn;
  if (k == "apply_dense_by_rows") return t.apply_dense_by_rows;
  if (k == "apply_tri_by_rows") return t.apply_tri_by_rows;
  if (k == "pass1_chunks") return t.pass1_chunks;
  if (k == "apply_pair") return t.apply_pair;
  return -1.0;
}
