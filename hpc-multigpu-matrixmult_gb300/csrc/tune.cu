// Scheme and tile selection for the FP64-accurate Ozaki GEMMs.
//
// Order of precedence for each choice: an environment variable, then the
// tuning table written by the autotuner (PHPC_TUNE_TABLE, or tune_table.txt
// next to the library), then a built-in default. Schemes: the modular one
// (PHPC_MODULI = 8..15 residue GEMMs; built-in default: the fewest moduli
// whose operand grid has at least 51 bits, Frobenius error about 2e-15 on
// inputs whose exponents spread over 2^+-20 inside a row) or, with
// PHPC_MODULI=0 or a table entry of 0 moduli, the digit scheme (PHPC_SLICES =
// 2..8 slices, default 7: 55-bit digit grids).
#include <dlfcn.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "phpc_host.hpp"

namespace phpc {
namespace {

constexpr int kMinModuliCount = 8, kMaxModuliCount = 15;  // range of the modular scheme

struct TuneEntry {
  long long max_mnk;  // entry applies to problems with m*n*k <= max_mnk (first match wins)
  int slices;
  int bn;
  int group_rows;     // L2 raster height of the persistent tile order (0 = default 8)
  int cluster;        // CTAs per cluster sharing B (1 or 2; 0 = default 1)
  int moduli;         // modular scheme with this many moduli; 0 = digit scheme; -1 = built-in rule
  int stages;         // K-stages of the tcgen05 ring (0 = the deepest that fits)
};

// "f32 max_mnk bn group_rows stages": the 3xBF16 FP32 GEMM; "plain max_mnk
// stages": the plain FP64 GEMM's ring depth.
struct F32Entry {
  long long max_mnk;
  int bn, group_rows, stages;
};
struct PlainEntry {
  long long max_mnk;
  int stages;
};

std::once_flag g_once;
std::vector<TuneEntry> g_table;    // single-problem entries
std::vector<TuneEntry> g_grouped;  // grouped-call entries (lines starting with "grouped")
std::vector<F32Entry> g_f32;       // 3xBF16 entries (lines starting with "f32")
std::vector<PlainEntry> g_plain;   // plain FP64 entries (lines starting with "plain")

std::string library_dir() {
  Dl_info info;
  if (dladdr(reinterpret_cast<void*>(&library_dir), &info) && info.dli_fname) {
    std::string p(info.dli_fname);
    const size_t s = p.rfind('/');
    if (s != std::string::npos) return p.substr(0, s);
  }
  return ".";
}

// Table format (text): one entry per line, "max_mnk slices bn [group_rows
// [cluster [moduli [stages]]]]" for single problems, "grouped max_mean_mnk
// slices bn [stages]" for grouped calls, "f32 max_mnk bn group_rows stages"
// for the 3xBF16 GEMM and "plain max_mnk stages" for the plain FP64 GEMM;
// '#' starts a comment line; the first entry whose max_mnk covers the
// problem applies. Written by autotune.py.
void load_table() {
  const char* env = getenv("PHPC_TUNE_TABLE");
  const std::string path = env ? std::string(env) : library_dir() + "/tune_table.txt";
  FILE* f = fopen(path.c_str(), "r");
  if (!f) return;
  char line[256];
  while (fgets(line, sizeof line, f)) {
    if (line[0] == '#') continue;
    TuneEntry e{};
    if (strncmp(line, "grouped", 7) == 0) {
      const int got = sscanf(line + 7, "%lld %d %d %d", &e.max_mnk, &e.slices, &e.bn, &e.stages);
      if (got >= 3 && e.slices >= 2 && e.slices <= 8 && (e.bn == 128 || e.bn == 256)) {
        if (got < 4 || e.stages < 2) e.stages = 0;
        g_grouped.push_back(e);
      }
      continue;
    }
    if (strncmp(line, "f32", 3) == 0) {
      F32Entry f{};
      if (sscanf(line + 3, "%lld %d %d %d", &f.max_mnk, &f.bn, &f.group_rows, &f.stages) == 4 &&
          (f.bn == 128 || f.bn == 256) && f.group_rows >= 1 && f.group_rows <= 64 && (f.stages == 0 || f.stages >= 2))
        g_f32.push_back(f);
      continue;
    }
    if (strncmp(line, "plain", 5) == 0) {
      PlainEntry pe{};
      if (sscanf(line + 5, "%lld %d", &pe.max_mnk, &pe.stages) == 2 && pe.stages >= 2 && pe.stages <= 6)
        g_plain.push_back(pe);
      continue;
    }
    const int got = sscanf(line, "%lld %d %d %d %d %d %d", &e.max_mnk, &e.slices, &e.bn, &e.group_rows, &e.cluster,
                           &e.moduli, &e.stages);
    if (got >= 3 && e.slices >= 2 && e.slices <= 8 && (e.bn == 128 || e.bn == 256)) {
      if (got < 4 || e.group_rows < 1 || e.group_rows > 64) e.group_rows = 0;
      if (got < 5 || (e.cluster != 1 && e.cluster != 2)) e.cluster = 0;
      if (got < 6 || (e.moduli != 0 && (e.moduli < kMinModuliCount || e.moduli > kMaxModuliCount))) e.moduli = -1;
      if (got < 7 || e.stages < 2) e.stages = 0;
      g_table.push_back(e);
    }
  }
  fclose(f);
}

const TuneEntry* lookup(int m, int k, int n) {
  std::call_once(g_once, load_table);
  const long long mnk = (long long)m * n * k;
  for (const TuneEntry& e : g_table)
    if (mnk <= e.max_mnk) return &e;
  return nullptr;
}

}  // namespace

int default_slices(int m, int k, int n) {
  const char* env = getenv("PHPC_SLICES");
  if (env) {
    const int s = atoi(env);
    if (s >= 2 && s <= 8) return s;
  }
  if (const TuneEntry* e = lookup(m, k, n)) return e->slices;
  return 7;
}

int default_moduli(int m, int k, int n) {
  const char* env = getenv("PHPC_MODULI");
  if (env) {
    const int q = atoi(env);
    if (q == 0 || (q >= kMinModuliCount && q <= kMaxModuliCount)) return q;
  }
  if (const TuneEntry* e = lookup(m, k, n))
    if (e->moduli >= 0) return e->moduli;
  for (int q = kMinModuliCount; q < kMaxModuliCount; ++q)
    if (ozaki2_bits(q, k) >= 51) return q;
  return kMaxModuliCount;
}

int default_bn(int m, int k, int n) {
  const char* env = getenv("PHPC_OZAKI_BN");
  if (env) {
    const int b = atoi(env);
    if (b == 128 || b == 256) return b;
  }
  if (const TuneEntry* e = lookup(m, k, n)) return e->bn;
  return 256;
}

// CTAs per cluster of the single-problem slice GEMM (1, or 2 = a CTA pair
// computing one 256-row tile with cta_group::2 MMAs, each CTA loading its own
// half of the operands): PHPC_CLUSTER, else the table, else 1.
int default_cluster(int m, int k, int n) {
  const char* env = getenv("PHPC_CLUSTER");
  if (env && (atoi(env) == 1 || atoi(env) == 2)) return atoi(env);
  if (const TuneEntry* e = lookup(m, k, n))
    if (e->cluster == 2) return 2;
  return 1;
}

int default_group_rows(int m, int k, int n) {
  const char* env = getenv("PHPC_GROUP_ROWS");
  if (env && atoi(env) > 0 && atoi(env) <= 64) return atoi(env);
  if (const TuneEntry* e = lookup(m, k, n))
    if (e->group_rows > 0) return e->group_rows;
  return 8;
}

// Tile width of the grouped slice GEMM: PHPC_GROUPED_BN, else the tuning
// table's entry for the batch's mean problem size, else 128 (small problems
// waste less of a 128-wide tile).
int default_grouped_bn(const phpc_gemm_problem* problems, int count) {
  const char* env = getenv("PHPC_GROUPED_BN");
  if (env) {
    const int b = atoi(env);
    if (b == 128 || b == 256) return b;
  }
  double mnk = 0;
  for (int i = 0; i < count; ++i) mnk += (double)problems[i].m * problems[i].n * problems[i].k;
  if (count > 0) {
    std::call_once(g_once, load_table);
    const long long mean = (long long)(mnk / count);
    for (const TuneEntry& e : g_grouped)
      if (mean <= e.max_mnk) return e.bn;
  }
  return 128;
}

// K-stages of the tcgen05 ring: PHPC_STAGES (>= 2; the launcher caps it at
// what fits), else the table, else 0 (the deepest ring that fits).
int default_stages(int m, int k, int n) {
  const char* env = getenv("PHPC_STAGES");
  if (env && atoi(env) >= 2) return atoi(env);
  if (const TuneEntry* e = lookup(m, k, n)) return e->stages;
  return 0;
}

int default_grouped_stages(const phpc_gemm_problem* problems, int count) {
  const char* env = getenv("PHPC_STAGES");
  if (env && atoi(env) >= 2) return atoi(env);
  double mnk = 0;
  for (int i = 0; i < count; ++i) mnk += (double)problems[i].m * problems[i].n * problems[i].k;
  if (count > 0) {
    std::call_once(g_once, load_table);
    const long long mean = (long long)(mnk / count);
    for (const TuneEntry& e : g_grouped)
      if (mean <= e.max_mnk) return e.stages;
  }
  return 0;
}

F32Tune default_f32(int m, int k, int n) {
  F32Tune t{256, 8, 0};
  std::call_once(g_once, load_table);
  const long long mnk = (long long)m * n * k;
  for (const F32Entry& e : g_f32)
    if (mnk <= e.max_mnk) {
      t = {e.bn, e.group_rows, e.stages};
      break;
    }
  if (const char* env = getenv("PHPC_F32_BN"))
    if (atoi(env) == 128 || atoi(env) == 256) t.bn = atoi(env);
  if (const char* env = getenv("PHPC_GROUP_ROWS"))
    if (atoi(env) > 0 && atoi(env) <= 64) t.group_rows = atoi(env);
  if (const char* env = getenv("PHPC_STAGES"))
    if (atoi(env) >= 2) t.stages = atoi(env);
  return t;
}

// Ring depth of the plain FP64 GEMM: PHPC_DMMA_STAGES (2 .. 6), else the
// table, else 4.
int default_plain_stages(int m, int k, int n) {
  const char* env = getenv("PHPC_DMMA_STAGES");
  if (env && atoi(env) >= 2 && atoi(env) <= 6) return atoi(env);
  std::call_once(g_once, load_table);
  const long long mnk = (long long)m * n * k;
  for (const PlainEntry& e : g_plain)
    if (mnk <= e.max_mnk) return e.stages;
  return 4;
}

}  // namespace phpc

extern "C" int phpc_default_slices(int m, int k, int n) { return phpc::default_slices(m, k, n); }

extern "C" int phpc_tuning(int m, int k, int n, int* cfg) {
  using namespace phpc;
  if (!cfg || m < 0 || k < 0 || n < 0) return PHPC_ERR_ARG;
  const F32Tune f = default_f32(m, k, n);
  const int v[10] = {default_moduli(m, k, n), default_slices(m, k, n), default_bn(m, k, n),
                     default_group_rows(m, k, n), default_cluster(m, k, n), default_stages(m, k, n),
                     f.bn, f.group_rows, f.stages, default_plain_stages(m, k, n)};
  for (int i = 0; i < 10; ++i) cfg[i] = v[i];
  return PHPC_OK;
}
