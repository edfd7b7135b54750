// Launch-shape table of this build, written by the autotuner
// (python -m molds_gb300.autotune) into molds_gb300/tuning.txt and read once
// per process.  Lines "<key> <threshold> <value>":
//   groups <n_mol> <g>            batches of at least n_mol molecules run as g
//                                 concurrent molecule groups
//   tridiag_threads <n> <t>       bases up to n: t threads per tridiagonalisation CTA
//   check_block <b>               SCF iterations enqueued per convergence check
//   vec_pairs <n> <p>             bases up to n: p eigenpairs (lane pairs) per CTA of
//                                 the tridiagonal eigenvector kernel (1..16)
//   vec_smem <n> <s>              bases up to n: that kernel keeps its inverse-iteration
//                                 factors in shared memory (1, when they fit) or in
//                                 the global workspace (0)
// MOLDS_GB300_TUNING names another table (the autotuner's candidates);
// missing entries keep the built-in defaults.
#include <dlfcn.h>

#include <algorithm>
#include <cstdlib>
#include <fstream>
#include <mutex>
#include <sstream>
#include <string>
#include <utility>
#include <vector>

#include "tuning.h"

namespace nddo {
namespace {

struct Table {
  std::vector<std::pair<int, int>> groups{{48, 1}, {96, 2}, {144, 3}, {192, 4}};
  std::vector<std::pair<int, int>> tridiag_threads{{1 << 30, 512}};
  std::vector<std::pair<int, int>> vec_pairs{{1 << 30, 16}};
  std::vector<std::pair<int, int>> vec_smem{{1 << 30, 1}};
  int check_block = 2;
};

std::once_flag g_once;
Table g_table;

std::string default_path() {
  Dl_info info;
  if (dladdr(reinterpret_cast<void*>(&tuned_groups), &info) && info.dli_fname) {
    std::string lib(info.dli_fname);
    const size_t a = lib.rfind('/');
    if (a != std::string::npos) {
      const std::string dir = lib.substr(0, a);            // molds_gb300/_build
      const size_t b = dir.rfind('/');
      if (b != std::string::npos) return dir.substr(0, b) + "/tuning.txt";
    }
  }
  return "tuning.txt";
}

void load() {
  const char* env = std::getenv("MOLDS_GB300_TUNING");
  std::ifstream f(env ? std::string(env) : default_path());
  if (!f) return;
  Table t;
  bool groups = false, threads = false, pairs = false, smem = false;
  std::string line;
  while (std::getline(f, line)) {
    if (line.empty() || line[0] == '#') continue;
    std::istringstream in(line);
    std::string key;
    int a = 0, b = 0;
    in >> key >> a;
    if (key == "check_block") {
      if (a >= 1 && a <= 16) t.check_block = a;
      continue;
    }
    if (!(in >> b)) continue;
    if (key == "groups" && a >= 1 && b >= 1 && b <= 16) {
      if (!groups) t.groups.clear();
      groups = true;
      t.groups.emplace_back(a, b);
    } else if (key == "tridiag_threads" && a >= 1 && b >= 32 && b <= 1024 && (b & (b - 1)) == 0) {
      if (!threads) t.tridiag_threads.clear();
      threads = true;
      t.tridiag_threads.emplace_back(a, b);
    } else if (key == "vec_pairs" && a >= 1 && b >= 1 && b <= 16) {
      if (!pairs) t.vec_pairs.clear();
      pairs = true;
      t.vec_pairs.emplace_back(a, b);
    } else if (key == "vec_smem" && a >= 1 && (b == 0 || b == 1)) {
      if (!smem) t.vec_smem.clear();
      smem = true;
      t.vec_smem.emplace_back(a, b);
    }
  }
  std::sort(t.groups.begin(), t.groups.end());
  std::sort(t.tridiag_threads.begin(), t.tridiag_threads.end());
  std::sort(t.vec_pairs.begin(), t.vec_pairs.end());
  std::sort(t.vec_smem.begin(), t.vec_smem.end());
  if (t.vec_smem.empty() || t.vec_smem.back().first < (1 << 30))
    t.vec_smem.emplace_back(1 << 30, t.vec_smem.empty() ? 1 : t.vec_smem.back().second);
  if (t.vec_pairs.empty() || t.vec_pairs.back().first < (1 << 30))
    t.vec_pairs.emplace_back(1 << 30, t.vec_pairs.empty() ? 16 : t.vec_pairs.back().second);
  if (t.tridiag_threads.empty() || t.tridiag_threads.back().first < (1 << 30))
    t.tridiag_threads.emplace_back(1 << 30, t.tridiag_threads.empty() ? 512 : t.tridiag_threads.back().second);
  g_table = t;
}

const Table& table() {
  std::call_once(g_once, load);
  return g_table;
}

}  // namespace

int tuned_groups(int n_mol) {
  int g = 1;
  for (const auto& e : table().groups)
    if (n_mol >= e.first) g = e.second;
  return std::max(1, std::min(g, std::max(1, n_mol)));
}

int tuned_tridiag_threads(int n) {
  for (const auto& e : table().tridiag_threads)
    if (n <= e.first) return e.second;
  return 512;
}

int tuned_check_block() { return table().check_block; }

int tuned_vec_pairs(int n) {
  for (const auto& e : table().vec_pairs)
    if (n <= e.first) return e.second;
  return 16;
}

bool tuned_vec_smem(int n) {
  for (const auto& e : table().vec_smem)
    if (n <= e.first) return e.second != 0;
  return true;
}

}  // namespace nddo
