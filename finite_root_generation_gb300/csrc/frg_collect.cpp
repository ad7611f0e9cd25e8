// Root collection, duplicate marking and persistence (include/frg_gb300.h).
//
// Replaces SortingDeletingMerging (frgsupport.cu:10-215) together with the
// driver's thrust ordering (frg.cu:432-435) and file handling (frg.cu:295-336,
// :472-480), with the same results:
//   - the round's roots are ordered by Re(root[0]), ties in path order (the
//     stable sort_by_key of frg.cu:434);
//   - in the merged order a new root precedes a collected root only when strictly
//     smaller (frgsupport.cu:37);
//   - a success (code 0) is a duplicate (code 6) when every real component is
//     within dup_tol of a collected root, or of a lower-index success of the same
//     round that is itself not a duplicate, among its neighbours whose Re(root[0])
//     is within dup_tol (frgsupport.cu:69-172);
//   - the remaining successes are folded into the sorted collection
//     (frgsupport.cu:191-211).
// The reference walks std::list/std::deque structures; here the collection is a
// flat sorted array and a round costs O((n_coll + n) + n log n).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <vector>

#include "../../include/frg_gb300.h"

namespace {
constexpr int kReals = 2 * FRG_NV;  // 42 doubles per root
}

struct frg_coll {
  double tol = 1e-6;
  std::vector<double> roots;  // size() / 42 roots, sorted by roots[42 i]
  int64_t size() const { return (int64_t)(roots.size() / kReals); }
};

extern "C" frg_status frg_coll_create(frg_coll** out, double dup_tol) {
  if (!out || !(dup_tol >= 0)) return FRG_ERR_ARG;
  frg_coll* c = new (std::nothrow) frg_coll();
  if (!c) return FRG_ERR_ALLOC;
  c->tol = dup_tol;
  *out = c;
  return FRG_OK;
}

extern "C" void frg_coll_destroy(frg_coll* c) { delete c; }

extern "C" int64_t frg_coll_size(const frg_coll* c) { return c ? c->size() : 0; }

extern "C" frg_status frg_coll_get(const frg_coll* c, double* out, int64_t capacity) {
  if (!c || (!out && c->size() > 0) || capacity < c->size()) return FRG_ERR_ARG;
  if (c->size()) std::memcpy(out, c->roots.data(), sizeof(double) * c->roots.size());
  return FRG_OK;
}

static bool same_root(const double* a, const double* b, double tol) {
  for (int k = 0; k < kReals; ++k)
    if (std::fabs(a[k] - b[k]) > tol) return false;
  return true;
}

extern "C" frg_status frg_coll_merge(frg_coll* c, const double* roots, int32_t* codes, int64_t n) {
  if (!c || n < 0 || (n > 0 && (!roots || !codes))) return FRG_ERR_ARG;
  if (n == 0) return FRG_OK;
  const double tol = c->tol;
  const int64_t nc = c->size();
  const double* coll = c->roots.data();
  // round order by Re(root[0]), ties in index order
  std::vector<int64_t> order(n);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(),
                   [&](int64_t a, int64_t b) { return roots[kReals * a] < roots[kReals * b]; });
  // merged order: >= 0 collection index, < 0 encodes -(new index) - 1
  std::vector<int64_t> merged;
  merged.reserve(nc + n);
  std::vector<int64_t> rank(n);
  int64_t ic = 0, in = 0;
  while (ic < nc || in < n) {
    if (in < n && (ic >= nc || roots[kReals * order[in]] < coll[kReals * ic])) {
      rank[order[in]] = (int64_t)merged.size();
      merged.push_back(-order[in] - 1);
      ++in;
    } else {
      merged.push_back(ic++);
    }
  }
  const int64_t total = (int64_t)merged.size();
  for (int64_t t = 0; t < n; ++t) {
    if (codes[t] != 0) continue;
    const double* rt = roots + kReals * t;
    const int64_t r = rank[t];
    for (int dir = -1; dir <= 1; dir += 2) {
      for (int64_t k = r + dir; k >= 0 && k < total; k += dir) {
        const int64_t e = merged[k];
        const double* ro = e >= 0 ? coll + kReals * e : roots + kReals * (-e - 1);
        if (std::fabs(rt[0] - ro[0]) > tol) break;
        if (e >= 0) {
          if (same_root(rt, ro, tol)) codes[t] = FRG_CODE_DUPLICATE;
        } else {
          const int64_t u = -e - 1;
          if (u < t && codes[u] == 0 && same_root(rt, ro, tol)) codes[t] = FRG_CODE_DUPLICATE;
        }
      }
    }
  }
  std::vector<double> out;
  out.reserve((size_t)kReals * (nc + n));
  for (int64_t k = 0; k < total; ++k) {
    const int64_t e = merged[k];
    if (e >= 0) out.insert(out.end(), coll + kReals * e, coll + kReals * (e + 1));
    else if (codes[-e - 1] == 0) out.insert(out.end(), roots + kReals * (-e - 1), roots + kReals * (-e));
  }
  c->roots.swap(out);
  return FRG_OK;
}

extern "C" frg_status frg_coll_save(const frg_coll* c, const char* path) {
  if (!c || !path) return FRG_ERR_ARG;
  FILE* f = std::fopen(path, "wb");
  if (!f) return FRG_ERR_IO;
  size_t w = c->roots.empty() ? 0 : std::fwrite(c->roots.data(), sizeof(double), c->roots.size(), f);
  int rc = std::fclose(f);
  return (w == c->roots.size() && rc == 0) ? FRG_OK : FRG_ERR_IO;
}

extern "C" frg_status frg_coll_load(frg_coll* c, const char* path) {
  if (!c || !path) return FRG_ERR_ARG;
  FILE* f = std::fopen(path, "rb");
  if (!f) return FRG_ERR_IO;
  std::fseek(f, 0, SEEK_END);
  long bytes = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  const long per = (long)(sizeof(double) * kReals);
  if (bytes < 0 || bytes % per != 0) { std::fclose(f); return FRG_ERR_IO; }  // truncated or corrupt
  std::vector<double> buf((size_t)bytes / sizeof(double));
  size_t r = buf.empty() ? 0 : std::fread(buf.data(), sizeof(double), buf.size(), f);
  std::fclose(f);
  if (r != buf.size()) return FRG_ERR_IO;
  for (size_t i = kReals; i < buf.size(); i += kReals)
    if (buf[i] < buf[i - kReals]) return FRG_ERR_IO;  // a collection file is sorted by Re(root[0])
  c->roots.swap(buf);
  return FRG_OK;
}

extern "C" frg_status frg_codes_append(const char* path, const int32_t* codes, int64_t n) {
  if (!path || n < 0 || (n > 0 && !codes)) return FRG_ERR_ARG;
  FILE* f = std::fopen(path, "ab");
  if (!f) return FRG_ERR_IO;
  size_t w = n ? std::fwrite(codes, sizeof(int32_t), (size_t)n, f) : 0;
  int rc = std::fclose(f);
  return (w == (size_t)n && rc == 0) ? FRG_OK : FRG_ERR_IO;
}

// Principal branch of Lambert W by Halley's iteration on w e^w = z (the reference
// uses Halley's method too, frgsupport.cu:249-272). Starting points: the series
// about the branch point -1/e, log(1+z) in the middle, log asymptotics for large z.
extern "C" double frg_lambertw0(double z) {
  const double inv_e = 0.36787944117144233;
  if (z == 0.0) return 0.0;
  if (z < -inv_e) return NAN;
  double w;
  if (z < -0.25) {
    const double p = std::sqrt(2.0 * (2.718281828459045 * z + 1.0));
    w = -1.0 + p * (1.0 + p * (-1.0 / 3.0 + p * (11.0 / 72.0)));
  } else if (z < 3.0) {
    w = 0.7 * std::log1p(z);
  } else {
    const double l1 = std::log(z), l2 = std::log(l1);
    w = l1 - l2 + l2 / l1;
  }
  for (int it = 0; it < 64; ++it) {
    const double ew = std::exp(w), f = w * ew - z, wp1 = w + 1.0;
    const double den = ew * wp1 - (w + 2.0) * f / (2.0 * wp1);
    if (den == 0.0 || !std::isfinite(den)) break;
    const double dw = f / den;
    w -= dw;
    if (std::fabs(dw) <= 1e-16 * (1.0 + std::fabs(w))) break;
  }
  return w;
}

extern "C" double frg_estimate_collected(int64_t successes, int64_t duplicates) {
  if (successes <= 0) return 0.0;
  const double s = (double)successes / ((double)successes + (double)duplicates);
  return s * frg_lambertw0((-1.0 / s) * std::exp(-1.0 / s)) + 1.0;
}
