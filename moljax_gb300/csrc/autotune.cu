// Registry of autotuned launch choices and the candidate generator for mixed-radix
// DFT schedules.  The timing loops live beside the kernels they tune
// (mjx_autotune_dft in dftn.cu, mjx_autotune_stencil2d in explicit.cu).
#include <map>
#include <mutex>
#include <tuple>
#include <vector>
#include <algorithm>
#include <string.h>

#include "autotune.cuh"
#include "moljax_gb300.h"

namespace mjx {

int elem_size(int dtype);

namespace {
std::mutex g_mu;
std::map<std::pair<int, int>, DftTune> g_dft;
std::map<std::tuple<int, int, int, int>, int> g_rows;
}  // namespace

bool tune_dft_get(int n, int elem, DftTune* t) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_dft.find({n, elem});
  if (it == g_dft.end()) return false;
  *t = it->second;
  return true;
}

void tune_dft_put(int n, int elem, const DftTune& t) {
  std::lock_guard<std::mutex> lk(g_mu);
  g_dft[{n, elem}] = t;
}

void tune_dft_clear(int n, int elem) {
  std::lock_guard<std::mutex> lk(g_mu);
  g_dft.erase({n, elem});
}

int tune_rows_get(int ny, int nx, int nf, int elem) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_rows.find(std::make_tuple(ny, nx, nf, elem));
  return it == g_rows.end() ? 0 : it->second;
}

void tune_rows_put(int ny, int nx, int nf, int elem, int rows) {
  std::lock_guard<std::mutex> lk(g_mu);
  g_rows[std::make_tuple(ny, nx, nf, elem)] = rows;
}

// Schedules of n = 2^a 3^b 5^c: the multisets with the most radix-4 passes and with one
// radix-4 pass traded for two radix-2 passes, each in four orders (the default 4,2,3,5;
// ascending; descending; odd radices first), without duplicates.
int dft_schedules(int n, int* out, int max) {
  if (n < 2 || (n & (n - 1)) == 0) return 0;
  int m = n, a = 0, b = 0, c = 0;
  while (m % 2 == 0) { m /= 2; ++a; }
  while (m % 3 == 0) { m /= 3; ++b; }
  while (m % 5 == 0) { m /= 5; ++c; }
  if (m != 1) return 0;
  std::vector<std::vector<int>> cands;
  auto add = [&](std::vector<int> v) {
    if (v.empty() || v.size() > 16) return;
    if (std::find(cands.begin(), cands.end(), v) == cands.end()) cands.push_back(v);
  };
  const int pmax = a / 2;
  for (int p = pmax; p >= 0 && p >= pmax - 1; --p) {
    const int q = a - 2 * p;
    std::vector<int> base;
    for (int i = 0; i < p; ++i) base.push_back(4);
    for (int i = 0; i < q; ++i) base.push_back(2);
    for (int i = 0; i < b; ++i) base.push_back(3);
    for (int i = 0; i < c; ++i) base.push_back(5);
    add(base);
    std::vector<int> asc = base, desc = base, odd;
    std::sort(asc.begin(), asc.end());
    std::sort(desc.begin(), desc.end(), [](int x, int y) { return x > y; });
    add(asc);
    add(desc);
    for (int r : base) if (r & 1) odd.push_back(r);
    for (int r : base) if (!(r & 1)) odd.push_back(r);
    add(odd);
  }
  int k = 0;
  for (const auto& v : cands) {
    if (k >= max) break;
    int* row = out + 17 * k;
    memset(row, 0, 17 * sizeof(int));
    row[0] = (int)v.size();
    for (size_t i = 0; i < v.size(); ++i) row[1 + i] = v[i];
    ++k;
  }
  return k;
}

}  // namespace mjx

using namespace mjx;

int mjx_dft_schedule_candidates(int n, int* out, int max) {
  if (out == nullptr || max < 1) return 0;
  return dft_schedules(n, out, max);
}

mjx_status mjx_dft_schedule_set(int n, int dtype, int nrad, const int* rad, int tpsm) {
  const int e = elem_size(dtype);
  if (!e) return MJX_BAD_DTYPE;
  if (n < 2 || n > 2048) return MJX_BAD_ARG;
  if (nrad == 0) { tune_dft_clear(n, e); return MJX_OK; }
  if (nrad < 0 || nrad > 16 || rad == nullptr || tpsm < 0 || tpsm > 256) return MJX_BAD_ARG;
  long long prod = 1;
  DftTune t;
  memset(&t, 0, sizeof(t));
  for (int i = 0; i < nrad; ++i) {
    if (rad[i] < 2 || rad[i] > 5) return MJX_BAD_ARG;
    prod *= rad[i];
    t.rad[i] = rad[i];
  }
  if (prod != n) return MJX_BAD_ARG;
  t.nrad = nrad;
  t.tpsm = tpsm;
  tune_dft_put(n, e, t);
  return MJX_OK;
}

mjx_status mjx_stencil_rows_set(int ny, int nx, int nfields, int dtype, int rows) {
  const int e = elem_size(dtype);
  if (!e) return MJX_BAD_DTYPE;
  if (ny < 1 || nx < 1 || nfields < 1 || nfields > 4) return MJX_BAD_ARG;
  // 64 selects the TMA-staged form (FP32 with 16-byte rows; other stages fall back to 8)
  if (rows != 0 && rows != 2 && rows != 4 && rows != 8 && rows != 16 && rows != 32 && rows != 64)
    return MJX_BAD_ARG;
  tune_rows_put(ny, nx, nfields, e, rows);
  return MJX_OK;
}

int mjx_stencil_rows_get(int ny, int nx, int nfields, int dtype) {
  const int e = elem_size(dtype);
  if (!e) return 0;
  return tune_rows_get(ny, nx, nfields, e);
}
