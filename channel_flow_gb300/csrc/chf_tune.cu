// chf_tune.cu -- the autotuner: launch shapes and FFT radix orders picked by
// measurement on the device, per (device, grid, product grid, precision).
//
// The reference's counterpart is FFTW's measured planning: its thirteen
// plans are created with FFTW_MEASURE (poiseuilleflow.f90:100-112), which
// times candidate algorithms once and keeps the fastest.  chf_autotune does
// the same for this library's choices:
//   * the radix order of every shared-memory FFT plan (spanwise and
//     streamwise lengths, the 2 nnz and 2 zpad wall-normal lengths): the
//     rule's order, its reverse and the odd radices first, where the rule is
//     the largest radices (16, 8, 9, ...) for the x / y lines and 4s, then
//     2, 3, 5 for the wall-normal ones; the x / y lines also try radices up to 4;
//   * the lines per CTA of the shared-memory FFT kernels (y: streamwise
//     modes per CTA; x: rows per CTA; FP64 z: modes per CTA), every shape the
//     launch rules accept;
//   * the increment solve's thread mapping (CHF_MIXED): modes per CTA (2 or
//     4), matrix columns per load batch (2, 3 or 4), block rows per thread
//     (1 or 2) and, where one row per thread at 288 threads would loop, one
//     pass in wide blocks or the loop.
// Every candidate computes the same results bit for bit (a plan change
// rewrites the plan's stage twiddle table first, with the same values).  The
// recovery's arithmetic (chf_set_launch_shape "recover_form") is not
// searched: its two forms differ in the last bits.
// Each knob is tuned in turn (coordinate descent), every candidate timed as
// whole time steps with CUDA events on the handle's stream, best of `reps`
// runs; a candidate replaces the current choice only when it is at least 1%
// faster.  The steps run on the handle's state, which is saved first and put
// back afterwards (data, history arrangement and flow word).
// The register FFTs of the 192-point lines and the tensor-core GEMM tiles
// (fixed by the 512 TMEM columns, k_tcgemm.cu) have no alternatives here.
// The choice is cached for the process: later handles of the same key start
// with it (chf_create).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "chf_internal.h"

using namespace chf;

struct chf_handle : public Handle {};

namespace {

struct Choice {
  Tuning t;
  FftPlan py, px, pz2, pzm;
  std::string report;
};

using Key = std::tuple<int, int, int, int, int, int>;  // device, nnx, nny, nnz, MZ, precision

std::mutex g_mu;
std::map<Key, Choice> g_cache;

Key key_of(const Handle* h) {
  return Key{h->device, h->d.nnx, h->d.nny, h->d.nnz, h->d.MZ, h->cfg.precision};
}

FftPlan plan_from(int L, const std::vector<int>& radices) {
  FftPlan p{};
  p.L = L;
  int Ns = 1;
  for (int r : radices) {
    p.R[p.nst] = r;
    p.Ns[p.nst] = Ns;
    ++p.nst;
    Ns *= r;
  }
  fft_plan_divisors(p);
  return p;
}

std::string radix_string(const FftPlan& p) {
  std::string s;
  for (int i = 0; i < p.nst; ++i) s += (i ? "." : "") + std::to_string(p.R[i]);
  return s.empty() ? "1" : s;
}

// radix orders of one length: the rule's, reversed, odd radices first
std::vector<FftPlan> plan_candidates(const FftPlan& rule) {
  const int L = rule.L;
  std::vector<int> r(rule.R, rule.R + rule.nst);
  std::vector<std::vector<int>> orders{r, std::vector<int>(r.rbegin(), r.rend())};
  std::vector<int> odd;
  for (int x : r)
    if (x % 2) odd.push_back(x);
  for (int x : r)
    if (x % 2 == 0) odd.push_back(x);
  orders.push_back(odd);
  std::vector<FftPlan> out;
  for (auto& o : orders) {
    bool seen = false;
    for (auto& p : out) seen = seen || (std::vector<int>(p.R, p.R + p.nst) == o);
    if (!seen) out.push_back(plan_from(L, o));
  }
  return out;
}

// mean device time of one step over `reps` runs of `nsteps` direct steps,
// the fastest run; < 0 on a launch error
double time_steps(Handle* h, int nsteps, int reps, cudaEvent_t e0, cudaEvent_t e1) {
  if (step_once(h) != CHF_OK) return -1.0;  // warm
  double best = 1e30;
  for (int r = 0; r < reps; ++r) {
    if (cudaEventRecord(e0, h->stream) != cudaSuccess) return -1.0;
    for (int s = 0; s < nsteps; ++s)
      if (step_once(h) != CHF_OK) return -1.0;
    if (cudaEventRecord(e1, h->stream) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess) return -1.0;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    best = std::min(best, (double)ms / nsteps);
  }
  return best;
}

std::string describe(const Handle* h, double ms_rule, double ms_best) {
  char buf[512];
  std::snprintf(buf, sizeof buf,
                "fft radices py %s px %s pz2 %s pzm %s; kxb %d xr %d zl_c2v %d zl_curl %d; "
                "increment solve %d modes x %d columns x %d rows per thread%s, %s recovery; step %.4f ms "
                "(rules %.4f ms)",
                radix_string(h->py).c_str(), radix_string(h->px).c_str(), radix_string(h->pz2).c_str(),
                radix_string(h->pzm).c_str(), h->tune.kxb, h->tune.xr, h->tune.zl_c2v, h->tune.zl_curl,
                h->tune.inc_mch, h->tune.inc_cb, h->tune.inc_rpt, h->tune.inc_wide ? "" : " (288-thread blocks)",
                (h->tune.rec_form >= 0 ? h->tune.rec_form == 1 : h->rec_df_rule) ? "double-float" : "FP64", ms_best,
                ms_rule);
  return buf;
}

}  // namespace

namespace chf {

// chf_create: start from the process's cached choice for this key, if any
void apply_cached_tuning(Handle* h) {
  std::lock_guard<std::mutex> lock(g_mu);
  auto it = g_cache.find(key_of(h));
  if (it == g_cache.end()) return;
  h->tune = it->second.t;
  h->py = it->second.py;
  h->px = it->second.px;
  h->pz2 = it->second.pz2;
  h->pzm = it->second.pzm;
}

}  // namespace chf

extern "C" {

int chf_autotune(chf_handle* h, int reps) {
  if (!h) return CHF_E_INVALID;
  if (!h->uploaded) {
    h->err = "chf_autotune before chf_upload_state (it times steps of the state)";
    return CHF_E_STATE;
  }
  if (reps <= 0) reps = 3;
  if (!cuda_ok(h, cudaSetDevice(h->device), "cudaSetDevice") ||
      !cuda_ok(h, cudaStreamSynchronize(h->stream), "cudaStreamSynchronize"))
    return CHF_E_CUDA;
  const Dims& d = h->d;
  const size_t fb = sizeof(cd) * d.field_elems(), mb = sizeof(double) * 2 * d.NZ * d.nch;
  // save the state: field data, arrangement, means, flow word
  cd* saved_ptr[F_COUNT];
  std::copy(h->f, h->f + F_COUNT, saved_ptr);
  void* save = nullptr;
  const size_t total = F_COUNT * fb + M_COUNT * mb + sizeof(double) * 4 * d.nch;
  if (!cuda_ok(h, cudaMalloc(&save, total), "autotune save")) return CHF_E_NOMEM;
  char* sp = static_cast<char*>(save);
  bool good = true;
  for (int i = 0; i < F_COUNT; ++i)
    good = good && cudaMemcpyAsync(sp + i * fb, h->f[i], fb, cudaMemcpyDeviceToDevice, h->stream) == cudaSuccess;
  for (int i = 0; i < M_COUNT; ++i)
    good = good && cudaMemcpyAsync(sp + F_COUNT * fb + i * mb, h->mean[i], mb, cudaMemcpyDeviceToDevice,
                                   h->stream) == cudaSuccess;
  good = good && cudaMemcpyAsync(sp + F_COUNT * fb + M_COUNT * mb, h->flow, sizeof(double) * 4 * d.nch,
                                 cudaMemcpyDeviceToDevice, h->stream) == cudaSuccess;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  good = good && cudaEventCreate(&e0) == cudaSuccess && cudaEventCreate(&e1) == cudaSuccess;
  const bool was_profiling = h->profiling;
  h->profiling = false;
  const int nsteps = 2;
  double best = good ? time_steps(h, nsteps, reps, e0, e1) : -1.0;
  const double rule = best;
  auto try_knob = [&](auto set, const auto& cands) {
    if (cands.size() < 2 || best < 0) return;
    auto keep = cands[0];
    for (const auto& c : cands) {
      set(c);
      const double t = time_steps(h, nsteps, reps, e0, e1);
      if (t < 0) {
        best = -1.0;
        return;
      }
      if (t < 0.99 * best) {
        best = t;
        keep = c;
      }
    }
    set(keep);
  };
  // each knob starts from the current choice (the first candidate is kept
  // unless another one is at least 1% faster)
  auto with_current = [](auto cur, auto cands) {
    std::vector<decltype(cur)> out{cur};
    for (auto& c : cands) out.push_back(c);
    return out;
  };
  bool tw_ok = true;
  const bool reg_xy = mixed_front(h) && xy_register_path(d);
  if (!reg_xy) {
    // two-buffer stages: the large-radix rule's orders, and radices up to 4
    const int maxr = h->cfg.precision == CHF_FP64 ? 8 : 16;
    auto xy_cands = [&](int L) {
      auto c = plan_candidates(make_plan_pp(L, maxr));
      for (auto& q : plan_candidates(make_plan(L))) c.push_back(q);
      return c;
    };
    // a plan change rewrites the plan's stage twiddle table before it runs
    try_knob([&](const FftPlan& p) { h->py = p, tw_ok = tw_ok && upload_stage_twiddles(h) == CHF_OK; },
             with_current(h->py, xy_cands(d.PY)));
    try_knob([&](const FftPlan& p) { h->px = p, tw_ok = tw_ok && upload_stage_twiddles(h) == CHF_OK; },
             with_current(h->px, xy_cands(d.PX)));
    try_knob([&](int v) { h->tune.kxb = v; }, with_current(h->tune.kxb, shape_candidates(h, 0)));
    try_knob([&](int v) { h->tune.xr = v; }, with_current(h->tune.xr, shape_candidates(h, 1)));
  }
  if (!mixed_front(h)) {
    try_knob([&](const FftPlan& p) { h->pzm = p; }, with_current(h->pzm, plan_candidates(make_plan(2 * d.MZ))));
    try_knob([&](int v) { h->tune.zl_c2v = v; }, with_current(h->tune.zl_c2v, shape_candidates(h, 2)));
    try_knob([&](int v) { h->tune.zl_curl = v; }, with_current(h->tune.zl_curl, shape_candidates(h, 3)));
  }
  // the 2 nnz DFTs of the FP64 solve (every mode in CHF_FP64 and
  // CHF_MIXED_F64SOLVE, the (0,0) mode in CHF_MIXED)
  try_knob([&](const FftPlan& p) { h->pz2 = p; }, with_current(h->pz2, plan_candidates(make_plan(2 * d.N))));
  if (increment_solve(h)) {
    struct IncMap {
      int mch, cb, rpt, wide;
    };
    std::vector<IncMap> maps{{h->tune.inc_mch, h->tune.inc_cb, h->tune.inc_rpt, h->tune.inc_wide}};
    const SolveLayout& sl = h->sl;
    const bool long_blocks = sl.ne_v + sl.no_v + sl.ne_w + sl.no_w > 288;  // the one-row block loops
    for (int wide : {1, 0}) {
      if (wide == 0 && !long_blocks) continue;
      for (int mch : {4, 2})
        for (int cb : {4, 3, 2}) maps.push_back({mch, cb, 1, wide});
    }
    for (int mch : {4, 2})
      for (int cb : {3, 2}) maps.push_back({mch, cb, 2, 1});
    try_knob(
        [&](const IncMap& m) {
          h->tune.inc_mch = m.mch, h->tune.inc_cb = m.cb, h->tune.inc_rpt = m.rpt, h->tune.inc_wide = m.wide;
        },
        maps);
  }
  h->profiling = was_profiling;
  // put the state back
  std::copy(saved_ptr, saved_ptr + F_COUNT, h->f);
  for (int i = 0; i < F_COUNT; ++i)
    good = good && cudaMemcpyAsync(h->f[i], sp + i * fb, fb, cudaMemcpyDeviceToDevice, h->stream) == cudaSuccess;
  for (int i = 0; i < M_COUNT; ++i)
    good = good && cudaMemcpyAsync(h->mean[i], sp + F_COUNT * fb + i * mb, mb, cudaMemcpyDeviceToDevice,
                                   h->stream) == cudaSuccess;
  good = good && cudaMemcpyAsync(h->flow, sp + F_COUNT * fb + M_COUNT * mb, sizeof(double) * 4 * d.nch,
                                 cudaMemcpyDeviceToDevice, h->stream) == cudaSuccess;
  good = good && cudaStreamSynchronize(h->stream) == cudaSuccess;
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(save);
  // the captured step graphs hold the old shapes
  for (auto& g : h->graphs) cudaGraphExecDestroy(g.exec);
  h->graphs.clear();
  if (!good || best < 0 || !tw_ok) {
    if (h->err.empty()) h->err = "chf_autotune: a timed step failed";
    return CHF_E_CUDA;
  }
  h->tune.tuned = true;
  h->tune.manual = false;
  Choice c{h->tune, h->py, h->px, h->pz2, h->pzm, describe(h, rule, best)};
  std::lock_guard<std::mutex> lock(g_mu);
  g_cache[key_of(h)] = c;
  return CHF_OK;
}

int chf_set_launch_shape(chf_handle* h, const char* name, int value) {
  if (!h) return CHF_E_INVALID;
  if (!name) {
    h->err = "chf_set_launch_shape: no name";
    return CHF_E_INVALID;
  }
  const std::string n(name);
  Tuning t = h->tune;
  auto bad = [&](const char* why) {
    h->err = "chf_set_launch_shape(" + n + ", " + std::to_string(value) + "): " + why;
    return CHF_E_INVALID;
  };
  if (n == "inc_modes") {
    if (value != 2 && value != 4) return bad("2 or 4 modes per CTA");
    t.inc_mch = value;
  } else if (n == "inc_columns") {
    if (value < 2 || value > 4) return bad("2, 3 or 4 columns per batch");
    t.inc_cb = value;
  } else if (n == "inc_rows") {
    if (value != 1 && value != 2) return bad("1 or 2 rows per thread");
    t.inc_rpt = value;
  } else if (n == "inc_wide") {
    if (value != 0 && value != 1) return bad("0 or 1");
    t.inc_wide = value;
  } else if (n == "recover_form") {
    if (value < -1 || value > 1) return bad("-1 (rule), 0 (FP64) or 1 (double-float)");
    t.rec_form = value;
  } else {
    static const char* knobs[] = {"kxb", "xr", "zl_c2v", "zl_curl"};
    int k = -1;
    for (int i = 0; i < 4; ++i)
      if (n == knobs[i]) k = i;
    if (k < 0) return bad("unknown name");
    if (value != 0) {
      const auto c = shape_candidates(h, k);
      if (std::find(c.begin(), c.end(), value) == c.end()) return bad("not a shape that fits this grid");
    }
    int* f[] = {&t.kxb, &t.xr, &t.zl_c2v, &t.zl_curl};
    *f[k] = value;
  }
  if (t.inc_rpt == 2 && t.inc_cb == 4) return bad("two rows per thread take 2 or 3 columns per batch");
  if (!cuda_ok(h, cudaSetDevice(h->device), "cudaSetDevice") ||
      !cuda_ok(h, cudaStreamSynchronize(h->stream), "cudaStreamSynchronize"))
    return CHF_E_CUDA;
  t.manual = true;
  h->tune = t;
  // the captured step graphs hold the old shapes
  for (auto& g : h->graphs) cudaGraphExecDestroy(g.exec);
  h->graphs.clear();
  return CHF_OK;
}

int chf_tuning(const chf_handle* h, char* buf, int len) {
  if (!h || !buf || len <= 0) return CHF_E_INVALID;
  std::string s;
  {
    std::lock_guard<std::mutex> lock(g_mu);
    auto it = g_cache.find(key_of(h));
    s = h->tune.manual ? describe(h, 0.0, 0.0) + " (set by chf_set_launch_shape)"
        : (h->tune.tuned || it != g_cache.end()) && it != g_cache.end()
            ? it->second.report
            : describe(h, 0.0, 0.0) + " (launch rules; not tuned)";
  }
  std::snprintf(buf, (size_t)len, "%s", s.c_str());
  return CHF_OK;
}

}  // extern "C"
