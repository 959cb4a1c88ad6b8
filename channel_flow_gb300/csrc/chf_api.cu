// chf_api.cu -- the C ABI declared in include/chflow.h.
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "chf_internal.h"

namespace chf {

bool cuda_ok(Handle* h, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return true;
  if (h) h->err = std::string(what) + ": " + cudaGetErrorString(e);
  return false;
}

FftPlan make_plan(int L) {
  FftPlan p{};
  p.L = L;
  int m = L, Ns = 1;
  while (m > 1) {
    int r = (m % 4 == 0) ? 4 : (m % 2 == 0) ? 2 : (m % 3 == 0) ? 3 : 5;
    p.R[p.nst] = r;
    p.Ns[p.nst] = Ns;
    ++p.nst;
    Ns *= r;
    m /= r;
  }
  fft_plan_divisors(p);
  return p;
}

// Plans of the two-buffer FFT stages (the x / y transforms, smem_fft_pp):
// the largest radices first (16 when allowed, then 8, 9, 4, 3, 5, 2), so
// that a line passes through shared memory as few times as possible; maxr
// bounds the radix (FP64 lines hold 8 complex values per thread at most)
FftPlan make_plan_pp(int L, int maxr) {
  FftPlan p{};
  p.L = L;
  int m = L, Ns = 1;
  while (m > 1) {
    int r = 2;
    for (int c : {16, 8, 9, 4, 3, 5, 2})
      if (c <= maxr && m % c == 0) {
        r = c;
        break;
      }
    p.R[p.nst] = r;
    p.Ns[p.nst] = Ns;
    ++p.nst;
    Ns *= r;
    m /= r;
  }
  fft_plan_divisors(p);
  return p;
}

static bool factors_235(int n) {
  if (n <= 0) return false;
  for (int p : {2, 3, 5})
    while (n % p == 0) n /= p;
  return n == 1;
}

int upload_stage_twiddles(Handle* h) {
  const bool f32 = mixed_front(h);
  struct Tab {
    void** dst;
    const FftPlan* p;
    bool f32;
  } tabs[] = {{&h->stw_py, &h->py, f32},
              {&h->stw_px, &h->px, f32},
              {(void**)&h->stw_py64, &h->py64, false},
              {(void**)&h->stw_px64, &h->px64, false}};
  for (const Tab& t : tabs) {
    if (!f32 && (t.dst == (void**)&h->stw_py64 || t.dst == (void**)&h->stw_px64)) continue;  // FP64 handle: py, px
    const int L = t.p->L;
    const size_t es = t.f32 ? sizeof(cf) : sizeof(cd);
    if (!*t.dst && !cuda_ok(h, cudaMalloc(t.dst, es * (size_t)L), "stage twiddles")) return CHF_E_NOMEM;
    const std::vector<cd> tw = twiddles(L);
    std::vector<unsigned char> host(es * (size_t)L, 0);
    if (t.f32)
      fft_stage_twiddles<float>(*t.p, tw, reinterpret_cast<cf*>(host.data()));
    else
      fft_stage_twiddles<double>(*t.p, tw, reinterpret_cast<cd*>(host.data()));
    if (!cuda_ok(h, cudaMemcpy(*t.dst, host.data(), host.size(), cudaMemcpyHostToDevice), "stage twiddles"))
      return CHF_E_CUDA;
  }
  return CHF_OK;
}

std::vector<cd> twiddles(int L) {
  std::vector<cd> t(L);
  const double twopi = 8.0 * std::atan(1.0);
  for (int k = 0; k < L; ++k) {
    double a = -twopi * (double)k / (double)L;
    t[k] = cd{std::cos(a), std::sin(a)};
  }
  return t;
}

const char* const kKernelNames[K_COUNT] = {
    "k_zc2v", "k_yinv", "k_xprod", "k_yfwd", "k_zcurl", "k_solve", "k_diag",
    "k_tc_split_z1", "k_tc_gemm_z1", "k_tc_split_z2", "k_tc_gemm_z2", "k_curl", "k_tc_gemm_gl",
    "k_meanfix", "k_inc_solve", "k_inc_recover", "k_solve_mean"};

static cudaEvent_t take_event(Handle* h) {
  if (!h->event_pool.empty()) {
    cudaEvent_t e = h->event_pool.back();
    h->event_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

void prof_begin(Handle* h, int kid, cudaEvent_t* a) {
  (void)kid;
  *a = nullptr;
  if (!h->profiling) return;
  *a = take_event(h);
  cudaEventRecord(*a, h->stream);
}

void prof_end(Handle* h, int kid, cudaEvent_t a) {
  if (!h->profiling || !a) return;
  cudaEvent_t b = take_event(h);
  cudaEventRecord(b, h->stream);
  h->pending.push_back({kid, a, b});
}

static void prof_collect(Handle* h) {
  if (h->pending.empty()) return;
  cudaStreamSynchronize(h->stream);
  for (auto& p : h->pending) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, p.a, p.b);
    h->prof[p.kid].launches += 1;
    h->prof[p.kid].ms += ms;
    h->event_pool.push_back(p.a);
    h->event_pool.push_back(p.b);
  }
  h->pending.clear();
}

}  // namespace chf

using namespace chf;

struct chf_handle : public Handle {};

static thread_local std::string g_create_error;

static std::string validate(const chf_config* c) {
  if (!c) return "config is NULL";
  if (c->nnx < 4 || c->nnx % 4) return "nnx must be a positive multiple of 4";
  if (c->nny < 4 || c->nny % 4) return "nny must be a positive multiple of 4";
  if (c->nnz < 4 || c->nnz % 2) return "nnz must be even and >= 4";
  // the solve kernels hold a column of nnz + 1 <= 256 values in one warp
  // (k_solve.cu: WD_EMAX) and two chunks of 2 nnz-point lines in a CTA
  if (c->nnz > 254) return "nnz must be <= 254";
  if (!(c->aphi > 0) || !(c->beta > 0)) return "aphi and beta must be positive";
  if (!(c->dt > 0) || !(c->re > 0)) return "dt and re must be positive";
  if (!std::isfinite(c->re_p)) return "re_p must be finite";
  if (c->precision != CHF_FP64 && c->precision != CHF_MIXED && c->precision != CHF_MIXED_F64SOLVE)
    return "precision must be CHF_FP64, CHF_MIXED or CHF_MIXED_F64SOLVE";
  int mz = c->zpad == 0 ? 2 * c->nnz : c->zpad;
  if (2 * mz <= 3 * c->nnz) return "zpad must satisfy 2*zpad > 3*nnz (exact dealiasing)";
  if (!factors_235(3 * c->nnx / 2) || !factors_235(3 * c->nny / 2) || !factors_235(2 * mz) ||
      !factors_235(2 * c->nnz))
    return "transform lengths 3nnx/2, 3nny/2, 2nnz and 2zpad must factor into 2, 3 and 5";
  return "";
}

static void release(chf_handle* h) {
  if (!h) return;
  if (h->device >= 0) cudaSetDevice(h->device);
  for (auto& p : h->f) cudaFree(p);
  for (auto& p : h->mean) cudaFree(p);
  void* ptrs[] = {h->iapha, h->ibeta, h->t0, h->t2, h->t4, h->k2vals, h->xinv, h->xmean,
                  h->group_start, h->group_modes, h->tw_py, h->tw_px, h->tw_z2, h->tw_zm,
                  h->twf_py, h->twf_px, h->stw_py, h->stw_px, h->stw_py64, h->stw_px64, h->incm, h->incx, h->incr_exp, h->inc_items, h->phi, h->flow, h->stats_buf, h->pres_buf, h->phys_buf, h->tw_pxu, h->tw_pyu, h->group_re, h->ubphi_dev, h->wz, h->wy, h->scratch, h->dev_status, h->az1, h->az2,
                  h->agl, h->bimg, h->wz32, h->wy32, h->lc64, h->aexp1, h->aexp2, h->aexp3, h->bexp, h->z2_tail, h->gl_tail};
  for (void* p : ptrs) cudaFree(p);
  for (auto& p : h->pending) {
    cudaEventDestroy(p.a);
    cudaEventDestroy(p.b);
  }
  for (auto e : h->event_pool) cudaEventDestroy(e);
  for (auto& g : h->graphs) cudaGraphExecDestroy(g.exec);
  for (cudaEvent_t e : {h->ev_ready, h->ev_inputs, h->ev_hist_in, h->ev_nonlinear, h->ev_vg, h->ev_done})
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : h->ev_field)
    if (e) cudaEventDestroy(e);
  if (h->copy_in) cudaStreamDestroy(h->copy_in);
  if (h->copy_out) cudaStreamDestroy(h->copy_out);
  if (h->ev_fork) cudaEventDestroy(h->ev_fork);
  if (h->ev_join) cudaEventDestroy(h->ev_join);
  if (h->side_stream) cudaStreamDestroy(h->side_stream);
  if (h->own_stream) cudaStreamDestroy(h->own_stream);
}

namespace chf {
bool mixed_front(const Handle* h) { return h->cfg.precision != CHF_FP64; }
bool increment_solve(const Handle* h) { return h->cfg.precision == CHF_MIXED; }

int launch_nonlinear(Handle* h, const cudaEvent_t* field_ready) {
  return mixed_front(h) ? launch_nonlinear_mixed(h, field_ready) : launch_nonlinear_fp64(h);
}

int launch_solve(Handle* h) { return increment_solve(h) ? launch_solve_mixed(h) : launch_solve_fp64(h); }

int step_once(Handle* h) {
  int rc = launch_nonlinear(h, nullptr);
  if (rc != CHF_OK) return rc;
  return launch_solve(h);
}
}  // namespace chf

// The graph of a pair of steps for the current history arrangement, captured
// on first use; *out = nullptr when steps must be launched directly: with
// per-kernel profiling on (its events are host-side bookkeeping), when the
// stream is already being captured by the caller (the direct launches then
// become part of the caller's graph), or after a capture failed.
static int pair_graph(chf_handle* h, cudaGraphExec_t* out) {
  *out = nullptr;
  if (h->graphs_off || h->profiling) return CHF_OK;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (!cuda_ok(h, cudaStreamIsCapturing(h->stream, &cs), "cudaStreamIsCapturing")) return CHF_E_CUDA;
  if (cs != cudaStreamCaptureStatusNone) return CHF_OK;
  for (auto& g : h->graphs)
    if (std::memcmp(g.f, h->f, sizeof g.f) == 0) {
      *out = g.exec;
      return CHF_OK;
    }
  Handle::StepGraph sg{};
  std::memcpy(sg.f, h->f, sizeof sg.f);
  if (cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeRelaxed) != cudaSuccess) {
    cudaGetLastError();
    h->graphs_off = true;
    return CHF_OK;
  }
  int rc = step_once(h);
  if (rc == CHF_OK) rc = step_once(h);
  cudaGraph_t graph = nullptr;
  cudaError_t e = cudaStreamEndCapture(h->stream, &graph);
  bool ok = rc == CHF_OK && e == cudaSuccess && graph &&
            cudaGraphInstantiate(&sg.exec, graph, 0) == cudaSuccess;
  if (graph) cudaGraphDestroy(graph);
  // the captured launches did not run; put the arrangement back either way
  std::memcpy(h->f, sg.f, sizeof sg.f);
  if (!ok) {
    cudaGetLastError();
    h->err.clear();
    h->graphs_off = true;
    return CHF_OK;
  }
  h->graphs.push_back(sg);
  *out = sg.exec;
  return CHF_OK;
}

extern "C" {

int chf_create(const chf_config* cfg, chf_handle** out) {
  if (!out) {
    g_create_error = "out is NULL";
    return CHF_E_INVALID;
  }
  *out = nullptr;
  std::string why = validate(cfg);
  if (!why.empty()) {
    g_create_error = why;
    return CHF_E_INVALID;
  }
  chf_handle* h = new (std::nothrow) chf_handle();
  if (!h) {
    g_create_error = "host allocation failed";
    return CHF_E_NOMEM;
  }
  h->cfg = *cfg;
  h->device = cfg->device;
  Dims& d = h->d;
  d.nnx = cfg->nnx;
  d.nny = cfg->nny;
  d.nnz = cfg->nnz;
  d.N = cfg->nnz;
  d.NZ = cfg->nnz + 1;
  d.KX = cfg->nnx / 2;
  d.KY = cfg->nny;
  d.NYQ = cfg->nny / 2;
  d.PX = 3 * cfg->nnx / 2;
  d.PY = 3 * cfg->nny / 2;
  d.MZ = cfg->zpad == 0 ? 2 * cfg->nnz : cfg->zpad;
  d.MP = d.MZ + 1;
  d.nch = 1;
  d.chm = d.modes();
  auto fail = [&](int code) {
    g_create_error = h->err.empty() ? "chf_create failed" : h->err;
    release(h);
    delete h;
    return code;
  };
  int ndev = 0;
  if (!cuda_ok(h, cudaGetDeviceCount(&ndev), "cudaGetDeviceCount")) return fail(CHF_E_CUDA);
  if (cfg->device < 0 || cfg->device >= ndev) {
    h->err = "device ordinal out of range";
    h->device = -1;
    return fail(CHF_E_INVALID);
  }
  if (!cuda_ok(h, cudaSetDevice(cfg->device), "cudaSetDevice") ||
      !cuda_ok(h, cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking), "cudaStreamCreate"))
    return fail(CHF_E_CUDA);
  h->stream = h->own_stream;
  if (!cuda_ok(h, cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, cfg->device),
               "cudaDeviceGetAttribute"))
    return fail(CHF_E_CUDA);
  h->prof.resize(K_COUNT);
  for (int k = 0; k < K_COUNT; ++k) h->prof[k] = {kKernelNames[k], 0, 0.0};
  const size_t fe = d.field_elems();
  for (int i = 0; i < F_COUNT; ++i) {
    if (!cuda_ok(h, cudaMalloc((void**)&h->f[i], sizeof(cd) * fe), "state alloc")) return fail(CHF_E_NOMEM);
    cudaMemsetAsync(h->f[i], 0, sizeof(cd) * fe, h->stream);
  }
  for (int i = 0; i < M_COUNT; ++i) {
    if (!cuda_ok(h, cudaMalloc((void**)&h->mean[i], sizeof(double) * 2 * d.NZ), "mean alloc"))
      return fail(CHF_E_NOMEM);
    cudaMemsetAsync(h->mean[i], 0, sizeof(double) * 2 * d.NZ, h->stream);
  }
  if (cfg->precision == CHF_FP64) {
    const size_t wz_elems = (size_t)6 * d.MP * d.modes();
    const size_t wy_elems = (size_t)6 * d.MP * d.PY * d.KX;
    if (!cuda_ok(h, cudaMalloc((void**)&h->wz, sizeof(cd) * wz_elems), "work alloc") ||
        !cuda_ok(h, cudaMalloc((void**)&h->wy, sizeof(cd) * wy_elems), "work alloc"))
      return fail(CHF_E_NOMEM);
  }
  if (!cuda_ok(h, cudaMalloc((void**)&h->dev_status, sizeof(int)), "status alloc") ||
      !cuda_ok(h, cudaMemsetAsync(h->dev_status, 0, sizeof(int), h->stream), "status init"))
    return fail(CHF_E_NOMEM);
  h->scratch_bytes = 4096;
  if (!cuda_ok(h, cudaMalloc(&h->scratch, h->scratch_bytes), "scratch alloc")) return fail(CHF_E_NOMEM);
  // radix 16 is built for FP32 lines only
  h->py64 = make_plan_pp(d.PY, 8);
  h->px64 = make_plan_pp(d.PX, 8);
  h->py = cfg->precision == CHF_FP64 ? h->py64 : make_plan_pp(d.PY, 16);
  h->px = cfg->precision == CHF_FP64 ? h->px64 : make_plan_pp(d.PX, 16);
  h->pz2 = make_plan(2 * d.N);
  h->pzm = make_plan(2 * d.MZ);
  struct {
    cd** dst;
    int L;
  } tws[] = {{&h->tw_py, d.PY}, {&h->tw_px, d.PX}, {&h->tw_z2, 2 * d.N}, {&h->tw_zm, 2 * d.MZ}};
  for (auto& t : tws) {
    std::vector<cd> v = twiddles(t.L);
    if (!cuda_ok(h, cudaMalloc((void**)t.dst, sizeof(cd) * v.size()), "twiddle alloc") ||
        !cuda_ok(h, cudaMemcpy(*t.dst, v.data(), sizeof(cd) * v.size(), cudaMemcpyHostToDevice),
                 "twiddle upload"))
      return fail(CHF_E_CUDA);
  }
  apply_cached_tuning(h);  // a measured choice for this grid earlier in the process
  if (upload_stage_twiddles(h) != CHF_OK) return fail(CHF_E_CUDA);
  int rc = setup_solver(h);
  if (rc != CHF_OK) return fail(rc);
  if (mixed_front(h)) {
    rc = setup_mixed(h);
    if (rc == CHF_OK && increment_solve(h)) rc = setup_solver_mixed(h);
    if (rc != CHF_OK) return fail(rc);
    if (!cuda_ok(h, cudaStreamCreateWithFlags(&h->side_stream, cudaStreamNonBlocking), "cudaStreamCreate") ||
        !cuda_ok(h, cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming), "cudaEventCreate") ||
        !cuda_ok(h, cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming), "cudaEventCreate"))
      return fail(CHF_E_CUDA);
  }
  if (!cuda_ok(h, cudaStreamCreateWithFlags(&h->copy_in, cudaStreamNonBlocking), "cudaStreamCreate") ||
      !cuda_ok(h, cudaStreamCreateWithFlags(&h->copy_out, cudaStreamNonBlocking), "cudaStreamCreate"))
    return fail(CHF_E_CUDA);
  for (cudaEvent_t* e : {&h->ev_ready, &h->ev_inputs, &h->ev_hist_in, &h->ev_nonlinear, &h->ev_vg, &h->ev_done})
    if (!cuda_ok(h, cudaEventCreateWithFlags(e, cudaEventDisableTiming), "cudaEventCreate")) return fail(CHF_E_CUDA);
  for (cudaEvent_t& e : h->ev_field)
    if (!cuda_ok(h, cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "cudaEventCreate")) return fail(CHF_E_CUDA);
  // FP64: k_zc2v, k_yinv, k_xprod, k_yfwd, k_zcurl, k_solve; mixed front:
  // two splits, three GEMMs, k_yinv_w, k_xprod_w, k_yfwd_w, k_curl,
  // k_meanfix; then k_solve, or k_inc_solve + k_inc_recover + the (0,0) mode
  h->kernels_per_step = !mixed_front(h) ? 6 : increment_solve(h) ? 13 : 11;
  if (!cuda_ok(h, cudaStreamSynchronize(h->stream), "create sync")) return fail(CHF_E_CUDA);
  *out = h;
  return CHF_OK;
}

int chf_destroy(chf_handle* h) {
  if (!h) return CHF_E_INVALID;
  release(h);
  delete h;
  return CHF_OK;
}

const char* chf_last_error(const chf_handle* h) {
  if (!h) return g_create_error.c_str();
  return h->err.c_str();
}

static int transfer(chf_handle* h, bool up, double* const* fields, double* const* means) {
  if (!h) return CHF_E_INVALID;
  if (!cuda_ok(h, cudaSetDevice(h->device), "cudaSetDevice")) return CHF_E_CUDA;
  const size_t fb = sizeof(cd) * h->d.field_elems();
  const size_t mb = sizeof(double) * 2 * h->d.NZ;
  for (int i = 0; i < F_COUNT; ++i) {
    if (!fields[i]) continue;
    cudaError_t e = up ? cudaMemcpyAsync(h->f[i], fields[i], fb, cudaMemcpyHostToDevice, h->stream)
                       : cudaMemcpyAsync(fields[i], h->f[i], fb, cudaMemcpyDeviceToHost, h->stream);
    if (!cuda_ok(h, e, up ? "upload" : "download")) return CHF_E_CUDA;
  }
  for (int i = 0; i < M_COUNT; ++i) {
    if (!means[i]) continue;
    cudaError_t e = up ? cudaMemcpyAsync(h->mean[i], means[i], mb, cudaMemcpyHostToDevice, h->stream)
                       : cudaMemcpyAsync(means[i], h->mean[i], mb, cudaMemcpyDeviceToHost, h->stream);
    if (!cuda_ok(h, e, up ? "upload" : "download")) return CHF_E_CUDA;
  }
  if (!cuda_ok(h, cudaStreamSynchronize(h->stream), up ? "upload sync" : "download sync"))
    return CHF_E_CUDA;
  if (up) h->uploaded = true;
  return CHF_OK;
}

int chf_upload_state(chf_handle* h, const double* vnp1, const double* omegaynp1, const double* unp1,
                     const double* wnp1, const double* omegaxnp1, const double* omegaznp1,
                     const double* rhsvn, const double* rhsomegayn, const double* clamb1n,
                     const double* clamb1nm1, const double* clamb3n, const double* clamb3nm1,
                     const double* au0, const double* w0) {
  double* f[F_COUNT] = {(double*)vnp1, (double*)omegaynp1, (double*)unp1, (double*)wnp1,
                        (double*)omegaxnp1, (double*)omegaznp1, (double*)rhsvn, (double*)rhsomegayn};
  double* m[M_COUNT] = {(double*)clamb1n, (double*)clamb1nm1, (double*)clamb3n,
                        (double*)clamb3nm1, (double*)au0, (double*)w0};
  return transfer(h, true, f, m);
}

int chf_download_state(chf_handle* h, double* vnp1, double* omegaynp1, double* unp1, double* wnp1,
                       double* omegaxnp1, double* omegaznp1, double* rhsvn, double* rhsomegayn,
                       double* clamb1n, double* clamb1nm1, double* clamb3n, double* clamb3nm1,
                       double* au0, double* w0) {
  double* f[F_COUNT] = {vnp1, omegaynp1, unp1, wnp1, omegaxnp1, omegaznp1, rhsvn, rhsomegayn};
  double* m[M_COUNT] = {clamb1n, clamb1nm1, clamb3n, clamb3nm1, au0, w0};
  return transfer(h, false, f, m);
}

int chf_getnonlinear(chf_handle* h) {
  if (!h) return CHF_E_INVALID;
  if (!h->uploaded) {
    h->err = "chf_getnonlinear before chf_upload_state";
    return CHF_E_STATE;
  }
  if (!cuda_ok(h, cudaSetDevice(h->device), "cudaSetDevice")) return CHF_E_CUDA;
  return launch_nonlinear(h, nullptr);
}

int chf_solve(chf_handle* h) {
  if (!h) return CHF_E_INVALID;
  if (!h->uploaded) {
    h->err = "chf_solve before chf_upload_state";
    return CHF_E_STATE;
  }
  if (!cuda_ok(h, cudaSetDevice(h->device), "cudaSetDevice")) return CHF_E_CUDA;
  return launch_solve(h);
}

int chf_step(chf_handle* h, int nsteps) {
  if (!h) return CHF_E_INVALID;
  if (nsteps < 0) {
    h->err = "nsteps must be >= 0";
    return CHF_E_INVALID;
  }
  if (!h->uploaded) {
    h->err = "chf_step before chf_upload_state";
    return CHF_E_STATE;
  }
  if (!cuda_ok(h, cudaSetDevice(h->device), "cudaSetDevice")) return CHF_E_CUDA;
  int s = 0;
  if (nsteps - s >= 2) {
    cudaGraphExec_t g = nullptr;
    int rc = pair_graph(h, &g);
    if (rc != CHF_OK) return rc;
    if (g)
      for (; s + 2 <= nsteps; s += 2)
        if (!cuda_ok(h, cudaGraphLaunch(g, h->stream), "cudaGraphLaunch")) return CHF_E_CUDA;
  }
  for (; s < nsteps; ++s) {
    int rc = step_once(h);
    if (rc != CHF_OK) return rc;
  }
  return CHF_OK;
}

static int check_status(chf_handle* h);

// One blocking call that advances host-resident module arrays in place:
// upload, nsteps steps, download, with the copies overlapped with the steps.
//   copy_in : the mean arrays and the six nonlinear inputs, one event per
//             field (the mixed path's first stages run field by field as
//             they land), then the N^{n-1} histories (only the solve reads
//             them: they land during the nonlinear term);
//   copy_out: after the last nonlinear term, the new histories (during the
//             solve); after the mixed path's increment solve, v and omega_y
//             (during the recovery); at the end u, w, omega_x, omega_z and the
//             mean arrays.
// Every module array crosses the link once each way, as with
// chf_upload_state + chf_step + chf_download_state, whose results this
// reproduces bit for bit.
static bool ev_rec(chf_handle* h, cudaEvent_t e, cudaStream_t s) {
  return cuda_ok(h, cudaEventRecord(e, s), "cudaEventRecord");
}
static bool ev_wait(chf_handle* h, cudaStream_t s, cudaEvent_t e) {
  return cuda_ok(h, cudaStreamWaitEvent(s, e, 0), "cudaStreamWaitEvent");
}

int chf_step_host(chf_handle* h, int nsteps, double* vnp1, double* omegaynp1, double* unp1, double* wnp1,
                  double* omegaxnp1, double* omegaznp1, double* rhsvn, double* rhsomegayn, double* clamb1n,
                  double* clamb1nm1, double* clamb3n, double* clamb3nm1, double* au0, double* w0) {
  if (!h) return CHF_E_INVALID;
  double* fh[F_COUNT] = {vnp1, omegaynp1, unp1, wnp1, omegaxnp1, omegaznp1, rhsvn, rhsomegayn};
  double* mh[M_COUNT] = {clamb1n, clamb1nm1, clamb3n, clamb3nm1, au0, w0};
  for (double* p : fh)
    if (!p) {
      h->err = "chf_step_host: every module array is required";
      return CHF_E_INVALID;
    }
  for (double* p : mh)
    if (!p) {
      h->err = "chf_step_host: every module array is required";
      return CHF_E_INVALID;
    }
  if (nsteps < 1) {
    h->err = "nsteps must be >= 1";
    return CHF_E_INVALID;
  }
  if (!cuda_ok(h, cudaSetDevice(h->device), "cudaSetDevice")) return CHF_E_CUDA;
  // mixed: the nonlinear front follows the fields as they land; inc: the
  // increment solve finishes v and omega_y before the recovery
  const bool mixed = mixed_front(h), inc = increment_solve(h);
  const size_t fb = sizeof(cd) * h->d.field_elems(), mb = sizeof(double) * 2 * h->d.NZ;
  cudaStream_t S = h->stream, ci = h->copy_in, co = h->copy_out;
  auto up = [&](void* dst, const void* src, size_t n) {
    return cuda_ok(h, cudaMemcpyAsync(dst, src, n, cudaMemcpyHostToDevice, ci), "upload");
  };
  auto down = [&](void* dst, const void* src, size_t n) {
    return cuda_ok(h, cudaMemcpyAsync(dst, src, n, cudaMemcpyDeviceToHost, co), "download");
  };
  // the device buffers may still be in use by earlier work on the handle's stream
  if (!ev_rec(h, h->ev_ready, S) || !ev_wait(h, ci, h->ev_ready) || !ev_wait(h, co, h->ev_ready)) return CHF_E_CUDA;
  for (int i = 0; i < M_COUNT; ++i)
    if (!up(h->mean[i], mh[i], mb)) return CHF_E_CUDA;
  {
    const int order[6] = {F_U, F_V, F_W, F_OX, F_OY, F_OZ};
    for (int k = 0; k < 6; ++k)
      if (!up(h->f[order[k]], fh[order[k]], fb) || !ev_rec(h, h->ev_field[k], ci)) return CHF_E_CUDA;
  }
  if (!ev_rec(h, h->ev_inputs, ci)) return CHF_E_CUDA;
  if (!up(h->f[F_RV], fh[F_RV], fb) || !up(h->f[F_RG], fh[F_RG], fb) || !ev_rec(h, h->ev_hist_in, ci))
    return CHF_E_CUDA;
  h->uploaded = true;
  // the mixed path's first stages follow the fields as they land
  if (!mixed && !ev_wait(h, S, h->ev_inputs)) return CHF_E_CUDA;
  if (mixed) {  // the mean arrays precede the fields on the copy stream
    if (!ev_wait(h, S, h->ev_field[0])) return CHF_E_CUDA;
  }
  for (int s = 0; s < nsteps; ++s) {
    const bool last = s == nsteps - 1;
    int rc = launch_nonlinear(h, (mixed && s == 0) ? h->ev_field : nullptr);
    if (rc != CHF_OK) return rc;
    if (s == 0 && !ev_wait(h, S, h->ev_hist_in)) return CHF_E_CUDA;
    if (last) {  // the new histories are final; the host buffers were read by the upload
      if (!ev_rec(h, h->ev_nonlinear, S) || !ev_wait(h, co, h->ev_nonlinear) || !ev_wait(h, co, h->ev_hist_in) ||
          !down(fh[F_RV], h->f[F_RV], fb) || !down(fh[F_RG], h->f[F_RG], fb))
        return CHF_E_CUDA;
    }
    h->after_inc = (last && inc) ? h->ev_vg : nullptr;
    rc = launch_solve(h);
    h->after_inc = nullptr;
    if (rc != CHF_OK) return rc;
    if (last && inc &&
        (!ev_wait(h, co, h->ev_vg) || !down(fh[F_V], h->f[F_V], fb) || !down(fh[F_OY], h->f[F_OY], fb)))
      return CHF_E_CUDA;
  }
  if (!ev_rec(h, h->ev_done, S) || !ev_wait(h, co, h->ev_done)) return CHF_E_CUDA;
  for (int i : {F_U, F_W, F_OX, F_OZ})
    if (!down(fh[i], h->f[i], fb)) return CHF_E_CUDA;
  if (!inc)
    for (int i : {F_V, F_OY})
      if (!down(fh[i], h->f[i], fb)) return CHF_E_CUDA;
  for (int i = 0; i < M_COUNT; ++i)
    if (!down(mh[i], h->mean[i], mb)) return CHF_E_CUDA;
  if (!cuda_ok(h, cudaStreamSynchronize(co), "cudaStreamSynchronize")) return CHF_E_CUDA;
  return check_status(h);
}

// Device-side error word: the tensor-core GEMM records a bounded-wait
// timeout there instead of hanging (11: a free ring stage, 12: a free
// accumulator set, 13: operands, 14: the final MMA drain, 15: accumulators
// ready, 16: copies landing at exit, 17: the resident A tile at exit).
static int check_status(chf_handle* h) {
  int st = 0;
  if (!cuda_ok(h, cudaMemcpyAsync(&st, h->dev_status, sizeof(int), cudaMemcpyDeviceToHost, h->stream),
               "status read") ||
      !cuda_ok(h, cudaStreamSynchronize(h->stream), "cudaStreamSynchronize"))
    return CHF_E_CUDA;
  if (st != 0) {
    h->err = "tensor-core pipeline wait timed out (code " + std::to_string(st) + ")";
    // reported once: the word is cleared so the handle stays usable (the
    // state of the failed step is not; upload or read a restart file)
    cudaMemsetAsync(h->dev_status, 0, sizeof(int), h->stream);
    cudaStreamSynchronize(h->stream);
    return CHF_E_CUDA;
  }
  return CHF_OK;
}

int chf_test_wait_timeout(chf_handle* h, int wait_us) {
  if (!h) return CHF_E_INVALID;
  if (!mixed_front(h)) {
    h->err = "chf_test_wait_timeout: only the mixed precisions run the tensor-core pipeline";
    return CHF_E_INVALID;
  }
  if (wait_us < 1 || wait_us > 1000000) {
    h->err = "chf_test_wait_timeout: wait_us must be 1 .. 1000000";
    return CHF_E_INVALID;
  }
  h->test_skip = 1;
  h->test_wait_ns = 1000L * wait_us;
  return CHF_OK;
}

int chf_synchronize(chf_handle* h) {
  if (!h) return CHF_E_INVALID;
  if (!cuda_ok(h, cudaSetDevice(h->device), "cudaSetDevice") ||
      !cuda_ok(h, cudaStreamSynchronize(h->stream), "cudaStreamSynchronize"))
    return CHF_E_CUDA;
  return check_status(h);
}

int chf_diagnostics(chf_handle* h, chf_diag* out) {
  if (!h || !out) return CHF_E_INVALID;
  if (!cuda_ok(h, cudaSetDevice(h->device), "cudaSetDevice")) return CHF_E_CUDA;
  int rc = launch_diagnostics(h, out);
  if (rc == CHF_E_NUMERIC) h->err = "non-finite values in the state";
  if (rc == CHF_OK) rc = check_status(h);
  return rc;
}

int chf_kernels_per_step(const chf_handle* h) { return h ? h->kernels_per_step : 0; }

int chf_set_flow_rate(chf_handle* h, double bulk_velocity) {
  if (!h) return CHF_E_INVALID;
  if (!(bulk_velocity >= 0.0) || !std::isfinite(bulk_velocity)) {
    h->err = "bulk velocity must be finite and >= 0 (0 switches the control off)";
    return CHF_E_INVALID;
  }
  if (!cuda_ok(h, cudaSetDevice(h->device), "cudaSetDevice") ||
      !cuda_ok(h, cudaMemcpyAsync(h->flow, &bulk_velocity, sizeof(double), cudaMemcpyHostToDevice, h->stream),
               "flow rate") ||
      !cuda_ok(h, cudaStreamSynchronize(h->stream), "flow rate"))
    return CHF_E_CUDA;
  return CHF_OK;
}

int chf_get_flow_rate(chf_handle* h, double* target, double* bulk_velocity, double* dpdx_correction) {
  if (!h) return CHF_E_INVALID;
  double w[4];
  if (!cuda_ok(h, cudaSetDevice(h->device), "cudaSetDevice") ||
      !cuda_ok(h, cudaMemcpyAsync(w, h->flow, sizeof(w), cudaMemcpyDeviceToHost, h->stream), "flow rate") ||
      !cuda_ok(h, cudaStreamSynchronize(h->stream), "flow rate"))
    return CHF_E_CUDA;
  if (target) *target = w[0];
  if (bulk_velocity) *bulk_velocity = w[3];
  if (dpdx_correction) *dpdx_correction = w[1];
  return CHF_OK;
}

int chf_set_stream(chf_handle* h, void* stream) {
  if (!h) return CHF_E_INVALID;
  if (!cuda_ok(h, cudaSetDevice(h->device), "cudaSetDevice")) return CHF_E_CUDA;
  // order the switch: work already queued on the old stream completes first
  if (!cuda_ok(h, cudaStreamSynchronize(h->stream), "cudaStreamSynchronize")) return CHF_E_CUDA;
  h->stream = stream ? (cudaStream_t)stream : h->own_stream;
  return CHF_OK;
}

int chf_profile_enable(chf_handle* h, int on) {
  if (!h) return CHF_E_INVALID;
  prof_collect(h);
  h->profiling = on != 0;
  return CHF_OK;
}

int chf_profile_reset(chf_handle* h) {
  if (!h) return CHF_E_INVALID;
  prof_collect(h);
  for (auto& r : h->prof) {
    r.launches = 0;
    r.ms = 0.0;
  }
  return CHF_OK;
}

int chf_profile_read(chf_handle* h, int idx, const char** name, int* launches, double* total_ms) {
  if (!h || idx < 0 || idx >= (int)h->prof.size()) return CHF_E_INVALID;
  prof_collect(h);
  if (name) *name = h->prof[idx].name;
  if (launches) *launches = h->prof[idx].launches;
  if (total_ms) *total_ms = h->prof[idx].ms;
  return CHF_OK;
}

int chf_device_field(chf_handle* h, int which, void** dptr) {
  if (!h || !dptr || which < 0 || which >= F_COUNT) return CHF_E_INVALID;
  *dptr = h->f[which];
  return CHF_OK;
}

}  // extern "C"
